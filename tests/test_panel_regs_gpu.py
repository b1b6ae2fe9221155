"""Leaf-panel kernels with the rows in registers (ELGB_OPT_PANEL_REGS = 2:
one thread-block cluster, 512 threads x 2 rows per CTA, panels of up to
16384 rows; taller ones keep the shared-memory kernels) against the
shared-memory kernels: the same lu::Panel steps
(src/lapack_like/factor/LU/Panel.hpp:15-59) in the same arithmetic order,
so pivots and factors must agree bit for bit, including ties and singular
columns; and P A = L U to FP32 accuracy."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _lu(ctx, A0, regs, nb=0, kind=2):
    A = A0.clone()  # keeps the column-major strides
    assert A.stride(0) == 1
    ctx.set_option("panel_regs", regs)
    try:
        piv = ctx.lu_mixed(A, gemm_kind=kind, nb=nb)
        ctx.check()
    finally:
        ctx.set_option("panel_regs", 2)
    return A, piv


def _matrix(m, n, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randn(n, m, device="cuda", generator=g).t()  # column-major m x n


@pytest.mark.parametrize("m,n,nb", [(300, 300, 0), (1000, 700, 0), (2100, 2100, 0),
                                    (5000, 1200, 0), (8192, 8192, 0), (16384, 640, 0),
                                    (4100, 3000, 1024), (6000, 4096, 768)])
def test_register_cluster_panels_match_shared_memory_panels(ctx, m, n, nb):
    A0 = _matrix(m, n, m + n)
    A1, p1 = _lu(ctx, A0, 0, nb=nb)
    A2, p2 = _lu(ctx, A0, 2, nb=nb)
    assert torch.equal(p1, p2)
    assert torch.equal(A1, A2)


@pytest.mark.parametrize("m,n", [(20000, 600), (32768, 544)])
def test_tall_panels_in_registers_factor_to_fp32_accuracy(ctx, m, n):
    """Panels taller than 16384 rows: 16-column leaves with four rows a
    thread in registers (ELGB_OPT_PANEL_REGS = 2) against the shared-memory
    kernels' 32-column leaves.  The recursion splits differently, so the
    rounding differs: both must give P A = L U to FP32 accuracy (checked in
    FP64 on the host) with the same first pivots."""
    A0 = _matrix(m, n, m + n)
    Ah = A0.double().cpu().numpy()
    piv0 = None
    for regs in (0, 2):
        A, piv = _lu(ctx, A0, regs)
        LU = A.double().cpu().numpy()
        k = min(m, n)
        L = np.tril(LU[:, :k], -1)
        L[:k, :k] += np.eye(k)
        U = np.triu(LU[:k, :])
        PA = O.permute_rows(piv.cpu().numpy(), Ah)
        assert np.linalg.norm(PA - L @ U) / np.linalg.norm(Ah) <= 4e-5, regs
        if piv0 is None:
            piv0 = piv.cpu().numpy()
        else:
            assert np.array_equal(piv.cpu().numpy()[:16], piv0[:16])


def test_register_cluster_panels_ties_and_zero_columns(ctx):
    """Exact ties (integer entries) pick the lowest row; a zero column is
    reported at its 1-based index and the factorization goes on."""
    m = n = 1536
    g = np.random.default_rng(3)
    A = g.integers(-3, 4, (m, n)).astype(np.float32)
    A[:, 77] = 0.0
    A0 = torch.from_numpy(A.T.copy()).cuda().t()
    outs = []
    for regs in (0, 2):
        Ac = A0.clone()
        ctx.set_option("panel_regs", regs)
        try:
            piv = ctx.lu_mixed(Ac, gemm_kind=2)
            info, err = ctx.status()
        finally:
            ctx.set_option("panel_regs", 2)
        outs.append((Ac, piv, info, err))
    assert outs[0][2] == outs[1][2] == 78 and outs[1][3] == 0
    assert torch.equal(outs[0][1], outs[1][1])
    assert torch.equal(outs[0][0], outs[1][0])


def test_register_cluster_panels_backward_error(ctx):
    """P A = L U to FP32 accuracy (exact-FP32 SIMT updates), checked in FP64
    on the host, with the first pivots equal to the oracle's FP32 El::LU
    (later ones may differ at near-ties that rounding breaks the other way)."""
    n = 2048
    A0 = _matrix(n, n, 11)
    A, piv = _lu(ctx, A0, 2, nb=256, kind=-1)
    Ah = A0.double().cpu().numpy()
    LU = A.double().cpu().numpy()
    L = np.tril(LU, -1) + np.eye(n)
    U = np.triu(LU)
    PA = O.permute_rows(piv.cpu().numpy(), Ah)
    assert np.linalg.norm(PA - L @ U) / np.linalg.norm(Ah) <= 4e-5
    _, pivr = O.lu(Ah.astype(np.float32), nb=256, dtype=np.float32)
    assert np.array_equal(piv.cpu().numpy()[:8], pivr[:8])


def test_product_form_trailing_solve_factors_to_fp32_accuracy(ctx):
    """ELGB_OPT_INV_TRSM = 1: the trailing update's U12 = L11^-1 A12 as
    A12 - N A12 with N = I - L11^-1 on the tensor cores.  Rounding differs
    from the substitution, so P A = L U is checked to FP32 accuracy and the
    first pivots against the default path."""
    n = 3000
    A0 = _matrix(n, n, 5)
    Ah = A0.double().cpu().numpy()
    A1, p1 = _lu(ctx, A0, 2)
    ctx.set_option("inv_trsm", 1)
    try:
        A2, p2 = _lu(ctx, A0, 2)
    finally:
        ctx.set_option("inv_trsm", 0)
    LU = A2.double().cpu().numpy()
    L = np.tril(LU, -1) + np.eye(n)
    U = np.triu(LU)
    PA = O.permute_rows(p2.cpu().numpy(), Ah)
    assert np.linalg.norm(PA - L @ U) / np.linalg.norm(Ah) <= 1e-4
    assert np.array_equal(p1.cpu().numpy()[:512], p2.cpu().numpy()[:512])
    assert not torch.equal(A1, A2)  # the option took the other path


def test_interchanges_on_the_swap_stream_change_nothing(ctx):
    """ELGB_OPT_SWAP_STREAM: the interchanges of the trailing update's second
    part run on a third stream beside the panel; each column sees the same
    row moves before the same update, so the factors are bit-identical."""
    n = 8192
    A0 = _matrix(n, n, 17)
    outs = []
    for v in (0, 1):
        ctx.set_option("swap_stream", v)
        try:
            outs.append(_lu(ctx, A0, 2))
        finally:
            ctx.set_option("swap_stream", 0)
    assert torch.equal(outs[0][1], outs[1][1])
    assert torch.equal(outs[0][0], outs[1][0])


@pytest.mark.parametrize("m,n", [(300, 300), (2100, 2100), (8192, 2048), (20000, 600)])
def test_push_exchange_matches_barrier_exchange(ctx, m, n):
    """ELGB_OPT_PANEL_PUSH: candidates pushed into every CTA on an mbarrier
    instead of read after a cluster barrier.  Only the exchange differs, so
    pivots and factors are bit-identical."""
    A0 = _matrix(m, n, 7 * m + n)
    outs = []
    for v in (0, 1):
        ctx.set_option("panel_push", v)
        try:
            outs.append(_lu(ctx, A0, 2))
        finally:
            ctx.set_option("panel_push", 1)
    assert torch.equal(outs[0][1], outs[1][1])
    assert torch.equal(outs[0][0], outs[1][0])
    info, err = ctx.status()
    assert err == 0


@pytest.mark.parametrize("m,n,nb", [(2100, 2100, 0), (8192, 1024, 0), (20000, 600, 0)])
def test_fused_node_update_matches_separate_launches(ctx, m, n, nb):
    """ELGB_OPT_PANEL_NODE = 1: the left leaf of a two-leaf recursion node
    applies the node's TRSM and update itself, with launch_trsm_block's and
    launch_gemm_simt's operations in their order, so the factors equal those
    of the separate launches bit for bit (and, up to 16384 rows, the
    shared-memory kernels')."""
    A0 = _matrix(m, n, 3 * m + n)
    A1, p1 = _lu(ctx, A0, 2, nb=nb)
    ctx.set_option("panel_node", 1)
    try:
        A2, p2 = _lu(ctx, A0, 2, nb=nb)
    finally:
        ctx.set_option("panel_node", 0)
    assert torch.equal(p1, p2)
    assert torch.equal(A1, A2)
    if m <= 16384:
        A0s, p0s = _lu(ctx, A0, 0, nb=nb)
        assert torch.equal(p0s, p2)
        assert torch.equal(A0s, A2)

"""ElGBResidualNoAlloc_d: the FP64 residual for callers that cannot allocate
device memory (a device heap budgeted up front or owned by another
allocator, or code that must not let cudaMalloc / cudaFree synchronize the
device).  Checked call after call against a host FP64 B - A X and against
the allocating entry point ElGBResidual_d, and checked to leave the device's
free memory unchanged (its scratch is a fixed device array).

This file is collected last on purpose (a failure here leaves every other
test already run)."""
import ctypes

import numpy as np
import pytest
import torch

from elemental_gb300 import _lib
from elemental_gb300 import device as D

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _noalloc(lib, A, X, B, R):
    n, q = B.shape
    s = torch.cuda.current_stream().cuda_stream
    return lib.ElGBResidualNoAlloc_d(n, q, _p(A), A.stride(1), _p(X), X.stride(1), _p(B),
                                     B.stride(1), _p(R), R.stride(1), ctypes.c_void_p(s))


def _inputs(n, q, seed):
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    A = D.colmajor(n, n)
    A.copy_(torch.randn(n, n, generator=g, device="cuda", dtype=torch.float64))
    B = D.colmajor(n, q)
    B.copy_(torch.randn(n, q, generator=g, device="cuda", dtype=torch.float64))
    return A, B, g


def _host_residual_bound(Ah, Xh, Bh):
    """Host FP64 residual and a bound on its rounding error: each entry is a
    length-n FP64 dot product, off by at most ~n eps sum_j |a_ij x_j| (taken
    with a margin of 4)."""
    Rh = Bh - Ah @ Xh
    bound = 4 * (Ah.shape[1] + 1) * EPS * (np.abs(Ah) @ np.abs(Xh) + np.abs(Bh))
    return Rh, bound


@pytest.mark.parametrize("n,q", [(3000, 5), (4097, 16), (1500, 20), (1, 1)])
def test_no_alloc_residual_matches_host_and_allocating_entry_point(ctx, n, q):
    lib = _lib.load()
    A, B, g = _inputs(n, q, n * 31 + q)
    Ah, Bh = A.cpu().numpy(), B.cpu().numpy()
    for call in range(2):  # two calls in a row share the static scratch
        X = D.colmajor(n, q)
        X.copy_(torch.randn(n, q, generator=g, device="cuda", dtype=torch.float64))
        R = D.colmajor(n, q)
        R.fill_(float("nan"))
        assert _noalloc(lib, A, X, B, R) == 0
        torch.cuda.synchronize()
        got = R.cpu().numpy()
        Rh, bound = _host_residual_bound(Ah, X.cpu().numpy(), Bh)
        assert np.all(np.abs(got - Rh) <= bound), (call, np.abs(got - Rh).max())
        # the allocating entry point gives the same result (same kernels,
        # same summation order)
        R_ref = ctx.residual(A, X, B).cpu().numpy()
        assert np.array_equal(got, R_ref), call


def test_no_alloc_residual_leaves_device_memory_unchanged(ctx):
    """Every call takes its scratch from the library's fixed array: with all
    tensors allocated up front and the kernels loaded by a first call, calls
    whose partial sums fill the array (n = 16384, 16 right-hand sides: 8 MiB)
    leave the device's free memory where it was."""
    lib = _lib.load()
    n, q = 16384, 16
    A, B, g = _inputs(n, q, 77)
    X = D.colmajor(n, q)
    X.copy_(torch.randn(n, q, generator=g, device="cuda", dtype=torch.float64))
    R = D.colmajor(n, q)
    small = [t[:256, :] for t in (B, X, R)]
    As = A[:256, :256]
    assert _noalloc(lib, As, *small) == 0  # loads the kernels
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        R.fill_(float("nan"))
        assert _noalloc(lib, A, X, B, R) == 0
        torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, (free0, free1)
    Rh, bound = _host_residual_bound(A.cpu().numpy(), X.cpu().numpy(), B.cpu().numpy())
    assert np.all(np.abs(R.cpu().numpy() - Rh) <= bound)


def test_no_alloc_rejects_oversize_before_touching_memory(ctx):
    lib = _lib.load()
    # 32768 rows x 16 right-hand sides x 8 column chunks exceeds the array;
    # the null pointers are never dereferenced because the size check fails first
    null = ctypes.c_void_p(0)
    rc = lib.ElGBResidualNoAlloc_d(32768, 16, null, 32768, null, 32768, null, 32768, null,
                                   32768, null)
    assert rc == 3
    torch.cuda.synchronize()

"""The C-ABI library loads and exports every symbol include/*.h declares, and
its host-only pieces (El::Matrix handles, El::Permutation swap sequences,
blocksize stack, error strings) behave like the reference's — no GPU calls."""
import ctypes
import subprocess

import numpy as np
import pytest

import elemental_gb300 as El
from elemental_gb300 import _lib
from elemental_gb300.build import LIB


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    assert lib is not None
    names = _lib.exported_symbols_from_headers()
    assert len(names) > 80
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True, text=True,
                         check=True).stdout
    syms = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    missing = [n for n in names if n not in syms]
    assert not missing, missing


def test_error_strings_and_blocksize_stack():
    lib = _lib.load()
    assert lib.ElErrorString(0) == b"EL_SUCCESS"
    assert lib.ElErrorString(5) == b"EL_RUNTIME_ERROR"
    assert El.Blocksize() == 128
    El.PushBlocksizeStack(96)
    assert El.Blocksize() == 96
    assert lib.ElGBBlocksize() == 96
    El.PopBlocksizeStack()
    assert El.Blocksize() == 128
    assert lib.ElGBBlocksize() == 128


def test_matrix_handles_attach_and_access():
    lib = _lib.load()
    a = np.asfortranarray(np.arange(12, dtype=np.float64).reshape(3, 4))
    M = El.Matrix(a)
    h, w, ld = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert lib.ElMatrixHeight_d(M.obj, ctypes.byref(h)) == 0 and h.value == 3
    assert lib.ElMatrixWidth_d(M.obj, ctypes.byref(w)) == 0 and w.value == 4
    assert lib.ElMatrixLDim_d(M.obj, ctypes.byref(ld)) == 0 and ld.value == 3
    buf = ctypes.c_void_p()
    assert lib.ElMatrixBuffer_d(M.obj, ctypes.byref(buf)) == 0
    assert buf.value == a.ctypes.data


def test_permutation_swap_sequence_host_logic():
    """Permutation::Swap / PermuteRows / ExplicitVector semantics
    (src/lapack_like/perm/Permutation.cpp:205-250, 544-586, 731-745)."""
    lib = _lib.load()
    P = El.Permutation()
    assert lib.ElPermutationMakeIdentity(P.obj, 5) == 0
    for o, d in enumerate([3, 1, 4, 4]):
        assert lib.ElPermutationSwap(P.obj, o, d) == 0
    p = P.ExplicitVector()
    ref = list(range(5))
    for o, d in enumerate([3, 1, 4, 4]):
        ref[o], ref[d] = ref[d], ref[o]
    assert list(p) == ref
    assert list(El._swap_dests_from_explicit(p)) == [3, 1, 4, 4, 4]
    B = El.Matrix(np.arange(10, dtype=np.float64).reshape(5, 2) * 1.0)
    P.PermuteRows(B)
    assert np.array_equal(B.array[:, 0], np.arange(0, 10, 2, dtype=np.float64)[ref])
    # an out-of-range swap is a logic error, as in the reference's debug check
    assert lib.ElPermutationSwap(P.obj, 4, 7) == 4


def test_swap_recovery_roundtrip_random():
    rng = np.random.default_rng(0)
    for n in (1, 2, 17, 200):
        d = np.array([rng.integers(i, n) for i in range(n)], dtype=np.int32)
        lab = np.arange(n)
        for i, j in enumerate(d):
            lab[[i, j]] = lab[[j, i]]
        assert np.array_equal(El._swap_dests_from_explicit(lab), d)


def test_device_api_fails_loudly_without_gpu():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.ElGBCreate(ctypes.byref(h), 0) != 0


def test_host_alloc_argument_handling():
    """ElGBHostAlloc / ElGBHostFree: zero bytes, NULL and foreign pointers
    (host logic only); without a GPU the driver refuses the registration
    and the call fails cleanly."""
    import torch

    lib = _lib.load()
    p = ctypes.c_void_p(1234)
    assert lib.ElGBHostAlloc(0, ctypes.byref(p)) == 0 and not p.value
    assert lib.ElGBHostFree(None) == 0
    buf = ctypes.create_string_buffer(64)
    assert lib.ElGBHostFree(ctypes.cast(buf, ctypes.c_void_p)) == 4  # EL_LOGIC_ERROR
    assert lib.ElGBHostAlloc(1 << 20, None) == 3  # EL_ARG_ERROR
    if not torch.cuda.is_available():
        assert lib.ElGBHostAlloc(1 << 20, ctypes.byref(p)) == 5  # EL_RUNTIME_ERROR
        assert not p.value


def test_profile_and_option_entry_points_reject_a_null_context():
    """The profiling and option entry points check their context before
    touching anything (host logic only)."""
    lib = _lib.load()
    cnt = ctypes.c_int(-1)
    assert lib.ElGBProfileStartTags(None, 1) == 3  # EL_ARG_ERROR
    assert lib.ElGBProfileRecords(None, 0, ctypes.byref(cnt), None, None, None, None) == 3
    assert cnt.value == -1
    for opt in range(1, 18):
        assert lib.ElGBSetOption(None, opt, 1) == 3


def test_python_matrix_views_share_memory():
    """El.Matrix slicing gives views through ElView_d (the reference's
    Matrix.__getitem__, python/core/Matrix.py:456-482); a permutation applied
    through a view moves the parent's rows."""
    lib = _lib.load()
    a = np.asfortranarray(np.arange(20, dtype=np.float64).reshape(5, 4))
    A = El.Matrix(a)
    V = A[1:4, 2:]
    h, w, ld = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert lib.ElMatrixHeight_d(V.obj, ctypes.byref(h)) == 0 and h.value == 3
    assert lib.ElMatrixWidth_d(V.obj, ctypes.byref(w)) == 0 and w.value == 2
    assert lib.ElMatrixLDim_d(V.obj, ctypes.byref(ld)) == 0 and ld.value == 5
    buf = ctypes.c_void_p()
    assert lib.ElMatrixBuffer_d(V.obj, ctypes.byref(buf)) == 0
    assert buf.value == a.ctypes.data + (1 + 2 * 5) * 8
    assert np.array_equal(V.array, a[1:4, 2:])
    P = El.Permutation()
    assert lib.ElPermutationMakeIdentity(P.obj, 3) == 0
    assert lib.ElPermutationSwap(P.obj, 0, 2) == 0
    before = a.copy()
    P.PermuteRows(V)
    assert np.array_equal(a[1, 2:], before[3, 2:]) and np.array_equal(a[3, 2:], before[1, 2:])
    assert np.array_equal(a[:, :2], before[:, :2])
    col = A[:, 1]
    assert col.array.shape == (5, 1) and col.array[4, 0] == a[4, 1]
    with pytest.raises(IndexError):
        A[::2, :]


def test_python_permutation_swap_sequence_api():
    """El.Permutation's swap-sequence methods (python/core/Permutation.py:56-187)
    over the C interface: implicit origins until a swap names another origin,
    parity, appending with an offset."""
    P = El.Permutation()
    P.MakeIdentity(4)
    P.ReserveSwaps(4)
    P.Swap(0, 2)
    P.Swap(1, 1)
    assert P.IsSwapSequence() and P.IsImplicitSwapSequence() and P.Parity()
    P.Swap(3, 0)  # origin 3 is not the swap count 2: explicit origins
    assert not P.IsImplicitSwapSequence() and not P.Parity()
    assert list(P.SwapDestinations()) == [2, 1, 0]
    lab = list(range(4))
    for o, d in ((0, 2), (1, 1), (3, 0)):
        lab[o], lab[d] = lab[d], lab[o]
    assert list(P.ExplicitVector()) == lab
    Q = El.Permutation()
    Q.MakeIdentity(6)
    Q.SwapSequence(P, 2)
    assert list(Q.SwapDestinations()) == [4, 3, 2] and Q.Height() == Q.Width() == 6
    B = El.Matrix(np.arange(6, dtype=np.float64).reshape(6, 1))
    Q.PermuteRows(B)
    assert list(B.array[:, 0]) == [0.0, 1.0] + [2.0 + v for v in lab]
    with pytest.raises(El.ElError):
        P.Swap(0, 9)
    P.Empty()
    assert P.Height() == 0 and len(P.SwapDestinations()) == 0

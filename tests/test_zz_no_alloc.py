"""ElGBResidualNoAlloc_d: the FP64 residual for callers that cannot allocate
device memory (for example while capturing a CUDA graph that must not
contain allocations, or when another allocator owns all device memory).
It must give the same result as the allocating entry point ElGBResidual_d,
call after call, with its scratch in a fixed device array.

This file is collected last on purpose (a failure here leaves every other
test already run)."""
import ctypes

import numpy as np
import pytest
import torch

from elemental_gb300 import _lib
from elemental_gb300 import device as D

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _noalloc(lib, A, X, B, R):
    n, q = B.shape
    s = torch.cuda.current_stream().cuda_stream
    return lib.ElGBResidualNoAlloc_d(n, q, _p(A), A.stride(1), _p(X), X.stride(1), _p(B),
                                     B.stride(1), _p(R), R.stride(1), ctypes.c_void_p(s))


@pytest.mark.parametrize("n,q", [(3000, 5), (4097, 16), (1, 1)])
def test_no_alloc_residual_matches_allocating_entry_point(ctx, n, q):
    lib = _lib.load()
    g = torch.Generator(device="cuda")
    g.manual_seed(n * 31 + q)
    A = D.colmajor(n, n)
    A.copy_(torch.randn(n, n, generator=g, device="cuda", dtype=torch.float64))
    B = D.colmajor(n, q)
    B.copy_(torch.randn(n, q, generator=g, device="cuda", dtype=torch.float64))
    for call in range(2):  # two calls in a row share the static scratch
        X = D.colmajor(n, q)
        X.copy_(torch.randn(n, q, generator=g, device="cuda", dtype=torch.float64))
        R_ref = ctx.residual(A, X, B)
        R = D.colmajor(n, q)
        R.fill_(float("nan"))
        assert _noalloc(lib, A, X, B, R) == 0
        torch.cuda.synchronize()
        ref = R_ref.cpu().numpy()
        got = R.cpu().numpy()
        scale = np.abs(A.cpu().numpy()).sum(axis=1).max() * np.abs(X.cpu().numpy()).max()
        assert np.abs(got - ref).max() <= 1e-13 * max(scale, 1.0), (call, np.abs(got - ref).max())


def test_no_alloc_rejects_oversize_before_touching_memory(ctx):
    lib = _lib.load()
    # 32768 rows x 16 right-hand sides x 8 column chunks exceeds the array;
    # the null pointers are never dereferenced because the size check fails first
    null = ctypes.c_void_p(0)
    rc = lib.ElGBResidualNoAlloc_d(32768, 16, null, 32768, null, 32768, null, 32768, null,
                                   32768, null)
    assert rc == 3
    torch.cuda.synchronize()

"""The selector MLP's hand-written FP32 kernels (mlp.cu) against the FP64
CPU oracle (oracle/mlp_oracle.py): forward probabilities, the batch gradient
of the mean cross-entropy, and a training run that lowers the loss."""
import ctypes

import numpy as np
import pytest
import torch

from elemental_gb300 import _lib
from oracle import mlp_oracle as MO

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def rand_params(seed):
    rng = np.random.default_rng(seed)
    th = []
    for name, shp in MO.SHAPES:
        fan_in = shp[0] if len(shp) == 2 else 1
        scale = np.sqrt(2.0 / fan_in) if len(shp) == 2 else 0.1
        th.append((rng.standard_normal(shp) * scale).ravel())
    return np.concatenate(th).astype(np.float32)


def test_param_count():
    assert _lib.load().ElGBMLPParamCount() == MO.NPARAM == 5443


@pytest.mark.parametrize("B", [1, 37, 256, 1000])
def test_forward_and_gradient_match_oracle(ctx, B):
    lib = _lib.load()
    rng = np.random.default_rng(B)
    theta = rand_params(B)
    X = rng.standard_normal((B, 16)).astype(np.float32)
    y = rng.integers(0, 3, B).astype(np.int32)
    dth, dX, dy = (torch.from_numpy(a).cuda() for a in (theta, X, y))
    probs = torch.empty(B, 3, device="cuda")
    am = torch.empty(B, dtype=torch.int32, device="cuda")
    ctx._bind()
    assert lib.ElGBMLPForward(ctx.h, _p(dth), _p(dX), B, _p(probs), _p(am)) == 0
    ref = MO.forward(theta.astype(np.float64), X.astype(np.float64))
    assert np.abs(probs.cpu().numpy() - ref["probs"]).max() < 1e-5
    assert np.array_equal(am.cpu().numpy(), ref["probs"].argmax(1))
    grad = torch.empty(MO.NPARAM, device="cuda")
    loss = ctypes.c_float()
    assert lib.ElGBMLPGradient(ctx.h, _p(dth), _p(dX), _p(dy), B, _p(grad),
                               ctypes.byref(loss)) == 0
    L, g = MO.loss_and_grad(theta.astype(np.float64), X.astype(np.float64), y)
    assert abs(loss.value - L) <= 1e-5 * max(1.0, abs(L))
    gg = grad.cpu().numpy().astype(np.float64)
    rel = np.linalg.norm(gg - g) / max(np.linalg.norm(g), 1e-30)
    assert rel < 1e-4, rel
    # and the oracle gradient is the gradient: central finite difference of
    # the oracle loss along a random direction (ReLU kinks crossed within
    # +-h make this approximate, hence the looser bound)
    d = rng.standard_normal(MO.NPARAM)
    h = 1e-6
    th64 = theta.astype(np.float64)
    fd = (MO.loss_and_grad(th64 + h * d, X, y)[0] - MO.loss_and_grad(th64 - h * d, X, y)[0]) / (2 * h)
    assert abs(fd - g @ d) <= 2e-3 * max(1.0, abs(fd))


def test_adam_training_lowers_loss(ctx):
    lib = _lib.load()
    rng = np.random.default_rng(0)
    B = 512
    X = rng.standard_normal((B, 16)).astype(np.float32)
    y = (X[:, 0] > 0).astype(np.int32) + (X[:, 1] > 1).astype(np.int32)
    theta = torch.from_numpy(rand_params(1)).cuda()
    m = torch.zeros_like(theta)
    v = torch.zeros_like(theta)
    g = torch.empty_like(theta)
    dX, dy = torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda()
    ctx._bind()
    losses = []
    for step in range(1, 301):
        loss = ctypes.c_float()
        assert lib.ElGBMLPGradient(ctx.h, _p(theta), _p(dX), _p(dy), B, _p(g),
                                   ctypes.byref(loss) if step % 50 == 1 else None) == 0
        if step % 50 == 1:
            losses.append(loss.value)
        assert lib.ElGBMLPAdamStep(ctx.h, _p(theta), _p(g), _p(m), _p(v), 1e-2, 0.9, 0.999,
                                   1e-8, 0.0, step) == 0
    assert losses[-1] < 0.5 * losses[0], losses

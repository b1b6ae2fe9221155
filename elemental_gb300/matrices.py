"""Seeded synthetic inputs for the factor-and-solve path (host, FP64).

Counterparts of the reference's generators in src/matrices, generated once in
FP64 on the host so that the GPU path and the CPU oracle see identical bits:

* gaussian(m, n, seed)        iid N(0,1)              (random/independent/Gaussian.cpp:15-21)
* spd(n, seed)                G^T G / n + I, G iid N(0,1)
* haar(n, seed)               Q of the QR of a Gaussian (random/misc/Haar.cpp:14-21)
* conditioned(n, kappa, seed) U diag(sigma) V^T, U, V Haar, sigma geometric 1 .. 1/kappa
* gepp_growth(n)              growth-2^(n-1) matrix    (deterministic/misc/GEPPGrowth.cpp:14-28)
* hermitian_uniform_spectrum  Q diag(U[lo,hi)) Q^T     (random/misc/HermitianUniformSpectrum.cpp:22-43)

All use numpy's PCG64 Generator seeded by an integer; the base seed of the
benchmark workloads is 20261204 (+ config index, + system index).
"""
from __future__ import annotations

import numpy as np

BASE_SEED = 20261204


def rng(seed):
    return np.random.default_rng(int(seed))


def gaussian(m, n, seed):
    return np.asfortranarray(rng(seed).standard_normal((n, m)).T)


def spd(n, seed):
    G = gaussian(n, n, seed)
    A = G.T @ G / n
    A[np.diag_indices(n)] += 1.0
    return np.asfortranarray(A)


def haar(n, seed):
    Q, R = np.linalg.qr(gaussian(n, n, seed))
    # sign fix so that the distribution is Haar (QR's R diagonal positive)
    Q = Q * np.sign(np.diag(R))[None, :]
    return np.asfortranarray(Q)


def conditioned(n, kappa, seed):
    """A = U diag(sigma) V^T with U, V Haar (two independent seeds) and
    sigma_i = kappa^(-i/(n-1)), so ||A||_2 = 1 and cond_2(A) = kappa."""
    U = haar(n, 2 * int(seed) + 1)
    V = haar(n, 2 * int(seed) + 2)
    if n > 1:
        sig = np.power(float(kappa), -np.arange(n) / (n - 1))
    else:
        sig = np.ones(1)
    return np.asfortranarray((U * sig[None, :]) @ V.T)


def gepp_growth(n):
    A = np.eye(n)
    if n <= 1:
        return np.asfortranarray(A)
    A[:, n - 1] = 1.0
    il = np.tril_indices(n, -1)
    A[il] = -1.0
    return np.asfortranarray(A)


def hermitian_uniform_spectrum(n, lower, upper, seed):
    g = rng(seed)
    d = g.uniform(lower, upper, n)
    Q = haar(n, int(seed) + 7919)
    return np.asfortranarray((Q * d[None, :]) @ Q.T)

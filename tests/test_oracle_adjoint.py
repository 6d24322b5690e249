"""Coefficient gradient of A_H on the CPU, oracle only (no GPU).

Pins the formula the GPU gradient kernel implements: at the solution of
G A u_i = 0 (u_i = X_i + E_i), dA_H[i, j] / da(v) = u_i(v) . u_j(v) / M for an
isotropic coefficient a, with no adjoint solve.  Checked against central
differences of the oracle's own A_H.
"""
import numpy as np

import oracle
from ffthompy_gb300 import workloads


def _ah_and_fields(a, N, tol=1e-13):
    d = len(N)
    A = np.einsum('ij,...->ij...', np.eye(d), a)
    G, _ = oracle.green_operator('scalar', np.asarray(N), np.ones(d), 'GaNi', 1)
    Afun = lambda v: oracle.apply_GA(G, A, v)
    us = []
    for l in range(d):
        E = np.zeros((d,) + tuple(N))
        E[l] = 1.
        X, _ = oracle.cg(Afun, Afun(-E), np.zeros_like(E), tol=tol, maxiter=2000)
        us.append(X + E)
    AH = oracle.assembly_matrix(A, us)
    return AH, us


def test_gradient_formula_matches_central_differences():
    N = (11, 9)
    a = np.exp(workloads.gaussian_field(N, 0.2, seed=4))
    AH, us = _ah_and_fields(a, N)
    M = np.prod(N)
    W = np.array([[1.0, 0.3], [0.3, -0.5]])  # a general adjoint seed
    grad = sum(W[i, j] * np.einsum('c...,c...->...', us[i], us[j])
               for i in range(2) for j in range(2)) / M
    rng = np.random.default_rng(0)
    for _ in range(4):
        v = tuple(int(rng.integers(n)) for n in N)
        h = 1e-4 * a[v]
        ap, am = a.copy(), a.copy()
        ap[v] += h
        am[v] -= h
        fd = (np.sum(W * _ah_and_fields(ap, N)[0]) - np.sum(W * _ah_and_fields(am, N)[0])) / (2 * h)
        assert abs(fd - grad[v]) < 1e-6 * abs(grad[v]) + 1e-12, (v, fd, grad[v])

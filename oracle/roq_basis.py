"""A synthetic reduced-order-quadrature basis for the tests: a reduced basis
of TaylorF2 waveforms (SVD of a seeded training set) with empirical-
interpolation nodes (greedy selection, the standard construction of
Field et al., arXiv:1308.3565, and Canizares et al., arXiv:1404.6284).

TEST INFRASTRUCTURE ONLY: ROQ basis files are not part of the reference tree
nor of this container; this seeded basis stands in for them so that the
reference's ROQGravitationalWaveTransient and the GPU ROQ likelihood can be
compared on the same weights.  The basis only needs to be the same for both,
not accurate.
"""
from __future__ import annotations

import numpy as np

from .taylorf2 import taylorf2_aligned


def empirical_interpolation(basis):
    """Greedy EIM nodes of an orthonormal basis (N x n) and the interpolant
    matrix B (n x N) with h(f) ~ sum_j h(F_j) B_j(f)."""
    N, n = basis.shape
    nodes = [int(np.argmax(np.abs(basis[:, 0])))]
    for j in range(1, n):
        E = basis[:, :j]
        V = E[nodes, :]
        coef = np.linalg.solve(V, basis[nodes, j])
        r = basis[:, j] - E @ coef
        nodes.append(int(np.argmax(np.abs(r))))
    V = basis[nodes, :]
    B = np.linalg.solve(V.T, basis.T)   # (E V^-1)^T
    return np.array(nodes), B


def build(frequencies, n_linear=40, n_quadratic=20, n_train=300, seed=2024, minimum_frequency=20.0,
          mass_range=(10.0, 40.0)):
    """(nodes_linear, B_linear (n_l x N complex), nodes_quadratic, B_quadratic (n_q x N real))
    on ``frequencies`` (the masked analysis frequencies)."""
    rng = np.random.default_rng(seed)
    f = np.asarray(frequencies, dtype=np.float64)
    lin, quad = [], []
    for _ in range(n_train):
        m1, m2 = np.sort(rng.uniform(*mass_range, 2))[::-1]
        h = taylorf2_aligned(f, m1, m2, rng.uniform(-0.05, 0.05), rng.uniform(-0.05, 0.05), 100.0, 0.0,
                             0.0, minimum_frequency=minimum_frequency)["plus"]
        lin.append(h / np.linalg.norm(h))
        q = np.abs(h) ** 2
        quad.append(q / np.linalg.norm(q))
    ul = np.linalg.svd(np.array(lin).T, full_matrices=False)[0][:, :n_linear]
    uq = np.linalg.svd(np.array(quad).T, full_matrices=False)[0][:, :n_quadratic]
    nl, bl = empirical_interpolation(ul)
    nq, bq = empirical_interpolation(uq)
    return f[nl], bl, f[nq], bq.real

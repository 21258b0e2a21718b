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


# Bands (duration T_b, f_lo, f_hi) of the seeded multi-banded basis for an
# 8 s segment sampled at 2048 Hz: each band on the grid k / T_b, the bands
# contiguous in frequency and the last one reaching the Nyquist frequency.
MULTIBAND_BANDS_8S = ((8.0, 20.0, 60.0), (4.0, 60.0, 200.0), (2.0, 200.0, 1024.0))


def multiband_layout(bands):
    """(durations T_b, start/end frequency bins [n_b, 2], the multi-banded
    frequencies) of ``bands`` = ((T_b, f_lo, f_hi), ...): band b holds the
    bins k / T_b with f_lo <= f < f_hi (f <= f_hi for the last band)."""
    durations, bins, freqs = [], [], []
    for b, (tb, lo, hi) in enumerate(bands):
        s = int(np.ceil(lo * tb))
        e = int(np.floor(hi * tb)) - (0 if b == len(bands) - 1 else 1)
        durations.append(tb)
        bins.append([s, e])
        freqs.append(np.arange(s, e + 1) / tb)
    return np.array(durations), np.array(bins, dtype=np.int64), np.concatenate(freqs)


def build_multiband(bands=MULTIBAND_BANDS_8S, n_linear=40, n_quadratic=20, seed=2024, minimum_frequency=20.0):
    """A multi-banded basis in the layout of an ROQ basis file (roq.py:793-1055
    reads it): ``multiband_<type>``, ``durations_s_<type>``,
    ``start_end_frequency_bins_<type>`` and ``basis_<type>["0"]`` with the
    basis on the multi-banded frequencies and its empirical-interpolation
    nodes.  Returns (linear_matrix, quadratic_matrix) as dictionaries."""
    durations, bins, f = multiband_layout(bands)
    nl, bl, nq, bq = build(f, n_linear=n_linear, n_quadratic=n_quadratic, seed=seed,
                           minimum_frequency=minimum_frequency)
    lin = {"multiband_linear": np.array(True), "durations_s_linear": durations,
           "start_end_frequency_bins_linear": bins, "basis_linear": {"0": {"basis": bl, "frequency_nodes": nl}}}
    quad = {"multiband_quadratic": np.array(True), "durations_s_quadratic": durations,
            "start_end_frequency_bins_quadratic": bins,
            "basis_quadratic": {"0": {"basis": bq, "frequency_nodes": nq}}}
    return lin, quad

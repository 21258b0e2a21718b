"""numpy restatement of bilby's relative-binning likelihood
(bilby/gw/likelihood/relative.py, Zackay, Dai & Venumadhav arXiv:1806.08792).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA relative-binning kernel.
Parity with the reference itself is pinned by
``tests/golden/tf2_128s_relbin.npz``, which the reference wrote through
``tests/golden/make_golden.py``.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import restate as R

GAMMA = np.array([-5 / 3, -2 / 3, 1, 5 / 3, 7 / 3])   # relative.py:146


@dataclass
class RelbinSetup:
    bin_inds: np.ndarray          # grid index of each bin edge
    bin_freqs: np.ndarray         # edge frequencies
    fiducial: list                # per detector: fiducial response on the full grid
    summary: list                 # per detector: (a0, a1, b0, b1), one value per bin
    maximum_frequency: float


def fiducial_waveforms(dets, source, fiducial_parameters):
    """relative.py:232-254: the fiducial responses, zero above the fiducial's
    last non-zero frequency."""
    p = dict(fiducial_parameters)
    pols = source(dets[0].frequency, **p)
    nz = np.where(pols["plus"] != 0j)[0][-1]
    fmax = dets[0].frequency[nz]
    out = []
    for det in dets:
        wf = R.detector_response(det, pols, p["ra"], p["dec"], p["geocent_time"], p["psi"])
        wf = wf * (det.frequency <= fmax)
        out.append(wf)
    return out, float(fmax)


def setup_bins(dets, frequency_array, fiducial_maximum_frequency, chi=1.0, epsilon=0.5,
               maximum_frequencies=None, minimum_frequencies=None):
    """relative.py:178-230.  ``maximum_frequencies`` / ``minimum_frequencies``
    are the interferometers' band limits (strain_data.py:103-110)."""
    gamma = GAMMA[:, np.newaxis]
    fmax = frequency_array[0]
    fmin = frequency_array[-1]
    for q, det in enumerate(dets):
        fmax = max(fmax, maximum_frequencies[q])
        fmin = min(fmin, minimum_frequencies[q])
    fmax = min(fmax, fiducial_maximum_frequency)
    useful = frequency_array[(frequency_array >= fmin) & (frequency_array <= fmax)]
    d_alpha = chi * 2 * np.pi / np.abs((fmin ** gamma) * np.heaviside(-gamma, 1)
                                       - (fmax ** gamma) * np.heaviside(gamma, 1))
    d_phi = np.sum(np.sign(gamma) * d_alpha * useful ** gamma, axis=0)
    d_phi_from_start = d_phi - d_phi[0]
    number_of_bins = int(d_phi_from_start[-1] // epsilon)
    bin_inds, bin_freqs = [], []
    last = -1
    for i in range(number_of_bins + 1):
        idx = np.where(d_phi_from_start >= ((i / number_of_bins) * d_phi_from_start[-1]))[0][0]
        if idx == last:
            continue
        f = useful[idx]
        last = idx
        bin_inds.append(np.where(frequency_array >= f)[0][0])
        bin_freqs.append(f)
    return np.array(bin_inds, dtype=int), np.array(bin_freqs)


def summary_data(dets, fiducial, bin_freqs):
    """relative.py:319-363: per bin a0 = <h0|d>, b0 = <h0|h0>, a1 = <h0|d df>,
    b1 = <h0|h0 df> over the masked grid, df measured from the bin centre."""
    out = []
    n_bins = len(bin_freqs) - 1
    for det, h0_full in zip(dets, fiducial):
        m = det.mask
        mf = det.frequency[m]
        inds = [int(np.where(mf == e)[0][0]) for e in bin_freqs]
        if inds[-1] < len(mf) - 1:
            inds[-1] += 1
        strain = det.masked_strain[m]
        h0 = np.asarray(h0_full[m])
        psd = det.psd[m]
        a0, b0, a1, b1 = np.zeros((4, n_bins), dtype=complex)
        for i in range(n_bins):
            s, e = inds[i], inds[i + 1]
            f = mf[s:e]
            df = f - (mf[s] + mf[e]) / 2
            a0[i] = R.noise_weighted_inner_product(h0[s:e], strain[s:e], psd[s:e], det.duration)
            b0[i] = R.noise_weighted_inner_product(h0[s:e], h0[s:e], psd[s:e], det.duration)
            a1[i] = R.noise_weighted_inner_product(h0[s:e], strain[s:e] * df, psd[s:e], det.duration)
            b1[i] = R.noise_weighted_inner_product(h0[s:e], h0[s:e] * df, psd[s:e], det.duration)
        out.append((a0, a1, b0, b1))
    return out


def setup(dets, source, fiducial_parameters, chi=1.0, epsilon=0.5, maximum_frequency=2048.0,
          minimum_frequency=20.0) -> RelbinSetup:
    fid, fmax = fiducial_waveforms(dets, source, fiducial_parameters)
    inds, freqs = setup_bins(dets, dets[0].frequency, fmax, chi, epsilon,
                             [min(maximum_frequency, d.frequency[-1]) for d in dets],
                             [minimum_frequency for _ in dets])
    return RelbinSetup(inds, freqs, fid, summary_data(dets, fid, freqs), fmax)


def terms(dets, source, setup: RelbinSetup, params):
    """relative.py:365-402: <d|h> (complex) and <h|h> summed over detectors,
    from the ratio of the waveform to the fiducial at the bin edges."""
    f = setup.bin_freqs
    pols = source(f, **params)
    widths = f[1:] - f[:-1]
    dh, hh = 0j, 0.0
    for det, h0_full, (a0, a1, b0, b1) in zip(dets, setup.fiducial, setup.summary):
        # get_detector_response with explicit frequencies: no mask (interferometer.py:329-333)
        signal = 0
        for mode, h in pols.items():
            signal = signal + h * R.antenna_response(det.tensor, params["ra"], params["dec"],
                                                     params["geocent_time"], params["psi"], mode)
        shift = R.time_delay_from_geocenter(det.vertex, params["ra"], params["dec"], params["geocent_time"])
        dt = (params["geocent_time"] - det.start_time) + shift
        strain = signal * np.exp(-1j * 2 * np.pi * dt * f)
        ratio = strain / h0_full[setup.bin_inds]
        r0 = (ratio[1:] + ratio[:-1]) / 2
        r1 = (ratio[1:] - ratio[:-1]) / widths
        dh = dh + (a0 * r0.conj() + a1 * r1.conj()).sum()
        hh = hh + (b0 * abs(r0) ** 2 + 2 * b1 * (r0 * r1.conj()).real).sum().real
    return dh, float(hh)


def log_likelihood_ratio(dets, source, setup: RelbinSetup, params, marg: R.Marginalization | None = None):
    """relative.py through base.py:448-477 (no time marginalisation)."""
    marg = marg or R.Marginalization()
    dh, hh = terms(dets, source, setup, params)
    return R._combine(dh, hh, None, params, marg, None)

"""numpy restatement of the per-evaluation part of bilby's multi-banded
likelihood (bilby/gw/likelihood/multiband.py:741-819), with linear
interpolation of <h|h> on the bands and coefficients the reference computed
(tests/golden/tf2_128s_multiband.npz), and with the IFFT-FFT <h|h>
(multiband.py:760-779) on given IFFT-FFT tables.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA multi-banding kernel.
"""
from __future__ import annotations

import numpy as np

from . import restate as R


def banded_strains(dets, source, weights, params):
    """The detector responses at the banded frequencies, one array per
    detector (multiband.py:741-758)."""
    pols = source(weights["waveform_frequencies"], **params)
    modes = {m: v[weights["unique_to_original_frequencies"]] for m, v in pols.items()}
    f = weights["banded_frequency_points"]
    out = []
    for det in dets:
        signal = 0
        for mode, h in modes.items():
            signal = signal + h * R.antenna_response(det.tensor, params["ra"], params["dec"],
                                                     params["geocent_time"], params["psi"], mode)
        shift = R.time_delay_from_geocenter(det.vertex, params["ra"], params["dec"], params["geocent_time"])
        out.append(signal * np.exp(-1j * 2 * np.pi * ((params["geocent_time"] - det.start_time) + shift) * f))
    return out


def hh_ifft_fft(strain, q, det, tables):
    """<h|h> of detector q by the IFFT-FFT sum (multiband.py:760-779): band 0
    directly, band b >= 1 by irfft of sqrt(w) h into the last M_b of 2 M_b
    samples, rfft and the weights Re I_b.  ``tables`` holds Ks_Ke,
    start_end_idxs, Mbs, Tbhats, windows, square_root_windows, duration and
    per detector Ibcs_<q> (a list over bands)."""
    hh = 0.0
    for b in range(len(tables["Mbs"])):
        ks, ke = (int(x) for x in tables["Ks_Ke"][b])
        s, e = (int(x) for x in tables["start_end_idxs"][b])
        mb = int(tables["Mbs"][b])
        if b == 0:
            with np.errstate(divide="ignore", invalid="ignore"):
                w = det.mask[ks:ke + 1] * tables["windows"][s:e + 1] / det.psd[ks:ke + 1]
            hh += (4. / tables["duration"]) * np.vdot(np.abs(strain[s:e + 1]) ** 2, w).real
        else:
            wth = np.zeros(mb // 2 + 1, dtype=complex)
            wth[ks:ke + 1] = tables["square_root_windows"][s:e + 1] * strain[s:e + 1]
            ibc = np.asarray(tables[f"Ibcs_{q}"][b])
            hbc = np.zeros(len(ibc) * 2 - 2)
            hbc[-mb:] = np.fft.irfft(wth)
            thbc = np.fft.rfft(hbc)
            hh += (4. / tables["Tbhats"][b]) * np.vdot(np.abs(thbc) ** 2, ibc.real).real
    return float(hh)


def log_likelihood_ratio_ifft_fft(dets, source, weights, tables, params, marg: R.Marginalization | None = None):
    """lnL with the IFFT-FFT <h|h> (no time marginalisation)."""
    marg = marg or R.Marginalization()
    dh, hh = 0j, 0.0
    for q, (det, strain) in enumerate(zip(dets, banded_strains(dets, source, weights, params))):
        dh = dh + np.conj(np.dot(strain, weights[f"linear_coeffs_{q}"]))
        hh += hh_ifft_fft(strain, q, det, tables)
    return R._combine(dh, hh, None, params, marg, None)


def terms(dets, source, weights, params):
    """<d|h> (complex) and <h|h> summed over detectors.  ``source`` maps
    (frequencies, **params) -> polarisations; ``weights`` holds
    ``waveform_frequencies``, ``unique_to_original_frequencies``,
    ``banded_frequency_points`` and per detector ``linear_coeffs_<q>`` /
    ``quadratic_coeffs_<q>``."""
    pols = source(weights["waveform_frequencies"], **params)
    modes = {m: v[weights["unique_to_original_frequencies"]] for m, v in pols.items()}
    f = weights["banded_frequency_points"]
    dh, hh = 0j, 0.0
    for q, det in enumerate(dets):
        # get_detector_response at explicit frequencies: no mask (interferometer.py:329-333)
        signal = 0
        for mode, h in modes.items():
            signal = signal + h * R.antenna_response(det.tensor, params["ra"], params["dec"],
                                                     params["geocent_time"], params["psi"], mode)
        shift = R.time_delay_from_geocenter(det.vertex, params["ra"], params["dec"], params["geocent_time"])
        strain = signal * np.exp(-1j * 2 * np.pi * ((params["geocent_time"] - det.start_time) + shift) * f)
        dh = dh + np.conj(np.dot(strain, weights[f"linear_coeffs_{q}"]))
        hh = hh + np.vdot(np.abs(strain) ** 2, weights[f"quadratic_coeffs_{q}"]).real
    return dh, float(hh)


def log_likelihood_ratio(dets, source, weights, params, marg: R.Marginalization | None = None):
    marg = marg or R.Marginalization()
    dh, hh = terms(dets, source, weights, params)
    return R._combine(dh, hh, None, params, marg, None)

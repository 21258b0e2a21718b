"""numpy restatement of the per-evaluation part of bilby's multi-banded
likelihood (bilby/gw/likelihood/multiband.py:741-819, linear interpolation of
<h|h>), on the bands and coefficients the reference computed
(tests/golden/tf2_128s_multiband.npz).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA multi-banding kernel.
"""
from __future__ import annotations

import numpy as np

from . import restate as R


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

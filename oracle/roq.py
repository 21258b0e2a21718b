"""numpy restatement of the per-evaluation part of bilby's ROQ likelihood
(bilby/gw/likelihood/roq.py:463-602, single basis, no time
marginalisation), on weights the reference computed.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA ROQ kernel.
"""
from __future__ import annotations

import numpy as np

from . import restate as R


def closest_time_indices(time, samples):
    """roq.py:552-575."""
    closest = int(np.floor((time - samples[0]) / (samples[1] - samples[0])))
    indices = [closest + k for k in (-2, -1, 0, 1, 2)]
    return indices, (indices[0] >= 0) and (indices[-1] < len(samples))


def interp_five_samples(ts, values, time):
    """roq.py:577-602 (LIGO-T2100224)."""
    r1 = (-values[0] + 8. * values[1] - 14. * values[2] + 8. * values[3] - values[4]) / 4.
    r2 = values[2] - 2. * values[3] + values[4]
    a = (ts[3] - time) / max(ts[1] - ts[0], 1e-12)
    b = 1. - a
    c = (a ** 3. - a) / 6.
    d = (b ** 3. - b) / 6.
    return a * values[2] + b * values[3] + c * r1 + d * r2


def terms(dets, source, roq, params):
    """<d|h> and <h|h> summed over detectors.  ``roq``: ``time_samples``,
    ``nodes_linear``, ``nodes_quadratic`` and per detector ``linear_<q>``
    (a callable row index -> weights row) and ``quadratic_<q>``."""
    pl = source(roq["nodes_linear"], **params)
    pq = source(roq["nodes_quadratic"], **params)
    ts = roq["time_samples"]
    dh, hh = 0j, 0.0
    for q, det in enumerate(dets):
        fp = R.antenna_response(det.tensor, params["ra"], params["dec"], params["geocent_time"], params["psi"], "plus")
        fx = R.antenna_response(det.tensor, params["ra"], params["dec"], params["geocent_time"], params["psi"], "cross")
        h_lin = pl["plus"] * fp + pl["cross"] * fx
        h_quad = pq["plus"] * fp + pq["cross"] * fx
        hh += np.vdot(np.abs(h_quad) ** 2, roq[f"quadratic_{q}"]).real
        delay = R.time_delay_from_geocenter(det.vertex, params["ra"], params["dec"], params["geocent_time"])
        t_ifo = params["geocent_time"] - det.start_time + delay
        idx, ok = closest_time_indices(t_ifo, ts)
        idx = np.clip(idx, 0, len(ts) - 1)
        vals = np.array([np.sum(np.conj(h_lin) * roq[f"linear_{q}"](j)) for j in idx])
        d = interp_five_samples(ts[idx], vals, t_ifo)
        with np.errstate(divide="ignore"):
            d = d + np.log(ok)
        dh += d
    return dh, float(hh)


def log_likelihood_ratio(dets, source, roq, params, marg: R.Marginalization | None = None):
    marg = marg or R.Marginalization()
    dh, hh = terms(dets, source, roq, params)
    return R._combine(dh, hh, None, params, marg, None)

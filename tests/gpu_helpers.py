"""Helpers shared by the GPU tests: build an oracle analysis and the matching
device-resident analysis from the same seeded data."""
from __future__ import annotations

import numpy as np

from bilby_gb300.analysis import Analysis, DetectorData, params_block
from bilby_gb300.workloads import WORKLOADS, Workload, draw_points, point
from oracle import data as OD
from oracle import restate as R

FP64_RTOL = 1e-9      # plain float64 kernel vs the oracle: |d lnL| <= 1e-9 * max(1, |Re<d|h>|, <h|h>/2)
MIXED_ATOL = 1e-3     # mixed-precision kernel vs the float64 oracle: |d lnL| <= 1e-3


def device_analysis(dets, model, w: Workload) -> Analysis:
    dd = [DetectorData(d.name, d.vertex, d.tensor, d.start_time, d.masked_strain, d.psd, d.mask) for d in dets]
    return Analysis(model, dets[0].frequency, dd, w.duration, w.sampling_frequency, w.minimum_frequency)


def oracle_plain(dets, w: Workload, params: dict, idx) -> tuple[np.ndarray, np.ndarray]:
    """Oracle lnL and parity scale for the points ``idx`` of ``params``."""
    src = OD.source_for(w.model, w.minimum_frequency)
    lnl, scale = [], []
    for i in idx:
        p = point(params, i)
        dh, hh = R.plain_terms(dets, src, p)
        lnl.append(float(np.real(dh) - hh / 2))
        scale.append(R.parity_scale(dh, hh))
    return np.array(lnl), np.array(scale)


_POOL: dict = {}


def _pool_init(w):
    import os
    os.environ["OMP_NUM_THREADS"] = "1"
    _POOL["dets"] = OD.build_workload(w)
    _POOL["src"] = OD.source_for(w.model, w.minimum_frequency)


def _pool_eval(p):
    dh, hh = R.plain_terms(_POOL["dets"], _POOL["src"], p)
    return float(np.real(dh) - hh / 2), R.parity_scale(dh, hh)


def oracle_plain_pool(w: Workload, params: dict, idx) -> tuple[np.ndarray, np.ndarray]:
    """``oracle_plain`` over the host cores: a pool of processes started with
    ``spawn`` (safe after CUDA is initialised), each building the workload's
    oracle data once."""
    import multiprocessing as mp
    import os
    pts = [point(params, i) for i in idx]
    n = max(1, min(len(os.sched_getaffinity(0)), 32, len(pts)))
    with mp.get_context("spawn").Pool(n, initializer=_pool_init, initargs=(w,)) as pool:
        res = pool.map(_pool_eval, pts, chunksize=max(1, len(pts) // (4 * n)))
    return np.array([r[0] for r in res]), np.array([r[1] for r in res])


def small_workload(base: str, **changes) -> Workload:
    from dataclasses import replace
    return replace(WORKLOADS[base], **changes)


__all__ = ["device_analysis", "oracle_plain", "oracle_plain_pool", "params_block", "draw_points", "point", "small_workload",
           "FP64_RTOL", "MIXED_ATOL", "WORKLOADS"]

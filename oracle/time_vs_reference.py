"""Time the oracle's numpy restatement against the reference bilby itself.

TEST INFRASTRUCTURE ONLY.  The CPU arm of the benchmark runs the oracle (the
reference cannot travel to the GPU host), so this recipe records, once, how
fast the restatement is relative to the reference's own
``GravitationalWaveTransient.log_likelihood_ratio`` on the same data, PSD and
parameters: one process, OMP_NUM_THREADS=1, the same prior draws through
both, after warm-up calls.  It needs the reference source tree (see
``oracle/ref_harness.py``).

    OMP_NUM_THREADS=1 python oracle/time_vs_reference.py [--points N]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _time(fn, pts, warm=3):
    for p in pts[:warm]:
        fn(p)
    t = []
    for p in pts:
        t0 = time.perf_counter()
        fn(p)
        t.append(time.perf_counter() - t0)
    return float(np.median(t)), [float(v) for v in t]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--points", type=int, default=40)
    args = ap.parse_args()
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_golden import build_reference, make_priors  # noqa: E402
    from oracle import data as OD
    from oracle import ref_harness
    from oracle import restate as R
    from oracle.taylorf2 import taylorf2_aligned
    from bilby_gb300.workloads import WORKLOADS, draw_points, point
    bilby = ref_harness.import_bilby()
    out = {}
    for name in ("sg_4s", "tf2_128s", "tf2_marg_8s"):
        w = WORKLOADS[name]
        source = bilby.gw.source.sinegaussian if w.model == "sinegaussian" else taylorf2_aligned
        ifos, wfg = build_reference(bilby, w, source)
        marg = name == "tf2_marg_8s"
        priors = make_priors(bilby, w, time=marg, phase=marg) if marg else None
        like = bilby.gw.likelihood.GravitationalWaveTransient(
            interferometers=ifos, waveform_generator=wfg, priors=priors, time_marginalization=marg,
            phase_marginalization=marg)
        params = draw_points(w, args.points, np.random.default_rng(99), fixed_extrinsic=False)
        pts = [point(params, i) for i in range(args.points)]
        dets = OD.build_workload(w)
        src = OD.source_for(w.model, w.minimum_frequency)
        m = None
        if marg:
            tc = w.injection["geocent_time"]
            m = R.Marginalization(time=True, phase=True)
            R.setup_time_marginalization(m, w.start_time, w.duration, w.sampling_frequency, tc - 0.1, tc + 0.1)
            for p in pts:
                p["geocent_time"] = float(priors["geocent_time"])
                p["phase"] = 0.0
        else:
            for p in pts:
                p.pop("time_jitter", None)
        lo, hi = (w.injection["geocent_time"] - 0.1, w.injection["geocent_time"] + 0.1)
        prior = (lambda t: ((t >= lo) & (t <= hi)) / (hi - lo)) if marg else None
        t_ref, _ = _time(lambda p: like.log_likelihood_ratio(dict(p)), pts)
        t_orc, _ = _time(lambda p: R.log_likelihood_ratio(dets, src, p, m, prior), pts)
        out[name] = {"reference_ms": t_ref * 1e3, "oracle_ms": t_orc * 1e3, "oracle_speed_over_reference": t_ref / t_orc,
                     "points": args.points, "marginalization": "time+phase" if marg else "none"}
        print(name, json.dumps(out[name]), flush=True)
    print(json.dumps(out))


if __name__ == "__main__":
    main()

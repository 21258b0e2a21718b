"""The oracle's ROQ restatement (oracle/roq.py) on the weights the reference's
ROQGravitationalWaveTransient computed (tests/golden/tf2_marg_8s_2k_roq.npz,
seeded synthetic basis) reproduces the reference's lnL."""
import numpy as np
import pytest

from tests.conftest import golden
from oracle import data as OD
from oracle import restate as R
from oracle import roq as RQ
from bilby_gb300.workloads import WORKLOADS, point


def golden_roq(z, n_det):
    t0, dt, n = z["roq_time_meta"]
    start = int(round(t0 / dt))
    roq = dict(time_samples=np.arange(start, start + int(n)) * dt, nodes_linear=z["roq_nodes_linear"],
               nodes_quadratic=z["roq_nodes_quadratic"])
    for q in range(n_det):
        rows = {int(r): k for k, r in enumerate(z[f"roq_linear_rows_{q}"])}
        w = z[f"roq_linear_{q}"]
        roq[f"linear_{q}"] = lambda j, rows=rows, w=w: w[rows[int(j)]]
        roq[f"quadratic_{q}"] = z[f"roq_quadratic_{q}"]
    return roq


@pytest.mark.parametrize("combo", ["none", "p"])
def test_oracle_reproduces_the_reference(combo):
    w = WORKLOADS["tf2_marg_8s_2k"]
    dets = OD.build_workload(w)
    z = golden("tf2_marg_8s_2k_roq")
    assert np.allclose(OD.strain_checksum(dets), z["checksum"], rtol=1e-14, atol=0)
    src = OD.source_for(w.model, w.minimum_frequency)
    roq = golden_roq(z, len(dets))
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    marg = R.Marginalization(phase="p" in combo)
    got = []
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        if "p" in combo:
            q["phase"] = 0.0
        got.append(RQ.log_likelihood_ratio(dets, src, roq, q, marg))
    ref = z["lnl_" + combo]
    assert np.all(np.abs(np.array(got) - ref) <= 1e-10 * np.maximum(1.0, np.abs(ref))), np.array(got) - ref

"""The oracle's relative-binning restatement (oracle/relbin.py) against the
values the reference's RelativeBinningGravitationalWaveTransient wrote
(tests/golden/tf2_128s_relbin.npz): same data, bins, summary data and lnL."""
import numpy as np
import pytest

from tests.conftest import golden
from oracle import data as OD
from oracle import relbin as RB
from oracle import restate as R
from bilby_gb300.workloads import WORKLOADS, point


@pytest.fixture(scope="module")
def rb():
    w = WORKLOADS["tf2_128s"]
    dets = OD.build_workload(w)
    src = OD.source_for(w.model, w.minimum_frequency)
    return w, dets, src, RB.setup(dets, src, dict(w.injection)), golden("tf2_128s_relbin")


def test_same_data_bins_and_summary(rb):
    w, dets, src, st, z = rb
    assert np.allclose(OD.strain_checksum(dets), z["checksum"], rtol=1e-14, atol=0)
    assert np.array_equal(st.bin_inds, z["bin_inds"])
    assert np.array_equal(st.bin_freqs, z["bin_freqs"])
    for q in range(len(dets)):
        ref = z[f"summary_{q}"]
        assert np.max(np.abs(np.stack(st.summary[q]) - ref)) <= 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("combo", ["none", "p"])
def test_lnl(rb, combo):
    w, dets, src, st, z = rb
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    marg = R.Marginalization(phase="p" in combo)
    got = []
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        if "p" in combo:
            q["phase"] = 0.0
        got.append(RB.log_likelihood_ratio(dets, src, st, q, marg))
    ref = z["lnl_" + combo]
    assert np.all(np.abs(np.array(got) - ref) <= 1e-11 * np.maximum(1.0, np.abs(ref)))

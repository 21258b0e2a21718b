"""The host construction of the GPU ROQ likelihood's weights
(bilby/gw/likelihood/roq.py:736-1005: time grid, linear weights by inverse
FFTs, quadratic weights) reproduces the reference's weights for the same
seeded synthetic basis (tests/golden/tf2_marg_8s_2k_roq.npz).  No GPU."""
import numpy as np

from tests.conftest import golden
from oracle import data as OD
from oracle import restate as R
from oracle import roq_basis
from bilby_gb300.workloads import WORKLOADS


class _StrainData:
    def __init__(self, det):
        self.frequency_array = det.frequency
        self.frequency_mask = det.mask
        self.frequency_domain_strain = det.masked_strain
        self.duration = det.duration
        self.start_time = det.start_time


class _Ifo:
    def __init__(self, det, snr):
        self.name = det.name
        self.strain_data = _StrainData(det)
        self.power_spectral_density_array = det.psd
        self.minimum_frequency = 20.0
        self.maximum_frequency = 1024.0
        self.meta_data = {"optimal_SNR": snr}


class _Uniform:
    def __init__(self, lo, hi):
        self.minimum, self.maximum = lo, hi


def test_weights_match_the_reference():
    from bilby_gb300.roq import ROQGravitationalWaveTransient
    w = WORKLOADS["tf2_marg_8s_2k"]
    dets = OD.build_workload(w)
    src = OD.source_for(w.model, w.minimum_frequency)
    pols = src(dets[0].frequency, **w.injection)
    ifos = []
    for d in dets:
        s = R.detector_response(d, pols, w.injection["ra"], w.injection["dec"], w.injection["geocent_time"],
                                w.injection["psi"])
        m = d.mask
        snr = np.sqrt(R.noise_weighted_inner_product(s[m], s[m], d.psd[m], d.duration).real)
        ifos.append(_Ifo(d, snr))
    fm = dets[0].frequency[dets[0].mask]
    nl, bl, nq, bq = roq_basis.build(fm, minimum_frequency=w.minimum_frequency)
    like = object.__new__(ROQGravitationalWaveTransient)
    like.interferometers = ifos
    tc = w.injection["geocent_time"]
    like._prior = {"geocent_time": _Uniform(tc - 0.1, tc + 0.1)}
    like.time_reference = "geocent"
    like.roq_params = None
    like.roq_scale_factor = 1
    like.weights = {}
    like._set_weights(like._parse_basis(bl.T, "linear"), like._parse_basis(bq.T, "quadratic"))
    z = golden("tf2_marg_8s_2k_roq")
    ts = like.weights["time_samples"]
    t0, dt, n = z["roq_time_meta"]
    assert len(ts) == int(n) and ts[0] == t0 and ts[1] - ts[0] == dt
    for q, ifo in enumerate(ifos):
        lin = like.weights[ifo.name + "_linear"][0][z[f"roq_linear_rows_{q}"]]
        ref = z[f"roq_linear_{q}"]
        assert np.max(np.abs(lin - ref)) <= 1e-10 * np.max(np.abs(ref))
        quad = like.weights[ifo.name + "_quadratic"][0]
        assert np.max(np.abs(quad - z[f"roq_quadratic_{q}"])) <= 1e-12 * np.max(np.abs(quad))

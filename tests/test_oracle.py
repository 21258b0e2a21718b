"""The oracle pinned against the reference's golden values (CPU only)."""
import json
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN, golden
from bilby_gb300.workloads import WORKLOADS, point
from oracle import data as OD
from oracle import restate as R


def test_known_answer_noise_log_likelihood():
    """test/gw/likelihood_test.py:195-201: H1, 4 s at 2048 Hz, seed 500."""
    dets = OD.build_detectors(["H1"], 2048.0, 4.0, 0.0, 500)
    nll = R.noise_log_likelihood(dets)
    assert nll == pytest.approx(-4014.1787704539474, rel=1e-13, abs=0)
    ka = json.load(open(os.path.join(GOLDEN, "known_answer.json")))
    assert nll == pytest.approx(ka["H1_seed500_4s_2048Hz_noise_log_likelihood"], rel=1e-13, abs=0)


def test_ln_i0_matches_scipy():
    """test/gw/utils_test.py:349-352."""
    from scipy.special import i0
    values = np.linspace(-10, 10, 101)
    assert np.max(np.abs(R.ln_i0(values) - np.log(i0(values)))) < 1e-10


@pytest.mark.parametrize("name", ["sg_4s", "tf2_128s"])
def test_oracle_regenerates_the_reference_data(name):
    w = WORKLOADS[name]
    z = golden(name)
    dets = OD.build_workload(w)
    assert np.allclose(OD.strain_checksum(dets), z["checksum"], rtol=1e-13, atol=0)
    assert R.noise_log_likelihood(dets) == pytest.approx(float(z["noise_lnl"]), rel=1e-13, abs=0)


@pytest.mark.parametrize("name", ["sg_4s", "tf2_128s"])
def test_oracle_matches_reference_log_likelihood_ratio(name):
    w = WORKLOADS[name]
    z = golden(name)
    dets = OD.build_workload(w)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    src = OD.source_for(w.model, w.minimum_frequency)
    n = len(z["lnl"]) if name == "sg_4s" else 4
    for i in range(n):
        p = point(params, i)
        got = R.log_likelihood_ratio(dets, src, p)
        scale = R.parity_scale(*R.plain_terms(dets, src, p))
        assert abs(got - z["lnl"][i]) <= 1e-12 * scale


@pytest.mark.parametrize("name", ["tf2_marg_8s_2k", "tf2_marg_8s", "tf2_marg_6s_2k"])
def test_oracle_time_and_phase_marginalization_matches_reference(name):
    """The reference's time / phase / time+phase marginalised values at FFT
    lengths 8192 and 16384."""
    w = WORKLOADS[name]
    z = golden(w.name)
    dets = OD.build_workload(w)
    assert np.allclose(OD.strain_checksum(dets), z["checksum"], rtol=1e-13, atol=0)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    src = OD.source_for(w.model, w.minimum_frequency)
    tc = w.injection["geocent_time"]
    for combo in ("t", "p", "tp"):
        m = R.Marginalization(time="t" in combo, phase="p" in combo)
        if m.time:
            R.setup_time_marginalization(m, w.start_time, w.duration, w.sampling_frequency, tc - 0.1, tc + 0.1)
        t_min, t_max = tc - 0.1, tc + 0.1
        # Uniform.prob (core/prior/analytical.py:231-242) divides by max - min at GPS magnitude
        prior = lambda t: ((t >= t_min) & (t <= t_max)) / (t_max - t_min)  # noqa: E731
        for i in range(len(params["mass_1"])):
            q = point(params, i)
            if m.time:
                q["geocent_time"] = w.start_time
            if m.phase:
                q["phase"] = 0.0
            got = R.log_likelihood_ratio(dets, src, q, m, prior)
            ref = z["lnl_" + combo][i]
            assert abs(got - ref) <= 1e-10 * max(1.0, abs(ref)), (combo, i, got, ref)


def test_oracle_geometry_is_bilbys():
    """Vertex and detector tensor of H1 computed by the restated formulas
    equal the values the package's detector module computes."""
    from bilby_gb300.detector import get_empty_interferometer
    for name in ("H1", "L1", "V1"):
        v, t = R.detector_geometry(name)
        ifo = get_empty_interferometer(name)
        assert np.allclose(ifo.geometry.vertex, v, rtol=1e-15, atol=0)
        assert np.allclose(ifo.geometry.detector_tensor, t, rtol=1e-14, atol=1e-16)


def test_oracle_time_prior_other_than_uniform_matches_reference():
    """The reference's time-marginalised values under a TruncatedGaussian
    geocent_time prior (tests/golden/tf2_marg_8s_2k_time_prior.npz)."""
    from bilby_gb300.prior import TruncatedGaussian
    w = WORKLOADS["tf2_marg_8s_2k"]
    z = golden("tf2_marg_8s_2k_time_prior")
    dets = OD.build_workload(w)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    src = OD.source_for(w.model, w.minimum_frequency)
    tc = w.injection["geocent_time"]
    prior = TruncatedGaussian(tc + 0.02, 0.04, tc - 0.1, tc + 0.1)
    for combo in ("t", "tp"):
        m = R.Marginalization(time=True, phase="p" in combo)
        R.setup_time_marginalization(m, w.start_time, w.duration, w.sampling_frequency, tc - 0.1, tc + 0.1)
        for i in range(len(params["mass_1"])):
            q = point(params, i)
            q["geocent_time"] = w.start_time
            if m.phase:
                q["phase"] = 0.0
            got = R.log_likelihood_ratio(dets, src, q, m, prior.prob)
            ref = z["lnl_" + combo][i]
            assert abs(got - ref) <= 1e-10 * max(1.0, abs(ref)), (combo, i, got, ref)


def test_time_prior_table_interpolates_the_density():
    """The kernels' 4-node Lagrange interpolation (restated here in numpy) of
    the table from time_prior_table reproduces the prior's density at any
    time of the window to 1e-10 relative, reads nodes exactly, and the node
    times are exact multiples of a power-of-two step."""
    from bilby_gb300.likelihood import time_prior_table
    from bilby_gb300.prior import Gaussian, TruncatedGaussian, Uniform
    tc, dtc = 1126259646.0, 2.0 / 4096
    assert time_prior_table(Uniform(tc - 0.1, tc + 0.1), tc - 4, tc + 4, dtc) is None
    for prior in (TruncatedGaussian(tc + 0.02, 0.04, tc - 0.1, tc + 0.1), Gaussian(tc, 0.5)):
        dens, t0, h = time_prior_table(prior, tc - 6, tc + 2, dtc)
        assert np.log2(h) == np.floor(np.log2(h)) and h <= dtc / 8 and t0 % h == 0.0
        n = len(dens)
        lo = max(prior.minimum, tc - 6)
        hi = min(prior.maximum, tc + 2)
        t = np.concatenate([np.random.default_rng(0).uniform(lo, hi, 2000), [lo, hi, t0 + 7 * h]])
        x = (t - t0) / h
        g = np.clip(np.floor(x).astype(np.int64) - 1, 0, n - 4)
        u = x - g
        p = [dens[g + q] for q in range(4)]
        v = (p[3] * u * (u - 1) * (u - 2) - p[0] * (u - 1) * (u - 2) * (u - 3)) / 6 \
            + (p[1] * u * (u - 2) * (u - 3) - p[2] * u * (u - 1) * (u - 3)) / 2
        ref = prior.prob(t)
        assert np.max(np.abs(v - ref) / ref) < 1e-10
        assert v[-1] == dens[7]

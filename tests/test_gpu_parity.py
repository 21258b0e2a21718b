"""Parity of the CUDA likelihood with the oracle (numpy restatement of the
reference) and with the reference's own golden values, on identical seeded
data, through the C ABI.

Tolerances (written here, used below):
* plain float64 kernels: |dlnL| <= 1e-9 * max(1, |Re<d|h>|, <h|h>/2);
* mixed-precision kernels: |dlnL| <= 1e-3 against the float64 oracle, for
  every point, templates far louder than the data included (their error
  control recomputes a point in float64 when its bound exceeds the tolerance).
"""
import numpy as np
import pytest

from tests.conftest import golden
from tests.gpu_helpers import (FP64_RTOL, MIXED_ATOL, WORKLOADS, device_analysis, draw_points, oracle_plain,
                               oracle_plain_pool, params_block, small_workload)
from oracle import data as OD

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg(gpu):
    w = WORKLOADS["sg_4s"]
    dets = OD.build_workload(w)
    return w, dets, device_analysis(dets, "sinegaussian", w)


@pytest.fixture(scope="module")
def tf2(gpu):
    w = WORKLOADS["tf2_128s"]
    dets = OD.build_workload(w)
    return w, dets, device_analysis(dets, "taylorf2", w)


@pytest.fixture(scope="module")
def tf2_small(gpu):
    # H1/L1/V1, 8 s at 2048 Hz, the 1-2 Msun TaylorF2 population
    w = small_workload("tf2_128s", sampling_frequency=2048.0, duration=8.0,
                       injection=dict(WORKLOADS["tf2_128s"].injection, geocent_time=WORKLOADS["tf2_128s"].start_time + 6.0))
    dets = OD.build_workload(w)
    return w, dets, device_analysis(dets, "taylorf2", w)


def test_noise_log_likelihood(sg, tf2):
    for w, dets, an in (sg, tf2):
        from oracle import restate as R
        ref = R.noise_log_likelihood(dets)
        assert abs(an.noise_log_likelihood() - ref) <= 1e-12 * abs(ref)
        assert abs(an.noise_log_likelihood() - float(golden(w.name)["noise_lnl"])) <= 1e-12 * abs(ref)


def test_known_answer_noise(gpu):
    """test/gw/likelihood_test.py:195-201: H1, 4 s at 2048 Hz, seed 500."""
    dets = OD.build_detectors(["H1"], 2048.0, 4.0, 0.0, 500)
    w = small_workload("sg_4s", detectors=("H1",), start_time=0.0)
    an = device_analysis(dets, "sinegaussian", w)
    assert an.noise_log_likelihood() == pytest.approx(-4014.1787704539474, rel=1e-12, abs=0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sine_gaussian_vs_reference_golden(sg, precision):
    w, dets, an = sg
    z = golden(w.name)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    got = an.log_likelihood_ratio_host(params_block(params), precision)
    ref = z["lnl"]
    _, scale = oracle_plain(dets, w, params, range(len(ref)))
    if precision == "fp64":
        assert np.all(np.abs(got - ref) <= FP64_RTOL * scale), np.max(np.abs(got - ref) / scale)
    else:
        assert np.all(np.abs(got - ref) <= MIXED_ATOL), np.abs(got - ref)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sine_gaussian_many_points(sg, precision):
    w, dets, an = sg
    params = draw_points(w, 300, np.random.default_rng(11))
    got = an.log_likelihood_ratio_host(params_block(params), precision)
    idx = range(0, 300, 3)
    ref, scale = oracle_plain(dets, w, params, idx)
    g = got[list(idx)]
    if precision == "fp64":
        assert np.all(np.abs(g - ref) <= FP64_RTOL * scale), np.max(np.abs(g - ref) / scale)
    else:
        assert np.max(np.abs(g - ref)) <= MIXED_ATOL, np.max(np.abs(g - ref))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_taylorf2_full_size_vs_reference_golden(tf2, precision):
    """128 s at 4096 Hz (262145 bins), H1/L1/V1: the reference's own lnL."""
    w, dets, an = tf2
    z = golden(w.name)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    got = an.log_likelihood_ratio_host(params_block(params), precision)
    ref = z["lnl"]
    _, scale = oracle_plain(dets, w, params, range(len(ref)))
    if precision == "fp64":
        assert np.all(np.abs(got - ref) <= FP64_RTOL * scale), np.max(np.abs(got - ref) / scale)
    else:
        assert np.max(np.abs(got - ref)) <= MIXED_ATOL, np.abs(got - ref)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_taylorf2_small_many_points(tf2_small, precision):
    w, dets, an = tf2_small
    params = draw_points(w, 200, np.random.default_rng(5))
    # put half the points on the injection so that <d|h> is large
    for k in ("mass_1", "mass_2", "chi_1", "chi_2", "luminosity_distance", "theta_jn", "phase", "ra", "dec", "psi",
              "geocent_time"):
        params[k][:100] = w.injection[k] + (params[k][:100] - params[k][:100].mean()) * 1e-4
    got = an.log_likelihood_ratio_host(params_block(params), precision)
    idx = list(range(0, 200, 5))
    ref, scale = oracle_plain(dets, w, params, idx)
    g = got[idx]
    assert np.max(np.abs(ref[:20])) > 10.0  # the injected points carry signal
    if precision == "fp64":
        assert np.all(np.abs(g - ref) <= FP64_RTOL * scale), np.max(np.abs(g - ref) / scale)
    else:
        assert np.max(np.abs(g - ref)) <= MIXED_ATOL, np.max(np.abs(g - ref))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_independence(tf2_small, precision):
    """A point's result does not depend on the batch it is evaluated in."""
    w, dets, an = tf2_small
    params = draw_points(w, 333, np.random.default_rng(9))
    block = params_block(params)
    full = an.log_likelihood_ratio_host(block, precision)
    for i in (0, 127, 128, 332):
        alone = an.log_likelihood_ratio_host(block[:, i:i + 1], precision)
        assert alone[0] == full[i]
    sub = an.log_likelihood_ratio_host(block[:, 100:229], precision)
    assert np.array_equal(sub, full[100:229])


def test_invalid_points_return_nan_to_num_minus_inf(tf2_small):
    """base.py:424-425: an undefined waveform gives np.nan_to_num(-np.inf)."""
    w, dets, an = tf2_small
    params = draw_points(w, 4, np.random.default_rng(1))
    params["mass_1"][1] = -1.0
    params["luminosity_distance"][2] = np.nan
    for precision in ("fp64", "mixed"):
        got = an.log_likelihood_ratio_host(params_block(params), precision)
        assert got[1] == np.nan_to_num(-np.inf) and got[2] == np.nan_to_num(-np.inf)
        assert np.isfinite(got[0]) and np.isfinite(got[3])


def test_source_polarizations_match_oracle(gpu):
    from bilby_gb300 import _capi
    from oracle import restate as R
    from oracle.taylorf2 import taylorf2_aligned
    f = np.linspace(0, 1024, 4097)
    p = params_block(dict(hrss=1e-22, Q=9.0, frequency=200.0))[:, 0]
    plus, cross = _capi.source_polarizations(_capi.MODEL_SINEGAUSSIAN, f, p)
    ref = R.sinegaussian(f, 1e-22, 9.0, 200.0)
    assert np.allclose(plus, ref["plus"], rtol=1e-12, atol=0)
    assert np.allclose(cross, ref["cross"], rtol=1e-12, atol=0)
    q = dict(mass_1=1.5, mass_2=1.3, chi_1=0.02, chi_2=-0.01, luminosity_distance=100.0, theta_jn=0.4, phase=1.3)
    plus, cross = _capi.source_polarizations(_capi.MODEL_TAYLORF2, f, params_block(q)[:, 0], 20.0)
    ref = taylorf2_aligned(f, **q, minimum_frequency=20.0)
    scale = np.max(np.abs(ref["plus"]))
    assert np.max(np.abs(plus - ref["plus"])) <= 1e-9 * scale
    assert np.max(np.abs(cross - ref["cross"])) <= 1e-9 * scale


@pytest.mark.parametrize("fixture", ["tf2", "sg"])
def test_mixed_at_the_injection(fixture, request):
    """The loudest points (on and around the injection, where <d|h> is
    largest) keep |dlnL| <= 1e-3 in mixed precision."""
    w, dets, an = request.getfixturevalue(fixture)
    keys = [k for k in w.injection]
    rng = np.random.default_rng(4)
    n = 16
    params = {k: np.full(n, float(w.injection[k])) for k in keys}
    params["geocent_time"] = params["geocent_time"] + rng.normal(0, 2e-4, n) * (np.arange(n) > 0)
    params["psi"] = params["psi"] + rng.normal(0, 0.05, n) * (np.arange(n) > 0)
    got = an.log_likelihood_ratio_host(params_block(params), "mixed")
    exact = an.log_likelihood_ratio_host(params_block(params), "fp64")
    ref, scale = oracle_plain(dets, w, params, range(0, n, 4))
    assert ref[0] > 20.0, ref[0]  # a loud signal
    assert np.all(np.abs(exact[::4] - ref) <= FP64_RTOL * scale)
    assert np.max(np.abs(got - exact)) <= MIXED_ATOL, np.abs(got - exact)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_staged_host_evaluation_matches(tf2_small, precision):
    """log_likelihood_ratio_staged (parameters written into the pinned staging
    buffer, gwl_eval_host_staged) gives the results of gwl_eval_host bit for
    bit, for a batch, a smaller batch after it, and a larger one."""
    w, dets, an = tf2_small
    for n in (300, 17, 700):
        p = draw_points(w, n, np.random.default_rng(60 + n))
        ref = an.log_likelihood_ratio_host(params_block(p), precision)
        got = an.log_likelihood_ratio_staged(p, precision)
        assert np.array_equal(ref, got)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sine_gaussian_all_ten_thousand_draws(sg, precision):
    """The sine-Gaussian configuration at its stated breadth: 10^4 prior draws
    (half at the injection's sky position and time, half with sky, psi and
    time drawn), every one against the oracle."""
    w, dets, an = sg
    rng = np.random.default_rng(2024)
    pf = draw_points(w, 5000, rng, fixed_extrinsic=True)
    pr = draw_points(w, 5000, rng, fixed_extrinsic=False)
    params = {k: np.concatenate([pf[k], pr[k]]) for k in pf}
    got = an.log_likelihood_ratio_host(params_block(params), precision)
    ref, scale = oracle_plain_pool(w, params, range(10000))
    if precision == "fp64":
        assert np.all(np.abs(got - ref) <= FP64_RTOL * scale), np.max(np.abs(got - ref) / scale)
    else:
        assert np.max(np.abs(got - ref)) <= MIXED_ATOL, np.max(np.abs(got - ref))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_taylorf2_full_size_512_draws(tf2, precision):
    """128 s at 4096 Hz (262145 bins), H1/L1/V1: 512 prior draws against the
    oracle."""
    w, dets, an = tf2
    params = draw_points(w, 512, np.random.default_rng(512))
    got = an.log_likelihood_ratio_host(params_block(params), precision)
    ref, scale = oracle_plain_pool(w, params, range(512))
    if precision == "fp64":
        assert np.all(np.abs(got - ref) <= FP64_RTOL * scale), np.max(np.abs(got - ref) / scale)
    else:
        assert np.max(np.abs(got - ref)) <= MIXED_ATOL, np.max(np.abs(got - ref))


def test_sine_gaussian_loud_templates_are_refined(sg):
    """Templates 10 to 100 times louder than the prior's loudest (<h|h> up to
    1e9): the error bound sends them to the float64 recomputation, and every
    mixed result stays within 1e-3 of the float64 kernel; the prior's own
    quiet draws need none."""
    w, dets, an = sg
    rng = np.random.default_rng(77)
    params = draw_points(w, 400, rng)
    params["hrss"] = 10 ** rng.uniform(-21, -19, 400)
    block = params_block(params)
    mixed = an.log_likelihood_ratio_host(block, "mixed")
    refined = an.last_refined()
    fp64 = an.log_likelihood_ratio_host(block, "fp64")
    assert refined > 0
    assert np.max(np.abs(mixed - fp64)) <= MIXED_ATOL, np.max(np.abs(mixed - fp64))
    quiet = draw_points(w, 400, np.random.default_rng(78))
    quiet["hrss"] = 10 ** rng.uniform(-23, -22, 400)
    an.log_likelihood_ratio_host(params_block(quiet), "mixed")
    assert an.last_refined() == 0

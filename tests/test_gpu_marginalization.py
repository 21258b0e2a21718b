"""Marginalised likelihoods on the GPU against the reference's own values
(tests/golden/tf2_marg_8s_2k.npz at 8 s and 2048 Hz, FFT length 8192, and
tests/golden/tf2_marg_8s.npz at 8 s and 4096 Hz, FFT length 16384; generated
by the reference with the oracle's TaylorF2 as its source model) and against
brute-force integrals of the
non-marginalised likelihood (the pattern of the reference's
test/gw/likelihood/marginalization_test.py:383-430).

Tolerances: float64 kernels |dlnL| <= 1e-8 * max(1, |lnL|); mixed precision
|dlnL| <= 1e-3.
"""
import numpy as np
import pytest

from tests.conftest import golden
from bilby_gb300.workloads import DISTANCE_PRIOR, WORKLOADS, point

pytestmark = pytest.mark.gpu

COMBOS = ["t", "p", "d", "tp", "td", "pd", "tpd"]


def make_likelihood(w, combo, precision, table_path, time_prior=None):
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.likelihood import GravitationalWaveTransient
    from bilby_gb300.prior import PowerLaw, Uniform
    from bilby_gb300.source import taylorf2_aligned
    from bilby_gb300.waveform_generator import WaveformGenerator
    grandom.seed(w.seed)
    ifos = InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=taylorf2_aligned,
                            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
    ifos.inject_signal(waveform_generator=wfg, parameters=dict(w.injection))
    tc = w.injection["geocent_time"]
    priors = {}
    if "t" in combo or time_prior is not None:
        priors["geocent_time"] = time_prior if time_prior is not None else Uniform(tc - 0.1, tc + 0.1)
    if "p" in combo:
        priors["phase"] = Uniform(0, 2 * np.pi, boundary="periodic")
    if "d" in combo:
        priors["luminosity_distance"] = PowerLaw(DISTANCE_PRIOR["alpha"], DISTANCE_PRIOR["minimum"],
                                                 DISTANCE_PRIOR["maximum"])
    like = GravitationalWaveTransient(ifos, wfg, priors=priors, time_marginalization="t" in combo or time_prior is not None,
                                      phase_marginalization="p" in combo, distance_marginalization="d" in combo,
                                      distance_marginalization_lookup_table=str(table_path), precision=precision)
    return like, priors


def golden_points(w, priors, combo):
    z = golden(w.name)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    pts = []
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        if "t" in combo:
            q["geocent_time"] = float(priors["geocent_time"])
        if "p" in combo:
            q["phase"] = 0.0
        if "d" in combo:
            q["luminosity_distance"] = float(priors["luminosity_distance"])
        if "t" not in combo:
            q.pop("time_jitter")
        pts.append(q)
    return pts, z["lnl_" + combo]


@pytest.mark.parametrize("workload", ["tf2_marg_8s_2k", "tf2_marg_8s", "tf2_marg_6s_2k"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("combo", COMBOS)
def test_marginalized_vs_reference_golden(gpu, tmp_path, combo, precision, workload):
    w = WORKLOADS[workload]
    like, priors = make_likelihood(w, combo, precision, tmp_path / "table.npz")
    pts, ref = golden_points(w, priors, combo)
    single = np.array([like.log_likelihood_ratio(q) for q in pts])
    batch = like.log_likelihood_ratio_batch({k: np.array([q[k] for q in pts]) for k in pts[0]})
    assert np.array_equal(single, batch)
    if precision == "fp64":
        tol = 1e-8 * np.maximum(1.0, np.abs(ref))
        assert np.all(np.abs(single - ref) <= tol), (combo, single - ref)
    else:
        assert np.max(np.abs(single - ref)) <= 1e-3, (combo, single - ref)


def test_priors_mutated_like_the_reference(gpu, tmp_path):
    """base.py:183-223: marginalised parameters are fixed in the caller's dict."""
    w = WORKLOADS["tf2_marg_8s_2k"]
    like, priors = make_likelihood(w, "tpd", "fp64", tmp_path / "table.npz")
    assert priors["geocent_time"] == w.start_time
    assert priors["phase"] == 0.0
    assert isinstance(priors["luminosity_distance"], float)
    assert "time_jitter" in priors
    assert like.marginalized_parameters == ["geocent_time", "phase", "luminosity_distance"]
    # the cached table is reused by a second likelihood with the same prior
    like2, _ = make_likelihood(w, "tpd", "fp64", tmp_path / "table.npz")
    assert np.array_equal(like2._dist_margd_loglikelihood_array, like._dist_margd_loglikelihood_array)


def test_distance_table_matches_the_reference_construction(gpu):
    """base.py:994-1018 restated row by row for a subset of rows."""
    from scipy.special import logsumexp
    from bilby_gb300 import _capi
    from bilby_gb300.likelihood import d_inner_h_ref_axis, optimal_snr_squared_ref_axis
    from bilby_gb300.prior import PowerLaw
    prior = PowerLaw(2.0, 100.0, 5000.0)
    dist = np.linspace(prior.minimum, prior.maximum, 10000)
    parr = np.array([prior.prob(d) for d in dist])
    ref_dist = prior.rescale(0.5)
    for phase in (False, True):
        table = _capi.distance_lookup_table(dist, parr, ref_dist, phase)
        scaling = ref_dist / dist
        dh = np.outer(d_inner_h_ref_axis(800, phase), scaling)
        if phase:
            from scipy.special import i0e
            dh = np.log(i0e(np.abs(dh))) + np.abs(dh)
        hh = np.outer(optimal_snr_squared_ref_axis(400), scaling ** 2)
        dd = dist[1] - dist[0]
        log_norm = logsumexp(0 / dist, b=parr * dd)
        for ii in (0, 57, 199, 311, 399):
            row = logsumexp(dh - hh[ii] / 2, b=parr * dd, axis=-1) - log_norm
            assert np.allclose(table[ii], row, rtol=1e-12, atol=1e-9), (phase, ii)


def test_phase_marginalization_vs_brute_force(gpu, tmp_path):
    """ln of the phase-averaged likelihood equals the marginalised value."""
    w = WORKLOADS["tf2_marg_8s_2k"]
    plain, _ = make_likelihood(w, "", "fp64", tmp_path / "t0.npz")
    marg, _ = make_likelihood(w, "p", "fp64", tmp_path / "t1.npz")
    z = golden(w.name)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    params.pop("time_jitter")
    # the injection itself, where the likelihood is large
    params = {k: np.r_[v, w.injection[k]] for k, v in params.items()}
    phases = np.linspace(0, 2 * np.pi, 1001)[:-1]
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        batch = {k: np.full(len(phases), v) for k, v in q.items()}
        batch["phase"] = phases
        lnl = plain.log_likelihood_ratio_batch(batch)
        brute = np.log(np.mean(np.exp(lnl - lnl.max()))) + lnl.max()
        q["phase"] = 0.0
        assert abs(marg.log_likelihood_ratio(q) - brute) < 1e-6 * max(1.0, abs(brute))


@pytest.mark.parametrize("combo", ["t", "tp", "tpd"])
def test_mixed_time_marginalized_matches_float64_fft16384(gpu, tmp_path, combo):
    """The mixed time-marginalised kernel at FFT length 16384 (8 s at 4096 Hz:
    an even number of stages, a radix-4 last pass pruned to the prior window)
    against the float64 kernel on 96 prior draws: |dlnL| <= 1e-3."""
    from bilby_gb300.workloads import draw_points
    w = WORKLOADS["tf2_marg_8s"]
    like, priors = make_likelihood(w, combo, "mixed", tmp_path / "table.npz")
    p = draw_points(w, 96, np.random.default_rng(71))
    p["geocent_time"] = np.full(96, float(priors["geocent_time"]))
    if "p" in combo:
        p["phase"] = np.zeros(96)
    if "d" in combo:
        p["luminosity_distance"] = np.full(96, float(priors["luminosity_distance"]))
    mixed = like.log_likelihood_ratio_batch(p, precision="mixed")
    fp64 = like.log_likelihood_ratio_batch(p, precision="fp64")
    assert np.all(np.abs(mixed - fp64) <= 1e-3), np.abs(mixed - fp64).max()


@pytest.mark.parametrize("combo", ["t", "tpd"])
def test_mixed_time_marginalized_error_control_on_loud_templates(gpu, tmp_path, combo):
    """Loud templates (the injection's masses and sky position at 20-800 Mpc,
    |<d|h>| up to 3e4), where the float32 transform alone errs by up to 6e-3:
    the mixed kernel marks the points over its error bound, the windowed
    float64 kernel recomputes them (split over CTAs), and every result is
    within 1e-3 of the float64 kernel's; with the control off the marks
    vanish."""
    w = WORKLOADS["tf2_marg_8s"]
    like, priors = make_likelihood(w, combo, "mixed", tmp_path / "table.npz")
    rng = np.random.default_rng(73)
    n = 1024
    p = {k: np.full(n, float(v)) for k, v in w.injection.items()}
    p["luminosity_distance"] = rng.uniform(20.0, 800.0, n)
    p["theta_jn"] = rng.uniform(0.0, np.pi, n)
    p["geocent_time"] = np.full(n, float(priors["geocent_time"]))
    p["time_jitter"] = rng.uniform(-1 / w.sampling_frequency, 1 / w.sampling_frequency, n)
    if "p" in combo:
        p["phase"] = np.zeros(n)
    if "d" in combo:
        p["luminosity_distance"] = np.full(n, float(priors["luminosity_distance"]))
    mixed = like.log_likelihood_ratio_batch(p, precision="mixed")
    refined = like.analysis.last_refined()
    fp64 = like.log_likelihood_ratio_batch(p, precision="fp64")
    assert np.all(np.abs(mixed - fp64) <= 1e-3), np.abs(mixed - fp64).max()
    if combo == "t":
        assert refined > 0
    like.analysis.refinement_tolerance = 0.0
    like.log_likelihood_ratio_batch(p, precision="mixed")
    assert like.analysis.last_refined() == 0


def test_mixed_time_marginalized_sine_gaussian(gpu, tmp_path):
    """Time marginalisation of the sine-Gaussian in mixed precision (the
    full-band integrand, the padded buffer, radix-16 passes and the pruned last
    pass; <h|h> in float-float from the mixed sine-Gaussian pass) against
    float64 on 64 draws (4 s at 2048 Hz, FFT length 4096): |dlnL| <= 1e-3."""
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.likelihood import GravitationalWaveTransient
    from bilby_gb300.prior import Uniform
    from bilby_gb300.source import sinegaussian
    from bilby_gb300.waveform_generator import WaveformGenerator
    from bilby_gb300.workloads import draw_points
    w = WORKLOADS["sg_4s"]
    grandom.seed(w.seed)
    ifos = InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=sinegaussian)
    ifos.inject_signal(waveform_generator=wfg, parameters=dict(w.injection))
    tc = w.injection["geocent_time"]
    priors = {"geocent_time": Uniform(tc - 0.1, tc + 0.1)}
    like = GravitationalWaveTransient(ifos, wfg, priors=priors, time_marginalization=True, precision="mixed")
    p = draw_points(w, 64, np.random.default_rng(73))
    p["geocent_time"] = np.full(64, float(priors["geocent_time"]))
    mixed = like.log_likelihood_ratio_batch(p, precision="mixed")
    fp64 = like.log_likelihood_ratio_batch(p, precision="fp64")
    assert np.all(np.abs(mixed - fp64) <= 1e-3), np.abs(mixed - fp64).max()


def test_concurrent_analyses_of_different_fft_lengths(gpu, tmp_path):
    """Two time-marginalised analyses of different FFT lengths (8192 and 4096)
    evaluated at the same time from two host threads give the values they give
    one after the other: each length keeps its own twiddle tables."""
    import threading
    from dataclasses import replace
    w8 = WORKLOADS["tf2_marg_8s_2k"]
    w4 = replace(w8, duration=4.0, start_time=w8.injection["geocent_time"] - 3.0)
    likes = []
    for w, sub in ((w8, "a"), (w4, "b")):
        (tmp_path / sub).mkdir()
        like, priors = make_likelihood(w, "tpd", "mixed", tmp_path / sub / "table.npz")
        z = golden(w8.name)
        params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
        params["geocent_time"] = np.full(len(params["mass_1"]), float(priors["geocent_time"]))
        params["phase"] = np.zeros(len(params["mass_1"]))
        params["luminosity_distance"] = np.full(len(params["mass_1"]), float(priors["luminosity_distance"]))
        likes.append((like, params))
    for precision in ("fp64", "mixed"):
        alone = [like.log_likelihood_ratio_batch(p, precision=precision) for like, p in likes]
        results = [[], []]

        def work(k):
            like, p = likes[k]
            for _ in range(20):
                results[k].append(like.log_likelihood_ratio_batch(p, precision=precision))

        threads = [threading.Thread(target=work, args=(k,)) for k in range(2)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for k in range(2):
            assert all(np.array_equal(r, alone[k]) for r in results[k]), (precision, k)


@pytest.mark.parametrize("combo", ["t", "tp"])
def test_sine_gaussian_marginalized_vs_reference_golden(gpu, tmp_path, combo):
    """The sine-Gaussian burst with time (and phase) marginalisation against
    the reference's values (tests/golden/sg_4s_marg.npz).  float64: 1e-8
    relative; mixed: 1e-3."""
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.likelihood import GravitationalWaveTransient
    from bilby_gb300.prior import Uniform
    from bilby_gb300.source import sinegaussian
    from bilby_gb300.waveform_generator import WaveformGenerator
    w = WORKLOADS["sg_4s"]
    z = golden("sg_4s_marg")
    for precision in ("fp64", "mixed"):
        grandom.seed(w.seed)
        ifos = InterferometerList(list(w.detectors))
        ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
        wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency,
                                start_time=w.start_time, frequency_domain_source_model=sinegaussian)
        ifos.inject_signal(waveform_generator=wfg, parameters=dict(w.injection))
        tc = w.injection["geocent_time"]
        priors = {"geocent_time": Uniform(tc - 0.1, tc + 0.1)}
        if "p" in combo:
            priors["phase"] = Uniform(0, 2 * np.pi, boundary="periodic")
        like = GravitationalWaveTransient(ifos, wfg, priors=priors, time_marginalization=True,
                                          phase_marginalization="p" in combo, precision=precision)
        params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
        n = len(params["hrss"])
        params["geocent_time"] = np.full(n, float(priors["geocent_time"]))
        if "p" in combo:
            params["phase"] = np.zeros(n)
        got = like.log_likelihood_ratio_batch(params)
        ref = z["lnl_" + combo]
        if precision == "fp64":
            assert np.all(np.abs(got - ref) <= 1e-8 * np.maximum(1.0, np.abs(ref))), got - ref
        else:
            assert np.all(np.abs(got - ref) <= 1e-3), got - ref


@pytest.mark.parametrize("combo", ["t", "d"])
def test_time_and_distance_marginalization_vs_brute_force(gpu, tmp_path, combo):
    """The pattern of the reference's marginalization_test.py:383-430: the
    marginalised lnL equals the log of the prior-weighted sum of the plain
    likelihood over a grid of the marginalised parameter (time: the
    marginalisation's own time samples; distance: the lookup table's
    distance grid), to the reference's delta of 0.5 (the plain likelihood on
    the time grid also moves the antenna patterns with the time)."""
    from scipy.special import logsumexp
    w = WORKLOADS["tf2_marg_8s_2k"]
    plain, _ = make_likelihood(w, "", "fp64", tmp_path / "t0.npz")
    marg, priors = make_likelihood(w, combo, "fp64", tmp_path / "t1.npz")
    z = golden(w.name)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    params.pop("time_jitter")
    params = {k: np.r_[v[:4], w.injection[k]] for k, v in params.items()}
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        if combo == "t":
            tp = marg.priors["geocent_time"]
            times = marg._times[(marg._times >= tp.minimum) & (marg._times <= tp.maximum)]
            grid = {k: np.full(len(times), v) for k, v in q.items()}
            grid["geocent_time"] = times
            brute = logsumexp(plain.log_likelihood_ratio_batch(grid), b=tp.prob(times) * marg._delta_tc)
            q["geocent_time"] = float(priors["geocent_time"])
            q["time_jitter"] = 0.0
        else:
            dist = marg._distance_array
            grid = {k: np.full(len(dist), v) for k, v in q.items()}
            grid["luminosity_distance"] = dist
            brute = logsumexp(plain.log_likelihood_ratio_batch(grid), b=marg.distance_prior_array * marg._delta_distance)
            q["luminosity_distance"] = float(priors["luminosity_distance"])
        got = marg.log_likelihood_ratio(q)
        assert abs(got - brute) < 0.5, (combo, i, got, brute)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("combo", ["t", "tp", "td", "tpd"])
def test_time_prior_other_than_uniform_vs_reference(gpu, tmp_path, combo, precision):
    """Time marginalisation under a TruncatedGaussian geocent_time prior (each
    jittered time sample weighted by prior(t) delta_tc, base.py:794-820)
    against the reference's values (tests/golden/tf2_marg_8s_2k_time_prior.npz):
    float64 |dlnL| <= 1e-8 max(1, |lnL|), mixed |dlnL| <= 1e-3."""
    from bilby_gb300.prior import TruncatedGaussian
    w = WORKLOADS["tf2_marg_8s_2k"]
    z = golden("tf2_marg_8s_2k_time_prior")
    tc = w.injection["geocent_time"]
    like, priors = make_likelihood(w, combo.replace("t", ""), precision, tmp_path / "table.npz",
                                   time_prior=TruncatedGaussian(tc + 0.02, 0.04, tc - 0.1, tc + 0.1))
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    n = len(params["mass_1"])
    params["geocent_time"] = np.full(n, float(priors["geocent_time"]))
    if "p" in combo:
        params["phase"] = np.zeros(n)
    if "d" in combo:
        params["luminosity_distance"] = np.full(n, float(priors["luminosity_distance"]))
    got = like.log_likelihood_ratio_batch(params)
    ref = z["lnl_" + combo]
    if precision == "fp64":
        assert np.all(np.abs(got - ref) <= 1e-8 * np.maximum(1.0, np.abs(ref))), got - ref
    else:
        assert np.max(np.abs(got - ref)) <= 1e-3, got - ref


def test_time_series_at_a_length_that_is_not_a_power_of_two(gpu):
    """The float64 transform d_inner_h_array of base.py:325-330 at FFT length
    6144 = 3 x 2048 (6 s at 2048 Hz: three radix-2 transforms of 2048 combined
    by a radix-3 step) against numpy's FFT in the oracle, summed over
    detectors, for points on and off the injection."""
    from oracle import data as OD
    from oracle import restate as R
    from tests.gpu_helpers import device_analysis, draw_points, params_block
    w = WORKLOADS["tf2_marg_6s_2k"]
    dets = OD.build_workload(w)
    an = device_analysis(dets, "taylorf2", w)
    tc = w.injection["geocent_time"]
    an.set_time_marginalization(True, False, tc - 0.1, tc + 0.1)
    p = draw_points(w, 6, np.random.default_rng(12))
    for k in ("mass_1", "mass_2", "chi_1", "chi_2", "luminosity_distance", "theta_jn", "phase", "ra", "dec", "psi",
              "geocent_time"):
        p[k][0] = w.injection[k]
    p["time_jitter"] = np.zeros(6)
    series, hh = an.time_series_host(params_block(p))
    assert series.shape == (6, 6144)
    src = OD.source_for(w.model, w.minimum_frequency)
    for i in range(6):
        q = point(p, i)
        pols = src(dets[0].frequency, **q)
        ref = sum(R.snrs(d, pols, q, True)[2] for d in dets)
        assert np.max(np.abs(series[i] - ref)) <= 1e-9 * np.max(np.abs(ref)), i
    an.close()

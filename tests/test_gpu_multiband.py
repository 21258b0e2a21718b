"""Multi-banding on the GPU against the reference's own MBGravitationalWaveTransient
(tests/golden/tf2_128s_multiband.npz, written by the reference with the
oracle's TaylorF2 as its source model): lnL ratios without marginalisation,
with phase, with distance, with time, and with time, phase and distance
marginalisation; batch equals single; the unsupported options are refused.

Tolerances: float64 |dlnL| <= 1e-9 * max(1, |lnL|) (1e-8 with the distance
table, as for the full likelihood)."""
import numpy as np
import pytest

from tests.conftest import golden
from bilby_gb300.workloads import DISTANCE_PRIOR, WORKLOADS, point

pytestmark = pytest.mark.gpu


def make(combo, tmp_path, **kw):
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.multiband import MBGravitationalWaveTransient
    from bilby_gb300.prior import PowerLaw, Uniform
    from bilby_gb300.source import taylorf2_aligned_frequency_sequence
    from bilby_gb300.waveform_generator import WaveformGenerator
    w = WORKLOADS["tf2_128s"]
    grandom.seed(w.seed)
    ifos = InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=taylorf2_aligned_frequency_sequence,
                            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
    ifos.inject_signal(waveform_generator=wfg, parameters=dict(w.injection))
    priors = {}
    if "t" in combo:
        tc = w.injection["geocent_time"]
        priors["geocent_time"] = Uniform(tc - 0.1, tc + 0.1)
    if "p" in combo:
        priors["phase"] = Uniform(0, 2 * np.pi, boundary="periodic")
    if "d" in combo:
        priors["luminosity_distance"] = PowerLaw(DISTANCE_PRIOR["alpha"], DISTANCE_PRIOR["minimum"],
                                                 DISTANCE_PRIOR["maximum"])
    like = MBGravitationalWaveTransient(ifos, wfg, reference_chirp_mass=0.87, priors=priors or None,
                                        time_marginalization="t" in combo,
                                        phase_marginalization="p" in combo, distance_marginalization="d" in combo,
                                        distance_marginalization_lookup_table=str(tmp_path / "table.npz"), **kw)
    return like, priors


@pytest.mark.parametrize("combo", ["none", "p", "d", "t", "tpd"])
def test_lnl_matches_the_reference(gpu, tmp_path, combo):
    like, priors = make(combo, tmp_path)
    z = golden("tf2_128s_multiband")
    if "t" not in combo:  # the time prior moves the bands (time_offset, multiband.py:197-225)
        assert len(like.banded_frequency_points) == len(z["mb_banded_frequency_points"])
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    pts = []
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        if "t" in combo:
            q["geocent_time"] = float(priors["geocent_time"])
            q["time_jitter"] = float(z["time_jitter"][i])
        if "p" in combo:
            q["phase"] = 0.0
        if "d" in combo:
            q["luminosity_distance"] = float(priors["luminosity_distance"])
        pts.append(q)
    ref = z["lnl_" + combo]
    single = np.array([like.log_likelihood_ratio(q) for q in pts])
    batch = like.log_likelihood_ratio_batch({k: np.array([q[k] for q in pts]) for k in pts[0]})
    assert np.array_equal(single, batch)
    rtol = 1e-8 if "d" in combo else 1e-9
    assert np.all(np.abs(single - ref) <= rtol * np.maximum(1.0, np.abs(ref))), single - ref


def test_weights_round_trip(gpu, tmp_path):
    from bilby_gb300.multiband import MBGravitationalWaveTransient
    like, _ = make("none", tmp_path)
    again = MBGravitationalWaveTransient(like.interferometers, like.waveform_generator, weights=like.weights)
    z = golden("tf2_128s_multiband")
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    a = like.log_likelihood_ratio_batch(params)
    b = again.log_likelihood_ratio_batch(params)
    assert np.array_equal(a, b)


def _golden_points(z, priors, combo):
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    pts = []
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        if "t" in combo:
            q["geocent_time"] = float(priors["geocent_time"])
            q["time_jitter"] = float(z["time_jitter"][i])
        if "p" in combo:
            q["phase"] = 0.0
        if "d" in combo:
            q["luminosity_distance"] = float(priors["luminosity_distance"])
        pts.append(q)
    return pts


@pytest.mark.parametrize("combo", ["none", "p", "t", "tpd"])
def test_ifft_fft_lnl_matches_the_reference(gpu, tmp_path, combo):
    """linear_interpolation=False: <h|h> by the IFFT-FFT sum (band 0 direct,
    even bins in the quadratic coefficients, odd bins by k_mb_hh_fft) against
    the reference's lnL (tests/golden/tf2_128s_multiband_ifft.npz), float64:
    |dlnL| <= 1e-9 max(1, |lnL|) (1e-8 with the distance table); batch equals
    single."""
    like, priors = make(combo, tmp_path, linear_interpolation=False)
    z = golden("tf2_128s_multiband_ifft")
    pts = _golden_points(z, priors, combo)
    ref = z["lnl_" + combo]
    single = np.array([like.log_likelihood_ratio(q) for q in pts])
    batch = like.log_likelihood_ratio_batch({k: np.array([q[k] for q in pts]) for k in pts[0]})
    assert np.array_equal(single, batch)
    rtol = 1e-8 if "d" in combo else 1e-9
    assert np.all(np.abs(single - ref) <= rtol * np.maximum(1.0, np.abs(ref))), single - ref


@pytest.mark.parametrize("combo", ["none", "tp", "tpd"])
def test_ifft_fft_mixed_precision_matches_float64(gpu, tmp_path, combo):
    """The mixed-precision multi-banded kernels with the IFFT-FFT <h|h> (its
    odd bins by float32 transforms with an error bound, the points over it
    recomputed in float64) against the float64 ones on 512 prior draws and
    on the golden points: |dlnL| <= 1e-3."""
    from bilby_gb300.analysis import params_block
    from bilby_gb300.workloads import draw_points
    w = WORKLOADS["tf2_128s"]
    like, priors = make(combo, tmp_path, linear_interpolation=False, precision="mixed")
    z = golden("tf2_128s_multiband_ifft")
    rng = np.random.default_rng(53)
    draws = draw_points(w, 512, rng)
    n = 512
    if "t" in combo:
        draws["geocent_time"] = np.full(n, float(priors["geocent_time"]))
        draws["time_jitter"] = rng.uniform(-1 / w.sampling_frequency, 1 / w.sampling_frequency, n)
    if "p" in combo:
        draws["phase"] = np.zeros(n)
    if "d" in combo:
        draws["luminosity_distance"] = np.full(n, float(priors["luminosity_distance"]))
    block = params_block(like._prepare(draws))
    mixed = like.analysis.log_likelihood_ratio_host(block, "mixed")
    fp64 = like.analysis.log_likelihood_ratio_host(block, "fp64")
    err = np.abs(mixed - fp64)
    assert np.all(np.isfinite(mixed)) and np.all(err <= 1e-3), (err.max(), fp64[np.argmax(err)])
    if "lnl_" + combo in z.files:
        pts = _golden_points(z, priors, combo)
        got = like.log_likelihood_ratio_batch({k: np.array([q[k] for q in pts]) for k in pts[0]})
        assert np.all(np.abs(got - z["lnl_" + combo]) <= 1e-3), got - z["lnl_" + combo]


def test_ifft_fft_mixed_refines_loud_templates(gpu, tmp_path):
    """The float32 odd-bin transforms on templates up to 10^4 times louder
    than the prior draws (5-120 Mpc, and 0.05-2 Mpc, at the injection's
    masses and sky position): the error bound sends the points it cannot
    hold to the float64 kernel, and every result stays within 1e-3 of
    float64."""
    from bilby_gb300.analysis import params_block
    w = WORKLOADS["tf2_128s"]
    like, _ = make("none", tmp_path, linear_interpolation=False, precision="mixed")
    rng = np.random.default_rng(59)
    for lo, hi in ((5.0, 120.0), (0.05, 2.0)):
        loud = {k: np.full(512, float(v)) for k, v in w.injection.items()}
        loud["luminosity_distance"] = 10 ** rng.uniform(np.log10(lo), np.log10(hi), 512)
        loud["theta_jn"] = rng.uniform(0.0, np.pi, 512)
        block = params_block(like._prepare(loud))
        mixed = like.analysis.log_likelihood_ratio_host(block, "mixed")
        fp64 = like.analysis.log_likelihood_ratio_host(block, "fp64")
        err = np.abs(mixed - fp64)
        assert np.all(np.isfinite(mixed)) and np.all(err <= 1e-3), (lo, err.max(), fp64[np.argmax(err)])


def test_ifft_fft_per_detector_snrs_sum_to_the_likelihood(gpu, tmp_path):
    """calculate_snrs per detector (one-detector analyses: the transform has
    no partner detector) gives <h|h> values whose sum is the three-detector
    analysis's <h|h> (detectors packed in pairs), and the lnL that
    compute_log_likelihood_from_snrs forms from them is the likelihood's."""
    like, priors = make("none", tmp_path, linear_interpolation=False)
    z = golden("tf2_128s_multiband_ifft")
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    from bilby_gb300.analysis import params_block
    block = params_block(like._prepare({k: np.asarray(v, dtype=float) for k, v in params.items()}))
    _, hh_all = like.analysis.inner_products_host(block, "fp64")
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        snrs = [like.calculate_snrs(None, ifo, parameters=dict(q)) for ifo in like.interferometers]
        hh = sum(float(s.optimal_snr_squared) for s in snrs)
        assert abs(hh - hh_all[i]) <= 1e-10 * max(1.0, abs(hh_all[i])), (i, hh, hh_all[i])
        dh = sum(complex(s.d_inner_h) for s in snrs)
        lnl = dh.real - hh / 2
        assert abs(lnl - z["lnl_none"][i]) <= 1e-9 * max(1.0, abs(z["lnl_none"][i])), (i, lnl, z["lnl_none"][i])


def test_ifft_fft_weights_round_trip(gpu, tmp_path):
    """The IFFT-FFT weights dictionary (Tbhats, windows, wths, hbcs, Ibcs by
    band) rebuilds a likelihood with identical results."""
    from bilby_gb300.multiband import MBGravitationalWaveTransient
    like, _ = make("none", tmp_path, linear_interpolation=False)
    weights = like.weights
    assert "quadratic_coeffs" not in weights and set(weights["Ibcs"]) == {i.name for i in like.interferometers}
    again = MBGravitationalWaveTransient(like.interferometers, like.waveform_generator, weights=weights)
    assert not again.linear_interpolation
    z = golden("tf2_128s_multiband_ifft")
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    assert np.array_equal(like.log_likelihood_ratio_batch(params), again.log_likelihood_ratio_batch(params))


@pytest.mark.parametrize("combo", ["none", "p", "d"])
def test_mixed_precision_matches_float64(gpu, tmp_path, combo):
    """The mixed-precision multi-banded kernel (float-float phase, fixed-point
    time shift, float32 products) against the float64 one on the same
    analysis: |dlnL| <= 1e-3 on the golden points and on 512 prior draws."""
    from bilby_gb300.analysis import params_block
    from bilby_gb300.workloads import draw_points
    like, priors = make(combo, tmp_path, precision="mixed")
    z = golden("tf2_128s_multiband")
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    draws = draw_points(WORKLOADS["tf2_128s"], 512, np.random.default_rng(41))
    for p in (params, draws):
        p = dict(p)
        n = len(p["mass_1"])
        if "p" in combo:
            p["phase"] = np.zeros(n)
        if "d" in combo:
            p["luminosity_distance"] = np.full(n, float(priors["luminosity_distance"]))
        block = params_block(like._prepare(p))
        mixed = like.analysis.log_likelihood_ratio_host(block, "mixed")
        fp64 = like.analysis.log_likelihood_ratio_host(block, "fp64")
        err = np.abs(mixed - fp64)
        assert np.all(err <= 1e-3), (err.max(), fp64[np.argmax(err)])


def test_mixed_precision_loud_points_run(gpu, tmp_path):
    """Templates far louder than the data (10 Mpc, well above the refinement
    bound of the full-grid kernels) go through the multi-banded mixed kernel
    without the full-grid kernels' marking and give finite results."""
    from bilby_gb300.analysis import params_block
    from bilby_gb300.workloads import draw_points
    like, _ = make("none", tmp_path, precision="mixed")
    p = draw_points(WORKLOADS["tf2_128s"], 4096, np.random.default_rng(43))
    p["luminosity_distance"] = np.full(4096, 10.0)
    block = params_block(like._prepare(p))
    mixed = like.analysis.log_likelihood_ratio_host(block, "mixed")
    assert np.all(np.isfinite(mixed))


def test_mixed_holds_1e3_and_refines_loud_templates(gpu, tmp_path):
    """The mixed-precision multi-banded kernel against the float64 one on
    prior draws and on templates 100 to 10^4 times louder (distances down to
    0.02 Mpc, <h|h> up to ~1e11): the error bound sends the loud ones to the
    float64 kernel and every result stays within 1e-3; of the prior draws
    (20-200 Mpc) at most 1% need recomputation."""
    from bilby_gb300.analysis import params_block
    from bilby_gb300.workloads import draw_points
    like, _ = make("none", tmp_path)
    an = like.analysis
    w = WORKLOADS["tf2_128s"]
    p = draw_points(w, 2000, np.random.default_rng(8))
    mixed = an.log_likelihood_ratio_host(params_block(p), "mixed")
    assert an.last_refined() <= 20
    fp64 = an.log_likelihood_ratio_host(params_block(p), "fp64")
    assert np.max(np.abs(mixed - fp64)) <= 1e-3, np.max(np.abs(mixed - fp64))
    loud = draw_points(w, 300, np.random.default_rng(9))
    loud["luminosity_distance"] = 10 ** np.random.default_rng(10).uniform(np.log10(0.02), np.log10(2.0), 300)
    mixed = an.log_likelihood_ratio_host(params_block(loud), "mixed")
    assert an.last_refined() > 0
    fp64 = an.log_likelihood_ratio_host(params_block(loud), "fp64")
    assert np.max(np.abs(mixed - fp64)) <= 1e-3, np.max(np.abs(mixed - fp64))


@pytest.mark.parametrize("combo", ["t", "tpd"])
def test_mixed_time_marginalized_matches_the_reference_and_float64(gpu, tmp_path, combo):
    """Time marginalisation in mixed precision (banded values with the exact
    fixed-point phase, windowed four-step transform in float32 with
    compensated window sums, float64 recomputation of the marked points):
    |dlnL| <= 1e-3 against the reference on the golden points, and against
    the float64 kernel on 1024 prior draws and on 1024 loud templates
    (5-120 Mpc at the injection's masses and sky position)."""
    from bilby_gb300.analysis import params_block
    from bilby_gb300.workloads import draw_points
    w = WORKLOADS["tf2_128s"]
    like, priors = make(combo, tmp_path, precision="mixed")
    z = golden("tf2_128s_multiband")
    params = {k[2:]: np.asarray(z[k], dtype=float) for k in z.files if k.startswith("p_")}
    rng = np.random.default_rng(47)

    def fix(p, jitter):
        p = dict(p)
        n = len(p["mass_1"])
        p["geocent_time"] = np.full(n, float(priors["geocent_time"]))
        p["time_jitter"] = jitter if jitter is not None else rng.uniform(-1 / w.sampling_frequency,
                                                                         1 / w.sampling_frequency, n)
        if "p" in combo:
            p["phase"] = np.zeros(n)
        if "d" in combo:
            p["luminosity_distance"] = np.full(n, float(priors["luminosity_distance"]))
        return p

    golden_pts = fix(params, np.asarray(z["time_jitter"], dtype=float))
    got = like.log_likelihood_ratio_batch(golden_pts)
    ref = z["lnl_" + combo]
    assert np.all(np.abs(got - ref) <= 1e-3), got - ref
    loud = {k: np.full(1024, float(v)) for k, v in w.injection.items()}
    loud["luminosity_distance"] = rng.uniform(5.0, 120.0, 1024)
    loud["theta_jn"] = rng.uniform(0.0, np.pi, 1024)
    for p in (fix(draw_points(w, 1024, rng), None), fix(loud, None)):
        block = params_block(like._prepare(p))
        mixed = like.analysis.log_likelihood_ratio_host(block, "mixed")
        fp64 = like.analysis.log_likelihood_ratio_host(block, "fp64")
        err = np.abs(mixed - fp64)
        assert np.all(np.isfinite(mixed))
        assert np.all(err <= 1e-3), (err.max(), fp64[np.argmax(err)])


def test_split_recomputation_equals_float64(gpu, tmp_path):
    """Every point marked (tolerance 1e-12) and recomputed by the split
    float64 recomputation: equal to the float64 kernel's results to rounding."""
    from bilby_gb300.analysis import params_block
    from bilby_gb300.workloads import draw_points
    w = WORKLOADS["tf2_128s"]
    like, priors = make("t", tmp_path, precision="mixed")
    rng = np.random.default_rng(29)
    p = draw_points(w, 8, rng)
    p["geocent_time"] = np.full(8, float(priors["geocent_time"]))
    p["time_jitter"] = rng.uniform(-1 / w.sampling_frequency, 1 / w.sampling_frequency, 8)
    block = params_block(like._prepare(p))
    like.analysis.refinement_tolerance = 1e-12
    mixed = like.analysis.log_likelihood_ratio_host(block, "mixed")
    assert like.analysis.last_refined() == 8
    fp64 = like.analysis.log_likelihood_ratio_host(block, "fp64")
    assert np.all(np.abs(mixed - fp64) <= 1e-10 * np.maximum(1.0, np.abs(fp64))), mixed - fp64

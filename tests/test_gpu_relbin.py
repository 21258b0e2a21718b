"""Relative binning on the GPU against the reference's own
RelativeBinningGravitationalWaveTransient (tests/golden/tf2_128s_relbin.npz,
written by the reference with the oracle's TaylorF2 as its source model):
the same bins and summary data, and lnL ratios without marginalisation, with
phase, with distance, with time, and with time, phase and distance
marginalisation.  Also: the relative-binning lnL agrees with the full
likelihood near the fiducial point, and batch equals single.

Tolerances: float64 |dlnL| <= 1e-9 * max(1, |lnL|) (1e-8 with the distance
table, as for the full likelihood); the mixed-precision time-marginalised
kernel (windowed four-step transform in float32, with error control) |dlnL| <=
1e-3 against the reference and against the float64 kernel."""
import numpy as np
import pytest

from tests.conftest import golden
from bilby_gb300.workloads import DISTANCE_PRIOR, WORKLOADS, point

pytestmark = pytest.mark.gpu


def make(combo, tmp_path, precision="fp64"):
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.prior import PowerLaw, Uniform
    from bilby_gb300.relative import RelativeBinningGravitationalWaveTransient
    from bilby_gb300.source import taylorf2_aligned_relative_binning
    from bilby_gb300.waveform_generator import WaveformGenerator
    w = WORKLOADS["tf2_128s"]
    grandom.seed(w.seed)
    ifos = InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=taylorf2_aligned_relative_binning,
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
    like = RelativeBinningGravitationalWaveTransient(
        ifos, wfg, fiducial_parameters=dict(w.injection), priors=priors or None,
        phase_marginalization="p" in combo, distance_marginalization="d" in combo,
        distance_marginalization_lookup_table=str(tmp_path / "table.npz"),
        time_marginalization="t" in combo, precision=precision)
    return w, ifos, wfg, like, priors


@pytest.fixture(scope="module")
def plain(gpu, tmp_path_factory):
    return make("none", tmp_path_factory.mktemp("rb"))


def test_bins_and_summary_match_the_reference(plain):
    w, ifos, wfg, like, _ = plain
    z = golden("tf2_128s_relbin")
    assert np.array_equal(like.bin_inds, z["bin_inds"])
    assert np.array_equal(like.bin_freqs, z["bin_freqs"])
    for q, ifo in enumerate(ifos):
        ours = np.stack(like.summary_data[ifo.name])
        ref = z[f"summary_{q}"]
        assert np.max(np.abs(ours - ref)) <= 1e-11 * np.max(np.abs(ref))


@pytest.mark.parametrize("combo", ["none", "p", "d", "t", "tpd"])
def test_lnl_matches_the_reference(gpu, tmp_path, combo):
    w, ifos, wfg, like, priors = make(combo, tmp_path)
    z = golden("tf2_128s_relbin")
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


def test_close_to_the_full_likelihood_near_the_fiducial(plain):
    from bilby_gb300.likelihood import GravitationalWaveTransient
    w, ifos, wfg, like, _ = plain
    full = GravitationalWaveTransient(ifos, wfg)
    inj = dict(w.injection)

    def points(scale):
        rng = np.random.default_rng(3)
        pts = {k: np.full(32, float(v)) for k, v in inj.items()}
        # mass ratio moved at fixed total mass (the ISCO cut-off stays put)
        dm = scale * inj["mass_1"] * rng.standard_normal(32)
        pts["mass_1"] = inj["mass_1"] + dm
        pts["mass_2"] = inj["mass_2"] - dm
        pts["luminosity_distance"] = inj["luminosity_distance"] * (1 + 0.1 * rng.standard_normal(32))
        pts["phase"] = inj["phase"] + 0.3 * rng.standard_normal(32)
        return pts

    # distance and phase alone leave the ratio to the fiducial constant: exact
    p0 = points(0.0)
    rb, ex = like.log_likelihood_ratio_batch(p0), full.log_likelihood_ratio_batch(p0)
    assert np.all(np.abs(rb - ex) <= 1e-8 * np.maximum(1.0, np.abs(ex))), rb - ex
    # a mass offset bends the ratio inside each bin; the interpolation error
    # shrinks with the offset (first order in the phase curvature)
    e = {}
    for scale in (1e-5, 1e-4):
        p = points(scale)
        e[scale] = np.max(np.abs(like.log_likelihood_ratio_batch(p) - full.log_likelihood_ratio_batch(p)))
    assert e[1e-5] < 0.05, e
    assert e[1e-5] < e[1e-4] / 5, e


@pytest.mark.parametrize("combo", ["t", "tpd"])
def test_mixed_time_marginalized_matches_the_reference(gpu, tmp_path, combo):
    w, ifos, wfg, like, priors = make(combo, tmp_path, precision="mixed")
    z = golden("tf2_128s_relbin")
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    n = len(params["mass_1"])
    batch = {k: np.asarray(v, dtype=float).copy() for k, v in params.items()}
    batch["geocent_time"] = np.full(n, float(priors["geocent_time"]))
    batch["time_jitter"] = np.asarray(z["time_jitter"], dtype=float)
    if "p" in combo:
        batch["phase"] = np.zeros(n)
    if "d" in combo:
        batch["luminosity_distance"] = np.full(n, float(priors["luminosity_distance"]))
    ref = z["lnl_" + combo]
    got = like.log_likelihood_ratio_batch(batch)
    assert np.all(np.abs(got - ref) <= 1e-3), got - ref


def test_mixed_time_marginalized_prior_draws_within_1e3_of_fp64(gpu, tmp_path):
    """2048 prior draws (sky, masses, spins, distance, inclination) with time,
    phase and distance marginalisation: the mixed kernel (with its refinement)
    against the float64 windowed kernel; the error bound marks few points."""
    from bilby_gb300.workloads import draw_points
    w, ifos, wfg, like, priors = make("tpd", tmp_path, precision="mixed")
    _, _, _, like64, _ = make("tpd", tmp_path, precision="fp64")
    rng = np.random.default_rng(17)
    p = draw_points(w, 2048, rng)
    p["geocent_time"] = np.full(2048, float(priors["geocent_time"]))
    p["phase"] = np.zeros(2048)
    p["luminosity_distance"] = np.full(2048, float(priors["luminosity_distance"]))
    p["time_jitter"] = rng.uniform(-1 / w.sampling_frequency, 1 / w.sampling_frequency, 2048)
    mx = like.log_likelihood_ratio_batch(p)
    refined = like.analysis.last_refined()
    f64 = like64.log_likelihood_ratio_batch(p)
    assert np.all(np.isfinite(mx))
    assert np.max(np.abs(mx - f64)) <= 1e-3, np.max(np.abs(mx - f64))
    assert refined <= 2048 // 10, refined
    # with the error control off, every point comes from the float32 kernel
    like.analysis.refinement_tolerance = 0.0
    raw = like.log_likelihood_ratio_batch(p)
    assert like.analysis.last_refined() == 0
    assert np.max(np.abs(raw - f64)) <= 1e-3, np.max(np.abs(raw - f64))


def test_split_recomputation_equals_float64(gpu, tmp_path):
    """With the tolerance at 1e-12 every point is marked and recomputed in
    float64 by the split recomputation (several CTAs per point, shares added
    in a fixed order): the results equal the float64 kernel's to rounding, and
    repeat bit for bit."""
    from bilby_gb300.workloads import draw_points
    w, ifos, wfg, like, priors = make("tpd", tmp_path, precision="mixed")
    _, _, _, like64, _ = make("tpd", tmp_path, precision="fp64")
    rng = np.random.default_rng(23)
    p = draw_points(w, 8, rng)
    p["geocent_time"] = np.full(8, float(priors["geocent_time"]))
    p["phase"] = np.zeros(8)
    p["luminosity_distance"] = np.full(8, float(priors["luminosity_distance"]))
    p["time_jitter"] = rng.uniform(-1 / w.sampling_frequency, 1 / w.sampling_frequency, 8)
    like.analysis.refinement_tolerance = 1e-12
    a = like.log_likelihood_ratio_batch(p)
    assert like.analysis.last_refined() == 8
    b = like.log_likelihood_ratio_batch(p)
    f64 = like64.log_likelihood_ratio_batch(p)
    assert np.array_equal(a, b)
    assert np.all(np.abs(a - f64) <= 1e-10 * np.maximum(1.0, np.abs(f64))), a - f64

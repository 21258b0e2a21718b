"""ROQ on the GPU against the reference's own ROQGravitationalWaveTransient
(tests/golden/tf2_marg_8s_2k_roq.npz: the reference's weights for a seeded
synthetic basis, stored for the time samples the points read, and its lnL
ratios without marginalisation, with phase, with distance, with time, and
with time, phase and distance marginalisation).  The rows of the linear
weights that were not stored are NaN, so reading any other time sample would
show.  With time marginalisation every row of the prior window is read, so
those likelihoods compute their weights from the same seeded basis.

Tolerances: float64 |dlnL| <= 1e-9 * max(1, |lnL|) (1e-8 with the distance
table, as for the full likelihood)."""
import numpy as np
import pytest

from tests.conftest import golden
from bilby_gb300.workloads import DISTANCE_PRIOR, WORKLOADS, point

pytestmark = pytest.mark.gpu


def golden_weights(z, names):
    t0, dt, n = z["roq_time_meta"]
    start = int(round(t0 / dt))
    weights = {"time_samples": np.arange(start, start + int(n)) * dt,
               "frequency_nodes_linear": [z["roq_nodes_linear"]],
               "frequency_nodes_quadratic": [z["roq_nodes_quadratic"]]}
    for q, name in enumerate(names):
        w = np.full((int(n), len(z["roq_nodes_linear"])), np.nan + 0j)
        w[z[f"roq_linear_rows_{q}"]] = z[f"roq_linear_{q}"]
        weights[name + "_linear"] = [w]
        weights[name + "_quadratic"] = [z[f"roq_quadratic_{q}"]]
    return weights


def make(combo, tmp_path, **kw):
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.prior import PowerLaw, Uniform
    from bilby_gb300.roq import ROQGravitationalWaveTransient
    from bilby_gb300.source import taylorf2_aligned_roq
    from bilby_gb300.waveform_generator import WaveformGenerator
    w = WORKLOADS["tf2_marg_8s_2k"]
    grandom.seed(w.seed)
    ifos = InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=taylorf2_aligned_roq,
                            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
    from bilby_gb300.source import taylorf2_aligned
    from bilby_gb300.waveform_generator import WaveformGenerator as WG
    inj = WG(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
             frequency_domain_source_model=taylorf2_aligned, waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
    ifos.inject_signal(waveform_generator=inj, parameters=dict(w.injection))
    tc = w.injection["geocent_time"]
    priors = {"geocent_time": Uniform(tc - 0.1, tc + 0.1)}
    if "p" in combo:
        priors["phase"] = Uniform(0, 2 * np.pi, boundary="periodic")
    if "d" in combo:
        priors["luminosity_distance"] = PowerLaw(DISTANCE_PRIOR["alpha"], DISTANCE_PRIOR["minimum"],
                                                 DISTANCE_PRIOR["maximum"])
    z = golden("tf2_marg_8s_2k_roq")
    from_basis = kw.pop("basis", False)
    if kw.pop("multiband", False):
        from oracle import roq_basis
        lin, quad = roq_basis.build_multiband(minimum_frequency=w.minimum_frequency)
        wfg.waveform_arguments.update(frequency_nodes_linear=lin["basis_linear"]["0"]["frequency_nodes"],
                                      frequency_nodes_quadratic=quad["basis_quadratic"]["0"]["frequency_nodes"])
        source = dict(linear_matrix=lin, quadratic_matrix=quad)
        z = golden("tf2_marg_8s_2k_roq_multiband")
    elif "t" in combo or from_basis:
        from oracle import roq_basis
        fm = ifos[0].frequency_array[ifos[0].frequency_mask]
        nl, bl, nq, bq = roq_basis.build(fm, minimum_frequency=w.minimum_frequency)
        wfg.waveform_arguments.update(frequency_nodes_linear=nl, frequency_nodes_quadratic=nq)
        source = dict(linear_matrix=bl.T, quadratic_matrix=bq.T)
    else:
        source = dict(weights=golden_weights(z, [i.name for i in ifos]))
    like = ROQGravitationalWaveTransient(ifos, wfg, priors, time_marginalization="t" in combo,
                                         phase_marginalization="p" in combo, distance_marginalization="d" in combo,
                                         distance_marginalization_lookup_table=str(tmp_path / "table.npz"),
                                         **source, **kw)
    return like, priors, z


@pytest.mark.parametrize("combo", ["none", "p", "d", "t", "tpd"])
def test_lnl_matches_the_reference(gpu, tmp_path, combo):
    like, priors, z = make(combo, tmp_path)
    if "t" in combo:  # the same marginalisation grid (roq.py:320-331)
        assert like._delta_tc == pytest.approx(float(z["roq_tm_delta_tc_" + combo]), rel=1e-12)
        assert len(like._times) == int(z["roq_tm_n_times_" + combo])
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



@pytest.mark.parametrize("combo", ["none", "t", "tpd"])
def test_multiband_basis_matches_the_reference(gpu, tmp_path, combo):
    """Weights built from a multi-banded basis (roq.py:920-974, 1007-1055; the
    seeded three-band basis of oracle/roq_basis.build_multiband) give the
    reference's lnL ratios (tests/golden/tf2_marg_8s_2k_roq_multiband.npz),
    without marginalisation, with time, and with time, phase and distance."""
    like, priors, z = make(combo, tmp_path, multiband=True)
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
    got = like.log_likelihood_ratio_batch({k: np.array([q[k] for q in pts]) for k in pts[0]})
    rtol = 1e-8 if "d" in combo else 1e-9
    assert np.all(np.abs(got - ref) <= rtol * np.maximum(1.0, np.abs(ref))), got - ref


def marginalized_points(params, priors, combo, jitter):
    """Prior draws as the marginalised likelihood takes them: the marginalised
    parameters at the values the constructor fixed in the priors."""
    pts = {k: np.asarray(v, dtype=np.float64).copy() for k, v in params.items()}
    n = len(pts["mass_1"])
    pts["geocent_time"] = np.full(n, float(priors["geocent_time"]))
    pts["time_jitter"] = np.asarray(jitter, dtype=np.float64)
    if "p" in combo:
        pts["phase"] = np.zeros(n)
    if "d" in combo:
        pts["luminosity_distance"] = np.full(n, float(priors["luminosity_distance"]))
    return pts


@pytest.mark.parametrize("combo", ["t", "tpd"])
def test_mixed_time_marginalized_matches_the_reference(gpu, tmp_path, combo):
    """Mixed precision (float32 weight-row products and marginalisation, the
    points over the error bound recomputed in float64): |dlnL| <= 1e-3 from
    the reference's values."""
    like, priors, z = make(combo, tmp_path)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    pts = marginalized_points(params, priors, combo, z["time_jitter"])
    got = like.log_likelihood_ratio_batch(pts, precision="mixed")
    ref = z["lnl_" + combo]
    assert np.all(np.abs(got - ref) <= 1e-3), got - ref


def test_mixed_time_marginalized_over_prior_draws(gpu, tmp_path):
    """5000 prior draws (three chunks of the mixed launch) and 64 templates
    near the injection, time, phase and distance marginalised: every mixed
    result within 1e-3 of the float64 kernel's."""
    from bilby_gb300.workloads import draw_points
    like, priors, z = make("tpd", tmp_path)
    w = WORKLOADS["tf2_marg_8s_2k"]
    rng = np.random.default_rng(11)
    p = draw_points(w, 5000, rng)
    loud = {k: np.full(64, float(w.injection[k])) for k in w.injection}
    loud["mass_1"] = loud["mass_1"] * (1 + rng.uniform(-2e-3, 2e-3, 64))
    for k in ("chi_1", "chi_2"):
        loud[k] = np.full(64, float(w.injection.get(k, 0.0)))
    p = {k: np.concatenate([np.asarray(p[k], dtype=np.float64), loud[k] if k in loud else p[k][:64]]) for k in p}
    pts = marginalized_points(p, priors, "tpd", p["time_jitter"])
    fp64 = like.log_likelihood_ratio_batch(pts, precision="fp64")
    mixed = like.log_likelihood_ratio_batch(pts, precision="mixed")
    refined = like.analysis.last_refined()
    assert np.all(np.isfinite(fp64))
    err = np.abs(mixed - fp64)
    assert np.all(err <= 1e-3), (err.max(), int(np.argmax(err)), refined)


def test_time_marginalized_with_many_nodes(gpu, tmp_path):
    """300 linear nodes: the nodes and each chunk's weight rows take more than
    48 KB of shared memory together with the kernel's static arrays."""
    from bilby_gb300.prior import Uniform
    from bilby_gb300.roq import ROQGravitationalWaveTransient
    from oracle import roq_basis
    like, priors, z = make("t", tmp_path)
    ifos, wfg = like.interferometers, like.waveform_generator
    fm = ifos[0].frequency_array[ifos[0].frequency_mask]
    w = WORKLOADS["tf2_marg_8s_2k"]
    nl, bl, nq, bq = roq_basis.build(fm, n_linear=300, n_quadratic=60, n_train=400,
                                     minimum_frequency=w.minimum_frequency)
    wfg.waveform_arguments.update(frequency_nodes_linear=nl, frequency_nodes_quadratic=nq)
    tc = w.injection["geocent_time"]
    big = ROQGravitationalWaveTransient(ifos, wfg, {"geocent_time": Uniform(tc - 0.1, tc + 0.1)},
                                        linear_matrix=bl.T, quadratic_matrix=bq.T, time_marginalization=True)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    params["geocent_time"] = np.full(len(params["mass_1"]), float(w.start_time))
    params["time_jitter"] = z["time_jitter"]
    batch = big.log_likelihood_ratio_batch(params)
    single = np.array([big.log_likelihood_ratio(point(params, i)) for i in range(len(batch))])
    assert np.all(np.isfinite(batch))
    assert np.array_equal(single, batch)


@pytest.mark.parametrize("combo", ["none", "pd"])
def test_per_detector_snrs_sum_to_the_likelihood(gpu, tmp_path, combo):
    """calculate_snrs per detector (one-detector analyses with that
    detector's weights) summed and passed to compute_log_likelihood_from_snrs
    equals the likelihood of the whole network."""
    like, priors, z = make(combo, tmp_path)
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    for i in range(4):
        q = point(params, i)
        if "p" in combo:
            q["phase"] = 0.0
        if "d" in combo:
            q["luminosity_distance"] = float(priors["luminosity_distance"])
        total = like._CalculatedSNRs()
        for ifo in like.interferometers:
            total += like.calculate_snrs(None, ifo, parameters=dict(q))
        lnl = like.compute_log_likelihood_from_snrs(total, dict(q))
        ref = like.log_likelihood_ratio(dict(q))
        rtol = 1e-8 if "d" in combo else 1e-9
        assert abs(lnl - ref) <= rtol * max(1.0, abs(ref)), (i, lnl, ref)


@pytest.mark.parametrize("combo", ["none", "t"])
def test_per_detector_snrs_match_reference(gpu, tmp_path, combo):
    """calculate_snrs per detector (with time marginalisation, the series of
    roq.py:535-541 on the marginalisation grid), per-detector lnL and the time
    draw of roq.py:1238-1271 against the reference
    (tests/golden/tf2_marg_8s_2k_roq_snrs.npz).  With time marginalisation the
    reference's scalar <d|h> sits at the segment start, outside the weight
    grid: its real part is -inf there, as here."""
    from bilby_gb300 import random as grandom
    like, priors, _ = make(combo if combo == "t" else "none", tmp_path, basis=True)
    z = golden("tf2_marg_8s_2k_roq_snrs")
    key = f"roq_{combo}"
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    names = [ifo.name for ifo in like.interferometers]
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        if combo == "t":
            q["geocent_time"] = float(priors["geocent_time"])
        else:
            q.pop("time_jitter")
        for k, ifo in enumerate(like.interferometers):
            s = like.calculate_snrs(None, ifo, parameters=dict(q))
            dh, hh = z[f"{key}_dh"][i, k], z[f"{key}_hh"][i, k]
            assert abs(s.optimal_snr_squared - hh) <= 1e-9 * max(1.0, hh)
            if np.isfinite(dh.real):
                assert abs(s.d_inner_h - dh) <= 1e-9 * max(1.0, abs(dh), hh)
            else:
                assert s.d_inner_h.real == dh.real
            if combo == "t":
                arr = s.d_inner_h_array
                assert len(arr) == int(z[f"{key}_series_len"])
                ref = z[f"{key}_series_{i}_{k}"]
                assert np.max(np.abs(arr[:400] - ref)) <= 1e-9 * max(1.0, np.max(np.abs(ref)))
                assert np.sum(np.abs(arr) ** 2) == pytest.approx(z[f"{key}_series_power"][i, k], rel=1e-9)
        res = like.compute_per_detector_log_likelihood(dict(q))
        got = np.array([res[f"{n}_log_likelihood"] for n in names])
        ref = z[f"{key}_per_det_lnl"][i]
        assert np.all(np.abs(got - ref) <= 1e-9 * np.maximum(1.0, np.abs(ref))), (i, got, ref)
        if combo == "t":
            grandom.seed(4321 + i)
            draw = like.generate_time_sample_from_marginalized_likelihood(parameters=dict(q))
            assert draw == z[f"{key}_time_draw"][i], (i, draw)


ROQ_BASES = [dict(seed=2024, mass_range=(10.0, 25.0)), dict(seed=2031, mass_range=(20.0, 40.0))]
PRIOR_RANGE_LINEAR = np.array([[8.0, 21.0], [19.0, 35.0]])
PRIOR_RANGE_QUADRATIC = np.array([[8.0, 25.0], [23.0, 35.0]])


def two_basis_likelihood(time_marginalization):
    """The two-basis ROQ likelihood of tests/golden/tf2_marg_8s_2k_roq_multibasis.npz:
    each basis' weights computed by this package from its seeded synthetic
    basis, merged into one weights dictionary with the chirp-mass ranges."""
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.prior import Uniform
    from bilby_gb300.roq import ROQGravitationalWaveTransient
    from bilby_gb300.source import taylorf2_aligned, taylorf2_aligned_roq
    from bilby_gb300.waveform_generator import WaveformGenerator
    from oracle import roq_basis
    w = WORKLOADS["tf2_marg_8s_2k"]
    grandom.seed(w.seed)
    ifos = InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
    inj = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=taylorf2_aligned,
                            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
    ifos.inject_signal(waveform_generator=inj, parameters=dict(w.injection))
    tc = w.injection["geocent_time"]
    fm = ifos[0].frequency_array[ifos[0].frequency_mask]
    single = []
    for b in ROQ_BASES:
        nl, bl, nq, bq = roq_basis.build(fm, minimum_frequency=w.minimum_frequency, seed=b["seed"],
                                        mass_range=b["mass_range"])
        wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                                frequency_domain_source_model=taylorf2_aligned_roq,
                                waveform_arguments=dict(minimum_frequency=w.minimum_frequency,
                                                        frequency_nodes_linear=nl, frequency_nodes_quadratic=nq))
        one = ROQGravitationalWaveTransient(ifos, wfg, {"geocent_time": Uniform(tc - 0.1, tc + 0.1)},
                                            linear_matrix=bl.T, quadratic_matrix=bq.T)
        single.append(one.weights)
        one.analysis.close()
    weights = {"time_samples": np.asarray(single[0]["time_samples"]),
               "prior_range_linear": {"chirp_mass": PRIOR_RANGE_LINEAR},
               "prior_range_quadratic": {"chirp_mass": PRIOR_RANGE_QUADRATIC}}
    for key in single[0]:
        if key.endswith("_linear") or key.endswith("_quadratic"):
            weights[key] = [np.asarray(s[key][0]) for s in single]
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=taylorf2_aligned_roq,
                            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
    priors = {"geocent_time": Uniform(tc - 0.1, tc + 0.1), "chirp_mass": Uniform(9.0, 34.0)}
    like = ROQGravitationalWaveTransient(ifos, wfg, priors, weights=weights,
                                         time_marginalization=time_marginalization)
    return like, priors


@pytest.mark.parametrize("combo", ["none", "t"])
def test_two_bases_selected_by_chirp_mass_match_the_reference(gpu, combo):
    """Several ROQ bases (roq.py:193-460): per point the same (linear,
    quadratic) basis pair as the reference, and its lnL ratio to
    1e-9 * max(1, |lnL|); the grouped batch equals the single calls."""
    z = golden("tf2_marg_8s_2k_roq_multibasis")
    like, priors = two_basis_likelihood(combo == "t")
    assert like.number_of_bases_linear == 2 and like.number_of_bases_quadratic == 2
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    n = len(params["chirp_mass"])
    if combo == "t":
        params["geocent_time"] = np.full(n, float(priors["geocent_time"]))
    else:
        params.pop("time_jitter")
    single, bl, bq = [], [], []
    for i in range(n):
        single.append(like.log_likelihood_ratio(point(params, i)))
        bl.append(like.basis_number_linear)
        bq.append(like.basis_number_quadratic)
    assert np.array_equal(bl, z["basis_linear_" + combo]) and np.array_equal(bq, z["basis_quadratic_" + combo])
    single = np.array(single)
    ref = z["lnl_" + combo]
    assert np.all(np.abs(single - ref) <= 1e-9 * np.maximum(1.0, np.abs(ref))), single - ref
    assert np.array_equal(like.log_likelihood_ratio_batch(params), single)
    # CUDA tensors convert chirp mass / mass ratio with torch's device arithmetic,
    # which differs from numpy's in the last bits of the masses
    import torch
    dev = {k: torch.from_numpy(np.asarray(v, dtype=np.float64)).cuda() for k, v in params.items()}
    got = like.log_likelihood_ratio_batch(dev).cpu().numpy()
    assert np.all(np.abs(got - single) <= 1e-9 * np.maximum(1.0, np.abs(single))), got - single

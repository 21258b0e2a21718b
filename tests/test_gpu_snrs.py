"""Per-detector inner products, per-detector likelihoods and the posterior
reconstruction of marginalised parameters, on the GPU, against the
reference's own values (tests/golden/tf2_marg_8s_2k_snrs.npz, generated by
tests/golden/make_golden.py --snrs-only).

Tolerances: inner products and per-detector lnL |d| <= 1e-9 * max(1, |x|)
(float64 kernels); the d_inner_h_array window |d| <= 1e-9 * max|series|;
reconstruction draws (the same uniform draws through an inverse CDF built
from float64 posteriors) within 1e-7 s, 1e-7 relative in distance, 1e-7 rad.
"""
import numpy as np
import pytest

from tests.conftest import golden
from tests.test_gpu_marginalization import make_likelihood
from bilby_gb300.workloads import WORKLOADS, point

pytestmark = pytest.mark.gpu

NAME = "tf2_marg_8s_2k"
RECON_SEED = 4321  # tests/golden/make_golden.py


def points(z, priors, combo):
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    out = []
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        if "t" in combo:
            q["geocent_time"] = float(priors["geocent_time"])
        else:
            q.pop("time_jitter")
        if "p" in combo:
            q["phase"] = 0.0
        if "d" in combo:
            q["luminosity_distance"] = float(priors["luminosity_distance"])
        out.append(q)
    return out


def close(a, b, rtol=1e-9):
    a, b = np.asarray(a), np.asarray(b)
    return np.all(np.abs(a - b) <= rtol * np.maximum(1.0, np.abs(b)))


def test_calculate_snrs_matches_reference(gpu, tmp_path):
    w = WORKLOADS[NAME]
    z = golden(NAME + "_snrs")
    like, priors = make_likelihood(w, "", "fp64", tmp_path / "table.npz")
    for i, q in enumerate(points(z, priors, "")):
        pols = like.waveform_generator.frequency_domain_strain(dict(q))
        total = like._CalculatedSNRs()
        for k, ifo in enumerate(like.interferometers):
            s = like.calculate_snrs(pols, ifo, parameters=dict(q))
            assert s.d_inner_h_array is None
            scale = max(1.0, abs(z["snr_dh"][i, k]), z["snr_hh"][i, k])
            assert abs(s.d_inner_h - z["snr_dh"][i, k]) <= 1e-9 * scale
            assert abs(s.optimal_snr_squared - z["snr_hh"][i, k]) <= 1e-9 * scale
            assert abs(s.complex_matched_filter_snr - z["snr_mf"][i, k]) <= 1e-9 * max(1.0, abs(z["snr_mf"][i, k]))
            total += s
        # the summed SNRs give the likelihood ratio
        lnl = like.compute_log_likelihood_from_snrs(total, dict(q))
        ref = like.log_likelihood_ratio(dict(q))
        assert abs(lnl - ref) <= 1e-9 * max(1.0, abs(ref))
        sample = total.snrs_as_sample
        assert sample["optimal_snr"] == pytest.approx(np.sqrt(z["snr_hh"][i].sum()), rel=1e-9)


@pytest.mark.parametrize("combo", ["", "t", "d", "p", "tpd"])
def test_per_detector_log_likelihood_matches_reference(gpu, tmp_path, combo):
    w = WORKLOADS[NAME]
    z = golden(NAME + "_snrs")
    like, priors = make_likelihood(w, combo, "fp64", tmp_path / "table.npz")
    ref = z["per_det_lnl" + ("_" + combo if combo else "")]
    names = [str(n) for n in z["detectors"]]
    for i, q in enumerate(points(z, priors, combo)):
        before = dict(q)
        res = like.compute_per_detector_log_likelihood(q)
        got = [res[f"{n}_log_likelihood"] for n in names]
        assert close(got, ref[i]), (combo, i, got, ref[i])
        # geocent_time is restored after the jitter is taken out again
        assert q["geocent_time"] == pytest.approx(before["geocent_time"], abs=1e-9)


def test_time_series_matches_reference(gpu, tmp_path):
    w = WORKLOADS[NAME]
    z = golden(NAME + "_snrs")
    like, priors = make_likelihood(w, "t", "fp64", tmp_path / "table.npz")
    for i, q in enumerate(points(z, priors, "t")):
        qq = dict(q)
        qq["geocent_time"] += qq["time_jitter"]
        idx = z[f"series_idx_{i}"]
        for k, ifo in enumerate(like.interferometers):
            s = like.calculate_snrs(None, ifo, parameters=dict(qq))
            arr = s.d_inner_h_array
            assert arr.shape == (len(ifo.frequency_array) - 1,)
            win = z[f"series_{i}"][k]
            scale = max(1.0, np.max(np.abs(win)))
            assert np.max(np.abs(arr[idx] - win)) <= 1e-9 * scale
            ssum, spow = z["series_sum"][i, k], z["series_power"][i, k]
            assert abs(arr.sum() - ssum) <= 1e-9 * max(1.0, np.sqrt(spow) * np.sqrt(len(arr)))
            assert np.sum(np.abs(arr) ** 2) == pytest.approx(spow, rel=1e-9)
        # the series and <h|h> summed over detectors give the marginalised lnL
        total = like._CalculatedSNRs()
        for ifo in like.interferometers:
            total += like.calculate_snrs(None, ifo, parameters=dict(qq))
        lnl = like.compute_log_likelihood_from_snrs(total, dict(qq))
        ref = like.log_likelihood_ratio(dict(q))
        assert abs(lnl - ref) <= 1e-8 * max(1.0, abs(ref))


@pytest.mark.parametrize("combo", ["t", "d", "p", "tpd"])
def test_posterior_reconstruction_matches_reference(gpu, tmp_path, combo):
    from bilby_gb300 import random as grandom
    w = WORKLOADS[NAME]
    z = golden(NAME + "_snrs")
    like, priors = make_likelihood(w, combo, "fp64", tmp_path / "table.npz")
    ref = z["recon_" + combo]
    for i, q in enumerate(points(z, priors, combo)):
        grandom.seed(RECON_SEED + i)
        s = like.generate_posterior_sample_from_marginalized_likelihood(dict(q))
        assert abs(s["geocent_time"] - ref[i, 0]) <= 1e-7, (combo, i)
        assert s["luminosity_distance"] == pytest.approx(ref[i, 1], rel=1e-7)
        assert abs(s["phase"] - ref[i, 2]) <= 1e-7, (combo, i)


def test_unmarginalized_reconstruction_returns_parameters(gpu, tmp_path):
    w = WORKLOADS[NAME]
    z = golden(NAME + "_snrs")
    like, priors = make_likelihood(w, "", "fp64", tmp_path / "table.npz")
    q = points(z, priors, "")[0]
    assert like.generate_posterior_sample_from_marginalized_likelihood(q) is q


def fast_likelihood(kind, combo, tmp_path):
    """The package's relative-binning or multi-banded likelihood on tf2_128s
    (fiducial = the injection; reference chirp mass 0.87), as the golden
    generator builds the reference's."""
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.multiband import MBGravitationalWaveTransient
    from bilby_gb300.prior import Uniform
    from bilby_gb300.relative import RelativeBinningGravitationalWaveTransient
    from bilby_gb300.source import taylorf2_aligned_frequency_sequence, taylorf2_aligned_relative_binning
    from bilby_gb300.waveform_generator import WaveformGenerator
    w = WORKLOADS["tf2_128s"]
    grandom.seed(w.seed)
    ifos = InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
    model = taylorf2_aligned_relative_binning if kind == "relbin" else taylorf2_aligned_frequency_sequence
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=model,
                            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
    ifos.inject_signal(waveform_generator=wfg, parameters=dict(w.injection))
    tc = w.injection["geocent_time"]
    t = combo == "t"
    priors = {"geocent_time": Uniform(tc - 0.1, tc + 0.1)} if t else None
    if kind == "relbin":
        like = RelativeBinningGravitationalWaveTransient(ifos, wfg, fiducial_parameters=dict(w.injection),
                                                         priors=priors, time_marginalization=t)
    else:
        like = MBGravitationalWaveTransient(ifos, wfg, reference_chirp_mass=0.87, priors=priors,
                                            time_marginalization=t)
    return like, priors


@pytest.mark.parametrize("kind", ["relbin", "multiband"])
@pytest.mark.parametrize("combo", ["none", "t"])
def test_fast_likelihood_snrs_match_reference(gpu, tmp_path, kind, combo):
    z = golden("tf2_128s_fast_snrs")
    like, priors = fast_likelihood(kind, combo, tmp_path)
    key = f"{kind}_{combo}"
    params = {k[2:]: z[k] for k in z.files if k.startswith("p_")}
    names = [ifo.name for ifo in like.interferometers]
    for i in range(len(params["mass_1"])):
        q = point(params, i)
        if combo == "t":
            q["geocent_time"] = float(priors["geocent_time"]) + q["time_jitter"]
        else:
            q.pop("time_jitter")
        for k, ifo in enumerate(like.interferometers):
            s = like.calculate_snrs(None, ifo, parameters=dict(q))
            dh, hh = z[f"{key}_dh"][i, k], z[f"{key}_hh"][i, k]
            scale = max(1.0, abs(dh), hh)
            assert abs(s.d_inner_h - dh) <= 1e-9 * scale, (key, i, k)
            assert abs(s.optimal_snr_squared - hh) <= 1e-9 * scale, (key, i, k)
            if combo == "t":
                arr = s.d_inner_h_array
                assert len(arr) == int(z[f"{key}_series_len"])
                win = z[f"{key}_series_{i}_{k}"]
                assert np.max(np.abs(arr[z[f"{key}_series_idx_{i}_{k}"]] - win)) <= 1e-9 * max(1.0, np.max(np.abs(win)))
                assert np.sum(np.abs(arr) ** 2) == pytest.approx(z[f"{key}_series_power"][i, k], rel=1e-9)
        qq = dict(q)
        if combo == "t":
            qq["geocent_time"] -= qq["time_jitter"]
        res = like.compute_per_detector_log_likelihood(dict(qq))
        got = [res[f"{n}_log_likelihood"] for n in names]
        assert close(got, z[f"{key}_per_det_lnl"][i]), (key, i, got)
        if kind == "multiband" and combo == "t":
            # multiband.py:822-855: a grid time drawn with numpy's global generator
            np.random.seed(RECON_SEED + i)
            draw = like.generate_time_sample_from_marginalized_likelihood(parameters=dict(qq))
            assert draw == z[f"{key}_time_draw"][i], (i, draw)
        if kind == "relbin" and combo == "t":
            # base.py:577-653 over the piecewise waveform of relative.py:380-396
            from bilby_gb300 import random as grandom
            grandom.seed(RECON_SEED + i)
            draw = like.generate_time_sample_from_marginalized_likelihood(parameters=dict(qq))
            assert abs(draw - z[f"{key}_time_draw"][i]) <= 1e-7, (i, draw)

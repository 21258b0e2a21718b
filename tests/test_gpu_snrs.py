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

"""Device prior rescaling and parameter conversion against the reference's
PriorDict.rescale + convert_to_lal_binary_black_hole_parameters
(tests/golden/priors.npz, which also holds the device programs compiled from
the reference's own prior objects), and the unit-cube batch path of the
likelihood against the host path."""
import numpy as np
import pytest

from tests.conftest import golden

pytestmark = pytest.mark.gpu


def golden_program(z, case):
    head, pars = z[f"{case}_prog_head"], z[f"{case}_prog_p"]
    prog = []
    for j, (k, t, c) in enumerate(head):
        tx = z[f"{case}_prog_tx_{j}"] if f"{case}_prog_tx_{j}" in z.files else None
        ty = z[f"{case}_prog_ty_{j}"] if f"{case}_prog_ty_{j}" in z.files else None
        prog.append((int(k), int(t), int(c), list(pars[j]), tx, ty))
    return prog


@pytest.mark.parametrize("case", ["a", "b"])
def test_rescale_matches_the_reference(gpu, case):
    import torch
    from bilby_gb300 import _capi
    from bilby_gb300.priors_device import DevicePriors
    z = golden("priors")
    keys = [str(k) for k in z[f"{case}_keys"]]
    dp = DevicePriors(keys=keys, program=golden_program(z, case))
    block = dp.rescale(torch.from_numpy(z[f"{case}_unit"]).cuda()).cpu().numpy()
    for k in keys:
        if k in _capi.SLOT:
            ref = z[f"{case}_v_{k}"]
            assert np.allclose(block[_capi.SLOT[k]], ref, rtol=1e-12, atol=1e-14 * np.max(np.abs(ref))), k
    for k in ("mass_1", "mass_2", "theta_jn"):
        if f"{case}_c_{k}" in z.files:
            assert np.allclose(block[_capi.SLOT[k]], z[f"{case}_c_{k}"], rtol=1e-12, atol=0), k


def test_unit_cube_batch_equals_host_batch(gpu):
    import torch
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.likelihood import GravitationalWaveTransient
    from bilby_gb300.prior import Cosine, PowerLaw, Sine, Uniform
    from bilby_gb300.priors_device import DevicePriors
    from bilby_gb300.source import taylorf2_aligned
    from bilby_gb300.waveform_generator import WaveformGenerator
    from bilby_gb300.workloads import WORKLOADS
    w = WORKLOADS["tf2_marg_8s_2k"]
    grandom.seed(w.seed)
    ifos = InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=taylorf2_aligned,
                            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
    ifos.inject_signal(waveform_generator=wfg, parameters=dict(w.injection))
    like = GravitationalWaveTransient(ifos, wfg)
    tc = w.injection["geocent_time"]
    priors = dict(mass_1=Uniform(10, 40), mass_2=Uniform(10, 40), chi_1=Uniform(-0.05, 0.05), chi_2=0.0,
                  luminosity_distance=PowerLaw(2, 20, 200), ra=Uniform(0, 2 * np.pi), dec=Cosine(),
                  psi=Uniform(0, np.pi), phase=Uniform(0, 2 * np.pi), theta_jn=Sine(),
                  geocent_time=Uniform(tc - 0.1, tc + 0.1))
    dp = DevicePriors(priors)
    u = np.random.default_rng(4).uniform(size=(len(dp.keys), 300))
    got = like.log_likelihood_ratio_from_unit_cube(torch.from_numpy(u).cuda(), dp).cpu().numpy()
    host = {k: priors[k].rescale(u[q]) for q, k in enumerate(dp.keys)}
    host["chi_2"] = np.zeros(300)
    ref = like.log_likelihood_ratio_batch(host)
    assert np.allclose(got, ref, rtol=1e-11, atol=1e-8)


def test_unit_cube_batch_in_a_detector_frame_equals_host_batch(gpu):
    """Detector-frame sampling on the batch path: zenith / azimuth in the
    H1-L1 frame and the arrival time at H1 become ra / dec and geocent_time on
    the device (get_sky_frame_parameters, base.py:1091-1137), and the lnL
    ratios equal the host path's, which converts the same draws with numpy."""
    import torch
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.likelihood import GravitationalWaveTransient
    from bilby_gb300.prior import PowerLaw, Sine, Uniform
    from bilby_gb300.priors_device import DevicePriors
    from bilby_gb300.source import taylorf2_aligned
    from bilby_gb300.waveform_generator import WaveformGenerator
    from bilby_gb300.workloads import WORKLOADS
    w = WORKLOADS["tf2_marg_8s_2k"]
    grandom.seed(w.seed)
    ifos = InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=taylorf2_aligned,
                            waveform_arguments=dict(minimum_frequency=w.minimum_frequency))
    ifos.inject_signal(waveform_generator=wfg, parameters=dict(w.injection))
    like = GravitationalWaveTransient(ifos, wfg, reference_frame="H1L1", time_reference="H1")
    tc = w.injection["geocent_time"]
    priors = dict(mass_1=Uniform(10, 40), mass_2=Uniform(10, 40), chi_1=Uniform(-0.05, 0.05), chi_2=0.0,
                  luminosity_distance=PowerLaw(2, 20, 200), zenith=Sine(), azimuth=Uniform(0, 2 * np.pi),
                  psi=Uniform(0, np.pi), phase=Uniform(0, 2 * np.pi), theta_jn=Sine(),
                  H1_time=Uniform(tc - 0.1, tc + 0.1))
    dp = DevicePriors(priors)
    u = np.random.default_rng(5).uniform(size=(len(dp.keys), 300))
    got = like.log_likelihood_ratio_from_unit_cube(torch.from_numpy(u).cuda(), dp).cpu().numpy()
    host = {k: priors[k].rescale(u[q]) for q, k in enumerate(dp.keys)}
    host["chi_2"] = np.zeros(300)
    ref = like.log_likelihood_ratio_batch(host)
    assert np.all(np.isfinite(ref))
    assert np.allclose(got, ref, rtol=1e-9, atol=1e-7), np.max(np.abs(got - ref))

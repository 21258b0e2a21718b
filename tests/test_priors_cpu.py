"""The device prior program compiled from the reference's own prior objects
equals the one stored with the golden values (so the GPU test, which runs
where bilby is absent, checks the same program); needs the reference tree,
skipped without it."""
import numpy as np
import pytest

from tests.conftest import golden


@pytest.mark.parametrize("case", ["a", "b"])
def test_compiled_program_matches_golden(case):
    ref_harness = pytest.importorskip("oracle.ref_harness")
    try:
        ref_harness.import_bilby()
    except Exception as e:  # pragma: no cover - reference tree absent
        pytest.skip(f"reference not importable: {e}")
    from bilby.core.prior import PriorDict
    from bilby_gb300.priors_device import compile_program
    z = golden("priors")
    keys = [str(k) for k in z[f"{case}_keys"]]
    # the reference priors exactly as tests/golden/make_golden.py builds them
    prog = compile_program(PriorDict(_cases()[case]), keys)
    head = np.array([[k, t, c] for k, t, c, _, _, _ in prog])
    assert np.array_equal(head, z[f"{case}_prog_head"])
    assert np.array_equal(np.array([p for _, _, _, p, _, _ in prog]), z[f"{case}_prog_p"])


def _cases():
    from bilby.core.prior import Cosine, Gaussian, LogUniform, PowerLaw, Sine, TruncatedGaussian, Uniform
    from bilby.gw.prior import AlignedSpin, UniformInComponentsChirpMass, UniformInComponentsMassRatio
    from bilby_gb300.workloads import WORKLOADS
    tc = WORKLOADS["tf2_128s"].injection["geocent_time"]
    return {
        "a": dict(chirp_mass=UniformInComponentsChirpMass(0.87, 1.74), mass_ratio=UniformInComponentsMassRatio(0.5, 1.0),
                  chi_1=AlignedSpin(a_prior=Uniform(0, 0.05)), chi_2=Uniform(-0.05, 0.05),
                  luminosity_distance=PowerLaw(2, 20, 200), dec=Cosine(), ra=Uniform(0, 2 * np.pi),
                  theta_jn=Sine(), psi=Uniform(0, np.pi), phase=Uniform(0, 2 * np.pi),
                  geocent_time=Uniform(tc - 0.1, tc + 0.1), hrss=LogUniform(1e-23, 1e-21), Q=Gaussian(10, 2),
                  frequency=TruncatedGaussian(200, 50, 50, 500)),
        "b": dict(chirp_mass=UniformInComponentsChirpMass(5, 30),
                  mass_ratio=UniformInComponentsMassRatio(0.125, 1.0, equal_mass=True),
                  cos_theta_jn=Uniform(-1, 1), luminosity_distance=PowerLaw(-1, 100, 1000)),
    }

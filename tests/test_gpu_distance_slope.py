"""Mixed precision under distance marginalisation without time
marginalisation: the lnL's slope in <d|h> is E[d_ref / d] under the point's
distance posterior, up to d_ref / d_min (about 40 for the workloads'
PowerLaw(2) prior on 100-5000 Mpc), so the mixed kernels scale their error
bounds by that bound (gwl_set_distance_slope).  Templates matching the
tf2_128s injection at 100 Mpc sit at the worst case (posterior at d_min);
every result stays within 1e-3 of float64, for the full-grid TaylorF2 kernel
and for multi-banding."""
import numpy as np
import pytest

from tests.test_gpu_marginalization import make_likelihood
from bilby_gb300.workloads import WORKLOADS

pytestmark = pytest.mark.gpu


def matching_templates(w, priors, combo, n, seed):
    rng = np.random.default_rng(seed)
    p = {k: np.full(n, float(v)) for k, v in w.injection.items()}
    p["mass_1"] = p["mass_1"] * (1.0 + rng.normal(0.0, 2e-4, n))
    p["mass_2"] = p["mass_2"] * (1.0 + rng.normal(0.0, 2e-4, n))
    p["chi_1"] = p["chi_1"] + rng.normal(0.0, 1e-3, n)
    p["theta_jn"] = rng.uniform(0.0, np.pi, n)
    p["luminosity_distance"] = np.full(n, float(priors["luminosity_distance"]))
    if "p" in combo:
        p["phase"] = np.zeros(n)
    return p


@pytest.mark.parametrize("combo", ["d", "pd"])
def test_full_grid_taylorf2_holds_1e3_at_the_slope_bound(gpu, tmp_path, combo):
    from bilby_gb300.analysis import params_block
    w = WORKLOADS["tf2_128s"]
    like, priors = make_likelihood(w, combo, "mixed", tmp_path / "table.npz")
    assert like._ref_dist / like._distance_array[0] > 30
    block = params_block(like._prepare(matching_templates(w, priors, combo, 256, 3)))
    mixed = like.analysis.log_likelihood_ratio_host(block, "mixed")
    fp64 = like.analysis.log_likelihood_ratio_host(block, "fp64")
    err = np.abs(mixed - fp64)
    assert np.all(np.isfinite(mixed)) and np.all(err <= 1e-3), (err.max(), fp64[np.argmax(err)])
    assert np.max(fp64) > 100.0   # the templates do match the loud injection


def test_multiband_holds_1e3_at_the_slope_bound(gpu, tmp_path):
    from bilby_gb300.analysis import params_block
    from tests.test_gpu_multiband import make
    w = WORKLOADS["tf2_128s"]
    like, priors = make("d", tmp_path, precision="mixed")
    block = params_block(like._prepare(matching_templates(w, priors, "d", 256, 4)))
    mixed = like.analysis.log_likelihood_ratio_host(block, "mixed")
    fp64 = like.analysis.log_likelihood_ratio_host(block, "fp64")
    err = np.abs(mixed - fp64)
    assert np.all(np.isfinite(mixed)) and np.all(err <= 1e-3), (err.max(), fp64[np.argmax(err)])

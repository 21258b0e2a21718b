"""Edge cases of the batch entry points on the GPU: empty batches, a single
point, large ragged batches (batch independence at B = 200,003), invalid
points under every marginalisation and in the device-tensor path.

An invalid point (negative mass, NaN distance) gives np.nan_to_num(-np.inf),
the reference's convention for an undefined waveform (base.py:424-425)."""
import numpy as np
import pytest

from tests.gpu_helpers import WORKLOADS, device_analysis, draw_points, params_block, small_workload
from oracle import data as OD

pytestmark = pytest.mark.gpu

NEG = np.nan_to_num(-np.inf)


@pytest.fixture(scope="module")
def small(gpu):
    w = small_workload("tf2_128s", sampling_frequency=2048.0, duration=8.0,
                       injection=dict(WORKLOADS["tf2_128s"].injection,
                                      geocent_time=WORKLOADS["tf2_128s"].start_time + 6.0))
    dets = OD.build_workload(w)
    return w, dets, device_analysis(dets, "taylorf2", w)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_empty_and_single_point_batches(small, precision):
    import torch
    w, dets, an = small
    empty = an.log_likelihood_ratio_host(np.zeros((params_block({}).shape[0], 0)), precision)
    assert empty.shape == (0,)
    one = params_block(draw_points(w, 1, np.random.default_rng(3)))
    a = an.log_likelihood_ratio_host(one, precision)
    b = an.log_likelihood_ratio_staged({k: one[i] for k, i in _slots().items()}, precision)
    assert a.shape == (1,) and np.isfinite(a[0]) and b[0] == a[0]
    # device path with no points: nothing launched, nothing written
    out = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    blk = torch.zeros((one.shape[0], 1), dtype=torch.float64, device="cuda")
    an.log_likelihood_ratio_device(blk.data_ptr(), 0, out.data_ptr(), precision,
                                   torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert out.item() == 7.0


def _slots():
    from bilby_gb300 import _capi
    return dict(_capi.SLOT)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_large_ragged_batch_matches_small_batches(small, precision):
    """200,003 points (not a multiple of any tile) in one launch sequence give
    the same values as the same points in batches of 1,000."""
    w, dets, an = small
    n = 200_003 if precision == "mixed" else 20_003
    block = params_block(draw_points(w, n, np.random.default_rng(17)))
    full = an.log_likelihood_ratio_host(block, precision)
    assert np.all(np.isfinite(full))
    for start in (0, n // 2, n - 1000):
        part = an.log_likelihood_ratio_host(block[:, start:start + 1000], precision)
        assert np.array_equal(part, full[start:start + 1000])


@pytest.mark.parametrize("combo", ["t", "p", "d", "tpd"])
def test_invalid_points_under_marginalisation(gpu, tmp_path, combo):
    from tests.test_gpu_marginalization import make_likelihood
    w = WORKLOADS["tf2_marg_8s_2k"]
    for precision in ("fp64", "mixed"):
        like, priors = make_likelihood(w, combo, precision, tmp_path / "table.npz")
        p = draw_points(w, 6, np.random.default_rng(5))
        if "t" in combo:
            p["geocent_time"] = np.full(6, float(priors["geocent_time"]))
            p["time_jitter"] = np.zeros(6)
        if "p" in combo:
            p["phase"] = np.zeros(6)
        if "d" in combo:
            p["luminosity_distance"] = np.full(6, float(priors["luminosity_distance"]))
        p["mass_1"][1] = -2.0
        p["mass_2"][4] = np.nan
        got = like.log_likelihood_ratio_batch(p, precision=precision)
        assert got[1] == NEG and got[4] == NEG, (combo, precision, got)
        assert np.all(np.isfinite(got[[0, 2, 3, 5]])), (combo, precision, got)


def test_invalid_points_through_device_tensors(small):
    import torch
    w, dets, an = small
    p = draw_points(w, 130, np.random.default_rng(8))
    p["mass_1"][129] = -1.0
    blk = torch.from_numpy(params_block(p)).cuda()
    out = torch.empty(130, dtype=torch.float64, device="cuda")
    for precision in ("fp64", "mixed"):
        an.log_likelihood_ratio_device(blk.data_ptr(), 130, out.data_ptr(), precision,
                                       torch.cuda.current_stream().cuda_stream)
        got = out.cpu().numpy()
        assert got[129] == NEG and np.all(np.isfinite(got[:129]))

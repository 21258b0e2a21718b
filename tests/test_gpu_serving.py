"""The serving loop on the GPU: a request's result is bit-identical whether
it runs alone or among many concurrent requests of other analyses, and
equals the direct evaluation."""
import numpy as np
import pytest

from bilby_gb300.analysis import params_block
from bilby_gb300.workloads import draw_points, uneven_analyses
from tests.test_gpu_batching import build

pytestmark = pytest.mark.gpu


def test_alone_and_in_the_mix(gpu):
    from bilby_gb300.serving import LikelihoodServer
    ws = [w for w in uneven_analyses(24, seed=11) if w.duration <= 16][:3]
    likes = [build(w) for w in ws]
    srv = LikelihoodServer(hbm_budget_bytes=20e9, max_points_per_step=20000).start()
    for q, lk in enumerate(likes):
        srv.add_analysis(q, lk)
    probe = params_block(draw_points(ws[0], 300, np.random.default_rng(0)))
    alone = srv.submit(0, probe).result(60)
    direct = likes[0].analysis.log_likelihood_ratio_host(probe, "mixed")
    assert np.array_equal(alone, direct)
    rng = np.random.default_rng(1)
    futs = []
    for r in range(60):
        q = int(rng.integers(0, len(ws)))
        b = params_block(draw_points(ws[q], int(rng.integers(1, 900)), rng))
        futs.append((q, b, srv.submit(q, b)))
        if r == 30:
            mixed = srv.submit(0, probe)
    for q, b, f in futs:
        assert np.array_equal(f.result(120), likes[q].analysis.log_likelihood_ratio_host(b, "mixed"))
    assert np.array_equal(mixed.result(60), alone)
    srv.stop()
    s = srv.stats.summary()
    assert s["failed"] == 0 and s["requests"] == 62
    assert s["steps"] < 62  # requests were batched together

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


@pytest.mark.parametrize("convert_on_client", [True, False])
def test_served_client_equals_direct_likelihood_for_sampler_dicts(gpu, tmp_path, convert_on_client):
    """A sampler dictionary in chirp mass / mass ratio, sent by the IPC client
    (one point and a batch; converted in the client or in the server), gives
    bit for bit what the direct likelihood's log_likelihood_ratio /
    log_likelihood_ratio_batch give, and the client's noise lnL is the
    likelihood's."""
    import threading
    from bilby_gb300.serving import LikelihoodServer, ServedLikelihood, serve_ipc
    w = [w for w in uneven_analyses(24, seed=11) if w.duration <= 16][0]
    like = build(w)
    srv = LikelihoodServer(hbm_budget_bytes=20e9, max_points_per_step=20000).start()
    srv.add_analysis("a", like)
    listener = serve_ipc(srv, str(tmp_path / "gwl.sock"))
    client = ServedLikelihood(str(tmp_path / "gwl.sock"), "a", convert_on_client=convert_on_client)
    p = draw_points(w, 64, np.random.default_rng(5))
    mc = (p["mass_1"] * p["mass_2"]) ** 0.6 / (p["mass_1"] + p["mass_2"]) ** 0.2
    sampler = {k: v for k, v in p.items() if k not in ("mass_1", "mass_2")}
    sampler["chirp_mass"] = mc
    sampler["mass_ratio"] = p["mass_2"] / p["mass_1"]
    served = client.log_likelihood_ratio_batch(sampler)
    assert np.array_equal(served, like.log_likelihood_ratio_batch(sampler))
    assert np.all(np.isfinite(served))
    one = {k: float(v[3]) for k, v in sampler.items()}
    assert client.log_likelihood_ratio(one) == like.log_likelihood_ratio(one)
    assert client.noise_log_likelihood() == like.noise_log_likelihood()
    threading.Thread(target=listener.close, daemon=True).start()
    srv.stop()

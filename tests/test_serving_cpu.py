"""The serving loop's host logic on the CPU (no GPU): continuous batching,
admission by the HBM budget, malformed requests, clients that go away, a
failing device step, and the local IPC front end with client processes."""
import multiprocessing as mp
import os
import tempfile
import threading
import time

import numpy as np
import pytest

from bilby_gb300 import _capi
from bilby_gb300.serving import AdmissionError, LikelihoodServer, ServedLikelihood, serve_ipc


class FakeAnalysis:
    def __init__(self, size, scale):
        self.size, self.scale, self.n_bins, self.n_detectors = size, scale, 1024, 2


class FakeBackend:
    """Evaluates lnL = scale * sum(params) on the CPU after `delay` seconds."""

    def __init__(self, delay=0.02, fail_on=None):
        self.delay, self.fail_on, self.launches = delay, fail_on, []

    def resident_bytes(self, an):
        return an.size

    def step_bytes(self, an, n):
        return 1000 * n

    def launch(self, slot, items):
        self.launches.append((slot, [b.shape[1] for _, b in items]))
        if self.fail_on is not None and len(self.launches) == self.fail_on:
            return ("fail", time.perf_counter() + self.delay)
        res = [an.scale * b.sum(axis=0) for an, b in items]
        return (res, time.perf_counter() + self.delay)

    def ready(self, h):
        return time.perf_counter() >= h[1]

    def results(self, h):
        if h[0] == "fail":
            raise TimeoutError("injected device failure")
        return h[0]


def block(n, seed):
    return np.random.default_rng(seed).normal(size=(_capi.NPARAM, n))


def expected(an, b):
    return an.scale * b.sum(axis=0)


def test_results_alone_and_in_the_mix():
    be = FakeBackend(delay=0.01)
    srv = LikelihoodServer(hbm_budget_bytes=1e9, backend=be).start()
    a, b = FakeAnalysis(1000, 2.0), FakeAnalysis(2000, -1.0)
    srv.add_analysis("a", a)
    srv.add_analysis("b", b)
    x = block(50, 1)
    alone = srv.submit("a", x).result(5)
    futs = [srv.submit("b" if q % 2 else "a", block(10 + q, q)) for q in range(40)]
    mixed = srv.submit("a", x)
    for q, f in enumerate(futs):
        assert np.array_equal(f.result(5), expected(b if q % 2 else a, block(10 + q, q)))
    assert np.array_equal(mixed.result(5), alone)
    srv.stop()
    s = srv.stats.summary()
    assert s["requests"] == 42 and s["failed"] == 0 and s["p50_ms"] > 0


def test_continuous_batching_packs_arrivals_during_a_step():
    be = FakeBackend(delay=0.05)
    srv = LikelihoodServer(hbm_budget_bytes=1e9, backend=be, n_streams=2).start()
    srv.add_analysis("a", FakeAnalysis(10, 1.0))
    first = srv.submit("a", block(5, 0))
    time.sleep(0.005)
    rest = [srv.submit("a", block(5, q)) for q in range(1, 30)]
    for f in [first] + rest:
        f.result(5)
    srv.stop()
    # all 30 requests ran in far fewer steps, and two steps overlapped on the two slots
    assert srv.stats.steps < 10
    assert {slot for slot, _ in be.launches} == {0, 1}


def test_admission_by_hbm_budget():
    srv = LikelihoodServer(hbm_budget_bytes=10_000, backend=FakeBackend())
    srv.add_analysis("a", FakeAnalysis(5_000, 1.0))
    with pytest.raises(AdmissionError):
        srv.add_analysis("b", FakeAnalysis(6_000, 1.0))
    srv.remove_analysis("a")
    srv.add_analysis("b", FakeAnalysis(6_000, 1.0))
    srv.start()
    too_big = srv.submit("b", block(5, 0))   # 5 points x 1000 B > 4000 B of room
    with pytest.raises(AdmissionError):
        too_big.result(1)
    assert srv.submit("b", block(3, 0)).result(5).shape == (3,)
    srv.stop()


def test_malformed_requests_fail_alone():
    srv = LikelihoodServer(hbm_budget_bytes=1e9, backend=FakeBackend()).start()
    srv.add_analysis("a", FakeAnalysis(10, 1.0))
    bad_key = srv.submit("zzz", block(4, 0))
    bad_shape = srv.submit("a", np.zeros((3, 4)))
    good = srv.submit("a", block(4, 0))
    with pytest.raises(KeyError):
        bad_key.result(1)
    with pytest.raises(ValueError):
        bad_shape.result(1)
    assert np.array_equal(good.result(5), expected(srv.analyses["a"], block(4, 0)))
    srv.stop()


def test_failed_device_step_fails_its_requests_only():
    be = FakeBackend(delay=0.01, fail_on=1)
    srv = LikelihoodServer(hbm_budget_bytes=1e9, backend=be).start()
    srv.add_analysis("a", FakeAnalysis(10, 1.0))
    f1 = srv.submit("a", block(4, 0))
    with pytest.raises(TimeoutError):
        f1.result(5)
    f2 = srv.submit("a", block(4, 1))
    assert f2.result(5).shape == (4,)
    srv.stop()


def test_client_that_goes_away_is_dropped():
    be = FakeBackend(delay=0.1)
    srv = LikelihoodServer(hbm_budget_bytes=1e9, backend=be, n_streams=1).start()
    srv.add_analysis("a", FakeAnalysis(10, 1.0))
    busy = srv.submit("a", block(4, 0))
    time.sleep(0.01)
    gone = object()
    queued = [srv.submit("a", block(4, q), client=gone) for q in range(5)]
    srv.cancel_client(gone)
    assert all(f.cancelled() for f in queued)
    assert busy.result(5).shape == (4,)
    assert srv.submit("a", block(2, 9)).result(5).shape == (2,)
    srv.stop()


def _client_proc(address, key, seed, conn):
    like = ServedLikelihood(address, key)
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(5):
        p = {k: rng.normal(size=3) for k in _capi.PARAM_SLOTS}
        out.append((p, like.log_likelihood_ratio_batch(p)))
    conn.send(out)


def _dying_client(address, key):
    from multiprocessing.connection import Client
    c = Client(address, authkey=b"gwlnl")
    c.send(("eval", key, np.ones((_capi.NPARAM, 2))))
    os._exit(0)  # leave without reading the reply


def test_ipc_front_end_with_client_processes():
    be = FakeBackend(delay=0.005)
    srv = LikelihoodServer(hbm_budget_bytes=1e9, backend=be).start()
    srv.add_analysis("a", FakeAnalysis(10, 3.0))
    path = os.path.join(tempfile.mkdtemp(), "gwl.sock")
    listener = serve_ipc(srv, path)
    ctx = mp.get_context("spawn")
    dying = ctx.Process(target=_dying_client, args=(path, "a"))
    dying.start()
    dying.join(30)
    pipes, procs = [], []
    for seed in range(2):
        r, w = ctx.Pipe(duplex=False)
        p = ctx.Process(target=_client_proc, args=(path, "a", seed, w))
        p.start()
        pipes.append(r)
        procs.append(p)
    from bilby_gb300.analysis import params_block
    for r, p in zip(pipes, procs):
        for params, got in r.recv():
            assert np.array_equal(got, 3.0 * params_block(params).sum(axis=0))
        p.join(30)
        assert p.exitcode == 0
    listener.close()
    srv.stop()

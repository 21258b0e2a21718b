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


def test_steps_grow_under_a_backlog():
    """Steps take up to max_points_per_step points, and up to
    backlog_points_per_step while more than that many wait; every request
    still gets its own results."""
    be = FakeBackend(delay=0.05)
    srv = LikelihoodServer(hbm_budget_bytes=1e9, backend=be, n_streams=1, max_points_per_step=100,
                           backlog_points_per_step=200)
    srv.add_analysis("a", FakeAnalysis(10, 1.0))
    futs = [srv.submit("a", block(20, q)) for q in range(30)]   # 600 points queued before the loop starts
    srv.start()
    for q, f in enumerate(futs):
        assert np.array_equal(f.result(5), expected(FakeAnalysis(10, 1.0), block(20, q)))
    srv.stop()
    sizes = [sum(n) for _, n in be.launches]
    assert sum(sizes) == 600 and max(sizes) <= 200
    assert sizes[0] == 200          # 600 waiting: a backlog step
    assert sizes[-1] <= 100         # the last 100 or fewer: an ordinary step
    assert srv._pending_points == 0


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
    from multiprocessing.connection import Client
    c = Client(address, authkey=b"gwlnl")
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(5):
        b = rng.normal(size=(_capi.NPARAM, 3))
        c.send(("eval", key, b))
        out.append((b, c.recv()[1]))
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
    for r, p in zip(pipes, procs):
        for b, got in r.recv():
            assert np.array_equal(got, 3.0 * b.sum(axis=0))
        p.join(30)
        assert p.exitcode == 0
    listener.close()
    srv.stop()


def _raw_client(address, key, seed, conn):
    """Packed blocks as raw bytes after an ``eval_raw`` header, twice the
    same connection (its receive buffer reused), then a header whose size
    does not match what follows."""
    from multiprocessing.connection import Client
    c = Client(address, authkey=b"gwlnl")
    rng = np.random.default_rng(seed)
    out = []
    for n in (7, 3, 1500):
        b = rng.normal(size=(_capi.NPARAM, n))
        c.send(("eval_raw", key, n))
        c.send_bytes(np.ascontiguousarray(b))
        out.append((b, c.recv()[1]))
    conn.send(out)
    c.send(("eval_raw", key, -4))   # malformed: the server drops this connection
    try:
        c.recv()
        dropped = False
    except (EOFError, OSError):
        dropped = True
    conn.send(dropped)


def test_ipc_raw_blocks_and_a_malformed_header():
    be = FakeBackend(delay=0.005)
    srv = LikelihoodServer(hbm_budget_bytes=1e9, backend=be).start()
    srv.add_analysis("a", FakeAnalysis(10, 2.0))
    path = os.path.join(tempfile.mkdtemp(), "gwl.sock")
    listener = serve_ipc(srv, path)
    ctx = mp.get_context("spawn")
    r, w = ctx.Pipe(duplex=False)
    p = ctx.Process(target=_raw_client, args=(path, "a", 5, w))
    p.start()
    for b, got in r.recv():
        assert np.array_equal(got, 2.0 * b.sum(axis=0))
    assert r.recv() is True
    p.join(30)
    assert p.exitcode == 0
    # the server still serves other clients
    r2, w2 = ctx.Pipe(duplex=False)
    p2 = ctx.Process(target=_client_proc, args=(path, "a", 9, w2))
    p2.start()
    for b, got in r2.recv():
        assert np.array_equal(got, 2.0 * b.sum(axis=0))
    p2.join(30)
    listener.close()
    srv.stop()


class _HostOnlyLikelihood:
    """A real likelihood's parameter preparation with a fake device analysis."""

    def __init__(self, like, analysis, noise):
        self.like, self.analysis, self._noise = like, analysis, noise

    def parameters_block(self, parameters):
        return self.like.parameters_block(parameters)

    @property
    def preparer(self):
        return self.like.preparer

    def noise_log_likelihood(self):
        return self._noise


def _tf2_likelihood(monkeypatch):
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.likelihood import GravitationalWaveTransient
    from bilby_gb300.source import taylorf2_aligned
    from bilby_gb300.waveform_generator import WaveformGenerator
    monkeypatch.setattr(GravitationalWaveTransient, "_build_analysis", lambda self: None)
    grandom.seed(3)
    ifos = InterferometerList(["H1", "L1"])
    ifos.set_strain_data_from_power_spectral_densities(2048.0, 4.0, 1126259640.0)
    wfg = WaveformGenerator(duration=4.0, sampling_frequency=2048.0, start_time=1126259640.0,
                            frequency_domain_source_model=taylorf2_aligned,
                            waveform_arguments=dict(minimum_frequency=20.0))
    return GravitationalWaveTransient(ifos, wfg)


SAMPLER_POINT = dict(chirp_mass=22.0, mass_ratio=0.7, chi_1=0.01, chi_2=-0.02, luminosity_distance=400.0,
                     theta_jn=0.3, phase=1.0, ra=1.0, dec=0.2, psi=0.5, geocent_time=1126259642.0)


def _sampler_client(address, key, convert_on_client, conn):
    like = ServedLikelihood(address, key, convert_on_client=convert_on_client)
    batch = {k: np.full(4, v) for k, v in SAMPLER_POINT.items()}
    batch["chirp_mass"] = np.array([15.0, 20.0, 25.0, 30.0])
    res = {"single": like.log_likelihood_ratio(dict(SAMPLER_POINT)), "batch": like.log_likelihood_ratio_batch(batch),
           "noise": like.noise_log_likelihood(), "log_likelihood": like.log_likelihood(dict(SAMPLER_POINT))}
    missing = dict(SAMPLER_POINT)
    missing.pop("psi")
    try:
        like.log_likelihood_ratio(missing)
        res["missing"] = None
    except KeyError as e:
        res["missing"] = str(e)
    conn.send((batch, res))


@pytest.mark.parametrize("convert_on_client", [True, False])
def test_served_client_prepares_sampler_parameters_like_the_likelihood(monkeypatch, convert_on_client):
    """A sampler dict in chirp mass / mass ratio through the IPC client gives
    the block the direct likelihood builds (sky frame, conversion, jitter run
    in the client with the likelihood's preparer, or in the server), the
    server's noise lnL, and KeyError for a missing psi."""
    like = _tf2_likelihood(monkeypatch)
    direct = like.parameters_block(dict(SAMPLER_POINT))
    assert direct[_capi.SLOT["mass_1"], 0] > direct[_capi.SLOT["mass_2"], 0] > 0
    with pytest.raises(KeyError):
        like.parameters_block({k: v for k, v in SAMPLER_POINT.items() if k != "psi"})
    srv = LikelihoodServer(hbm_budget_bytes=1e9, backend=FakeBackend(delay=0.002)).start()
    an = FakeAnalysis(10, 3.0)
    srv.add_analysis("tf2", _HostOnlyLikelihood(like, an, -123.5))
    srv.add_analysis("bare", an)
    with pytest.raises(TypeError):
        srv.submit_parameters("bare", dict(SAMPLER_POINT)).result(5)
    path = os.path.join(tempfile.mkdtemp(), "gwl.sock")
    listener = serve_ipc(srv, path)
    ctx = mp.get_context("spawn")
    r, w = ctx.Pipe(duplex=False)
    proc = ctx.Process(target=_sampler_client, args=(path, "tf2", convert_on_client, w))
    proc.start()
    batch, res = r.recv()
    proc.join(60)
    assert proc.exitcode == 0
    assert res["single"] == 3.0 * direct.sum(axis=0)[0]
    assert np.array_equal(res["batch"], 3.0 * like.parameters_block(batch).sum(axis=0))
    assert res["noise"] == -123.5
    assert res["log_likelihood"] == res["single"] - 123.5
    assert res["missing"] is not None and "psi" in res["missing"]
    listener.close()
    srv.stop()

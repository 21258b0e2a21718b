"""Serving: one process owns the GPU and evaluates likelihood-batch requests
from many concurrent sampler clients with continuous batching.

* Analyses are registered once (data, PSD and tables stay resident) and are
  admitted against an HBM budget; a registration that would exceed it is
  refused with ``MemoryError``.
* Requests (analysis, batch of points) queue up; whenever one of the
  ``n_streams`` step slots is free the scheduler packs pending requests (FIFO,
  up to ``max_points_per_step`` points -- ``backlog_points_per_step`` while
  more than that many wait -- and the remaining work-space budget) into one
  step: one batched launch over all their analyses on that slot's
  CUDA stream.  Requests that arrive while steps are running are admitted as
  slots free up; up to ``n_streams`` steps are on the device at once.
* Each request's result is bit-identical whether it ran alone or in a mix
  (the batched kernels never mix points of different requests).
* Latency (submission to result) is recorded per request; ``stats()``
  reports p50 / p99 and throughput.

The device work goes through a backend; :class:`GpuBackend` uses the CUDA
batcher, and a CPU stand-in with the same interface lets the scheduling,
admission and failure paths be tested without a GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import contextlib
import threading
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import _capi


class AdmissionError(MemoryError):
    """An analysis or a request does not fit in the HBM budget."""


@dataclass
class Request:
    key: object
    block: np.ndarray            # [NPARAM, B] float64
    future: cf.Future
    t_submit: float
    client: object = None

    @property
    def n(self) -> int:
        return self.block.shape[1]


@dataclass
class _Step:
    slot: int
    requests: list
    handle: object
    t_launch: float
    points: int = 0


@dataclass
class ServerStats:
    latencies: list = field(default_factory=list)
    points_done: int = 0
    steps: int = 0
    step_points: list = field(default_factory=list)
    t_first: float | None = None
    t_last: float | None = None
    failed: int = 0

    def summary(self) -> dict:
        lat = np.array(self.latencies) * 1e3
        span = (self.t_last - self.t_first) if self.t_first is not None and self.t_last is not None else 0.0
        return {"requests": len(self.latencies), "failed": self.failed, "points": self.points_done,
                "steps": self.steps,
                "mean_points_per_step": float(np.mean(self.step_points)) if self.step_points else 0.0,
                "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
                "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
                "evals_per_s": self.points_done / span if span > 0 else None}


class GpuBackend:
    """Device side of the server: per step slot one CUDA stream, one batcher
    and a staging arena (pinned host and device buffers for the parameter
    blocks and results of a step, grown on demand and reused), so that a step
    costs one host memcpy per request, one host-to-device and one
    device-to-host copy, and the batched launch."""

    def __init__(self, n_slots: int, precision: str = "mixed", use_graphs: bool = False):
        import torch
        from .batching import Batcher
        self.torch = torch
        self.precision = precision
        self.streams = [torch.cuda.Stream() for _ in range(n_slots)]
        self.batchers = [Batcher(use_graphs=use_graphs) for _ in range(n_slots)]
        self._arenas = [None] * n_slots

    @staticmethod
    @contextlib.contextmanager
    def trace(name: str):
        """An NVTX range (a no-op unless a profiler is attached)."""
        lib = _capi.load()
        lib.gwl_trace_push(name.encode())
        try:
            yield
        finally:
            lib.gwl_trace_pop()

    @staticmethod
    def resident_bytes(analysis) -> int:
        return analysis.resident_bytes()

    @staticmethod
    def step_bytes(analysis, n_points: int) -> int:
        """Device work space of n points of an analysis in one step."""
        groups = max(1, -(-analysis.n_bins // 512))
        return n_points * (8 * _capi.NPARAM + 8 + 640) + groups * analysis.n_detectors * 6 * 8 * n_points

    def _arena(self, slot: int, n_points: int):
        torch = self.torch
        a = self._arenas[slot]
        if a is None or a[0] < n_points:
            cap = max(n_points, 4096)
            a = (cap,
                 torch.empty(_capi.NPARAM * cap, dtype=torch.float64, pin_memory=True),
                 torch.empty(_capi.NPARAM * cap, dtype=torch.float64, device="cuda"),
                 torch.empty(cap, dtype=torch.float64, device="cuda"),
                 torch.empty(cap, dtype=torch.float64, pin_memory=True))
            self._arenas[slot] = a
        return a

    def launch(self, slot: int, items):
        """items: [(Analysis, host block)] -> handle; asynchronous.  The slot's
        arena is free: the scheduler hands a slot out only after its previous
        step was retired."""
        torch = self.torch
        n_total = sum(b.shape[1] for _, b in items)
        _, pin_in, dev_in, dev_out, pin_out = self._arena(slot, n_total)
        host = pin_in.numpy()
        raw, spans, off = [], [], 0
        for an, block in items:
            n = block.shape[1]
            host[_capi.NPARAM * off:_capi.NPARAM * (off + n)].reshape(_capi.NPARAM, n)[...] = block
            raw.append((an, dev_in.data_ptr() + 8 * _capi.NPARAM * off, n, dev_out.data_ptr() + 8 * off))
            spans.append((off, n))
            off += n
        stream = self.streams[slot]
        with torch.cuda.stream(stream):
            with self.trace("h2d"):
                dev_in[:_capi.NPARAM * off].copy_(pin_in[:_capi.NPARAM * off], non_blocking=True)
            with self.trace("launch"):
                self.batchers[slot].eval_device(raw, self.precision, stream.cuda_stream)
            with self.trace("readback"):
                pin_out[:off].copy_(dev_out[:off], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(stream)
        return (ev, spans, pin_out, None, slot)

    @staticmethod
    def ready(handle) -> bool:
        return handle[0].query()

    def results(self, handle):
        ev, spans, pin_out, _, slot = handle
        ev.synchronize()
        self.batchers[slot].check()
        out = pin_out.numpy()
        return [out[o:o + n].copy() for o, n in spans]


class LikelihoodServer:
    def __init__(self, hbm_budget_bytes: float = 160e9, max_points_per_step: int = 1 << 15, n_streams: int = 3,
                 backend=None, precision: str = "mixed", use_graphs: bool = False, poll_s: float = 5e-5,
                 backlog_points_per_step: int | None = None):
        self.budget = float(hbm_budget_bytes)
        self.max_points = int(max_points_per_step)
        # while more points than this wait, a step may take this many: larger
        # steps under a backlog (fewer per-step costs), short ones otherwise
        self.backlog_points = int(backlog_points_per_step or 2 * self.max_points)
        self.n_streams = int(n_streams)
        self.backend = backend if backend is not None else GpuBackend(n_streams, precision, use_graphs)
        self.poll_s = poll_s
        self.analyses: dict = {}
        self.likelihoods: dict = {}
        self.resident = 0
        self.pending: deque = deque()
        self._pending_points = 0          # points of the queued requests
        self.inflight: list = []
        self.cv = threading.Condition()
        self.stats = ServerStats()
        self._thread = None
        self._running = False
        self._busy_slots: set = set()

    # -- analyses ----------------------------------------------------------
    def add_analysis(self, key, analysis):
        """Register a device-resident analysis (an ``Analysis`` or a likelihood
        holding one); refused with AdmissionError beyond the HBM budget.  A
        likelihood also serves sampler parameter dictionaries
        (``submit_parameters``) and its noise log-likelihood."""
        an = getattr(analysis, "analysis", analysis)
        size = self.backend.resident_bytes(an)
        with self.cv:
            if key in self.analyses:
                raise ValueError(f"analysis {key!r} is already registered")
            if self.resident + size + self.backend.step_bytes(an, 1) > self.budget:
                raise AdmissionError(f"analysis {key!r} ({size / 1e9:.3f} GB) does not fit in the "
                                     f"{self.budget / 1e9:.1f} GB budget ({self.resident / 1e9:.3f} GB resident)")
            self.analyses[key] = an
            self.likelihoods[key] = analysis if hasattr(analysis, "parameters_block") else None
            self.resident += size

    def remove_analysis(self, key):
        with self.cv:
            an = self.analyses.pop(key)
            self.likelihoods.pop(key, None)
            self.resident -= self.backend.resident_bytes(an)

    def _likelihood(self, key):
        if key not in self.analyses:
            raise KeyError(f"unknown analysis {key!r}")
        like = self.likelihoods.get(key)
        if like is None:
            raise TypeError(f"analysis {key!r} was registered without a likelihood: send packed parameter blocks")
        return like

    def preparer(self, key):
        """The registered likelihood's parameter preparation (a picklable
        ``ParameterPreparer``), for clients that convert in their own process."""
        return self._likelihood(key).preparer

    def noise_log_likelihood(self, key) -> float:
        """The noise log-likelihood of a registered analysis (base.py:413-417)."""
        like = self.likelihoods.get(key)
        if like is not None:
            return float(like.noise_log_likelihood())
        if key not in self.analyses:
            raise KeyError(f"unknown analysis {key!r}")
        return float(self.analyses[key].noise_log_likelihood())

    # -- requests ----------------------------------------------------------
    def submit(self, key, block, client=None) -> cf.Future:
        """Queue a batch: ``block`` is a [NPARAM, B] float64 array (see
        ``analysis.params_block``).  Returns a Future of the B log-likelihood ratios."""
        fut: cf.Future = cf.Future()
        try:
            if key not in self.analyses:
                raise KeyError(f"unknown analysis {key!r}")
            block = np.ascontiguousarray(block, dtype=np.float64)
            if block.ndim != 2 or block.shape[0] != _capi.NPARAM or block.shape[1] < 1:
                raise ValueError(f"request block must have shape ({_capi.NPARAM}, B>=1), got {block.shape}")
            if self.backend.step_bytes(self.analyses[key], block.shape[1]) > self.budget - self.resident:
                raise AdmissionError("request larger than the work-space budget")
        except Exception as e:  # malformed request: fail it alone
            fut.set_exception(e)
            with self.cv:
                self.stats.failed += 1
            return fut
        req = Request(key, block, fut, time.perf_counter(), client)
        with self.cv:
            self.pending.append(req)
            self._pending_points += req.n
            self.cv.notify()
        return fut

    def submit_parameters(self, key, parameters, client=None) -> cf.Future:
        """Queue a sampler's parameter dictionary (scalars or equal-length
        arrays) for a registered likelihood.  The likelihood's own preparation
        runs first (sky frame, parameter conversion, time jitter), so the
        result equals its ``log_likelihood_ratio`` / ``log_likelihood_ratio_batch``;
        a dictionary that lacks a needed parameter fails with ``KeyError``."""
        try:
            block = self._likelihood(key).parameters_block(parameters)
        except Exception as e:
            fut: cf.Future = cf.Future()
            fut.set_exception(e)
            with self.cv:
                self.stats.failed += 1
            return fut
        return self.submit(key, block, client)

    def cancel_client(self, client):
        """Drop the queued requests of a client that went away (their futures are cancelled)."""
        with self.cv:
            keep = deque()
            for r in self.pending:
                if r.client is client:
                    r.future.cancel()
                    self._pending_points -= r.n
                else:
                    keep.append(r)
            self.pending = keep

    # -- scheduler ---------------------------------------------------------
    def _take(self):
        """FIFO requests for one step, within the point and work-space
        limits: max_points_per_step, or backlog_points_per_step while more
        points than that are queued."""
        take, pts, ws = [], 0, 0
        room = self.budget - self.resident
        limit = self.backlog_points if self._pending_points > self.backlog_points else self.max_points
        while self.pending:
            r = self.pending[0]
            if r.future.cancelled():
                self.pending.popleft()
                self._pending_points -= r.n
                continue
            need = self.backend.step_bytes(self.analyses[r.key], r.n)
            if take and (pts + r.n > limit or ws + need > room):
                break
            self.pending.popleft()
            self._pending_points -= r.n
            take.append(r)
            pts += r.n
            ws += need
        return take, pts

    def _retire(self, step: _Step):
        try:
            res = self.backend.results(step.handle)
            now = time.perf_counter()
            for r, out in zip(step.requests, res):
                if not r.future.cancelled():
                    r.future.set_result(out)
                self.stats.latencies.append(now - r.t_submit)
            self.stats.points_done += step.points
            self.stats.t_last = now
        except Exception as e:
            for r in step.requests:
                if not r.future.done():
                    r.future.set_exception(e)
            self.stats.failed += len(step.requests)

    def _loop(self):
        while True:
            with self.cv:
                if not self._running and not self.pending and not self.inflight:
                    return
            # retire finished steps
            done = [s for s in self.inflight if self.backend.ready(s.handle)]
            for s in done:
                self.inflight.remove(s)
                self._busy_slots.discard(s.slot)
                self._retire(s)
            launched = False
            with self.cv:
                if len(self.inflight) < self.n_streams and self.pending:
                    slot = min(set(range(self.n_streams)) - self._busy_slots)
                    trace = getattr(self.backend, "trace", None)
                    with trace("admission") if trace else contextlib.nullcontext():
                        take, pts = self._take()
                    if take:
                        self._busy_slots.add(slot)
                    else:
                        slot = None
                elif not self.pending and not self.inflight:
                    if not self._running:
                        continue
                    self.cv.wait(timeout=0.01)
                    continue
                else:
                    take = None
            if take:
                if self.stats.t_first is None:
                    self.stats.t_first = min(r.t_submit for r in take)
                try:
                    handle = self.backend.launch(slot, [(self.analyses[r.key], r.block) for r in take])
                    self.inflight.append(_Step(slot, take, handle, time.perf_counter(), pts))
                    self.stats.steps += 1
                    self.stats.step_points.append(pts)
                    launched = True
                except Exception as e:
                    self._busy_slots.discard(slot)
                    for r in take:
                        r.future.set_exception(e)
                    self.stats.failed += len(take)
            if not launched and self.inflight:
                time.sleep(self.poll_s)

    def start(self):
        self._running = True
        self._thread = threading.Thread(target=self._loop, name="gwl-server", daemon=True)
        self._thread.start()
        return self

    def stop(self, timeout: float = 60.0):
        with self.cv:
            self._running = False
            self.cv.notify_all()
        if self._thread is not None:
            self._thread.join(timeout)
            if self._thread.is_alive():
                raise TimeoutError("server thread did not drain in time")

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()


# ---------------------------------------------------------------------------
# local IPC front end for sampler processes
# ---------------------------------------------------------------------------
def serve_ipc(server: LikelihoodServer, address, authkey: bytes = b"gwlnl"):
    """Accept client processes on ``address`` (a Unix socket path or
    (host, port)).  Each connection sends one of

    * ``("eval", key, block)``: a packed [NPARAM, B] block;
    * ``("eval_raw", key, B)`` followed by the block's raw float64 bytes
      (``send_bytes``): the same without pickling, received straight into a
      buffer the connection reuses (its one request in flight keeps it
      until the step has copied it);
    * ``("eval_parameters", key, parameters)``: a sampler's dictionary,
      prepared by the registered likelihood (``submit_parameters``);
    * ``("noise", key, None)``: the analysis's noise log-likelihood;
    * ``("spec", key, None)``: the registered likelihood's parameter
      preparation (``ParameterPreparer``), so that the client converts;

    and receives ``("ok", results)`` or ``("error", message)``.  One thread
    accepts connections; one thread waits on all of them at once, reads each
    request and queues it; the reply is sent when its result is set (from the
    thread that retires the step), so no thread per client waits on a
    future.  A client has at most one request in flight, so each connection
    has one writer at a time.  Returns the listener (close it to stop
    accepting)."""
    import socket
    from multiprocessing.connection import Listener, wait
    listener = Listener(address, authkey=authkey)
    lock = threading.Lock()
    watched = {}                      # connection -> client token
    buffers = {}                      # connection -> its receive buffer (float64)
    wake_r, wake_w = socket.socketpair()
    wake_r.setblocking(False)

    def reply(conn, fut):
        try:
            try:
                msg = ("ok", fut.result())
            except Exception as e:
                msg = ("error", f"{type(e).__name__}: {e}")
            conn.send(msg)
        except (OSError, ValueError):
            pass                       # the client went away; the receiver drops it

    def drop(conn):
        buffers.pop(conn, None)
        with lock:
            token = watched.pop(conn, None)
        if token is not None:
            server.cancel_client(token)   # the client went away mid-request
        try:
            conn.close()
        except OSError:
            pass

    def handle(conn, msg):
        if not isinstance(msg, tuple) or len(msg) != 3 or \
                msg[0] not in ("eval", "eval_raw", "eval_parameters", "noise", "spec"):
            conn.send(("error", "malformed message"))
            return
        if msg[0] == "eval_raw":
            n = int(msg[2])
            if not 0 < n <= (1 << 26):
                raise ValueError("eval_raw: bad batch size")   # the stream is out of step: drop the client
            buf = buffers.get(conn)
            if buf is None or buf.size < _capi.NPARAM * n:
                buf = buffers[conn] = np.empty(_capi.NPARAM * max(n, 1024), dtype=np.float64)
            view = buf[:_capi.NPARAM * n]
            conn.recv_bytes_into(view)
            fut = server.submit(msg[1], view.reshape(_capi.NPARAM, n), client=watched.get(conn))
            fut.add_done_callback(lambda f, c=conn: reply(c, f))
            return
        if msg[0] in ("noise", "spec"):
            try:
                what = server.noise_log_likelihood if msg[0] == "noise" else server.preparer
                conn.send(("ok", what(msg[1])))
            except Exception as e:
                conn.send(("error", f"{type(e).__name__}: {e}"))
            return
        token = watched.get(conn)
        if msg[0] == "eval":
            fut = server.submit(msg[1], msg[2], client=token)
        else:
            fut = server.submit_parameters(msg[1], msg[2], client=token)
        fut.add_done_callback(lambda f, c=conn: reply(c, f))

    def receive():
        while True:
            with lock:
                conns = list(watched)
            try:
                ready = wait(conns + [wake_r], timeout=0.5)
            except OSError:
                ready = []
            for conn in ready:
                if conn is wake_r:
                    try:
                        while wake_r.recv(64):
                            pass
                    except (BlockingIOError, OSError):
                        pass
                    continue
                try:
                    msg = conn.recv()
                except (EOFError, OSError):
                    drop(conn)
                    continue
                try:
                    handle(conn, msg)
                except (OSError, ValueError, EOFError):
                    drop(conn)

    def accept():
        while True:
            try:
                conn = listener.accept()
            except OSError:
                return
            with lock:
                watched[conn] = object()
            try:
                wake_w.send(b"x")
            except OSError:
                pass

    threading.Thread(target=receive, daemon=True).start()
    threading.Thread(target=accept, daemon=True).start()
    return listener


class ServedLikelihood:
    """A sampler-side likelihood that sends each call to the serving process.

    ``log_likelihood_ratio(parameters)`` evaluates one point and
    ``log_likelihood_ratio_batch(parameters)`` a batch (a dict of equal-length
    arrays).  The dictionary is prepared exactly as the registered likelihood
    prepares it (sky frame, parameter conversion, time jitter): by default in
    this process, with the likelihood's ``ParameterPreparer`` fetched from the
    server on first use, so that only the packed float64 block travels; with
    ``convert_on_client=False`` the server converts.  Either way any parameter
    set the direct ``GravitationalWaveTransient`` accepts (e.g. ``chirp_mass``
    / ``mass_ratio``) gives the same result here, and a set that lacks a
    needed parameter raises ``KeyError``.  ``noise_log_likelihood()`` is the
    server's value for the analysis, fetched once."""

    def __init__(self, address, key, authkey: bytes = b"gwlnl", convert_on_client: bool = True):
        self.address, self.key, self.authkey = address, key, authkey
        self.convert_on_client = convert_on_client
        self._noise = None
        self._preparer = None
        self._conn = None

    def _connection(self):
        if self._conn is None:
            from multiprocessing.connection import Client
            self._conn = Client(self.address, authkey=self.authkey)
        return self._conn

    def __getstate__(self):
        st = dict(self.__dict__)
        st["_conn"] = None
        return st

    def _call(self, kind, payload):
        conn = self._connection()
        conn.send((kind, self.key, payload))
        status, result = conn.recv()
        if status != "ok":
            if result.startswith("KeyError"):
                raise KeyError(result)
            raise RuntimeError(result)
        return result

    @property
    def preparer(self):
        if self._preparer is None:
            self._preparer = self._call("spec", None)
        return self._preparer

    def log_likelihood_ratio_batch(self, parameters) -> np.ndarray:
        if self.convert_on_client:
            # the packed block as raw bytes after a small header (no pickling)
            block = np.ascontiguousarray(self.preparer.block(parameters), dtype=np.float64)
            conn = self._connection()
            conn.send(("eval_raw", self.key, int(block.shape[1])))
            conn.send_bytes(block)
            status, result = conn.recv()
            if status != "ok":
                if result.startswith("KeyError"):
                    raise KeyError(result)
                raise RuntimeError(result)
            return result
        return self._call("eval_parameters", {k: (v if isinstance(v, str) else np.asarray(v, dtype=np.float64))
                                              for k, v in dict(parameters).items()})

    def log_likelihood_ratio(self, parameters) -> float:
        return float(self.log_likelihood_ratio_batch(parameters)[0])

    def noise_log_likelihood(self) -> float:
        if self._noise is None:
            self._noise = float(self._call("noise", None))
        return self._noise

    def log_likelihood(self, parameters) -> float:
        return self.log_likelihood_ratio(parameters) + self.noise_log_likelihood()

"""Benchmark of the GW-transient likelihood hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

The metric is the served mixed-precision likelihood against the plain float64
kernel on the mixed-duration TaylorF2 workload: 64 analyses (durations 4-128
s, 2048 or 4096 Hz, 2-3 detectors, 256-4096 points each, 75,945 points in
all), served to 200 sampler clients.

* ``value``: one step is one batched launch sequence over all 64 analyses
  (one persistent kernel per detector count, replayed from a CUDA graph) with
  the parameter blocks resident in HBM; mixed precision with its error
  control; CUDA events on the launching stream; inputs larger than L2 and the
  L2 flushed (256 MiB write) before every timed step.
* ``e2e``: the served path end to end: 200 clients in 8 spawned processes send
  sampler parameter dictionaries (chirp mass / mass ratio) through the IPC
  client ``ServedLikelihood``; the server converts them, copies them to the
  device, runs continuously batched steps and copies the results back.
  ``e2e.value`` is the saturated throughput (every client back to back);
  ``p50_ms`` / ``p99_ms`` are the clients' latencies at 80% of it (Poisson
  arrivals).
* ``fp64``: the plain float64 kernel (the drop-in) over the whole uneven
  batch; ``served_over_fp64`` = e2e / fp64.
* Sub-objects: the single-analysis TaylorF2 launch (128 s at 4096 Hz,
  4096 points: the kernel the roofline is measured on), the sine-Gaussian
  configuration, the time+phase+distance marginalised configuration, the fast
  likelihoods, the single-point drop-in call, and CPU baselines measured in
  this run on the host cores (the oracle's numpy restatement of bilby's path).

``--impl reference`` times the reference algorithm on the host cores (the
oracle, one process per core) over the same 64-analysis mix.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import math
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "lnL evals/s, served mixed-precision vs plain FP64 @|ΔlnL|≤1e-3; p50/p99 ms"
FLUSH_BYTES = 256 << 20
WORKLOAD = "uneven64_served"

# Issue slots (thread instructions) per (point, in-band bin) of the mixed
# TaylorF2 inner loop, frozen from ncu's executed-instruction count of
# k_mixed_tf2 at tf2_128s, B = 4096 (H1/L1/V1): 739 M warp instructions x
# 31.76 active lanes / (4096 points x 259,585 in-band bins) = 22.1.  Counted
# for three detectors only (the single-analysis workload's); another
# detector count gets no issue roofline.
ISSUE_PER_POINT_BIN = {3: 22.1}
# files that define k_mixed_tf2: the DRAM traffic of a committed ncu capture
# is used only while their hash matches the one recorded with it
KERNEL_SOURCES = ["bilby_gb300/csrc/gwl_kernels.cu", "bilby_gb300/csrc/gwl_phase.cuh",
                  "bilby_gb300/csrc/gwl_device.cuh", "bilby_gb300/csrc/gwl_math.cuh",
                  "bilby_gb300/csrc/gwl_internal.h"]


def kernel_source_hash() -> str:
    h = hashlib.sha256()
    for rel in KERNEL_SOURCES:
        with open(os.path.join(ROOT, rel), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n-analyses", type=int, default=64)
    ap.add_argument("--fp64-steps", type=int, default=2, help="timed steps of the float64 uneven batch")
    ap.add_argument("--single-workload", default="tf2_128s", help="the single-analysis (roofline) workload")
    ap.add_argument("--batch", type=int, default=0, help="points per single-analysis launch (default: the workload's)")
    ap.add_argument("--fp64-batch", type=int, default=512, help="points per float64 single-analysis launch")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=6.0, help="pool time per CPU baseline sample")
    ap.add_argument("--cpu-latency-draws", type=int, default=200, help="single-process draws per CPU latency")
    ap.add_argument("--no-serving", action="store_true", help="skip both serving runs")
    ap.add_argument("--no-ipc", action="store_true", help="skip the IPC serving run")
    ap.add_argument("--serve-seconds", type=float, default=6.0, help="duration of each serving run")
    ap.add_argument("--ipc-procs", type=int, default=8, help="client processes of the IPC serving run")
    ap.add_argument("--serve-streams", type=int, default=3, help="serving steps in flight")
    ap.add_argument("--serve-max-points", type=int, default=1 << 15, help="points per serving step at most")
    ap.add_argument("--no-single", action="store_true", help="skip the single-analysis launch")
    ap.add_argument("--no-uneven", action="store_true",
                    help="profiling runs: skip the 64-analysis step and the served runs (the line's value is null)")
    ap.add_argument("--no-sg", action="store_true", help="skip the sine-Gaussian workload")
    ap.add_argument("--no-marg", action="store_true", help="skip the marginalised workload")
    ap.add_argument("--no-relbin", action="store_true", help="skip the relative-binning workload")
    ap.add_argument("--no-multiband", action="store_true", help="skip the multi-banding workload")
    ap.add_argument("--no-roq", action="store_true", help="skip the ROQ workload")
    ap.add_argument("--no-drop-in", action="store_true", help="skip the single-point call latency")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "10",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() in ("active", "1"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# workload construction through the library's own API
# ---------------------------------------------------------------------------
def build_likelihood(w, precision="mixed"):
    """A likelihood for workload ``w`` built through the library's public API."""
    from bilby_gb300 import random as grandom
    from bilby_gb300.detector import InterferometerList
    from bilby_gb300.likelihood import GravitationalWaveTransient
    from bilby_gb300.source import sinegaussian, taylorf2_aligned
    from bilby_gb300.waveform_generator import WaveformGenerator
    grandom.seed(w.seed)
    ifos = InterferometerList(list(w.detectors))
    ifos.set_strain_data_from_power_spectral_densities(w.sampling_frequency, w.duration, w.start_time)
    model = sinegaussian if w.model == "sinegaussian" else taylorf2_aligned
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=model,
                            waveform_arguments=dict(minimum_frequency=w.minimum_frequency)
                            if w.model == "taylorf2" else None)
    ifos.inject_signal(waveform_generator=wfg, parameters=dict(w.injection))
    return GravitationalWaveTransient(ifos, wfg, precision=precision)


def uneven_launches_per_step(ws) -> int:
    """Kernels one batched step launches: prologue, ordering scan and scatter,
    per detector count the fast kernel and the accurate kernel of the error
    control, the split-K reduction and the finalize."""
    classes = {len(w.detectors) for w in ws}
    return 3 + 2 * len(classes) + 2


def bench_uneven(likes, ws, steps, warmup, fp64_steps, seed=17):
    """Value of the line: one batched launch over all analyses per step
    (CUDA graph replay), then the plain float64 kernel over the same whole
    batch, and |dlnL| between the two for every point."""
    import torch
    from bilby_gb300.analysis import params_block
    from bilby_gb300.batching import Batcher
    from bilby_gb300.workloads import draw_points
    rng = np.random.default_rng(seed)
    stream = torch.cuda.Stream()
    bat = Batcher(use_graphs=True)
    blocks = [torch.from_numpy(params_block(draw_points(w, w.batch, rng))).cuda() for w in ws]
    outs = [torch.empty(w.batch, dtype=torch.float64, device="cuda") for w in ws]
    items = [(lk.analysis, b.data_ptr(), b.shape[1], o.data_ptr()) for lk, b, o in zip(likes, blocks, outs)]
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    tuned = [lk.analysis.autotune(b.data_ptr(), b.shape[1], stream.cuda_stream)[0] for lk, b in zip(likes, blocks)]
    torch.cuda.synchronize()

    def run(precision, n_steps, n_warm):
        for _ in range(n_warm):
            bat.eval_device(items, precision, stream.cuda_stream)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n_steps)]
        for s in range(n_steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(s))
            ev[s][0].record(stream)
            bat.eval_device(items, precision, stream.cuda_stream)
            ev[s][1].record(stream)
        torch.cuda.synchronize()
        bat.check()
        return [a.elapsed_time(b) for a, b in ev]

    ms = run("mixed", steps, warmup)
    refined = bat.last_refined(stream.cuda_stream)
    mixed = torch.cat([o.clone() for o in outs])
    ms64 = run("fp64", fp64_steps, 1)
    fp64 = torch.cat(outs)
    pts = sum(w.batch for w in ws)
    pbd = sum(w.batch * (w.n_bins - int(w.minimum_frequency * w.duration)) * len(w.detectors) for w in ws)
    value = pts * steps / (sum(ms) / 1e3)
    value64 = pts * fp64_steps / (sum(ms64) / 1e3)
    errs = (mixed - fp64).abs().cpu().numpy()
    lnls = fp64.cpu().numpy()
    j = int(np.argmax(errs))
    bat.close()
    return {"analyses": len(ws), "points_per_step": pts, "value": value, "unit": "evals/s",
            "ms_per_step": float(np.mean(ms)), "ms_steps": ms,
            "point_bin_detector_per_s": pbd * steps / (sum(ms) / 1e3),
            "launch": "one persistent kernel per detector count, CUDA-graph replay",
            "launches_per_step": uneven_launches_per_step(ws),
            "refined_points_per_step": refined,
            "autotuned_chunks_per_group": {str(c): tuned.count(c) for c in sorted(set(tuned))},
            "fp64": {"value": value64, "unit": "evals/s", "points_per_step": pts, "steps": fp64_steps,
                     "ms_per_step": float(np.mean(ms64)), "sample": "the whole uneven batch, one batched launch"},
            "mixed_over_fp64": value / value64,
            "max_abs_dlnl_mixed_vs_fp64": float(errs[j]), "lnl_at_max_dlnl": float(lnls[j]),
            "fraction_of_points_with_abs_dlnl_le_1e-3": float(np.mean(errs <= 1e-3)),
            "points_compared": int(len(errs))}


# ---------------------------------------------------------------------------
# serving: in-process submissions and IPC clients in other processes
# ---------------------------------------------------------------------------
def make_server(likes, n_streams, max_points):
    from bilby_gb300.serving import LikelihoodServer
    srv = LikelihoodServer(hbm_budget_bytes=160e9, max_points_per_step=max_points, n_streams=n_streams)
    for q, lk in enumerate(likes):
        srv.add_analysis(q, lk)
    return srv.start()


def bench_serving(srv, ws, seconds, capacity, n_clients=200, seed=23):
    """200 clients with Poisson arrivals (rate for ~80% load), batches
    log-uniform in [64, 8192] points, submitted in-process as packed blocks."""
    from bilby_gb300.analysis import params_block
    from bilby_gb300.workloads import draw_points
    rng = np.random.default_rng(seed)
    mean_b = (8192 - 64) / math.log(128)
    rate = 0.8 * capacity / mean_b
    pool = [params_block(draw_points(w, 8192, rng)) for w in ws]
    for q in range(len(ws)):
        srv.submit(q, pool[q][:, :64]).result(120)
    srv.stats = type(srv.stats)()
    futs = []
    t0 = time.perf_counter()
    t_next = t0
    while t_next - t0 < seconds:
        t_next += rng.exponential(1.0 / rate)
        now = time.perf_counter()
        if t_next > now:
            time.sleep(t_next - now)
        q = int(rng.integers(0, len(ws)))
        b = int(round(math.exp(rng.uniform(math.log(64), math.log(8192)))))
        off = int(rng.integers(0, 8192 - b + 1))
        futs.append(srv.submit(q, pool[q][:, off:off + b], client=int(rng.integers(0, n_clients))))
    for f in futs:
        f.result(300)
    out = srv.stats.summary()
    out.update({"clients": n_clients, "arrival_rate_per_s": rate, "target_load": 0.8,
                "batch": "log-uniform [64, 8192]", "submission": "in-process, packed parameter blocks"})
    return out


def _sampler_pool(w, n, rng):
    """Prior draws of an analysis as a sampler sends them: chirp mass and
    mass ratio instead of component masses."""
    from bilby_gb300.workloads import draw_points
    p = draw_points(w, n, rng)
    m1, m2 = p.pop("mass_1"), p.pop("mass_2")
    p["chirp_mass"] = (m1 * m2) ** 0.6 / (m1 + m2) ** 0.2
    p["mass_ratio"] = m2 / m1
    return p


def _ipc_client_proc(address, ws, clients, rate_per_client, t_start, seconds, closed_loop, seed, conn):
    """Sampler clients of one process, one thread and one connection each,
    each bound to one analysis; per request: (scheduled arrival, completion,
    points)."""
    from bilby_gb300.serving import ServedLikelihood
    rng0 = np.random.default_rng(seed)
    pools = {}
    for c in clients:
        q = c % len(ws)
        if q not in pools:
            pools[q] = _sampler_pool(ws[q], 8192, rng0)
    records = []
    lock = threading.Lock()

    def client(c):
        q = c % len(ws)
        like = ServedLikelihood(address, q)
        rng = np.random.default_rng(seed * 1000 + c)
        pool = pools[q]
        like.log_likelihood_ratio_batch({k: v[:8] for k, v in pool.items()})  # connect
        t_arr = t_start
        mine = []
        while True:
            if closed_loop:
                t_arr = max(time.perf_counter(), t_start)
            else:
                t_arr += rng.exponential(1.0 / rate_per_client)
            if t_arr - t_start >= seconds:
                break
            now = time.perf_counter()
            if t_arr > now:
                time.sleep(t_arr - now)
            b = int(round(math.exp(rng.uniform(math.log(64), math.log(8192)))))
            off = int(rng.integers(0, 8192 - b + 1))
            res = like.log_likelihood_ratio_batch({k: v[off:off + b] for k, v in pool.items()})
            t_done = time.perf_counter()
            ok = bool(np.all(np.isfinite(res))) and len(res) == b
            mine.append((t_arr, t_done, b, ok))
        with lock:
            records.extend(mine)

    threads = [threading.Thread(target=client, args=(c,)) for c in clients]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    conn.send(records)
    conn.close()


def bench_serving_ipc(srv, ws, seconds, procs=8, n_clients=200, seed=29):
    """The served path end to end: client processes send sampler dictionaries
    through ServedLikelihood over a Unix socket.  Phase 1: every client back to
    back (saturated throughput); phase 2: Poisson arrivals at 80% of it
    (latency)."""
    from bilby_gb300.serving import serve_ipc
    address = os.path.join(tempfile.mkdtemp(), "gwl.sock")
    listener = serve_ipc(srv, address)
    ctx = mp.get_context("spawn")
    groups = [list(range(p, n_clients, procs)) for p in range(procs)]

    def phase(closed_loop, rate_per_client, dur):
        srv.stats = type(srv.stats)()
        t_start = time.perf_counter() + 6.0   # time for the client processes to start and connect
        pipes, ps = [], []
        for p, cl in enumerate(groups):
            r, w_ = ctx.Pipe(duplex=False)
            pr = ctx.Process(target=_ipc_client_proc,
                             args=(address, ws, cl, rate_per_client, t_start, dur, closed_loop, seed + p, w_))
            pr.start()
            pipes.append(r)
            ps.append(pr)
        recs = []
        for r in pipes:
            recs.extend(r.recv())
        for pr in ps:
            pr.join(60)
        lat = np.array([d - a for a, d, _, _ in recs]) * 1e3
        pts = sum(b for _, _, b, _ in recs)
        span = max(d for _, d, _, _ in recs) - t_start
        return {"requests": len(recs), "points": int(pts), "evals_per_s": pts / span,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "all_finite": all(ok for *_, ok in recs), "server": srv.stats.summary()}

    sat = phase(True, 0.0, seconds)
    mean_b = (8192 - 64) / math.log(128)
    rate = 0.8 * sat["evals_per_s"] / mean_b
    loaded = phase(False, rate / n_clients, seconds)
    threading.Thread(target=listener.close, daemon=True).start()
    return {"clients": n_clients, "client_processes": procs, "batch": "log-uniform [64, 8192]",
            "request": "sampler dict (chirp_mass, mass_ratio, spins, distance, angles, time) through "
                       "ServedLikelihood; converted in the server by the analysis's likelihood",
            "saturated": sat, "at_80pct": dict(loaded, arrival_rate_per_s=rate, target_load=0.8)}


def bench_single(args, like, w, B, steps, warmup, sptr):
    """The single-analysis launch (the roofline's kernel): mixed precision at
    B points, the plain float64 kernel at a smaller batch, |dlnL| between
    them, and the public batch API with host arrays."""
    import torch
    from bilby_gb300.analysis import params_block
    from bilby_gb300.workloads import draw_points
    an = like.analysis
    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(w.draw_seed + 7919)
    host_params = [draw_points(w, B, rng) for _ in range(4)]
    blocks = [torch.from_numpy(params_block(p)).cuda() for p in host_params]
    out = torch.empty(B, dtype=torch.float64, device="cuda")
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    tuned_cpg, _ = an.autotune(blocks[0].data_ptr(), B, sptr)
    an.set_profiling(True)

    def timed(precision, bl, n_steps, warm):
        for s in range(warm):
            an.log_likelihood_ratio_device(bl[s % len(bl)].data_ptr(), bl[0].shape[1], out.data_ptr(), precision,
                                           sptr)
        torch.cuda.synchronize()
        an.last_kernel_ms()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n_steps)]
        kms = []
        for s in range(n_steps):
            flush.fill_(float(s))
            ev[s][0].record(stream)
            an.log_likelihood_ratio_device(bl[(warm + s) % len(bl)].data_ptr(), bl[0].shape[1], out.data_ptr(),
                                           precision, sptr)
            ev[s][1].record(stream)
            kms.append(an.last_kernel_ms())
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in ev], kms

    ms, kms = timed("mixed", blocks, steps, warmup)
    refined = an.last_refined(sptr)
    Bf = min(args.fp64_batch, B)
    fblocks = [b[:, :Bf].contiguous() for b in blocks[:3]]
    fms, _ = timed("fp64", fblocks, 3, 1)
    an.set_profiling(False)
    res64 = torch.empty(Bf, dtype=torch.float64, device="cuda")
    resmx = torch.empty(Bf, dtype=torch.float64, device="cuda")
    an.log_likelihood_ratio_device(fblocks[0].data_ptr(), Bf, res64.data_ptr(), "fp64", sptr)
    an.log_likelihood_ratio_device(fblocks[0].data_ptr(), Bf, resmx.data_ptr(), "mixed", sptr)
    torch.cuda.synchronize()
    e2e = []
    for s in range(warmup + steps):
        p = host_params[s % len(host_params)]
        t0 = time.perf_counter()
        res = like.log_likelihood_ratio_batch(p)
        if s >= warmup:
            e2e.append(time.perf_counter() - t0)
        assert res.shape == (B,)
    value = B * steps / (sum(ms) / 1e3)
    fp64_value = Bf * 3 / (sum(fms) / 1e3)
    return {"workload": w.name, "model": w.model, "detectors": list(w.detectors), "n_bins": w.n_bins, "batch": B,
            "value": value, "unit": "evals/s", "ms_per_launch": float(np.mean(ms)),
            "kernel_ms": float(np.mean(kms)), "autotuned_chunks_per_group": tuned_cpg,
            "refined_points_per_launch": refined,
            "fp64": {"value": fp64_value, "unit": "evals/s", "batch": Bf},
            "mixed_over_fp64": value / fp64_value,
            "max_abs_dlnl_mixed_vs_fp64": float((res64 - resmx).abs().max().item()),
            "e2e": {"value": B * steps / sum(e2e), "unit": "evals/s", "h2d_bytes_per_step": 8 * 15 * B,
                    "d2h_bytes_per_step": 8 * B,
                    "call": "GravitationalWaveTransient.log_likelihood_ratio_batch(dict of host numpy arrays)"}}


def bench_sine_gaussian(steps, warmup, batch=10000, seed=43):
    """The sine-Gaussian configuration: H1+L1, 4 s at 2048 Hz, 10^4 prior
    draws per launch; mixed and float64 kernels and |dlnL| between them."""
    import torch
    from bilby_gb300.analysis import params_block
    from bilby_gb300.workloads import WORKLOADS, draw_points
    w = WORKLOADS["sg_4s"]
    like = build_likelihood(w, precision="mixed")
    an = like.analysis
    rng = np.random.default_rng(seed)
    half = batch // 2
    pf = draw_points(w, half, rng, fixed_extrinsic=True)
    pr = draw_points(w, batch - half, rng, fixed_extrinsic=False)
    block = torch.from_numpy(params_block({k: np.concatenate([pf[k], pr[k]]) for k in pf})).cuda()
    res = {}
    outs = {}
    for precision in ("mixed", "fp64"):
        ms, finite = time_launches(an, block, batch, steps, warmup, precision)
        res[precision] = {"value": batch / (ms / 1e3), "unit": "evals/s", "ms_per_launch": ms}
        o = torch.empty(batch, dtype=torch.float64, device="cuda")
        an.log_likelihood_ratio_device(block.data_ptr(), batch, o.data_ptr(), precision,
                                       torch.cuda.current_stream().cuda_stream)
        outs[precision] = o
    torch.cuda.synchronize()
    err = (outs["mixed"] - outs["fp64"]).abs()
    return {"workload": w.name, "batch": batch, "draws": "half at the injection's sky position and time, half "
            "with sky, psi and time drawn", "mixed": res["mixed"], "fp64": res["fp64"],
            "mixed_over_fp64": res["mixed"]["value"] / res["fp64"]["value"],
            "max_abs_dlnl_mixed_vs_fp64": float(err.max().item()),
            "refined_points_per_launch": an.last_refined(torch.cuda.current_stream().cuda_stream)}


def bench_drop_in(like, w, n_calls=200, seed=47):
    """log_likelihood_ratio(dict): one point per call, the call samplers make
    unchanged; p50 / p99 milliseconds per call for each precision."""
    from bilby_gb300.workloads import draw_points, point
    p = draw_points(w, n_calls + 10, np.random.default_rng(seed))
    out = {}
    for precision in ("fp64", "mixed"):
        like.precision = precision
        lat = []
        for i in range(n_calls + 10):
            t0 = time.perf_counter()
            v = like.log_likelihood_ratio(point(p, i))
            if i >= 10:
                lat.append(time.perf_counter() - t0)
            assert np.isfinite(v)
        lat = np.array(lat) * 1e3
        out[precision] = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                          "calls": n_calls}
    like.precision = "mixed"
    return {"workload": w.name, "call": "GravitationalWaveTransient.log_likelihood_ratio(dict of floats)",
            **out}


def time_launches(an, block, n, steps, warmup, precision="fp64"):
    """Mean CUDA-event milliseconds of one evaluation launch of ``n`` points
    (the device block ``block``), L2 flushed before every timed launch."""
    import torch
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for s in range(warmup):
        an.log_likelihood_ratio_device(block.data_ptr(), n, out.data_ptr(), precision, stream.cuda_stream)
    torch.cuda.synchronize()
    ms = []
    for s in range(steps):
        flush.fill_(float(s))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        an.log_likelihood_ratio_device(block.data_ptr(), n, out.data_ptr(), precision, stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return float(np.mean(ms)), bool(torch.isfinite(out).all().item())


def time_marginalized_block(w, n, rng):
    """``n`` prior draws of workload ``w`` with geocent_time at the segment
    start (the marginalised likelihood's fixed value) and a time jitter."""
    import torch
    from bilby_gb300.analysis import params_block
    from bilby_gb300.workloads import draw_points
    p = draw_points(w, n, rng)
    p["geocent_time"] = np.full(n, float(w.start_time))
    p["time_jitter"] = rng.uniform(-1 / w.sampling_frequency, 1 / w.sampling_frequency, n)
    return torch.from_numpy(params_block(p)).cuda()


def bench_relbin(name, steps, warmup, batch=65536, seed=31):
    """Relative binning (bilby/gw/likelihood/relative.py) on the GPU: fiducial
    = the injection, default chi = 1 and epsilon = 0.5; float64 throughout."""
    import torch
    from bilby_gb300.analysis import params_block
    from bilby_gb300.relative import RelativeBinningGravitationalWaveTransient
    from bilby_gb300.workloads import WORKLOADS, draw_points
    w = WORKLOADS[name]
    base = build_likelihood(w, precision="fp64")
    t0 = time.perf_counter()
    like = RelativeBinningGravitationalWaveTransient(base.interferometers, base.waveform_generator,
                                                     fiducial_parameters=dict(w.injection))
    setup_s = time.perf_counter() - t0
    an = like.analysis
    rng = np.random.default_rng(seed)
    blocks = [torch.from_numpy(params_block(draw_points(w, batch, rng))).cuda() for _ in range(2)]
    out = torch.empty(batch, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for s in range(warmup):
        an.log_likelihood_ratio_device(blocks[s % 2].data_ptr(), batch, out.data_ptr(), "fp64", stream.cuda_stream)
    torch.cuda.synchronize()
    ms = []
    for s in range(steps):
        flush.fill_(float(s))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        an.log_likelihood_ratio_device(blocks[s % 2].data_ptr(), batch, out.data_ptr(), "fp64", stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    res = {"workload": name, "bins": int(like.number_of_bins), "batch": batch,
           "value": batch * steps / (sum(ms) / 1e3), "unit": "evals/s", "ms_per_launch": float(np.mean(ms)),
           "precision": "fp64", "setup_s": setup_s,
           "launch": "prologue + one warp per point over the bin edges"}
    # with time marginalisation (relative.py:380-420): the float64 FFT of
    # length n_bins - 1 over the rebuilt piecewise-linear waveform, per point
    from bilby_gb300.prior import Uniform
    tc = w.injection["geocent_time"]
    priors = {"geocent_time": Uniform(tc - 0.1, tc + 0.1)}
    like_t = RelativeBinningGravitationalWaveTransient(base.interferometers, base.waveform_generator,
                                                       fiducial_parameters=dict(w.injection), priors=priors,
                                                       time_marginalization=True)
    bt = 2048
    block = time_marginalized_block(w, bt, rng)
    tm = {"batch": bt, "fft_length": int(like_t.analysis.n_bins - 1),
          "launch": "prologue + windowed four-step transform, one CTA per point (float32 with refinement "
                    "of the marked points in float64, or float64)"}
    outs = {}
    for precision in ("fp64", "mixed"):
        ms_t, finite = time_launches(like_t.analysis, block, bt, steps, warmup, precision=precision)
        o = torch.empty(bt, dtype=torch.float64, device="cuda")
        like_t.analysis.log_likelihood_ratio_device(block.data_ptr(), bt, o.data_ptr(), precision, stream.cuda_stream)
        torch.cuda.synchronize()
        outs[precision] = o
        tm[precision] = {"value": bt / (ms_t / 1e3), "unit": "evals/s", "ms_per_launch": ms_t, "finite": finite}
        if precision == "mixed":
            tm[precision]["refined_points_per_launch"] = int(like_t.analysis.last_refined())
    tm["mixed_over_fp64"] = tm["mixed"]["value"] / tm["fp64"]["value"]
    tm["max_abs_dlnl_mixed_vs_fp64"] = float((outs["mixed"] - outs["fp64"]).abs().max().item())
    res["time_marginalized"] = tm
    return res


def bench_multiband(name, steps, warmup, batch=16384, seed=37):
    """Multi-banding (bilby/gw/likelihood/multiband.py, linear interpolation
    of <h|h>) on the GPU: reference chirp mass 0.87 (the 1+1 Msun prior
    corner); the float64 kernel and the mixed-precision one, with |dlnL|
    between them on the first batch."""
    import torch
    from bilby_gb300.analysis import params_block
    from bilby_gb300.multiband import MBGravitationalWaveTransient
    from bilby_gb300.workloads import WORKLOADS, draw_points
    w = WORKLOADS[name]
    base = build_likelihood(w, precision="fp64")
    t0 = time.perf_counter()
    like = MBGravitationalWaveTransient(base.interferometers, base.waveform_generator, reference_chirp_mass=0.87)
    setup_s = time.perf_counter() - t0
    an = like.analysis
    rng = np.random.default_rng(seed)
    blocks = [torch.from_numpy(params_block(draw_points(w, batch, rng))).cuda() for _ in range(2)]
    out = torch.empty(batch, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    res = {}
    for precision in ("fp64", "mixed"):
        for s in range(warmup):
            an.log_likelihood_ratio_device(blocks[s % 2].data_ptr(), batch, out.data_ptr(), precision,
                                           stream.cuda_stream)
        torch.cuda.synchronize()
        ms = []
        for s in range(steps):
            flush.fill_(float(s))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            an.log_likelihood_ratio_device(blocks[s % 2].data_ptr(), batch, out.data_ptr(), precision,
                                           stream.cuda_stream)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        res[precision] = {"value": batch * steps / (sum(ms) / 1e3), "unit": "evals/s",
                          "ms_per_launch": float(np.mean(ms))}
    o64 = torch.empty(batch, dtype=torch.float64, device="cuda")
    omx = torch.empty(batch, dtype=torch.float64, device="cuda")
    an.log_likelihood_ratio_device(blocks[0].data_ptr(), batch, o64.data_ptr(), "fp64", stream.cuda_stream)
    an.log_likelihood_ratio_device(blocks[0].data_ptr(), batch, omx.data_ptr(), "mixed", stream.cuda_stream)
    torch.cuda.synchronize()
    # with time marginalisation (multiband.py:714-726, 792-800): the float64
    # FFT of length Nbs[-1] / 2 over the scattered banded strain, per point
    from bilby_gb300.prior import Uniform
    tc = w.injection["geocent_time"]
    like_t = MBGravitationalWaveTransient(base.interferometers, base.waveform_generator, reference_chirp_mass=0.87,
                                          priors={"geocent_time": Uniform(tc - 0.1, tc + 0.1)},
                                          time_marginalization=True)
    bt = 2048
    block_t = time_marginalized_block(w, bt, rng)
    tm = {"batch": bt, "fft_length": int(like_t._mb_tm[0]),
          "banded_frequencies": int(len(like_t.banded_frequency_points)),
          "launch": "prologue + windowed four-step transform, one CTA per point (float32 banded values and "
                    "transform with refinement of the marked points in float64, or float64)"}
    outs = {}
    for precision in ("fp64", "mixed"):
        ms_t, finite = time_launches(like_t.analysis, block_t, bt, steps, warmup, precision=precision)
        o = torch.empty(bt, dtype=torch.float64, device="cuda")
        like_t.analysis.log_likelihood_ratio_device(block_t.data_ptr(), bt, o.data_ptr(), precision,
                                                    stream.cuda_stream)
        torch.cuda.synchronize()
        outs[precision] = o
        tm[precision] = {"value": bt / (ms_t / 1e3), "unit": "evals/s", "ms_per_launch": ms_t, "finite": finite}
        if precision == "mixed":
            tm[precision]["refined_points_per_launch"] = int(like_t.analysis.last_refined())
    tm["mixed_over_fp64"] = tm["mixed"]["value"] / tm["fp64"]["value"]
    tm["max_abs_dlnl_mixed_vs_fp64"] = float((outs["mixed"] - outs["fp64"]).abs().max().item())
    for ifo in base.interferometers:  # the MB time set-up fixes the antenna time on the interferometers
        ifo.reference_time = None
    # the IFFT-FFT <h|h> (linear_interpolation=False, multiband.py:760-779):
    # the odd-bin float64 transforms of bands 1.. per point and detector pair
    like_f = MBGravitationalWaveTransient(base.interferometers, base.waveform_generator, reference_chirp_mass=0.87,
                                          linear_interpolation=False)
    bf, bfm = 2048, 8192
    block_f = torch.from_numpy(params_block(draw_points(w, bf, rng))).cuda()
    block_fm = torch.from_numpy(params_block(draw_points(w, bfm, rng))).cuda()
    ifft = {"batch": bf, "batch_mixed": bfm, "transform_lengths": [int(m) for m in like_f.Mbs[1:]],
            "launch": "prologue + per band k_mb_hh_fft (float64) or k_mb_hh_fft32 (float32 with an error bound, "
                      "the marked points recomputed by k_mb_hh_fft), packed detector pairs, + the multi-banding "
                      "kernel"}
    outs_f = {}
    for precision in ("fp64", "mixed"):
        blk, nb = (block_f, bf) if precision == "fp64" else (block_fm, bfm)
        ms_f, finite = time_launches(like_f.analysis, blk, nb, steps, warmup, precision=precision)
        ifft[precision] = {"value": nb / (ms_f / 1e3), "unit": "evals/s", "ms_per_launch": ms_f, "finite": finite}
        o = torch.empty(bf, dtype=torch.float64, device="cuda")
        like_f.analysis.log_likelihood_ratio_device(block_f.data_ptr(), bf, o.data_ptr(), precision,
                                                    stream.cuda_stream)
        torch.cuda.synchronize()
        outs_f[precision] = o
    ifft["mixed_over_fp64"] = ifft["mixed"]["value"] / ifft["fp64"]["value"]
    ifft["max_abs_dlnl_mixed_vs_fp64"] = float((outs_f["mixed"] - outs_f["fp64"]).abs().max().item())
    return {"workload": name, "bands": int(like.number_of_bands),
            "banded_frequencies": int(len(like.banded_frequency_points)), "batch": batch,
            "value": res["fp64"]["value"], "unit": "evals/s", "ms_per_launch": res["fp64"]["ms_per_launch"],
            "precision": "fp64", "mixed": res["mixed"], "mixed_over_fp64": res["mixed"]["value"] / res["fp64"]["value"],
            "max_abs_dlnl_mixed_vs_fp64": float((omx - o64).abs().max().item()), "setup_s": setup_s,
            "launch": "prologue + one warp per point over the banded frequencies",
            "time_marginalized": tm, "ifft_fft": ifft}


def eim_basis(f, n_linear, n_quadratic, n_train, seed, fmin, mass_range=(10.0, 40.0)):
    """A seeded ROQ basis of the stated size on frequencies ``f``: reduced
    bases (SVD) of normalised TaylorF2 training waveforms (and of their
    squared moduli) with greedy empirical-interpolation nodes, the standard
    construction (Field et al., arXiv:1308.3565).  Returns (linear nodes,
    linear basis N x n, quadratic nodes, quadratic basis N x m)."""
    from bilby_gb300.source import taylorf2_aligned
    rng = np.random.default_rng(seed)
    lin, quad = [], []
    for _ in range(n_train):
        m1, m2 = np.sort(rng.uniform(*mass_range, 2))[::-1]
        h = taylorf2_aligned(f, m1, m2, rng.uniform(-0.05, 0.05), rng.uniform(-0.05, 0.05), 100.0, 0.0, 0.0,
                             minimum_frequency=fmin)["plus"]
        lin.append(h / np.linalg.norm(h))
        q = np.abs(h) ** 2
        quad.append(q / np.linalg.norm(q))

    def eim(basis):
        nodes = [int(np.argmax(np.abs(basis[:, 0])))]
        for j in range(1, basis.shape[1]):
            coef = np.linalg.solve(basis[nodes, :j], basis[nodes, j])
            nodes.append(int(np.argmax(np.abs(basis[:, j] - basis[:, :j] @ coef))))
        return np.array(nodes), np.linalg.solve(basis[nodes, :].T, basis.T).T

    ul = np.linalg.svd(np.array(lin).T, full_matrices=False)[0][:, :n_linear]
    uq = np.linalg.svd(np.array(quad).T, full_matrices=False)[0][:, :n_quadratic]
    nl, bl = eim(ul)
    nq, bq = eim(uq)
    order_l, order_q = np.argsort(nl), np.argsort(nq)
    return f[nl][order_l], bl[:, order_l], f[nq][order_q], bq[:, order_q].real


def bench_roq(name, steps, warmup, batch=65536, n_linear=400, n_quadratic=100, seed=41):
    """Reduced-order quadrature on the GPU (bilby/gw/likelihood/roq.py, one
    basis).  ROQ bases are data files the container does not have, so a
    seeded empirical-interpolation basis of TaylorF2 waveforms of the stated
    size stands in (eim_basis).  The float64 cost depends on the numbers of
    nodes and time samples only; the mixed-precision error bound, and so the
    share of points recomputed in float64, on the sizes of the weight-node
    products, which a basis of real waveforms gives."""
    import torch
    from bilby_gb300.analysis import params_block
    from bilby_gb300.prior import Uniform
    from bilby_gb300.roq import ROQGravitationalWaveTransient
    from bilby_gb300.source import taylorf2_aligned_roq
    from bilby_gb300.waveform_generator import WaveformGenerator
    from bilby_gb300.workloads import WORKLOADS, draw_points
    w = WORKLOADS[name]
    base = build_likelihood(w, precision="fp64")
    ifos = base.interferometers
    rng = np.random.default_rng(seed)
    fm = np.asarray(ifos[0].strain_data.frequency_array)[np.asarray(ifos[0].strain_data.frequency_mask)]
    nl, lin, nq, quad = eim_basis(fm, n_linear, n_quadratic, 2 * n_linear + 100, seed, w.minimum_frequency)
    wfg = WaveformGenerator(duration=w.duration, sampling_frequency=w.sampling_frequency, start_time=w.start_time,
                            frequency_domain_source_model=taylorf2_aligned_roq,
                            waveform_arguments=dict(minimum_frequency=w.minimum_frequency,
                                                    frequency_nodes_linear=nl, frequency_nodes_quadratic=nq))
    tc = w.injection["geocent_time"]
    t0 = time.perf_counter()
    like = ROQGravitationalWaveTransient(ifos, wfg, {"geocent_time": Uniform(tc - 0.1, tc + 0.1)},
                                         linear_matrix=lin, quadratic_matrix=quad)
    setup_s = time.perf_counter() - t0
    an = like.analysis
    p = draw_points(w, batch, rng)
    p["geocent_time"] = tc + rng.uniform(-0.1, 0.1, batch)
    blocks = [torch.from_numpy(params_block(p)).cuda() for _ in range(2)]
    out = torch.empty(batch, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for s in range(warmup):
        an.log_likelihood_ratio_device(blocks[s % 2].data_ptr(), batch, out.data_ptr(), "fp64", stream.cuda_stream)
    torch.cuda.synchronize()
    ms = []
    for s in range(steps):
        flush.fill_(float(s))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        an.log_likelihood_ratio_device(blocks[s % 2].data_ptr(), batch, out.data_ptr(), "fp64", stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    res = {"workload": name, "linear_nodes": n_linear, "quadratic_nodes": n_quadratic,
           "time_samples": int(len(like.weights["time_samples"])), "batch": batch,
           "value": batch * steps / (sum(ms) / 1e3), "unit": "evals/s", "ms_per_launch": float(np.mean(ms)),
           "precision": "fp64", "setup_s": setup_s,
           "basis": "seeded empirical-interpolation basis of TaylorF2 waveforms of the stated size",
           "launch": "prologue + one warp per point over the nodes"}
    # with time marginalisation (roq.py:320-331, 604-651): every weight row of
    # the prior window contracted per point, five-sample interpolation per time
    like_t = ROQGravitationalWaveTransient(ifos, wfg, {"geocent_time": Uniform(tc - 0.1, tc + 0.1)},
                                           linear_matrix=lin, quadratic_matrix=quad, time_marginalization=True)
    bt, bm = 1024, 8192
    blk_t = time_marginalized_block(w, bt, rng)   # parameter blocks are [slot][point]: one per batch size
    blk_m = time_marginalized_block(w, bm, rng)
    an_t = like_t.analysis
    ms_t, finite = time_launches(an_t, blk_t, bt, steps, warmup)
    ms_m, finite_m = time_launches(an_t, blk_m, bm, steps, warmup, "mixed")
    refined = an_t.last_refined()
    o64 = torch.empty(bt, dtype=torch.float64, device="cuda")
    omx = torch.empty(bt, dtype=torch.float64, device="cuda")
    an_t.log_likelihood_ratio_device(blk_t.data_ptr(), bt, o64.data_ptr(), "fp64", stream.cuda_stream)
    an_t.log_likelihood_ratio_device(blk_t.data_ptr(), bt, omx.data_ptr(), "mixed", stream.cuda_stream)
    torch.cuda.synchronize()
    res["time_marginalized"] = {
        "marginalization_samples": int(len(like_t._times)), "weight_rows": int(len(like_t.weights["time_samples"])),
        "launch": "prologue + per point the model at the nodes, one complex float32 GEMM per detector over every "
                  "weight row (cuBLAS, pedantic float32), per point the interpolation and marginalisation in "
                  "float32 with the error bound, float64 recomputation of the marked points",
        "fp64": {"batch": bt, "value": bt / (ms_t / 1e3), "unit": "evals/s", "ms_per_launch": ms_t,
                 "finite": finite},
        "mixed": {"batch": bm, "value": bm / (ms_m / 1e3), "unit": "evals/s", "ms_per_launch": ms_m,
                  "finite": finite_m, "refined_points_per_launch": refined},
        "mixed_over_fp64": (bm / ms_m) / (bt / ms_t),
        "max_abs_dlnl_mixed_vs_fp64": float((omx - o64).abs().max().item()),
        "points_compared": bt}
    return res


def bench_marginalized(name, steps, warmup, fp64_batch=256, seed=29):
    """Time + phase + distance marginalisation (length-L FFT per point, ln I0,
    bicubic distance table) on the 8 s TaylorF2 workload."""
    import torch
    from bilby_gb300.analysis import params_block
    from bilby_gb300.likelihood import GravitationalWaveTransient
    from bilby_gb300.prior import PowerLaw, Uniform
    from bilby_gb300.workloads import DISTANCE_PRIOR, WORKLOADS, draw_points
    w = WORKLOADS[name]
    base = build_likelihood(w, precision="mixed")
    tc = w.injection["geocent_time"]
    priors = dict(geocent_time=Uniform(tc - 0.1, tc + 0.1), phase=Uniform(0, 2 * np.pi, boundary="periodic"),
                  luminosity_distance=PowerLaw(DISTANCE_PRIOR["alpha"], DISTANCE_PRIOR["minimum"],
                                               DISTANCE_PRIOR["maximum"]))
    import tempfile
    t0 = time.perf_counter()
    like = GravitationalWaveTransient(base.interferometers, base.waveform_generator, priors=priors,
                                      time_marginalization=True, phase_marginalization=True,
                                      distance_marginalization=True, precision="mixed",
                                      distance_marginalization_lookup_table=os.path.join(tempfile.mkdtemp(), "t.npz"))
    setup_s = time.perf_counter() - t0
    rng = np.random.default_rng(seed)
    p = draw_points(w, w.batch, rng)
    p["geocent_time"] = np.full(w.batch, priors["geocent_time"])
    p["phase"] = np.zeros(w.batch)
    p["luminosity_distance"] = np.full(w.batch, priors["luminosity_distance"])
    block = torch.from_numpy(params_block(p)).cuda()
    out = torch.empty(w.batch, dtype=torch.float64, device="cuda")
    an = like.analysis
    stream = torch.cuda.current_stream()
    res = {}
    for precision, B in (("mixed", w.batch), ("fp64", fp64_batch)):
        for _ in range(warmup):
            an.log_likelihood_ratio_device(block.data_ptr(), B, out.data_ptr(), precision, stream.cuda_stream)
        torch.cuda.synchronize()
        ms = []
        n = steps if precision == "mixed" else 3
        bl = block[:, :B].contiguous()
        for _ in range(n):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            an.log_likelihood_ratio_device(bl.data_ptr(), B, out.data_ptr(), precision, stream.cuda_stream)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        res[precision] = {"value": B * n / (sum(ms) / 1e3), "unit": "evals/s", "batch": B,
                          "ms_per_launch": float(np.mean(ms))}
        if precision == "mixed":
            res[precision]["refined_points_per_launch"] = int(an.last_refined())
    m = torch.empty(fp64_batch, dtype=torch.float64, device="cuda")
    f = torch.empty(fp64_batch, dtype=torch.float64, device="cuda")
    bl = block[:, :fp64_batch].contiguous()
    an.log_likelihood_ratio_device(bl.data_ptr(), fp64_batch, m.data_ptr(), "mixed", stream.cuda_stream)
    an.log_likelihood_ratio_device(bl.data_ptr(), fp64_batch, f.data_ptr(), "fp64", stream.cuda_stream)
    torch.cuda.synchronize()
    return {"workload": name, "n_bins": w.n_bins, "fft_length": w.n_bins - 1, "marginalization": "time+phase+distance",
            "mixed": res["mixed"], "fp64": res["fp64"], "mixed_over_fp64": res["mixed"]["value"] / res["fp64"]["value"],
            "max_abs_dlnl_mixed_vs_fp64": float((m - f).abs().max().item()),
            "setup_s_incl_distance_table": setup_s}


# ---------------------------------------------------------------------------
# CPU baselines: the oracle's numpy restatement of the reference path on the
# host cores (one spawned process per core, OMP_NUM_THREADS=1)
# ---------------------------------------------------------------------------
_CPU: dict = {}


def _cpu_init(kind):
    """Worker state for one CPU configuration (built once per process)."""
    os.environ["OMP_NUM_THREADS"] = "1"
    from bilby_gb300.workloads import DISTANCE_PRIOR, WORKLOADS
    from oracle import data as OD
    from oracle import restate as R
    name = {"sg": "sg_4s", "tf2": "tf2_128s", "marg": "tf2_marg_8s", "relbin": "tf2_128s"}[kind]
    w = WORKLOADS[name]
    _CPU.update(kind=kind, w=w, dets=OD.build_workload(w), src=OD.source_for(w.model, w.minimum_frequency))
    if kind == "marg":
        tc = w.injection["geocent_time"]
        lo, hi = tc - 0.1, tc + 0.1
        m = R.Marginalization(time=True, phase=True, distance=True)
        R.setup_time_marginalization(m, w.start_time, w.duration, w.sampling_frequency, lo, hi)
        dist = np.linspace(DISTANCE_PRIOR["minimum"], DISTANCE_PRIOR["maximum"], 10000)
        prior = dist ** 2 / np.sum(dist ** 2 * (dist[1] - dist[0]))
        ref = float(np.interp(0.5, np.cumsum(prior) / np.sum(prior), dist))
        # a table of the reference's shape (400 x 800): the spline's per-sample
        # cost does not depend on its values; its one-off build is not timed
        R.setup_distance_marginalization(m, dist, prior, ref, table=np.zeros((400, 800)))
        _CPU.update(marg=m, prior=lambda t: ((t >= lo) & (t <= hi)) / (hi - lo))
    if kind == "relbin":
        from oracle import relbin as RB
        _CPU["relbin"] = RB.setup(_CPU["dets"], _CPU["src"], dict(w.injection))


def _cpu_eval(p):
    from oracle import restate as R
    k = _CPU["kind"]
    if k == "marg":
        return R.log_likelihood_ratio(_CPU["dets"], _CPU["src"], p, _CPU["marg"], _CPU["prior"])
    if k == "relbin":
        from oracle import relbin as RB
        return RB.log_likelihood_ratio(_CPU["dets"], _CPU["src"], _CPU["relbin"], p)
    return R.log_likelihood_ratio(_CPU["dets"], _CPU["src"], p)


def _cpu_eval_timed(p):
    t0 = time.perf_counter()
    _cpu_eval(p)
    return time.perf_counter() - t0


def _cpu_points(kind, n, seed=123):
    from bilby_gb300.workloads import WORKLOADS, draw_points, point
    name = {"sg": "sg_4s", "tf2": "tf2_128s", "marg": "tf2_marg_8s", "relbin": "tf2_128s"}[kind]
    w = WORKLOADS[name]
    p = draw_points(w, n, np.random.default_rng(seed))
    pts = [point(p, i) for i in range(n)]
    for q in pts:
        if kind == "marg":
            q["geocent_time"], q["phase"] = float(w.start_time), 0.0
            q["luminosity_distance"] = 1000.0
        else:
            q.pop("time_jitter", None)
    return pts


def cpu_config(kind, pool_seconds, latency_draws):
    """(i) one process, ``latency_draws`` draws after 10 warm-up calls: p50 /
    p99 milliseconds; (ii) a pool of one process per core for about
    ``pool_seconds``: evaluations per second."""
    cores = len(os.sched_getaffinity(0))
    ctx = mp.get_context("spawn")
    pts = _cpu_points(kind, max(latency_draws + 10, 4 * cores))
    with ctx.Pool(1, initializer=_cpu_init, initargs=(kind,)) as one:
        lat = np.array(one.map(_cpu_eval_timed, pts[:latency_draws + 10], chunksize=latency_draws + 10))[10:] * 1e3
    per = float(np.median(lat)) / 1e3
    n = int(min(20000, max(4 * cores, pool_seconds * cores / max(per, 1e-6))))
    pool_pts = [pts[i % len(pts)] for i in range(n)]
    with ctx.Pool(cores, initializer=_cpu_init, initargs=(kind,)) as pool:
        pool.map(_cpu_eval, pool_pts[:cores], chunksize=1)
        t0 = time.perf_counter()
        pool.map(_cpu_eval, pool_pts, chunksize=max(1, n // (8 * cores)))
        dt = time.perf_counter() - t0
    what = {"sg": "sg_4s, plain", "tf2": "tf2_128s, plain", "marg": "tf2_marg_8s, time+phase+distance",
            "relbin": "tf2_128s, relative binning (fiducial = injection), plain"}[kind]
    return {"value": n / dt, "unit": "evals/s", "cores": cores, "kind": "port",
            "latency_ms_p50": float(np.percentile(lat, 50)), "latency_ms_p99": float(np.percentile(lat, 99)),
            "sample": f"{what}: {latency_draws} draws in one process for the latency; {n} draws over {cores} "
                      f"processes in {dt:.1f} s for the throughput; oracle (numpy restatement of bilby's "
                      f"log_likelihood_ratio), OMP_NUM_THREADS=1"}


def _mix_worker(n_analyses, mine, conn):
    """Owns the oracle analyses ``mine`` of the 64-analysis mix; per command
    evaluates one draw of each and sends back the seconds of each evaluation."""
    os.environ["OMP_NUM_THREADS"] = "1"
    from bilby_gb300.workloads import draw_points, point, uneven_analyses
    from oracle import data as OD
    from oracle import restate as R
    ws = uneven_analyses(n_analyses)
    own = {}
    for q in mine:
        w = ws[q]
        own[q] = (OD.build_workload(w), OD.source_for(w.model, w.minimum_frequency),
                  draw_points(w, 64, np.random.default_rng(500 + q)))
    conn.send("ready")
    it = 0
    while True:
        msg = conn.recv()
        if msg is None:
            break
        times = []
        for q in mine:
            dets, src, p = own[q]
            t0 = time.perf_counter()
            R.log_likelihood_ratio(dets, src, point(p, it % 64))
            times.append((q, time.perf_counter() - t0))
        it += 1
        conn.send(times)
    conn.close()


class CpuMix:
    """The 64-analysis mix on the host cores: analyses spread over one
    process per core by their cost (bins x detectors, longest first onto the
    least-loaded process); one step evaluates one draw of every analysis
    (the uniform mix the served requests draw from), all processes at once."""

    def __init__(self, n_analyses=64):
        from bilby_gb300.workloads import uneven_analyses
        self.cores = len(os.sched_getaffinity(0))
        ws = uneven_analyses(n_analyses)
        cost = [w.n_bins * len(w.detectors) for w in ws]
        n_proc = min(self.cores, n_analyses)
        loads, owned = [0] * n_proc, [[] for _ in range(n_proc)]
        for q in sorted(range(n_analyses), key=lambda q: -cost[q]):
            j = int(np.argmin(loads))
            owned[j].append(q)
            loads[j] += cost[q]
        ctx = mp.get_context("spawn")
        self.conns, self.procs = [], []
        for mine in owned:
            a, b = ctx.Pipe()
            p = ctx.Process(target=_mix_worker, args=(n_analyses, mine, b))
            p.start()
            self.conns.append(a)
            self.procs.append(p)
        for c in self.conns:
            assert c.recv() == "ready"
        self.n = n_analyses

    def step(self):
        t0 = time.perf_counter()
        for c in self.conns:
            c.send(1)
        times = []
        for c in self.conns:
            times.extend(c.recv())
        return time.perf_counter() - t0, times

    def close(self):
        for c in self.conns:
            c.send(None)
        for p in self.procs:
            p.join(30)

    def run(self, steps, warmup):
        for _ in range(warmup):
            self.step()
        walls, evals = [], []
        for _ in range(steps):
            wall, t = self.step()
            walls.append(wall)
            evals.extend(s for _, s in t)
        lat = np.array(evals) * 1e3
        return {"value": self.n * steps / sum(walls), "unit": "evals/s", "cores": len(self.procs), "kind": "port",
                "latency_ms_p50": float(np.percentile(lat, 50)), "latency_ms_p99": float(np.percentile(lat, 99)),
                "sample": f"{steps} steps of one draw of each of the {self.n} analyses of the mix, {len(self.procs)} "
                          f"processes (analyses assigned by bins x detectors), oracle (numpy restatement of bilby's "
                          f"log_likelihood_ratio), OMP_NUM_THREADS=1, {sum(walls):.1f} s"}


# ---------------------------------------------------------------------------
def mix_config(n):
    from bilby_gb300.workloads import uneven_analyses
    ws = uneven_analyses(n)
    return {"workload": WORKLOAD, "analyses": n, "points_per_step": sum(w.batch for w in ws),
            "durations_s": [4, 8, 16, 32, 64, 128], "sampling_frequencies": [2048, 4096],
            "detectors": "2 or 3 of H1, L1, V1", "model": "taylorf2 (3.5PN aligned spin)",
            "clients": 200, "batch_per_request": "log-uniform [64, 8192]"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    mix = CpuMix(args.n_analyses)
    try:
        steps = max(args.steps, 10)
        r = mix.run(steps, max(1, args.warmup))
    finally:
        mix.close()
    line = {"metric": METRIC, "value": r["value"], "unit": "evals/s", "impl": "reference", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * args.n_analyses / r["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded noise from the bundled aLIGO O4 / AdV PSDs, one injection per analysis)",
            "config": dict(mix_config(args.n_analyses), parallelism=f"host cores x{r['cores']}"),
            "p50_ms": r["latency_ms_p50"], "p99_ms": r["latency_ms_p99"],
            "cpu_baseline": {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": r["value"], "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args, rank, world, local):
    import torch
    from bilby_gb300 import _build, _capi
    from bilby_gb300.workloads import WORKLOADS, uneven_analyses

    torch.cuda.set_device(local)
    _build.build()
    from bilby_gb300.replicas import ReplicaGroup
    dist = ReplicaGroup(world, backend="nccl")
    cpu = {}
    if rank == 0 and not args.no_cpu_baseline:
        # spawned before any CUDA work of this process
        mix = CpuMix(args.n_analyses)
        try:
            cpu["mix"] = mix.run(10, 2)
        finally:
            mix.close()
        for kind in ("sg", "tf2", "marg", "relbin"):
            cpu[kind] = cpu_config(kind, args.cpu_seconds, args.cpu_latency_draws)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    # -- the line's value: the 64-analysis batched step, device resident -------
    uneven = value = total_ms = None
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.05)
    if not args.no_uneven:
        uws = uneven_analyses(args.n_analyses)
        ulikes = [build_likelihood(uw, precision="mixed") for uw in uws]
        dist.barrier()
        uneven = bench_uneven(ulikes, uws, args.steps, args.warmup, args.fp64_steps)
        dist.barrier()
        total_ms = dist.max(float(np.sum(uneven["ms_steps"])))
        value = world * uneven["points_per_step"] * args.steps / (total_ms / 1e3)
    clk = clocks.stop()

    # -- served: in-process and through IPC client processes -------------------
    served = ipc = None
    if world == 1 and not args.no_serving and uneven is not None:
        srv = make_server(ulikes, args.serve_streams, args.serve_max_points)
        served = bench_serving(srv, uws, args.serve_seconds, uneven["value"])
        if not args.no_ipc:
            ipc = bench_serving_ipc(srv, uws, args.serve_seconds, procs=args.ipc_procs)
        srv.stop()

    # -- the single-analysis launch: the roofline's kernel ----------------------
    single = drop_in = None
    w = WORKLOADS[args.single_workload]
    if not args.no_single:
        like = build_likelihood(w, precision="mixed")
        single = bench_single(args, like, w, args.batch or w.batch, args.steps, args.warmup, sptr)
        if not args.no_drop_in:
            drop_in = bench_drop_in(like, w)
        like.analysis.close()
    sg = bench_sine_gaussian(max(3, args.steps // 2), args.warmup) if world == 1 and not args.no_sg else None
    relbin = bench_relbin("tf2_128s", max(3, args.steps // 2), args.warmup) \
        if world == 1 and not args.no_relbin else None
    multiband = bench_multiband("tf2_128s", max(3, args.steps // 4), args.warmup) \
        if world == 1 and not args.no_multiband else None
    roq = bench_roq("tf2_marg_8s_2k", max(3, args.steps // 2), args.warmup) if world == 1 and not args.no_roq else None
    marg = bench_marginalized("tf2_marg_8s", max(3, args.steps // 4), args.warmup) \
        if world == 1 and not args.no_marg else None

    # -- roofline of the mixed TaylorF2 inner loop -----------------------------
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peaks = json.load(open(peaks_path)) if os.path.exists(peaks_path) else {}
    hbm_peak = peaks.get("hbm_gbs")
    peak_src = "MEASURED_PEAKS.json (of measured)"
    if hbm_peak is None:
        hbm_peak, peak_src = 6800.0, "fallback 6.8 TB/s (of fallback)"
    roofline = roofline_hbm = None
    if single is not None:
        D = len(w.detectors)
        n_in = w.n_bins - int(math.ceil(w.minimum_frequency * w.duration))
        B = single["batch"]
        kernel_ms = single["kernel_ms"]
        sm_mhz = clk.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
        props = torch.cuda.get_device_properties(local)
        lanes = props.multi_processor_count * 128
        issue_peak = lanes * sm_mhz * 1e6 / 1e12
        per_bin = ISSUE_PER_POINT_BIN.get(D)
        achieved = per_bin * n_in * B / (kernel_ms / 1e3) / 1e12 if per_bin else None
        n_groups = int(math.ceil(math.ceil(n_in / 512) / single["autotuned_chunks_per_group"]))
        bytes_launch = n_in * 8 * D + 15 * 8 * B + n_groups * B * D * 8
        traffic, traffic_note = None, "no ncu capture recorded for this kernel source"
        tpath = os.path.join(ROOT, "profiles", f"{w.name}_mixed_traffic.json")
        if os.path.exists(tpath):
            t = json.load(open(tpath))
            if t.get("batch") != B:
                traffic_note = f"ncu capture at batch {t.get('batch')}, not {B}"
            elif t.get("kernel_source_sha16") != kernel_source_hash():
                traffic_note = "ncu capture of another kernel source (hash mismatch): not used"
            else:
                traffic = t["traffic_bytes_per_launch"]
                traffic_note = "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch, " + tpath[len(ROOT) + 1:]
        roofline = {"bound": "issue", "achieved": achieved, "peak": issue_peak, "unit": "Tinst/s",
                    "frac": achieved / issue_peak if achieved else None, "traffic": traffic, "kernel": "k_mixed_tf2",
                    "workload": f"{w.name}, B = {B}", "kernel_ms": kernel_ms,
                    "work": f"{per_bin} thread instructions per (point, in-band bin), frozen from "
                            f"ncu's executed-instruction count; {n_in} in-band bins",
                    "peak_source": f"{props.multi_processor_count} SMs x 128 lanes x sampled SM clock {sm_mhz} MHz",
                    "traffic_note": traffic_note,
                    "note": "the served step runs the same inner loop (k_multi_tf2); tables are reused from shared "
                            "memory by every point of a CTA, so DRAM is not the bound"}
        roofline_hbm = {"bound": "hbm", "achieved": bytes_launch / (kernel_ms / 1e3) / 1e9, "peak": hbm_peak,
                        "unit": "GB/s", "frac": bytes_launch / (kernel_ms / 1e3) / 1e9 / hbm_peak,
                        "traffic": traffic, "peak_source": peak_src,
                        "work": "compulsory bytes: polar weight tables (8 B per bin and detector), the parameter "
                                "block and the partial sums"}

    if rank == 0:
        e2e_v = ipc["saturated"]["evals_per_s"] if ipc else None
        ue = uneven or {"fp64": {"value": None}, "mixed_over_fp64": None, "max_abs_dlnl_mixed_vs_fp64": None,
                        "fraction_of_points_with_abs_dlnl_le_1e-3": None, "launches_per_step": 0}
        line = {
            "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps if total_ms else None,
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (exact 0.64 fixed-point phase recurrence, float-float anchors, error control to 1e-3)",
            "data": "synthetic (seeded noise from the bundled aLIGO O4 / AdV PSDs, one injection per analysis)",
            "config": dict(mix_config(args.n_analyses), parallelism=f"replicas x{world}",
                           l2="inputs larger than L2 and flushed before every timed step (256 MiB write)"),
            "fp64": ue["fp64"],
            "mixed_over_fp64": ue["mixed_over_fp64"],
            "served_over_fp64": (e2e_v / ue["fp64"]["value"]) if e2e_v else None,
            "max_abs_dlnl_mixed_vs_fp64": ue["max_abs_dlnl_mixed_vs_fp64"],
            "fraction_of_points_with_abs_dlnl_le_1e-3": ue["fraction_of_points_with_abs_dlnl_le_1e-3"],
            "gpu_launches": ue["launches_per_step"] * args.steps * world,
            "p50_ms": ipc["at_80pct"]["p50_ms"] if ipc else None,
            "p99_ms": ipc["at_80pct"]["p99_ms"] if ipc else None,
            "clocks": clk,
            "uneven": uneven,
        }
        if ipc:
            srv_stats = ipc["saturated"]["server"]
            pts_step = srv_stats.get("mean_points_per_step") or 0.0
            line["e2e"] = {"value": e2e_v, "unit": "evals/s",
                           "h2d_bytes_per_step": int(8 * _capi.NPARAM * pts_step), "d2h_bytes_per_step": int(8 * pts_step),
                           "path": "sampler dicts from 200 clients in 8 processes -> ServedLikelihood (IPC) -> "
                                   "server conversion -> pinned staging -> H2D -> batched step -> D2H -> client"}
        if roofline:
            line["roofline"] = roofline
            line["roofline_hbm"] = roofline_hbm
        if cpu:
            line["cpu_baseline"] = cpu["mix"]
            line["cpu_baselines"] = {"sg_4s": cpu["sg"], "tf2_128s": cpu["tf2"], "tf2_marg_8s_tpd": cpu["marg"],
                                     "tf2_128s_relative_binning": cpu["relbin"]}
            line["gpu_over_cpu"] = {
                "mixed_mix_value": value / cpu["mix"]["value"] if value else None,
                "fp64_mix_precision_matched": ue["fp64"]["value"] / cpu["mix"]["value"] if uneven else None,
                "served_e2e": (e2e_v / cpu["mix"]["value"]) if e2e_v else None}
        if served:
            line["served"] = {"in_process": served, "ipc": ipc}
        if single:
            line["single_analysis"] = single
            if cpu:
                single["fp64_over_cpu"] = single["fp64"]["value"] / cpu["tf2"]["value"]
                single["mixed_over_cpu"] = single["value"] / cpu["tf2"]["value"]
        if drop_in:
            line["drop_in_call"] = drop_in
        if sg:
            line["sine_gaussian"] = sg
            if cpu:
                sg["fp64_over_cpu"] = sg["fp64"]["value"] / cpu["sg"]["value"]
                sg["mixed_over_cpu"] = sg["mixed"]["value"] / cpu["sg"]["value"]
        if marg:
            line["marginalized"] = marg
            if cpu:
                marg["fp64_over_cpu"] = marg["fp64"]["value"] / cpu["marg"]["value"]
                marg["mixed_over_cpu"] = marg["mixed"]["value"] / cpu["marg"]["value"]
        if relbin:
            line["relative_binning"] = relbin
            if cpu:
                relbin["fp64_over_cpu"] = relbin["value"] / cpu["relbin"]["value"]
        if multiband:
            line["multiband"] = multiband
        if roq:
            line["roq"] = roq
        print(json.dumps(line))
    dist.close()


def main():
    from bilby_gb300.replicas import dist_info
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()

"""The multi-GPU replica path's host logic with two gloo ranks on the CPU:
each rank evaluates its share of a batch (here with the oracle, standing in
for its GPU), the max-over-ranks timing reduction and the gather give the
single-process answer."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from bilby_gb300.replicas import shard


def test_shard_covers_everything():
    for n in (0, 1, 7, 4096, 4097):
        for world in (1, 2, 3, 8):
            parts = [shard(n, r, world) for r in range(world)]
            assert sum(p.stop - p.start for p in parts) == n
            assert all(parts[r].stop == parts[r + 1].start for r in range(world - 1))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    from bilby_gb300.replicas import ReplicaGroup, shard
    from bilby_gb300.workloads import WORKLOADS, draw_points, point
    from oracle import data as OD
    from oracle import restate as R
    grp = ReplicaGroup(world, backend="gloo")
    w = WORKLOADS["sg_4s"]
    dets = OD.build_workload(w)
    src = OD.source_for(w.model)
    params = draw_points(w, 11, np.random.default_rng(3))
    sl = shard(11, rank, world)
    local = np.array([R.log_likelihood_ratio(dets, src, point(params, i)) for i in range(sl.start, sl.stop)])
    grp.barrier()
    full = grp.gather(local, 11)
    tmax = grp.max(float(rank + 1))
    grp.close()
    q.put((rank, full, tmax))


@pytest.mark.timeout(300)
def test_two_gloo_ranks_gather_the_full_batch():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    from bilby_gb300.workloads import WORKLOADS, draw_points, point
    from oracle import data as OD
    from oracle import restate as R
    w = WORKLOADS["sg_4s"]
    dets = OD.build_workload(w)
    params = draw_points(w, 11, np.random.default_rng(3))
    ref = np.array([R.log_likelihood_ratio(dets, OD.source_for(w.model), point(params, i)) for i in range(11)])
    for rank, full, tmax in res:
        assert np.array_equal(full, ref)
        assert tmax == 2.0

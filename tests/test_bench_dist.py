"""Multi-rank host logic of bench.py on CPU (gloo, world_size 2).

Ranks are replicas: each maps its own read shard against a full index copy,
so the only cross-rank traffic is the timing barrier and the max/sum of the
counters. These tests check that aggregation, that shards differ, and that
the sum of per-shard mapped counts equals mapping all shards at once (the
property that lets the path shard with no data exchange).
"""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(ws)
    d.barrier()
    # rank r: time r + 1 s, mapped 10 (r + 1), cells 7
    t, mapped, cells = bench.aggregate(d, rank + 1.0, [10 * (rank + 1), 7])
    d.barrier()
    d.close()
    q.put((rank, t, mapped, cells, bench.shard_seed(rank)))


def test_two_rank_aggregate_max_time_sum_counts():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    for rank, t, mapped, cells, _ in out:
        assert t == 2.0            # slowest rank's time
        assert mapped == 30.0      # 10 + 20
        assert cells == 14.0
    assert out[0][4] != out[1][4]  # each rank its own read shard


def test_shards_map_independently():
    """Mapped reads summed over two shards == mapping both shards together."""
    sys.path.insert(0, ROOT)
    import bench
    from oracle import pyoracle as po
    from swmapper_gb300 import synth
    from tests.helpers import oracle_index
    g = synth.reference(300_000, seed=11, kind="repeats100m")
    _, mix = oracle_index(g)
    shards = [synth.reads(g, 300, 150, 150, 0.03, seed=bench.shard_seed(r))[:2] for r in range(2)]
    assert not np.array_equal(shards[0][0], shards[1][0])
    per = [po.map_reads(mix, rd, ln, 7, nthreads=2).stats["mapped_reads"] for rd, ln in shards]
    allr = np.concatenate([s[0] for s in shards])
    alll = np.concatenate([s[1] for s in shards])
    whole = po.map_reads(mix, allr, alll, 7, nthreads=2).stats["mapped_reads"]
    assert sum(per) == whole


def test_reference_arm_nonzero_rank_exits_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""

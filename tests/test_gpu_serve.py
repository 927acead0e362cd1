"""The request loop (swm_serve_*) through the C ABI (gpu).

Requests that arrive while other blocks are on the GPU are coalesced into the
next free block slot; every request's records and unmapped ids must be the
same as mapping that request alone (integer results: exactly equal), with
several blocks in flight at once. Admission refusals are forced on the host
(a device-memory limit below one slot; a queue limit), with no device fault.
"""
import math

import numpy as np
import pytest

from swmapper_gb300 import synth
from tests.helpers import genome

pytestmark = pytest.mark.gpu

SWM_ERR_ARG, SWM_ERR_OOM, SWM_ERR_STATE = -1, -3, -7


def _requests(g, nreq, seed, max_size=300):
    rng = np.random.default_rng(seed)
    sizes = np.maximum(1, np.minimum(max_size, np.exp(rng.uniform(0, math.log(max_size), nreq)).astype(int)))
    reads, lens, _, _ = synth.reads(g, int(sizes.sum()), 50, 250, 0.03, seed=seed + 1, stride=250)
    eper = np.minimum(np.ceil(0.05 * lens), 15).astype(np.uint8)
    out, off = [], 0
    for sz in sizes:
        sl = slice(off, off + int(sz))
        out.append((reads[sl], lens[sl], eper[sl]))
        off += int(sz)
    return out


def _alone(m, req):
    reads, lens, eper = req
    res = m.map(reads, lens, int(eper.max()), errors_per_read=eper)
    return res.records(), [int(u) for u in res.unmapped]


def _serve_all(srv, reqs):
    ids = [srv.submit(r, ln, int(e.max()), errors_per_read=e) for r, ln, e in reqs]
    got = {}
    while len(got) < len(ids):
        res = srv.poll(timeout_ms=60_000)
        assert res is not None, "a request did not finish within a minute"
        rid, recs, info = res
        got[rid] = (recs, [int(u) for u in srv._buf.unmapped[:srv._buf.c.n_unmapped]], info)
    return [got[i] for i in ids]


def test_serve_same_alone_and_in_the_mix(cuda_lib):
    g = genome(2_000_000, 81, "repeats100m")
    reqs = _requests(g, 80, 82)
    ix = cuda_lib.Index.build(g)
    m = cuda_lib.Mapper(ix, max_reads=300)
    want = [_alone(m, r) for r in reqs]
    srv = cuda_lib.Server(ix, block_reads=512, max_slots=4, stride=256)
    try:
        _serve_all(srv, reqs)            # first pass makes the slots
        got = _serve_all(srv, reqs)      # second pass: every slot exists, blocks go out back to back
        for i, ((recs, unm, info), (wrecs, wunm)) in enumerate(zip(got, want)):
            assert recs == wrecs, i
            assert unm == wunm, i
            assert info["reads"] == reqs[i][0].shape[0] and info["block_reads"] >= info["reads"]
        st = srv.stats()
        assert st["slots"] >= 3 and st["max_blocks_in_flight"] >= 3, st
        assert st["requests_done"] == 2 * len(reqs) and st["refused_memory"] == 0
        # requests were coalesced: fewer blocks than requests
        assert st["blocks"] < 2 * len(reqs)
    finally:
        srv.close()


def test_serve_refuses_when_no_slot_fits_the_memory_limit(cuda_lib):
    g = genome(500_000, 83)
    ix = cuda_lib.Index.build(g)
    srv = cuda_lib.Server(ix, block_reads=1024, max_slots=2, stride=256, device_mem_limit=1 << 20)
    try:
        reads, lens, _, _ = synth.reads(g, 10, 100, 100, 0.02, seed=84)
        with pytest.raises(cuda_lib.SwmError) as ei:
            srv.submit(reads, lens, 5)
        assert ei.value.rc == SWM_ERR_OOM
        st = srv.stats()
        assert st["refused_memory"] == 1 and st["slots"] == 0 and st["slot_bytes"] > 1 << 20
    finally:
        srv.close()


def test_serve_refuses_when_the_queue_is_full(cuda_lib):
    """One slot, a queue of one block: requests submitted while it is busy
    beyond that are refused with SWM_ERR_STATE; the admitted ones finish with
    the same records as alone."""
    g = genome(3_000_000, 85, "human", nrun_min=2000, nrun_max=20000, copies_per_family=300)
    reads, lens, _, _ = synth.reads(g, 4096 * 12, 150, 150, 0.03, seed=86)
    ix = cuda_lib.Index.build(g)
    srv = cuda_lib.Server(ix, block_reads=4096, max_slots=1, stride=256, max_queued_reads=4096)
    admitted, refused = [], 0
    try:
        for i in range(12):
            sl = slice(4096 * i, 4096 * (i + 1))
            try:
                admitted.append((srv.submit(reads[sl], lens[sl], 7), sl))
            except cuda_lib.SwmError as e:
                assert e.rc == SWM_ERR_STATE
                refused += 1
        assert refused >= 1 and srv.stats()["refused_queue"] == refused
        got = {}
        while len(got) < len(admitted):
            rid, recs, _ = srv.poll(timeout_ms=60_000)
            got[rid] = recs
        m = cuda_lib.Mapper(ix, max_reads=4096)
        for rid, sl in admitted:
            assert got[rid] == m.map(reads[sl], lens[sl], 7).records()
    finally:
        srv.close()


def test_serve_rejects_bad_requests(cuda_lib):
    g = genome(300_000, 87)
    ix = cuda_lib.Index.build(g)
    srv = cuda_lib.Server(ix, block_reads=64, max_slots=1, stride=256)
    try:
        with pytest.raises(cuda_lib.SwmError) as ei:   # more reads than a block
            srv.submit(np.zeros((65, 100), np.uint8), np.full(65, 100, np.uint32), 5)
        assert ei.value.rc == SWM_ERR_ARG
        with pytest.raises(cuda_lib.SwmError) as ei:   # read longer than the envelope
            srv.submit(np.zeros((1, 300), np.uint8), np.array([255], np.uint32), 5)
        assert ei.value.rc == SWM_ERR_ARG
        assert srv.poll(timeout_ms=0) is None
    finally:
        srv.close()

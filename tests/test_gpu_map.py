"""GPU mapping against the oracle and the reference's recorded outputs (gpu)."""
import json
import math
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from swmapper_gb300 import synth
from tests.helpers import first_diff, genome, oracle_index, records_by_e

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_outputs.json")))


def _gpu(swm, g, reads, lens, e, eper=None, max_reads=None, table=True):
    """Map on the GPU; table=True builds the index's candidate table (the
    library builds it on its own only for large genomes), table=False drops
    it, so the candidate stage filters every fetched entry (the path for
    k != 12 and for genomes of small buckets)."""
    ix = swm.Index.build(g)
    if table:
        assert ix.candidate_table(True) > 0
    else:
        assert ix.candidate_table(False) == 0
    m = swm.Mapper(ix, max_reads=max_reads or max(1, reads.shape[0]))
    out = m.map(reads, lens, e, errors_per_read=eper)
    return out, m, ix


def _check(out, ref_records, ref_unmapped):
    got = out.records()
    d = first_diff(got, ref_records)
    assert d is None, d
    assert [int(x) for x in out.unmapped] == [int(x) for x in ref_unmapped]


@pytest.mark.parametrize("key", sorted(GOLD["map"]))
def test_gpu_equals_reference_outputs(cuda_lib, key):
    cases = {c[0]: c for c in GOLD["cases"]["map"]}
    name, e = key.rsplit("_e", 1)
    _, n, gseed, kind, over, nreads, lmin, lmax, err, es, rseed = cases[name]
    g = synth.reference(n, seed=gseed, kind=kind, **over)
    reads, lens, _, _ = synth.reads(g, nreads, lmin, lmax, err, seed=rseed)
    out, _, _ = _gpu(cuda_lib, g, reads, lens, int(e))
    want = [(r[0], r[1], tuple(r[2]), bytes.fromhex(r[3])) for r in GOLD["map"][key]["records"]]
    _check(out, want, GOLD["map"][key]["unmapped"])


def test_gpu_plain_1mbp(cuda_lib):
    """Plain workload shape: 1 Mbp uniform, 100 bp reads, 2% error, e=5."""
    g = genome(1_000_000, 1)
    reads, lens, _, _ = synth.reads(g, 4096, 100, 100, 0.02, seed=2)
    _, mix = oracle_index(g)
    ref = po.map_reads(mix, reads, lens, 5, nthreads=8)
    out, m, _ = _gpu(cuda_lib, g, reads, lens, 5)
    _check(out, ref.records(), ref.unmapped)
    st = m.stats()
    assert st["candidates"] == ref.stats["candidates"]
    assert st["mapped_reads"] == ref.stats["mapped_reads"]
    # every passing candidate runs all 100 read bases through the recurrence;
    # a candidate runs at most all of them, and (streaming form, the default)
    # all of them once more when its traceback needs checkpoints
    assert m.verify() == "stream16"
    assert 100 * st["passed"] <= st["myers_steps"] <= 100 * (st["candidates"] + st["passed"])
    assert st["myers_steps"] >= 16 * st["candidates"] // 2
    # the two-pass form runs no candidate past its last base
    m.set_verify("head64")
    out2 = m.map(reads, lens, 5)
    _check(out2, ref.records(), ref.unmapped)
    st2 = m.stats()
    assert 100 * st2["passed"] <= st2["myers_steps"] <= 100 * st2["candidates"]
    assert st2["myers_steps"] >= 64 * st2["candidates"] // 2


@pytest.mark.parametrize("table", [True, False])
def test_gpu_repeats_multibatch(cuda_lib, table):
    """Heavy repeats: refills, several batches per strand, buffer growth; with
    the candidate table and with entry-by-entry filtering."""
    g = genome(3_000_000, 7, "human", nrun_min=2000, nrun_max=20000, copies_per_family=300)
    reads, lens, _, _ = synth.reads(g, 3000, 150, 150, 0.03, seed=8)
    _, mix = oracle_index(g)
    for e in (7, 12):
        ref = po.map_reads(mix, reads, lens, e, nthreads=8)
        out, m, _ = _gpu(cuda_lib, g, reads, lens, e, table=table)
        _check(out, ref.records(), ref.unmapped)
        assert m.stats()["batches"] == ref.stats["batches"]


@pytest.mark.parametrize("table", [True, False])
def test_gpu_single_batch_items_near_the_limit(cuda_lib, table):
    """Close repeat copies: many items with refills on both sides of the
    single-batch limit (2017 selected positions), which the planner handles
    without the seed heap below it and with the heap above it."""
    g = genome(3_000_000, 7, "human", copies_per_family=1000, div_min=0.005, div_max=0.03, repeat_frac=0.6,
               rep_len_max=3000)
    reads, lens, _, _ = synth.reads(g, 600, 150, 150, 0.03, seed=21)
    _, mix = oracle_index(g)
    for e in (7, 12):
        ref = po.map_reads(mix, reads, lens, e, nthreads=8)
        out, m, _ = _gpu(cuda_lib, g, reads, lens, e, table=table)
        _check(out, ref.records(), ref.unmapped)
        assert m.stats()["batches"] == ref.stats["batches"]
        assert m.stats()["candidates"] == ref.stats["candidates"]


def test_gpu_uneven_per_read_e(cuda_lib):
    """Read lengths U[50, 250] with e = ceil(0.05 L) per read."""
    g = genome(2_000_000, 9, "repeats100m")
    reads, lens, _, _ = synth.reads(g, 3000, 50, 250, 0.04, seed=10, stride=250)
    eper = np.array([math.ceil(0.05 * int(L)) for L in lens], np.uint8)
    _, mix = oracle_index(g)
    ref_recs, ref_unm = records_by_e(mix, reads, lens, eper)
    out, _, _ = _gpu(cuda_lib, g, reads, lens, 0, eper=eper)
    _check(out, ref_recs, ref_unm)


@pytest.mark.parametrize("e", [0, 1, 3, 15])
def test_gpu_error_thresholds_and_odd_reads(cuda_lib, e):
    g = genome(500_000, 11, "repeats100m", copies_per_family=30, rep_len_max=3000)
    reads, lens, _, _ = synth.reads(g, 1500, 15, 254, 0.05, seed=12, stride=254)
    reads[::5, 7] = ord("N")
    reads[1::7, 20] = ord("a")
    lens[::50] = 14       # shorter than one long seed: no seeds, unmapped
    _, mix = oracle_index(g)
    ref = po.map_reads(mix, reads, lens, e, nthreads=8)
    out, _, _ = _gpu(cuda_lib, g, reads, lens, e)
    _check(out, ref.records(), ref.unmapped)


def test_gpu_reads_at_genome_ends(cuda_lib):
    g = genome(200_000, 13)
    reads = np.zeros((6, 120), np.uint8)
    lens = np.full(6, 120, np.uint32)
    reads[0] = g[:120]
    reads[1] = g[3:123]
    reads[2] = g[-120:]
    reads[3, :100] = g[-100:]
    lens[3] = 100
    reads[4] = g[50_000:50_120]
    reads[5] = g[1:121]
    _, mix = oracle_index(g)
    ref = po.map_reads(mix, reads, lens, 6)
    out, _, _ = _gpu(cuda_lib, g, reads, lens, 6)
    _check(out, ref.records(), ref.unmapped)


@pytest.mark.parametrize("table", [True, False])
def test_gpu_candidates_equal_oracle_trace(cuda_lib, table):
    g = genome(1_000_000, 14, "repeats100m", copies_per_family=20)
    reads, lens, _, _ = synth.reads(g, 64, 150, 150, 0.03, seed=15)
    _, mix = oracle_index(g)
    out, m, _ = _gpu(cuda_lib, g, reads, lens, 7, table=table)
    item, pos, err, loc = m.debug_candidates()
    for it in range(128):
        r, strand = it >> 1, it & 1
        s = bytes(reads[r, :lens[r]])
        if strand:
            s = s[::-1].translate(bytes.maketrans(b"ACGT", b"TGCA"))
        tr = po.trace_item(mix, s, 7)
        sel = item == it
        assert np.array_equal(pos[sel], tr["pos"]), it
        assert np.array_equal(err[sel], tr["err"]), it
        assert np.array_equal(loc[sel], tr["loc"]), it


def test_gpu_empty_and_async(cuda_lib):
    g = genome(300_000, 16)
    ix = cuda_lib.Index.build(g)
    m = cuda_lib.Mapper(ix, max_reads=512)
    empty = m.map(np.zeros((0, 100), np.uint8), np.zeros(0, np.uint32), 5)
    assert empty.ref_pos.shape[0] == 0 and empty.unmapped.size == 0
    reads, lens, _, _ = synth.reads(g, 500, 100, 100, 0.02, seed=17)
    a = m.map(reads, lens, 5).records()
    b = m.map(reads, lens, 5).records()
    assert a == b


def test_gpu_rejects_out_of_envelope(cuda_lib):
    g = genome(100_000, 18)
    ix = cuda_lib.Index.build(g)
    m = cuda_lib.Mapper(ix, max_reads=4)
    with pytest.raises(cuda_lib.SwmError):
        m.map(np.zeros((1, 300), np.uint8), np.array([255], np.uint32), 5)
    with pytest.raises(cuda_lib.SwmError):
        m.map(np.zeros((1, 100), np.uint8), np.array([100], np.uint32), 16)
    with pytest.raises(cuda_lib.SwmError):
        m.map(np.zeros((5, 100), np.uint8), np.full(5, 100, np.uint32), 5)


@pytest.mark.parametrize("serial", [False, True])
def test_gpu_packed_pingpong_equals_strided(cuda_lib, serial):
    """submit / wait_packed on two mappers (the host double-buffering of
    mapper_mpe.c:972-1106; with serial the two mappers' kernels run one block
    at a time) gives the same records as swm_map_batch."""
    g = genome(2_000_000, 19, "repeats100m")
    reads, lens, _, _ = synth.reads(g, 6000, 150, 150, 0.03, seed=20)
    ix = cuda_lib.Index.build(g)
    ix.serialize_mappers(serial)
    ma, mb = cuda_lib.Mapper(ix, max_reads=2000), cuda_lib.Mapper(ix, max_reads=2000)
    want = []
    for b0 in range(0, 6000, 2000):
        recs = ma.map(reads[b0:b0 + 2000], lens[b0:b0 + 2000], 7).records()
        want.extend((r[0] + 2 * b0,) + r[1:] for r in recs)
    got = []
    bufs = [cuda_lib.PackedBuffers(2000), cuda_lib.PackedBuffers(2000)]
    ms = [ma, mb]
    ms[0].submit(reads[0:2000], lens[0:2000], 7)
    ms[1].submit(reads[2000:4000], lens[2000:4000], 7)
    ms[0].wait_packed(bufs[0])
    got.extend((r[0],) + r[1:] for r in bufs[0].records())
    ms[0].submit(reads[4000:6000], lens[4000:6000], 7)
    ms[1].wait_packed(bufs[1])
    got.extend((r[0] + 4000,) + r[1:] for r in bufs[1].records())
    ms[0].wait_packed(bufs[0])
    got.extend((r[0] + 8000,) + r[1:] for r in bufs[0].records())
    assert got == want


def _even(x):
    x = np.uint64(x) & np.uint64(0x55555555)
    x = (x | (x >> np.uint64(1))) & np.uint64(0x33333333)
    x = (x | (x >> np.uint64(2))) & np.uint64(0x0F0F0F0F)
    x = (x | (x >> np.uint64(4))) & np.uint64(0x00FF00FF)
    x = (x | (x >> np.uint64(8))) & np.uint64(0x0000FFFF)
    return int(x)


def test_gpu_read_encoding_every_length(cuda_lib):
    """Per-item read words against the oracle's literal get_seed_from_reads
    state machine, for every read length 15..254 on both strands, with N and
    lowercase bases mixed in (covers every tail-encoder case)."""
    g = genome(300_000, 21)
    rng = np.random.default_rng(22)
    lens = np.arange(15, 255, dtype=np.uint32)
    n = lens.size * 2
    lens = np.concatenate([lens, lens])
    reads = np.zeros((n, 254), np.uint8)
    for i in range(n):
        L = int(lens[i])
        st = int(rng.integers(0, g.size - 300))
        reads[i, :L] = g[st:st + L]
        if i >= n // 2:
            for _ in range(int(rng.integers(1, 4))):
                reads[i, int(rng.integers(0, L))] = ord("N")
            reads[i, int(rng.integers(0, L))] = ord("c")
    ix = cuda_lib.Index.build(g)
    m = cuda_lib.Mapper(ix, max_reads=n)
    m.map(reads, lens, 4)
    words = m.debug_read_words(n)
    comp = bytes.maketrans(b"ACGT", b"TGCA")
    for it in range(2 * n):
        r, strand = it >> 1, it & 1
        s = bytes(reads[r, :lens[r]])
        if strand:
            s = s[::-1].translate(comp)
        w = po.encode_read(s)
        want = np.zeros(32, np.uint64)
        for b in range(8):
            a0, a1 = int(w[2 * b]), int(w[2 * b + 1])
            want[2 * b] = _even(a0) | (_even(a1) << 16)
            want[2 * b + 1] = _even(a0 >> 1) | (_even(a1 >> 1) << 16)
        want[16:] = w[16:]
        assert np.array_equal(words[it].astype(np.uint64), want), (it, int(lens[r]))


def test_gpu_pinned_buffers_direct_copy(cuda_lib):
    """Page-locked caller buffers take the direct-copy path; same records."""
    import ctypes
    rt = None
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            pass
    assert rt is not None
    rt.cudaHostRegister.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint]
    rt.cudaHostUnregister.argtypes = [ctypes.c_void_p]
    g = genome(1_000_000, 23, "repeats100m")
    reads, lens, _, _ = synth.reads(g, 3000, 150, 150, 0.03, seed=24)
    ix = cuda_lib.Index.build(g)
    m = cuda_lib.Mapper(ix, max_reads=3000)
    want = m.map(reads, lens, 7).records()
    buf = cuda_lib.PackedBuffers(3000)
    arrs = [reads, lens, buf.words, buf.cigar, buf.rlen]
    for a in arrs:
        assert rt.cudaHostRegister(a.ctypes.data, a.nbytes, 0) == 0
    try:
        m.submit(reads, lens, 7)
        m.wait_packed(buf)
        got = buf.records()
    finally:
        for a in arrs:
            rt.cudaHostUnregister(a.ctypes.data)
    assert got == want


@pytest.mark.parametrize("serial", [False, True])
def test_gpu_device_submit_two_mappers(cuda_lib, serial):
    """swm_map_device_submit / swm_map_device_wait on two mappers in turn
    (blocks overlapping on the GPU, or with serial their kernels one block at
    a time: swm_index_serialize_mappers) give the same records and unmapped
    ids as swm_map_device one block at a time."""
    import ctypes
    rt = None
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            pass
    assert rt is not None
    rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    rt.cudaFree.argtypes = [ctypes.c_void_p]
    g = genome(3_000_000, 31, "human", nrun_min=2000, nrun_max=20000, copies_per_family=300)
    reads, lens, _, _ = synth.reads(g, 6000, 150, 150, 0.03, seed=32)
    ix = cuda_lib.Index.build(g)
    ix.serialize_mappers(serial)
    d_reads, d_lens = ctypes.c_void_p(), ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(d_reads), reads.nbytes) == 0
    assert rt.cudaMalloc(ctypes.byref(d_lens), lens.nbytes) == 0
    try:
        assert rt.cudaMemcpy(d_reads, reads.ctypes.data, reads.nbytes, 1) == 0
        assert rt.cudaMemcpy(d_lens, lens.ctypes.data, lens.nbytes, 1) == 0
        stride = reads.shape[1]
        blk = [(b0, d_reads.value + b0 * stride, d_lens.value + b0 * 4) for b0 in (0, 2000, 4000)]

        def out_of(m):
            o = m.fetch(2000)
            return o.records(), [int(x) for x in o.unmapped]

        ref = cuda_lib.Mapper(ix, max_reads=2000)
        want = []
        for _, dr, dl in blk:
            ref.map_device(dr, dl, stride, 2000, 7)
            want.append(out_of(ref))
        ma, mb = cuda_lib.Mapper(ix, max_reads=2000), cuda_lib.Mapper(ix, max_reads=2000)
        got = [None] * 3
        ma.submit_device(blk[0][1], blk[0][2], stride, 2000, 7)
        mb.submit_device(blk[1][1], blk[1][2], stride, 2000, 7)
        ma.wait_device()
        got[0] = out_of(ma)
        ma.submit_device(blk[2][1], blk[2][2], stride, 2000, 7)
        mb.wait_device()
        got[1] = out_of(mb)
        ma.wait_device()
        got[2] = out_of(ma)
        assert got == want
        assert any(u for _, u in want) and all(r for r, _ in want)
    finally:
        rt.cudaFree(d_reads)
        rt.cudaFree(d_lens)


def test_gpu_requests_same_alone_and_in_the_mix(cuda_lib):
    """Serving coalesces requests that arrive together into one block: every
    request's records and unmapped ids are the same mapped alone and in the
    mix (read ids shifted by the request's offset in the block)."""
    g = genome(2_000_000, 61, "repeats100m")
    sizes = [1, 7, 300, 64, 1000, 5, 2]
    reads, lens, _, _ = synth.reads(g, sum(sizes), 50, 250, 0.03, seed=63)
    eper = np.minimum(np.ceil(0.05 * lens), 15).astype(np.uint8)
    ix = cuda_lib.Index.build(g)
    m = cuda_lib.Mapper(ix, max_reads=sum(sizes))
    mixed = m.map(reads, lens, int(eper.max()), errors_per_read=eper)
    got_mix = {}
    for rec in mixed.records():
        got_mix.setdefault(rec[0] >> 1, []).append(rec)
    unm_mix = set(int(u) >> 1 for u in mixed.unmapped)
    off = 0
    for sz in sizes:
        sl = slice(off, off + int(sz))
        alone = m.map(reads[sl], lens[sl], int(eper[sl].max()), errors_per_read=eper[sl])
        for rec in alone.records():
            r = (rec[0] >> 1) + off
            want = ((2 * r + (rec[0] & 1)),) + tuple(rec[1:])
            assert want in got_mix.get(r, []), (sz, r)
        for u in alone.unmapped:
            assert (int(u) >> 1) + off in unm_mix
        n_alone = sum(1 for _ in alone.records())
        n_mix = sum(len(got_mix.get(r, [])) for r in range(off, off + int(sz)))
        assert n_alone == n_mix
        off += int(sz)


@pytest.mark.parametrize("k,e", [(10, 7), (11, 5), (13, 7), (14, 3)])
def test_gpu_mapping_other_seed_lengths(cuda_lib, k, e):
    """-s other than 12: the generic seed kernel (long seeds of k + 3 bases,
    one warp per 32 items) and the rest of the pipeline, against the oracle."""
    g = genome(2_000_000, 70 + k, "repeats100m", copies_per_family=40)
    lmax = min(250, 17 * (k + 3) - 1)  # at most 16 long seeds of k + 3 bases (mapper_cpe.c:2515)
    reads, lens, _, _ = synth.reads(g, 2000, 50, lmax, 0.03, seed=80 + k, stride=250)
    reads[::9, 33] = ord("N")
    hix, mix = oracle_index(g, k)
    ref = po.map_reads(mix, reads, lens, e, nthreads=8)
    ix = cuda_lib.Index.build(g, k=k)
    m = cuda_lib.Mapper(ix, max_reads=reads.shape[0])
    out = m.map(reads, lens, e)
    _check(out, ref.records(), ref.unmapped)
    assert m.stats()["candidates"] == ref.stats["candidates"]


@pytest.mark.parametrize("mode", ["head32", "head64", "stream8", "stream16", "pair16"])
def test_gpu_verify_forms(cuda_lib, mode):
    """The form of the verification stage (an autotuner knob) changes no
    result: reads of 50-250 bp, per-read e up to 13 (the two-per-lane form
    runs these blocks one per lane), against the oracle."""
    g = genome(2_000_000, 90, "human", nrun_min=2000, nrun_max=20000, copies_per_family=200)
    reads, lens, _, _ = synth.reads(g, 3000, 50, 250, 0.04, seed=91, stride=250)
    eper = np.array([math.ceil(0.05 * int(L)) for L in lens], np.uint8)
    _, mix = oracle_index(g)
    ref_recs, ref_unm = records_by_e(mix, reads, lens, eper)
    ix = cuda_lib.Index.build(g)
    m = cuda_lib.Mapper(ix, max_reads=reads.shape[0])
    m.set_verify(mode)
    assert m.verify() == mode
    out = m.map(reads, lens, 0, errors_per_read=eper)
    _check(out, ref_recs, ref_unm)
    with pytest.raises(cuda_lib.SwmError):
        m.set_verify("head48")
    assert m.verify() == mode


@pytest.mark.parametrize("mode", ["stream8", "stream16", "pair16"])
def test_gpu_streaming_verify_uniform_e(cuda_lib, mode):
    """Streaming verification at one e for every read (150 bp, e = 7) on a
    repeat-rich genome: records, candidate counts and passing counts equal the
    oracle's and the two-pass form's."""
    g = genome(3_000_000, 93, "human", nrun_min=2000, nrun_max=20000, copies_per_family=300)
    reads, lens, _, _ = synth.reads(g, 4000, 150, 150, 0.03, seed=94, stride=160)
    ref, mix = oracle_index(g)
    want = po.map_reads(mix, reads, lens, 7)
    ix = cuda_lib.Index.build(g)
    m = cuda_lib.Mapper(ix, max_reads=reads.shape[0])
    m.set_verify("head64")
    base = m.map(reads, lens, 7)
    st64 = m.stats()
    m.set_verify(mode)
    out = m.map(reads, lens, 7)
    st = m.stats()
    _check(out, want.records(), want.unmapped)
    _check(out, base.records(), base.unmapped)
    assert st["candidates"] == st64["candidates"] == want.stats["candidates"]
    assert st["passed"] == st64["passed"]
    assert st["cells"] == st64["cells"]
    assert st["myers_steps"] < st64["myers_steps"]


@pytest.mark.parametrize("e", [0, 2, 5, 7])
def test_gpu_pair_verify_every_length(cuda_lib, e):
    """Two candidates per lane (15-bit halves of one word) at every e the form
    takes, reads of 15-254 bp (shorter than one 16-base chunk too) on a
    repeat-rich genome, and reads placed at both genome ends: records equal
    the oracle's and the one-per-lane streaming form's, step for step."""
    g = genome(1_500_000, 95 + e, "human", nrun_min=2000, nrun_max=20000, copies_per_family=200)
    reads, lens, _, _ = synth.reads(g, 3000, 15, 254, 0.03, seed=96 + e, stride=256)
    ends = np.zeros((4, 256), np.uint8)
    for r, (st, L) in enumerate([(0, 150), (3, 100), (g.size - 150, 150), (g.size - 40, 40)]):
        ends[r, :L] = g[st:st + L]
    reads = np.concatenate([reads, ends])
    lens = np.concatenate([lens, np.array([150, 100, 150, 40], np.uint32)])
    _, mix = oracle_index(g)
    want = po.map_reads(mix, reads, lens, e, nthreads=8)
    ix = cuda_lib.Index.build(g)
    m = cuda_lib.Mapper(ix, max_reads=reads.shape[0])
    m.set_verify("stream16")
    one = m.map(reads, lens, e)
    st1 = m.stats()
    m.set_verify("pair16")
    assert m.verify() == "pair16"
    two = m.map(reads, lens, e)
    st2 = m.stats()
    _check(two, want.records(), want.unmapped)
    _check(two, one.records(), one.unmapped)
    for k in ("candidates", "passed", "cells", "myers_steps"):
        assert st2[k] == st1[k], k


def test_gpu_records_split_past_the_record_limit(cuda_lib):
    """Reads from a unit copied 320 times (some copies with a substitution or
    an indel) have more locations than one record holds (SWM_MAX_CIGAR), so
    the records kernel's sequential path (flushes after groups of 8, dedup
    reset after a flush, primary flag on the first record only) runs beside
    its one-record fast path."""
    rng = np.random.default_rng(61)
    g = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 600_000)]
    unit = g[1000:1400].copy()
    starts = np.sort(rng.choice(np.arange(5_000, 590_000, 1_700), 320, replace=False))
    for i, s in enumerate(starts):
        cp = unit.copy()
        if i % 5 == 1:    # one substitution
            cp[200] = ord("A") if cp[200] != ord("A") else ord("C")
        elif i % 5 == 2:  # one deletion: the copy shifts by a base
            cp = np.concatenate([cp[:180], cp[181:], unit[-1:]])
        g[s:s + cp.size] = cp
    reads = np.zeros((40, 150), np.uint8)
    lens = np.full(40, 150, np.uint32)
    for r in range(40):
        o = 20 + 5 * r
        s = unit[o:o + 150].copy()
        if r % 3 == 1:
            s[70] = ord("G") if s[70] != ord("G") else ord("T")
        if r % 2:
            s = s[::-1].copy()
            s = np.frombuffer(bytes(s).translate(bytes.maketrans(b"ACGT", b"TGCA")), np.uint8)
        reads[r] = s
    _, mix = oracle_index(g)
    ref = po.map_reads(mix, reads, lens, 7)
    per_item = {}
    for rec in ref.records():
        per_item[rec[0]] = per_item.get(rec[0], 0) + 1
    assert max(per_item.values()) >= 2, "the workload should split some item's locations over records"
    out, _, _ = _gpu(cuda_lib, g, reads, lens, 7)
    _check(out, ref.records(), ref.unmapped)

"""Parity on the benchmarked genomes (gpu).

The benchmark's human-scale workload is a 3.1 Gbp genome: positions run
past 2^31 and ref_length (= 4 x the bytes of .base_2bits, mapper_mpe.c:288)
past 2^32, buckets hold hundreds of positions and a read fetches thousands of
index entries in several batches. These tests build the benchmark's own
genomes (same generator, same seeds) and compare the GPU index and mapping
with the oracle there: the index arrays in full, and the records of tens of
thousands of reads, including reads placed past 2^31, across N-run edges and
at the genome's end. The oracle's index build runs on every host core (the
threaded build gives the serial restatement's arrays exactly).
"""
import math
import os
import shutil

import numpy as np
import pytest

from oracle import pyoracle as po
from swmapper_gb300 import synth
from tests.helpers import first_diff, records_by_e

pytestmark = pytest.mark.gpu

HUMAN = dict(n=3_100_000_000, seed=31, kind="human", read_seed=13)
BATCHED = dict(n=100_000_000, seed=20261203, kind="repeats100m", read_seed=7)


def _threads():
    return max(1, os.cpu_count() or 1)


def _n_run_edges(g, lo, hi, limit):
    """Starts and ends of N runs between lo and hi (at most limit of each)."""
    seg = g[lo:hi] == ord("N")
    d = np.flatnonzero(np.diff(seg.astype(np.int8)))
    return [lo + int(x) + 1 for x in d[:limit]]


def _edge_reads(g, L=150):
    """Reads that straddle N-run edges below and above 2^31, sit in the last
    bases of the genome, and start exactly at 2^31 and 2^32 / 2."""
    starts = []
    for lo, hi in ((50_000_000, 1_000_000_000), (2**31, 2**31 + 1_000_000_000)):
        for e in _n_run_edges(g, lo, hi, 12):
            starts += [e - L // 2, e - L, e + 1]
    starts += [g.size - L, g.size - L - 7, 2**31, 2**31 - 75, 2**31 + 4]
    starts = [s for s in starts if 0 <= s <= g.size - L]
    reads = np.stack([g[s:s + L] for s in starts]).astype(np.uint8)
    return reads, np.full(len(starts), L, np.uint32)


@pytest.fixture(scope="module")
def human(cuda_lib):
    g = synth.reference(HUMAN["n"], seed=HUMAN["seed"], kind=HUMAN["kind"])
    ix = cuda_lib.Index.build(g, k=12)
    hix = po.build_index(g, 12, nthreads=_threads())
    yield g, ix, hix
    ix.close()


def test_human_index_equals_oracle(human):
    g, ix, hix = human
    got = ix.download()
    assert got["positions"].size > 700_000_000
    assert int(got["positions"].max()) > 2**31
    for key, want in (("hash_count", hix.hash_count), ("hash_offset", hix.hash_offset_end),
                      ("positions", hix.positions), ("pos_lseeds", hix.pos_lseeds),
                      ("base_2bits", hix.base_2bits), ("base_3bits", hix.base_3bits)):
        assert np.array_equal(got[key], want), key
    assert ix.info().ref_length > 2**32


@pytest.mark.parametrize("table", [True, False])
def test_human_mapping_equals_oracle(cuda_lib, human, table):
    """20,000 reads of the benchmark's read stream plus reads at N-run edges,
    past 2^31 and at the genome's end; e = 7 as in the benchmark; with the
    candidate table and with entry-by-entry filtering."""
    g, ix, hix = human
    ix.candidate_table(table)
    assert (ix.candidate_table(table) > 0) == table
    reads, lens, tpos, _ = synth.reads(g, 20_000, 150, 150, 0.03, seed=HUMAN["read_seed"])
    er, el = _edge_reads(g)
    reads = np.concatenate([reads, er])
    lens = np.concatenate([lens, el])
    assert (tpos >= 2**31).sum() > 4000
    mix = po.MapIndex(hix)
    ref = po.map_reads(mix, reads, lens, 7, nthreads=_threads())
    m = cuda_lib.Mapper(ix, max_reads=reads.shape[0])
    out = m.map(reads, lens, 7)
    got = out.records()
    d = first_diff(got, ref.records())
    assert d is None, d
    assert [int(x) for x in out.unmapped] == [int(x) for x in ref.unmapped]
    st = m.stats()
    assert st["candidates"] == ref.stats["candidates"] and st["batches"] == ref.stats["batches"]
    locs = [p for r in got for p in r[2]]
    assert sum(1 for p in locs if p > 2**31) > 0.2 * len(locs)
    # the reads above the edges include multi-batch items and N-run edges
    assert st["batches"] > st["items"]


def test_human_uneven_reads_equal_oracle(cuda_lib, human):
    """Reads of 50-250 bp with e = ceil(0.05 L) on the human-scale genome
    (the serving workload's shape)."""
    g, ix, hix = human
    ix.candidate_table(True)
    reads, lens, _, _ = synth.reads(g, 6000, 50, 250, 0.03, seed=17, stride=250)
    eper = np.array([min(15, math.ceil(0.05 * int(x))) for x in lens], np.uint8)
    recs, unm = records_by_e(po.MapIndex(hix), reads, lens, eper, nthreads=_threads())
    m = cuda_lib.Mapper(ix, max_reads=reads.shape[0])
    out = m.map(reads, lens, int(eper.max()), errors_per_read=eper)
    d = first_diff(out.records(), recs)
    assert d is None, d
    assert [int(x) for x in out.unmapped] == unm


def test_human_index_files_round_trip(cuda_lib, human, tmp_path):
    """The 5.7 GB index written by swm_index_save and loaded back by the
    chunked loader equals the built index."""
    _, ix, _ = human
    if shutil.disk_usage(str(tmp_path)).free < 12 * 2**30:
        pytest.skip("less than 12 GiB free for the index files")
    prefix = str(tmp_path / "human")
    ix.save(prefix, b"3100000000\n4\nchrS\n")
    back = cuda_lib.Index.open(prefix)
    try:
        a, b = ix.download(), back.download()
        for key in a:
            assert np.array_equal(a[key], b[key]), key
    finally:
        back.close()
        for f in os.listdir(str(tmp_path)):
            os.remove(os.path.join(str(tmp_path), f))


@pytest.fixture(scope="module")
def batched(cuda_lib):
    g = synth.reference(BATCHED["n"], seed=BATCHED["seed"], kind=BATCHED["kind"])
    ix = cuda_lib.Index.build(g, k=12)
    hix = po.build_index(g, 12, nthreads=_threads())
    yield g, ix, hix
    ix.close()


def test_batched_100m_index_and_mapping_equal_oracle(cuda_lib, batched):
    """The batched workload's 100 Mbp genome: index arrays and the records of
    20,000 reads of the benchmark's read stream (150 bp, 3% error, e = 7)."""
    g, ix, hix = batched
    got = ix.download()
    for key, want in (("positions", hix.positions), ("pos_lseeds", hix.pos_lseeds),
                      ("hash_count", hix.hash_count), ("base_2bits", hix.base_2bits)):
        assert np.array_equal(got[key], want), key
    reads, lens, _, _ = synth.reads(g, 20_000, 150, 150, 0.03, seed=BATCHED["read_seed"])
    ref = po.map_reads(po.MapIndex(hix), reads, lens, 7, nthreads=_threads())
    m = cuda_lib.Mapper(ix, max_reads=reads.shape[0])
    out = m.map(reads, lens, 7)
    d = first_diff(out.records(), ref.records())
    assert d is None, d
    assert [int(x) for x in out.unmapped] == [int(x) for x in ref.unmapped]


def test_batched_100m_uneven_equal_oracle(cuda_lib, batched):
    """The uneven workload's reads (50-250 bp, 4% error, e = ceil(0.05 L))."""
    g, ix, hix = batched
    reads, lens, _, _ = synth.reads(g, 8000, 50, 250, 0.04, seed=11, stride=250)
    eper = np.array([min(15, math.ceil(0.05 * int(x))) for x in lens], np.uint8)
    recs, unm = records_by_e(po.MapIndex(hix), reads, lens, eper, nthreads=_threads())
    m = cuda_lib.Mapper(ix, max_reads=reads.shape[0])
    out = m.map(reads, lens, int(eper.max()), errors_per_read=eper)
    d = first_diff(out.records(), recs)
    assert d is None, d
    assert [int(x) for x in out.unmapped] == unm

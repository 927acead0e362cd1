"""The oracle against the reference's own outputs (CPU).

tests/golden/reference_outputs.json holds outputs of the reference source
compiled on the host (tests/golden/make_golden.py); where the compiled
reference is present (oracle/_ref) the oracle is also compared with it live.
"""
import hashlib
import json
import os
import tempfile

import numpy as np
import pytest

from oracle import pyoracle as po
from swmapper_gb300 import synth

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_outputs.json")))


def _genome(n, seed, kind, over, nruns=(), lower=False):
    g = synth.reference(n, seed=seed, kind=kind, **over)
    for a, b in nruns:
        g[a:b] = ord("N")
    if lower:
        g[::7] += 32
        g[5::97] = ord("R")
    return g


def _fasta(path, g, splits):
    pts = [0] + list(splits) + [g.size]
    with open(path, "wb") as f:
        for i in range(len(pts) - 1):
            f.write(b">rec%d some comment\n" % i)
            seg = g[pts[i]:pts[i + 1]]
            for j in range(0, seg.size, 61):
                f.write(seg[j:j + 61].tobytes() + b"\n")


@pytest.mark.parametrize("case", GOLD["cases"]["index"], ids=lambda c: c[0])
def test_index_files_match_reference(case, tmp_path):
    name, n, seed, kind, over, nruns, splits = case
    g = _genome(n, seed, kind, over, nruns, lower=(name == "lower_iupac"))
    fa = str(tmp_path / "x.fa")
    _fasta(fa, g, splits)
    seq, ref_info = po.read_fasta(fa)
    assert np.array_equal(seq, g)
    hix = po.build_index(seq, 12)
    files = hix.files()
    files[".ref_info"] = ref_info
    want = GOLD["index"][name]
    for ext in po.FILE_EXTS:
        assert hashlib.sha256(files[ext]).hexdigest() == want[ext], ext
    assert hix.n_seeds == want["n_seeds"]


@pytest.mark.parametrize("key", sorted(GOLD["map"]))
def test_mapping_records_match_reference(key):
    cases = {c[0]: c for c in GOLD["cases"]["map"]}
    name, e = key.rsplit("_e", 1)
    _, n, gseed, kind, over, nreads, lmin, lmax, err, es, rseed = cases[name]
    g = _genome(n, gseed, kind, over)
    mix = po.MapIndex(po.build_index(g, 12))
    reads, lens, _, _ = synth.reads(g, nreads, lmin, lmax, err, seed=rseed)
    res = po.map_reads(mix, reads, lens, int(e))
    got = [[r[0], r[1], list(r[2]), r[3].hex()] for r in res.records()]
    assert got == GOLD["map"][key]["records"]
    assert [int(x) for x in res.unmapped] == GOLD["map"][key]["unmapped"]


def test_threaded_oracle_is_deterministic():
    g = _genome(200_000, 5, "repeats100m", {"copies_per_family": 30, "rep_len_max": 2000})
    mix = po.MapIndex(po.build_index(g, 12))
    reads, lens, _, _ = synth.reads(g, 400, 60, 180, 0.03, seed=9)
    a = po.map_reads(mix, reads, lens, 6, nthreads=1).records()
    b = po.map_reads(mix, reads, lens, 6, nthreads=4).records()
    assert a == b


needs_ref = pytest.mark.skipif(not po.have_ref(), reason="reference source not compiled here")


@needs_ref
@pytest.mark.parametrize("kind,lmin,lmax,e", [("uniform", 100, 100, 5), ("repeats100m", 150, 150, 7),
                                              ("human", 45, 190, 4), ("human", 60, 120, 10)])
def test_oracle_equals_reference_live(kind, lmin, lmax, e):
    over = {"copies_per_family": 60, "rep_len_max": 3000}
    if kind == "human":
        over.update(nrun_min=500, nrun_max=5000)
    g = _genome(600_000, 77, kind, over if kind != "uniform" else {})
    mix = po.MapIndex(po.build_index(g, 12))
    reads, lens, _, _ = synth.reads(g, 800, lmin, lmax, 0.04, seed=13)
    reads[::9, 3] = ord("N")
    a = po.map_reads(mix, reads, lens, e, nthreads=4)
    b = po.ref_map_reads(mix, reads, lens, e)
    assert a.records() == b.records()
    assert list(a.unmapped) == list(b.unmapped)


@needs_ref
def test_verbatim_reference_build_is_corrupt_where_documented(tmp_path):
    """The unpatched x86 build of serial_index.c (UB shift at s == 0) differs
    from the defined build exactly in positions / lseeds / offsets."""
    g = _genome(70_001, 22, "uniform", {})
    fa = str(tmp_path / "v.fa")
    _fasta(fa, g, [])
    d = po.ref_index_files(fa, str(tmp_path / "d"))
    v = po.ref_index_files(fa, str(tmp_path / "v"), verbatim=True)
    for ext in (".ref_info", ".hash_count", ".base_2bits", ".base_3bits"):
        assert d[ext] == v[ext], ext
    assert d[".positions"] != v[".positions"]


def test_block_merge_equals_sort_unique():
    """The reference's heap merge of filtered runs (block_heap_sort) yields the
    sorted unique union: checked through the per-item trace."""
    g = _genome(300_000, 8, "repeats100m", {"copies_per_family": 60, "rep_len_max": 2500})
    mix = po.MapIndex(po.build_index(g, 12))
    reads, lens, _, _ = synth.reads(g, 200, 150, 150, 0.03, seed=4)
    for r in range(200):
        tr = po.trace_item(mix, bytes(reads[r, :lens[r]]), 7)
        for b in np.unique(tr["batch"]):
            p = tr["pos"][tr["batch"] == b]
            assert np.all(np.diff(p.astype(np.int64)) > 0)


@pytest.mark.parametrize("n,kind,k", [(3_000_013, "human", 12), (2_000_032, "repeats100m", 12),
                                      (1_500_001, "uniform", 10)])
def test_threaded_oracle_index_equals_serial(n, kind, k):
    """The threaded oracle build (used for genomes of billions of bases) gives
    the serial restatement's arrays exactly, with N runs, lowercase bases and
    slices that split N runs and k-mers."""
    over = dict(nrun_min=2000, nrun_max=50_000) if kind == "human" else {}
    g = _genome(n, 91, kind, over, nruns=[(1_000_000 - 5, 1_000_000 + 7)], lower=True)
    a = po.build_index(g, k)
    for threads in (3, 8):
        b = po.build_index(g, k, nthreads=threads)
        for key in ("hash_count", "hash_offset_end", "positions", "pos_lseeds", "base_2bits", "base_3bits"):
            assert np.array_equal(getattr(a, key), getattr(b, key)), (threads, key)

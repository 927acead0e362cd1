"""Generate the golden fixtures that pin the oracle (run where the reference is present).

The reference ships no test data, so the fixtures are outputs of the
reference's own source compiled on the host (oracle/build_ref.sh):
  * SHA-256 of the seven index files written by serial_index.c (with the
    defined-shift / guarded-flush build) for seeded synthetic FASTA files;
  * the mapping records of the reference's get_positions() for seeded reads.
Inputs are regenerated from their seeds by swmapper_gb300.synth, so the
fixtures stay a few kilobytes.

Usage: python tests/golden/make_golden.py   (writes tests/golden/*.json)
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402
from swmapper_gb300 import synth  # noqa: E402
from oracle import build as obuild  # noqa: E402
from swmapper_gb300 import _build  # noqa: E402

# index cases: (name, n, seed, kind, overrides, N runs to paint, record split points)
INDEX_CASES = [
    ("uniform_n32", 65536, 21, "uniform", {}, [], [20000]),           # n % 32 == 0 (final-flush case)
    ("uniform_odd", 70001, 22, "uniform", {}, [(100, 130), (40000, 40003)], [123, 50000]),
    ("repeats", 120017, 23, "repeats100m", {"copies_per_family": 8, "rep_len_max": 3000}, [(7, 9)], []),
    ("lower_iupac", 40013, 24, "uniform", {}, [], [1000]),
]

# mapping cases: (name, genome n, genome seed, kind, overrides, nreads, lmin, lmax, err, e list, read seed)
MAP_CASES = [
    ("plain100", 300_000, 31, "uniform", {}, 300, 100, 100, 0.02, [5, 2], 41),
    ("rep150", 400_000, 32, "repeats100m", {"copies_per_family": 24, "rep_len_max": 4000}, 300, 150, 150, 0.03,
     [7], 42),
    ("var", 300_000, 33, "human", {"nrun_min": 500, "nrun_max": 3000, "copies_per_family": 40}, 300, 40, 200, 0.04,
     [3, 8], 43),
]


def genome(n, seed, kind, over, nruns=(), lower=False):
    g = synth.reference(n, seed=seed, kind=kind, **over)
    for a, b in nruns:
        g[a:b] = ord("N")
    if lower:
        g[::7] += 32          # lowercase bases (serial_index.c:152 upper-cases them)
        g[5::97] = ord("R")   # IUPAC code, indexed as N
    return g


def write_fasta(path, g, splits):
    pts = [0] + list(splits) + [g.size]
    with open(path, "wb") as f:
        for i in range(len(pts) - 1):
            f.write(b">rec%d some comment\n" % i)
            seg = g[pts[i]:pts[i + 1]]
            for j in range(0, seg.size, 61):
                f.write(seg[j:j + 61].tobytes() + b"\n")


def canon(recs):
    return [[r[0], r[1], list(r[2]), r[3].hex()] for r in recs]


def main():
    _build.build_synth()
    obuild.build_oracle()
    if obuild.build_ref() is None:
        raise SystemExit("reference source not available: cannot make golden fixtures")
    out = {"index": {}, "map": {}}
    with tempfile.TemporaryDirectory() as td:
        for name, n, seed, kind, over, nruns, splits in INDEX_CASES:
            g = genome(n, seed, kind, over, nruns, lower=(name == "lower_iupac"))
            fa = os.path.join(td, name + ".fa")
            write_fasta(fa, g, splits)
            files = po.ref_index_files(fa, os.path.join(td, name))
            out["index"][name] = {ext: hashlib.sha256(files[ext]).hexdigest() for ext in po.FILE_EXTS}
            out["index"][name]["n_seeds"] = len(files[".positions"]) // 4
    for name, n, gseed, kind, over, nreads, lmin, lmax, err, es, rseed in MAP_CASES:
        g = genome(n, gseed, kind, over)
        mix = po.MapIndex(po.build_index(g, 12))
        reads, lens, _, _ = synth.reads(g, nreads, lmin, lmax, err, seed=rseed)
        for e in es:
            res = po.ref_map_reads(mix, reads, lens, e)
            out["map"][f"{name}_e{e}"] = {"records": canon(res.records()),
                                          "unmapped": [int(x) for x in res.unmapped]}
    with open(os.path.join(HERE, "reference_outputs.json"), "w") as f:
        json.dump({"cases": {"index": INDEX_CASES, "map": MAP_CASES}, **out}, f, separators=(",", ":"))
    print("wrote", os.path.join(HERE, "reference_outputs.json"))


if __name__ == "__main__":
    main()

"""Shared helpers for the test-suite: seeded workloads and record comparison."""
from __future__ import annotations

import numpy as np

from oracle import pyoracle as po
from swmapper_gb300 import synth


def genome(n, seed, kind="uniform", nruns=(), **over):
    g = synth.reference(n, seed=seed, kind=kind, **over)
    for a, b in nruns:
        g[a:b] = ord("N")
    return g


def oracle_index(g, k=12):
    hix = po.build_index(g, k)
    return hix, po.MapIndex(hix)


def records_by_e(mix, reads, lens, eper, nthreads=4):
    """Oracle records for reads with per-read thresholds (mapped per e group)."""
    out = {}
    for e in sorted(set(int(x) for x in eper)):
        idx = np.nonzero(eper == e)[0]
        res = po.map_reads(mix, reads[idx], lens[idx], e, nthreads=nthreads)
        for rec in res.records():
            cur = rec[0]
            read = int(idx[cur >> 1])
            out.setdefault(read, []).append((2 * read + (cur & 1),) + rec[1:])
        for u in res.unmapped:
            out.setdefault(int(idx[u >> 1]), [])
    flat = []
    unm = []
    for r in sorted(out):
        if not out[r]:
            unm.append(2 * r + 1)
        flat.extend(out[r])
    return flat, unm


def first_diff(a, b):
    for i, (x, y) in enumerate(zip(a, b)):
        if x != y:
            return i, x, y
    if len(a) != len(b):
        return min(len(a), len(b)), len(a), len(b)
    return None

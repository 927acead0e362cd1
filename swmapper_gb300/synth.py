"""Seeded synthetic workloads (ctypes view of libswm_synth.so).

The named workloads, with the shapes the benchmark configurations give:
  plain       1 Mbp uniform ACGT, 100 bp reads, 2% error, e=5
  batched     100 Mbp, 41% GC, 10% repeat copies (300 bp-6 kb, 1% divergence),
              150 bp reads, 3% error, e=7
  uneven      same genome, reads U[50, 250] bp, 4% error, e=ceil(0.05 L)
  human       3.1 Gbp, 41% GC, 5% N runs (10 kb-1 Mb), 50% repeat families
              (2-15% divergence), 150 bp reads, 3% error, e=7
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build


class RefCfg(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("gc", C.c_double), ("repeat_frac", C.c_double),
                ("rep_len_min", C.c_uint64), ("rep_len_max", C.c_uint64),
                ("copies_per_family", C.c_uint64), ("div_min", C.c_double), ("div_max", C.c_double),
                ("n_frac", C.c_double), ("nrun_min", C.c_uint64), ("nrun_max", C.c_uint64)]


class ReadCfg(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("nreads", C.c_uint64), ("len_min", C.c_uint32),
                ("len_max", C.c_uint32), ("err_rate", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB_SYNTH):
            _build.build_synth()
        _lib = C.CDLL(_build.LIB_SYNTH)
        _lib.swm_synth_reference.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(RefCfg)]
        _lib.swm_synth_reads.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(ReadCfg), C.c_void_p,
                                         C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p]
    return _lib


GENOMES = {
    "uniform": dict(gc=0.5),
    "repeats100m": dict(gc=0.41, repeat_frac=0.10, rep_len_min=300, rep_len_max=6000,
                        copies_per_family=16, div_min=0.01, div_max=0.01),
    "human": dict(gc=0.41, repeat_frac=0.50, rep_len_min=300, rep_len_max=6000,
                  copies_per_family=400, div_min=0.02, div_max=0.15,
                  n_frac=0.05, nrun_min=10_000, nrun_max=1_000_000),
}


def reference(n: int, seed: int = 1, kind: str = "uniform", **over) -> np.ndarray:
    """Synthetic genome of n bases (uint8 array of A/C/G/T/N)."""
    cfg = dict(seed=seed, gc=0.5, repeat_frac=0.0, rep_len_min=0, rep_len_max=0, copies_per_family=0,
               div_min=0.0, div_max=0.0, n_frac=0.0, nrun_min=0, nrun_max=0)
    cfg.update(GENOMES[kind])
    cfg.update(over)
    out = np.empty(n, dtype=np.uint8)
    rc = lib().swm_synth_reference(out.ctypes.data, n, C.byref(RefCfg(**cfg)))
    if rc != 0:
        raise RuntimeError(f"swm_synth_reference failed ({rc})")
    return out


def reads(genome: np.ndarray, nreads: int, len_min: int, len_max: int, err_rate: float, seed: int = 7,
          stride: int | None = None):
    """Reads from genome: (buffer[nreads, stride] uint8, lens uint32, truth_pos, truth_strand)."""
    stride = stride or len_max
    buf = np.zeros((nreads, stride), dtype=np.uint8)
    lens = np.zeros(nreads, dtype=np.uint32)
    pos = np.zeros(nreads, dtype=np.uint32)
    strand = np.zeros(nreads, dtype=np.uint8)
    cfg = ReadCfg(seed=seed, nreads=nreads, len_min=len_min, len_max=len_max, err_rate=err_rate)
    rc = lib().swm_synth_reads(genome.ctypes.data, genome.size, C.byref(cfg), buf.ctypes.data, stride,
                               lens.ctypes.data, pos.ctypes.data, strand.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"swm_synth_reads failed ({rc})")
    return buf, lens, pos, strand

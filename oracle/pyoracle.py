"""ctypes view of the CPU oracle and of the compiled reference (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and the cpu_baseline / reference legs of
bench.py import this module. It is the checker, never the thing measured as
the product.

  Oracle          libswm_oracle.so   restatement of serial_index.c + mapper_cpe.c
  RefMapper       libswref.so        the reference's own get_positions() compiled
                                     for the host (oracle/build_ref.sh)
  ref_index_files run oracle/_ref/serial_index[_verbatim] on a FASTA
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from .build import LIB_ORACLE, LIB_SWREF, REF_DIR

RECORD_WORDS = 258
CIGAR_STRIDE = 4096
PAD_WORDS = 64

FILE_EXTS = (".ref_info", ".hash_count", ".hash_offset", ".positions", ".pos_lseeds", ".base_2bits",
             ".base_3bits")


class _Index(C.Structure):
    _fields_ = [("k", C.c_uint32), ("n", C.c_uint64), ("n_seeds", C.c_uint64),
                ("hash_count", C.POINTER(C.c_uint32)), ("hash_offset", C.POINTER(C.c_uint32)),
                ("positions", C.POINTER(C.c_uint32)), ("pos_lseeds", C.POINTER(C.c_uint16)),
                ("base_2bits", C.POINTER(C.c_uint32)), ("base_3bits", C.POINTER(C.c_uint32))]


class _MapIdx(C.Structure):
    _fields_ = [("k", C.c_uint32), ("hash_offset", C.c_void_p), ("positions", C.c_void_p),
                ("pos_lseeds", C.c_void_p), ("base_2bits", C.c_void_p), ("n_words2", C.c_uint64),
                ("ref_length", C.c_uint64)]


class _Out(C.Structure):
    _fields_ = [("ref_pos", C.c_void_p), ("cigar", C.c_void_p), ("unmapped", C.c_void_p),
                ("cap_records", C.c_uint64), ("cap_unmapped", C.c_uint64),
                ("n_records", C.c_uint64), ("n_unmapped", C.c_uint64), ("overflow", C.c_int)]


STAT_FIELDS = ["items", "batches", "fetched", "candidates", "cells", "passed", "hamming", "traceback",
               "emitted", "mapped_reads", "ub_shift_out", "ub_walk_stop", "ub_empty_merge",
               "ub_short_seeds", "ub_err0_traceback"]


class _Stats(C.Structure):
    _fields_ = [(f, C.c_uint64) for f in STAT_FIELDS]


class _Trace(C.Structure):
    _fields_ = [("n", C.c_uint32), ("batch", C.POINTER(C.c_uint32)), ("pos", C.POINTER(C.c_uint32)),
                ("err", C.POINTER(C.c_int32)), ("loc", C.POINTER(C.c_int32)), ("nbatches", C.c_uint32),
                ("nsel", C.c_uint32), ("sel_start", C.c_uint32 * 64), ("sel_count", C.c_uint32 * 64),
                ("sel_base", C.c_uint32 * 64), ("sel_shift", C.c_uint8 * 64), ("sel_rl", C.c_uint8 * 64),
                ("sel_rh", C.c_uint8 * 64), ("w", C.c_uint32 * 32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_ORACLE):
            from .build import build_oracle
            build_oracle()
        L = C.CDLL(LIB_ORACLE)
        L.swo_index_build.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.POINTER(_Index)]
        L.swo_index_build_mt.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.POINTER(_Index)]
        L.swo_index_free.argtypes = [C.POINTER(_Index)]
        L.swo_map_reads.argtypes = [C.POINTER(_MapIdx), C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                    C.c_uint32, C.c_uint32, C.POINTER(_Out), C.POINTER(_Stats)]
        L.swo_encode_read.argtypes = [C.c_char_p, C.c_uint32, C.c_uint32, C.c_void_p]
        L.swo_banded_myers.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                       C.c_uint32, C.POINTER(C.c_int)]
        L.swo_trace_item.argtypes = [C.POINTER(_MapIdx), C.c_char_p, C.c_uint32, C.c_uint32,
                                     C.POINTER(_Trace)]
        L.swo_trace_free.argtypes = [C.POINTER(_Trace)]
        L.swo_read_fasta.argtypes = [C.c_char_p, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64),
                                     C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)]
        L.swo_index_write.argtypes = [C.POINTER(_Index), C.c_char_p, C.c_char_p, C.c_size_t]
        _lib = L
    return _lib


class HostIndex:
    """Index arrays as numpy (copies), in the reference's file layout."""

    def __init__(self, k, n, hash_count, hash_offset_end, positions, pos_lseeds, base_2bits, base_3bits):
        self.k, self.n = k, n
        self.hash_count = hash_count
        self.hash_offset_end = hash_offset_end
        self.positions = positions
        self.pos_lseeds = pos_lseeds
        self.base_2bits = base_2bits
        self.base_3bits = base_3bits

    @property
    def n_seeds(self):
        return int(self.positions.size)

    def start_offsets(self) -> np.ndarray:
        """hash_offset the way the mapper rebuilds it from counts (mapper_mpe.c:250-255)."""
        off = np.zeros(self.hash_count.size + 1, dtype=np.uint64)
        np.cumsum(self.hash_count, dtype=np.uint64, out=off[1:])
        return off.astype(np.uint32)

    def files(self) -> dict:
        return {".hash_count": self.hash_count.tobytes(), ".hash_offset": self.hash_offset_end.tobytes(),
                ".positions": self.positions.tobytes(), ".pos_lseeds": self.pos_lseeds.tobytes(),
                ".base_2bits": self.base_2bits.tobytes(), ".base_3bits": self.base_3bits.tobytes()}


def build_index(seq: np.ndarray, k: int = 12, nthreads: int = 1) -> HostIndex:
    """The oracle's index (serial_index.c:157-445); nthreads > 1 splits its
    loops over host threads with identical output (swo_index_build_mt)."""
    seq = np.ascontiguousarray(seq, dtype=np.uint8)
    ix = _Index()
    if nthreads > 1:
        rc = lib().swo_index_build_mt(seq.ctypes.data, seq.size, k, nthreads, C.byref(ix))
    else:
        rc = lib().swo_index_build(seq.ctypes.data, seq.size, k, C.byref(ix))
    if rc != 0:
        raise RuntimeError(f"swo_index_build failed ({rc})")
    try:
        nb = 1 << (2 * k)
        W = (seq.size + 31) // 32
        S = ix.n_seeds

        def arr(ptr, count, dt):
            if count == 0:
                return np.zeros(0, dtype=dt)
            return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dt, copy=True)

        return HostIndex(k, seq.size, arr(ix.hash_count, nb, np.uint32), arr(ix.hash_offset, nb + 1, np.uint32),
                         arr(ix.positions, S, np.uint32), arr(ix.pos_lseeds, S, np.uint16),
                         arr(ix.base_2bits, 2 * W, np.uint32), arr(ix.base_3bits, W, np.uint32))
    finally:
        lib().swo_index_free(C.byref(ix))


class MapIndex:
    """Mapper view: start offsets, padded base_2bits, ref_length = bytes * 16."""

    def __init__(self, hix: HostIndex):
        self.k = hix.k
        self.hash_offset = hix.start_offsets()
        self.positions = np.concatenate([hix.positions, np.zeros(8, np.uint32)])
        self.pos_lseeds = np.concatenate([hix.pos_lseeds, np.zeros(8, np.uint16)])
        self.base_2bits = np.concatenate([hix.base_2bits, np.zeros(PAD_WORDS, np.uint32)])
        self.n_words2 = hix.base_2bits.size
        self.ref_length = hix.base_2bits.size * 4 * 16
        self._c = _MapIdx(self.k, self.hash_offset.ctypes.data, self.positions.ctypes.data,
                          self.pos_lseeds.ctypes.data, self.base_2bits.ctypes.data, self.n_words2,
                          self.ref_length)


class MapResult:
    def __init__(self, ref_pos, cigar, unmapped, stats=None):
        self.ref_pos = ref_pos      # [n_records, 258] uint32
        self.cigar = cigar          # [n_records, 4096] uint8
        self.unmapped = unmapped    # [n_unmapped] uint32
        self.stats = stats or {}

    def records(self):
        """Canonical form: list of (cur_read, primary, locs tuple, cigar bytes)."""
        out = []
        for r in range(self.ref_pos.shape[0]):
            rec = self.ref_pos[r]
            n = int(rec[1] & 0x0FFFFFFF)
            locs = tuple(int(x) for x in rec[2:2 + n])
            cb = self.cigar[r]
            p = 0
            parts = []
            for _ in range(n):
                ln = int(cb[p + 1])
                parts.append(bytes(cb[p:p + 2 + ln]))
                p += 2 + ln
            out.append((int(rec[0]), int(rec[1]) >> 31, locs, b"".join(parts)))
        return out


def map_reads(mix: MapIndex, reads: np.ndarray, lens: np.ndarray, e: int, nthreads: int = 1,
              cap_records: int | None = None) -> MapResult:
    reads = np.ascontiguousarray(reads, dtype=np.uint8)
    lens = np.ascontiguousarray(lens, dtype=np.uint32)
    nreads, stride = reads.shape
    cap = cap_records or max(16, 4 * nreads + 64)
    ref_pos = np.zeros((cap, RECORD_WORDS), dtype=np.uint32)
    cigar = np.zeros((cap, CIGAR_STRIDE), dtype=np.uint8)
    unm = np.zeros(max(1, nreads), dtype=np.uint32)
    out = _Out(ref_pos.ctypes.data, cigar.ctypes.data, unm.ctypes.data, cap, unm.size, 0, 0, 0)
    st = _Stats()
    rc = lib().swo_map_reads(C.byref(mix._c), reads.ctypes.data, stride, lens.ctypes.data, nreads, e, nthreads,
                             C.byref(out), C.byref(st))
    if rc != 0:
        raise RuntimeError(f"swo_map_reads failed ({rc})")
    stats = {f: int(getattr(st, f)) for f in STAT_FIELDS}
    return MapResult(ref_pos[:out.n_records], cigar[:out.n_records], unm[:out.n_unmapped], stats)


def encode_read(seq: bytes, k: int = 12) -> np.ndarray:
    w = np.zeros(32, dtype=np.uint32)
    lib().swo_encode_read(seq, len(seq), k, w.ctypes.data)
    return w


def trace_item(mix: MapIndex, seq: bytes, e: int) -> dict:
    tr = _Trace()
    rc = lib().swo_trace_item(C.byref(mix._c), seq, len(seq), e, C.byref(tr))
    if rc != 0:
        raise RuntimeError("trace failed")
    try:
        n = tr.n

        def a(p, dt):
            return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True) if n else np.zeros(0, dt)

        ns = tr.nsel
        return dict(batch=a(tr.batch, np.uint32), pos=a(tr.pos, np.uint32), err=a(tr.err, np.int32),
                    loc=a(tr.loc, np.int32), nbatches=tr.nbatches, nsel=ns,
                    sel_start=np.array(tr.sel_start[:ns], np.uint32),
                    sel_count=np.array(tr.sel_count[:ns], np.uint32),
                    sel_base=np.array(tr.sel_base[:ns], np.uint32),
                    sel_shift=np.array(tr.sel_shift[:ns], np.uint8),
                    sel_rl=np.array(tr.sel_rl[:ns], np.uint8), sel_rh=np.array(tr.sel_rh[:ns], np.uint8),
                    w=np.array(tr.w[:], np.uint32))
    finally:
        lib().swo_trace_free(C.byref(tr))


def read_fasta(path: str):
    seq = C.c_void_p()
    n = C.c_uint64()
    info = C.c_void_p()
    ilen = C.c_size_t()
    rc = lib().swo_read_fasta(path.encode(), C.byref(seq), C.byref(n), C.byref(info), C.byref(ilen))
    if rc != 0:
        raise RuntimeError(f"cannot read {path}")
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    s = np.ctypeslib.as_array(C.cast(seq, C.POINTER(C.c_uint8)), shape=(n.value,)).copy() if n.value else \
        np.zeros(0, np.uint8)
    ri = C.string_at(info, ilen.value)
    libc.free(seq)
    libc.free(info)
    return s, ri


# ---------------------------------------------------------------- reference

def have_ref() -> bool:
    return os.path.exists(LIB_SWREF)


_ref = None


def reflib():
    global _ref
    if _ref is None:
        if not have_ref():
            raise RuntimeError("reference harness not built (oracle/build_ref.sh)")
        L = C.CDLL(LIB_SWREF)
        L.swref_map.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint32,
                                C.c_uint32, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_int,
                                C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64),
                                C.POINTER(C.c_uint64)]
        _ref = L
    return _ref


def out_buffers(nreads: int):
    """Output buffers in the reference layout for blocks of up to nreads reads."""
    cap = max(16, 4 * nreads + 64)
    return (np.zeros((cap, RECORD_WORDS), dtype=np.uint32), np.zeros((cap, CIGAR_STRIDE), dtype=np.uint8),
            np.zeros(max(1, 2 * nreads), dtype=np.uint32))


def ref_map_reads(mix: MapIndex, reads: np.ndarray, lens: np.ndarray, e: int, nthreads: int = 1,
                  out=None) -> MapResult:
    """The reference's own get_positions() over the reads (records sorted canonically)."""
    reads = np.ascontiguousarray(reads, dtype=np.uint8)
    lens = np.ascontiguousarray(lens, dtype=np.uint32)
    nreads, stride = reads.shape
    ref_pos, cigar, unm = out if out is not None else out_buffers(nreads)
    cap = ref_pos.shape[0]
    if cap < 4 * nreads + 16 or unm.size < 2 * nreads:
        raise ValueError("output buffers too small for this block")
    nrec = C.c_uint64()
    nun = C.c_uint64()
    rc = reflib().swref_map(mix.hash_offset.ctypes.data, mix.positions.ctypes.data, mix.pos_lseeds.ctypes.data,
                            mix.base_2bits.ctypes.data, mix.ref_length, mix.k, e, reads.ctypes.data, stride,
                            lens.ctypes.data, nreads, nthreads, ref_pos.ctypes.data, cigar.ctypes.data,
                            unm.ctypes.data, C.byref(nrec), C.byref(nun))
    if rc != 0:
        raise RuntimeError(f"swref_map failed ({rc})")
    n = nrec.value
    rp, cg = ref_pos[:n], cigar[:n]
    # canonical order: by (cur_read, arrival) -- a single worker keeps arrival order per read
    order = np.argsort(rp[:, 0], kind="stable")
    return MapResult(rp[order], cg[order], np.sort(unm[:nun.value]))


def ref_index_files(fasta: str, prefix: str, verbatim: bool = False, k: int = 12) -> dict:
    exe = os.path.join(REF_DIR, "serial_index_verbatim" if verbatim else "serial_index")
    subprocess.run([exe, "-i" + fasta, "-p" + prefix, f"-s{k}"], check=True, capture_output=True)
    out = {}
    for ext in FILE_EXTS:
        with open(prefix + ext, "rb") as f:
            out[ext] = f.read()
    return out

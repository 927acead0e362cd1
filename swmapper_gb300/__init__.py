"""GB300 short-read mapper hot path (SWMapper's index build + mapping kernel).

Thin ctypes view of the C ABI in include/swmapper.h (libswmapper_gb300.so).
There is no CPU fallback: importing the classes below on a machine where the
CUDA library was not built raises.

    ix = Index.build(seq_bytes, k=12)            # GPU k-mer index
    m = Mapper(ix, max_reads=65536)
    res = m.map(reads, lens, errors=7)            # reference output layout
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

RECORD_WORDS = 258
CIGAR_STRIDE = 4096
MAX_READ_LEN = 254
MAX_ERRORS = 15


class IndexInfo(C.Structure):
    _fields_ = [("k", C.c_uint32), ("n", C.c_uint64), ("n_seeds", C.c_uint64), ("n_words2", C.c_uint64),
                ("n_words3", C.c_uint64), ("ref_length", C.c_uint64), ("device", C.c_int)]


class Batch(C.Structure):
    _fields_ = [("reads", C.c_void_p), ("reads_len", C.c_void_p), ("stride", C.c_uint64),
                ("reads_num", C.c_uint64), ("errors", C.c_uint32), ("errors_per_read", C.c_void_p)]


class Result(C.Structure):
    _fields_ = [("ref_pos_buffer", C.c_void_p), ("cigar_buffer", C.c_void_p), ("unmapped", C.c_void_p),
                ("records_cap", C.c_uint64), ("unmapped_cap", C.c_uint64), ("n_records", C.c_uint64),
                ("n_unmapped", C.c_uint64)]


class PackedResult(C.Structure):
    _fields_ = [("words", C.c_void_p), ("cigar", C.c_void_p), ("record_cigar_len", C.c_void_p),
                ("unmapped", C.c_void_p), ("words_cap", C.c_uint64), ("cigar_cap", C.c_uint64),
                ("records_cap", C.c_uint64), ("unmapped_cap", C.c_uint64), ("n_words", C.c_uint64),
                ("n_cigar", C.c_uint64), ("n_records", C.c_uint64), ("n_unmapped", C.c_uint64)]


STAT_FIELDS = ["reads", "items", "chunks", "batches", "fetched", "candidates", "cells", "passed", "records",
               "locations", "mapped_reads", "retries", "h2d_bytes", "d2h_bytes", "myers_steps", "kept"]


class MapStats(C.Structure):
    _fields_ = [(f, C.c_uint64) for f in STAT_FIELDS]


class ServeConfig(C.Structure):
    _fields_ = [("block_reads", C.c_uint64), ("max_slots", C.c_uint32), ("stride", C.c_uint64),
                ("max_queued_reads", C.c_uint64), ("device_mem_limit", C.c_uint64),
                ("device_mem_reserve", C.c_uint64)]


SERVE_FIELDS = ["slots", "slot_bytes", "blocks", "max_blocks_in_flight", "requests_admitted", "requests_done",
                "reads_done", "refused_memory", "refused_queue", "queued_reads"]


class ServeCounters(C.Structure):
    _fields_ = [(f, C.c_uint64) for f in SERVE_FIELDS]


class RequestInfo(C.Structure):
    _fields_ = [("id", C.c_uint64), ("reads", C.c_uint64), ("block_reads", C.c_uint64),
                ("latency_ms", C.c_double)]


class SwmError(RuntimeError):
    def __init__(self, msg, rc=None):
        super().__init__(msg)
        self.rc = rc


_lib = None


class Tuning(C.Structure):
    """swm_tuning (include/swmapper.h)."""
    _fields_ = [("verify_head_bases", C.c_uint32), ("verify_chunk", C.c_uint32), ("verify_pairs", C.c_uint32)]


# verification forms: name -> (verify_head_bases, verify_chunk, verify_pairs)
VERIFY_MODES = {"head32": (32, 0, 0), "head64": (64, 0, 0), "stream8": (64, 8, 0), "stream16": (64, 16, 0),
                "pair16": (64, 16, 1)}


def lib():
    """Load the CUDA library; raise if it was not built (no fallback path)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB_CUDA):
            raise SwmError(f"{_build.LIB_CUDA} is missing: run __graft_entry__.build() first")
        L = C.CDLL(_build.LIB_CUDA)
        vp, u32, u64 = C.c_void_p, C.c_uint32, C.c_uint64
        L.swm_last_error.restype = C.c_char_p
        L.swm_index_build.argtypes = [vp, u64, u32, C.c_int, C.POINTER(vp)]
        L.swm_index_build_device.argtypes = [vp, u64, u32, C.c_int, C.POINTER(vp)]
        L.swm_index_build_fasta.argtypes = [C.c_char_p, C.c_char_p, u32, C.c_int]
        L.swm_index_open.argtypes = [C.c_char_p, u32, C.c_int, C.POINTER(vp)]
        L.swm_index_save.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_size_t]
        L.swm_index_get_info.argtypes = [vp, C.POINTER(IndexInfo)]
        L.swm_index_download.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.swm_index_candidate_table.argtypes = [vp, C.c_int, C.POINTER(u64)]
        L.swm_index_serialize_mappers.argtypes = [vp, C.c_int]
        L.swm_index_free.argtypes = [vp]
        L.swm_index_free.restype = None
        L.swm_mapper_create.argtypes = [vp, u64, C.POINTER(vp)]
        L.swm_map_batch.argtypes = [vp, C.POINTER(Batch), C.POINTER(Result)]
        L.swm_map_submit.argtypes = [vp, C.POINTER(Batch)]
        L.swm_map_wait.argtypes = [vp, C.POINTER(Result)]
        L.swm_map_device.argtypes = [vp, vp, vp, u64, u64, u32, vp]
        L.swm_map_device_submit.argtypes = [vp, vp, vp, u64, u64, u32, vp]
        L.swm_map_device_wait.argtypes = [vp]
        L.swm_map_fetch.argtypes = [vp, C.POINTER(Result)]
        L.swm_map_fetch_packed.argtypes = [vp, C.POINTER(PackedResult)]
        L.swm_map_wait_packed.argtypes = [vp, C.POINTER(PackedResult)]
        L.swm_mapper_stats.argtypes = [vp, C.POINTER(MapStats)]
        L.swm_mapper_stage_ms.argtypes = [vp, C.c_char_p, C.POINTER(C.c_float)]
        L.swm_mapper_tuning.argtypes = [vp, C.POINTER(Tuning), C.POINTER(Tuning)]
        L.swm_mapper_launches.argtypes = [vp]
        L.swm_mapper_launches.restype = u64
        L.swm_mapper_stream.argtypes = [vp]
        L.swm_mapper_stream.restype = vp
        L.swm_mapper_debug_candidates.argtypes = [vp, vp, vp, vp, vp, u64, C.POINTER(u64)]
        L.swm_mapper_debug_read_words.argtypes = [vp, vp, u64]
        L.swm_mapper_free.argtypes = [vp]
        L.swm_mapper_free.restype = None
        L.swm_probe_random_reads.argtypes = [C.c_int, u64, C.POINTER(C.c_double)]
        L.swm_serve_open.argtypes = [vp, C.POINTER(ServeConfig), C.POINTER(vp)]
        L.swm_serve_submit.argtypes = [vp, C.POINTER(Batch), C.POINTER(u64)]
        L.swm_serve_poll.argtypes = [vp, C.c_int, C.POINTER(u64), C.POINTER(PackedResult), C.POINTER(RequestInfo)]
        L.swm_serve_stats.argtypes = [vp, C.POINTER(ServeCounters)]
        L.swm_serve_close.argtypes = [vp]
        _lib = L
    return _lib


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise SwmError(f"{what} failed ({rc}): {lib().swm_last_error().decode(errors='replace')}", rc)


def probe_random_reads(nbytes: int, device: int = 0) -> float:
    """Random 32-byte reads per second the device serves from a buffer of
    nbytes (swm_probe_random_reads)."""
    v = C.c_double()
    _check(lib().swm_probe_random_reads(device, nbytes, C.byref(v)), "swm_probe_random_reads")
    return float(v.value)


class Index:
    """Device-resident k-mer index (swm_index)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def build(cls, seq, k: int = 12, device: int = 0) -> "Index":
        seq = np.ascontiguousarray(np.frombuffer(seq, np.uint8) if isinstance(seq, (bytes, bytearray)) else seq,
                                   dtype=np.uint8)
        h = C.c_void_p()
        _check(lib().swm_index_build(seq.ctypes.data, seq.size, k, device, C.byref(h)), "swm_index_build")
        return cls(h)

    @classmethod
    def build_device(cls, d_seq: int, n: int, k: int = 12, device: int = 0) -> "Index":
        """Index n bases already in device memory (swm_index_build_device)."""
        h = C.c_void_p()
        _check(lib().swm_index_build_device(d_seq, n, k, device, C.byref(h)), "swm_index_build_device")
        return cls(h)

    @classmethod
    def open(cls, prefix: str, k: int = 12, device: int = 0) -> "Index":
        h = C.c_void_p()
        _check(lib().swm_index_open(prefix.encode(), k, device, C.byref(h)), "swm_index_open")
        return cls(h)

    @staticmethod
    def build_fasta(fasta: str, prefix: str, k: int = 12, device: int = 0) -> None:
        _check(lib().swm_index_build_fasta(fasta.encode(), prefix.encode(), k, device), "swm_index_build_fasta")

    def save(self, prefix: str, ref_info: bytes = b"") -> None:
        _check(lib().swm_index_save(self._h, prefix.encode(), ref_info, len(ref_info)), "swm_index_save")

    def info(self) -> IndexInfo:
        inf = IndexInfo()
        _check(lib().swm_index_get_info(self._h, C.byref(inf)), "swm_index_get_info")
        return inf

    def download(self) -> dict:
        inf = self.info()
        nb = 1 << (2 * inf.k)
        out = dict(hash_count=np.zeros(nb, np.uint32), hash_offset=np.zeros(nb + 1, np.uint32),
                   positions=np.zeros(inf.n_seeds, np.uint32), pos_lseeds=np.zeros(inf.n_seeds, np.uint16),
                   base_2bits=np.zeros(inf.n_words2, np.uint32), base_3bits=np.zeros(inf.n_words3, np.uint32))
        _check(lib().swm_index_download(self._h, *(out[k].ctypes.data for k in
                                                   ("hash_count", "hash_offset", "positions", "pos_lseeds",
                                                    "base_2bits", "base_3bits"))), "swm_index_download")
        return out

    def candidate_table(self, enable: bool | None = None) -> int:
        """Build (True) or drop (False) the device-only candidate table, or
        only report it (None) (swm_index_candidate_table); returns its device
        bytes (0: none)."""
        nbytes = C.c_uint64()
        mode = -1 if enable is None else (1 if enable else 0)
        _check(lib().swm_index_candidate_table(self._h, mode, C.byref(nbytes)), "swm_index_candidate_table")
        return int(nbytes.value)

    def serialize_mappers(self, on: bool = True) -> None:
        """Run the mappers' blocks one at a time on the GPU, their copies
        overlapping the other mappers' kernels (swm_index_serialize_mappers)."""
        _check(lib().swm_index_serialize_mappers(self._h, 1 if on else 0), "swm_index_serialize_mappers")

    def close(self) -> None:
        if self._h:
            lib().swm_index_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MapOutput:
    """Records in the reference layout plus the unmapped read ids."""

    def __init__(self, ref_pos, cigar, unmapped, stats):
        self.ref_pos, self.cigar, self.unmapped, self.stats = ref_pos, cigar, unmapped, stats

    def records(self):
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


class Mapper:
    """Mapping context (swm_mapper): one CUDA stream and its work buffers."""

    def __init__(self, index: Index, max_reads: int = 65536):
        self.index = index
        self.max_reads = max_reads
        h = C.c_void_p()
        _check(lib().swm_mapper_create(index._h, max_reads, C.byref(h)), "swm_mapper_create")
        self._h = h

    def _result(self, nreads: int, records_cap: int | None = None):
        cap = records_cap or max(64, 4 * nreads + 64)
        ref_pos = np.zeros((cap, RECORD_WORDS), np.uint32)
        cigar = np.zeros((cap, CIGAR_STRIDE), np.uint8)
        unm = np.zeros(max(1, nreads), np.uint32)
        res = Result(ref_pos.ctypes.data, cigar.ctypes.data, unm.ctypes.data, cap, unm.size, 0, 0)
        return res, ref_pos, cigar, unm

    def map(self, reads: np.ndarray, lens: np.ndarray, errors: int, errors_per_read=None,
            records_cap: int | None = None) -> MapOutput:
        """Map a block of reads held in host memory (swm_map_batch)."""
        reads = np.ascontiguousarray(reads, np.uint8)
        lens = np.ascontiguousarray(lens, np.uint32)
        n, stride = reads.shape
        epr = None if errors_per_read is None else np.ascontiguousarray(errors_per_read, np.uint8)
        b = Batch(reads.ctypes.data, lens.ctypes.data, stride, n, errors, epr.ctypes.data if epr is not None else None)
        res, ref_pos, cigar, unm = self._result(n, records_cap)
        _check(lib().swm_map_batch(self._h, C.byref(b), C.byref(res)), "swm_map_batch")
        return MapOutput(ref_pos[:res.n_records], cigar[:res.n_records], unm[:res.n_unmapped], self.stats())

    def submit(self, reads: np.ndarray, lens: np.ndarray, errors: int, errors_per_read=None) -> None:
        """Queue a block (swm_map_submit); the inputs are copied before it returns."""
        reads = np.ascontiguousarray(reads, np.uint8)
        lens = np.ascontiguousarray(lens, np.uint32)
        n, stride = reads.shape
        epr = None if errors_per_read is None else np.ascontiguousarray(errors_per_read, np.uint8)
        b = Batch(reads.ctypes.data, lens.ctypes.data, stride, n, errors, epr.ctypes.data if epr is not None else None)
        _check(lib().swm_map_submit(self._h, C.byref(b)), "swm_map_submit")

    def wait_packed(self, out: "PackedBuffers") -> "PackedBuffers":
        """Wait for the queued block and copy its records out packed (swm_map_wait_packed)."""
        _check(lib().swm_map_wait_packed(self._h, C.byref(out.c)), "swm_map_wait_packed")
        return out

    def map_device(self, d_reads: int, d_lens: int, stride: int, nreads: int, errors: int, d_errors: int | None = None):
        """Map reads already resident in device memory (pointers as ints)."""
        _check(lib().swm_map_device(self._h, d_reads, d_lens, stride, nreads, errors, d_errors),
               "swm_map_device")

    def submit_device(self, d_reads: int, d_lens: int, stride: int, nreads: int, errors: int,
                      d_errors: int | None = None):
        """Queue a block of device-resident reads and return (swm_map_device_submit)."""
        _check(lib().swm_map_device_submit(self._h, d_reads, d_lens, stride, nreads, errors, d_errors),
               "swm_map_device_submit")

    def wait_device(self):
        """Wait for the block queued by submit_device (swm_map_device_wait)."""
        _check(lib().swm_map_device_wait(self._h), "swm_map_device_wait")

    def fetch(self, nreads: int, records_cap: int | None = None) -> MapOutput:
        res, ref_pos, cigar, unm = self._result(nreads, records_cap)
        _check(lib().swm_map_fetch(self._h, C.byref(res)), "swm_map_fetch")
        return MapOutput(ref_pos[:res.n_records], cigar[:res.n_records], unm[:res.n_unmapped], self.stats())

    def stats(self) -> dict:
        s = MapStats()
        _check(lib().swm_mapper_stats(self._h, C.byref(s)), "swm_mapper_stats")
        return {f: int(getattr(s, f)) for f in STAT_FIELDS}

    def stage_ms(self, stage: str) -> float:
        v = C.c_float()
        _check(lib().swm_mapper_stage_ms(self._h, stage.encode(), C.byref(v)), "swm_mapper_stage_ms")
        return float(v.value)

    def set_verify(self, mode: str) -> None:
        """Form of the verification stage (swm_mapper_tuning): "head32" /
        "head64" (a first pass over that many bases of every candidate, then
        the rest), "stream8" / "stream16" (each lane runs its own candidate
        and tests the stop bound every 8 / 16 bases) or "pair16" (two
        candidates per lane when every threshold is <= 7). Results never
        change."""
        if mode not in VERIFY_MODES:
            raise SwmError(f"unknown verification form {mode!r} (one of {', '.join(VERIFY_MODES)})", -1)
        head, chunk, pairs = VERIFY_MODES[mode]
        t = Tuning(verify_head_bases=head, verify_chunk=chunk, verify_pairs=pairs)
        _check(lib().swm_mapper_tuning(self._h, C.byref(t), None), "swm_mapper_tuning")

    def verify(self) -> str:
        t = Tuning()
        _check(lib().swm_mapper_tuning(self._h, None, C.byref(t)), "swm_mapper_tuning")
        for name, (head, chunk, pairs) in VERIFY_MODES.items():
            if chunk == t.verify_chunk and pairs == t.verify_pairs and (chunk or head == t.verify_head_bases):
                return name
        raise SwmError(f"unexpected tuning {t.verify_head_bases}/{t.verify_chunk}", -1)

    def launches(self) -> int:
        return int(lib().swm_mapper_launches(self._h))

    def stream(self) -> int:
        return int(lib().swm_mapper_stream(self._h) or 0)

    def debug_candidates(self):
        n = C.c_uint64()
        _check(lib().swm_mapper_debug_candidates(self._h, None, None, None, None, 0, C.byref(n)), "debug")
        k = n.value
        item = np.zeros(k, np.uint32)
        pos = np.zeros(k, np.uint32)
        err = np.zeros(k, np.int32)
        loc = np.zeros(k, np.int32)
        _check(lib().swm_mapper_debug_candidates(self._h, item.ctypes.data, pos.ctypes.data, err.ctypes.data,
                                                 loc.ctypes.data, k, C.byref(n)), "debug")
        return item, pos, err, loc

    def debug_read_words(self, nreads: int) -> np.ndarray:
        w = np.zeros((2 * nreads, 32), np.uint32)
        _check(lib().swm_mapper_debug_read_words(self._h, w.ctypes.data, 2 * nreads), "debug_read_words")
        return w

    def close(self) -> None:
        if self._h:
            lib().swm_mapper_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PackedBuffers:
    """Host buffers for packed results (swm_packed_result), reusable across blocks."""

    def __init__(self, nreads: int, words_per_read: int = 16, cigar_per_read: int = 64, records_per_read: int = 4):
        self.words = np.zeros(max(64, nreads * words_per_read), np.uint32)
        self.cigar = np.zeros(max(256, nreads * cigar_per_read), np.uint8)
        self.rlen = np.zeros(max(16, nreads * records_per_read), np.uint32)
        self.unmapped = np.zeros(max(1, nreads), np.uint32)
        self.c = PackedResult(self.words.ctypes.data, self.cigar.ctypes.data, self.rlen.ctypes.data,
                              self.unmapped.ctypes.data, self.words.size, self.cigar.size, self.rlen.size,
                              self.unmapped.size, 0, 0, 0, 0)

    def records(self):
        """Same canonical form as MapOutput.records()."""
        out = []
        w = self.words[:self.c.n_words]
        cg = self.cigar[:self.c.n_cigar]
        wp = cp = 0
        for q in range(self.c.n_records):
            n = int(w[wp + 1] & 0x0FFFFFFF)
            locs = tuple(int(x) for x in w[wp + 2:wp + 2 + n])
            ln = int(self.rlen[q])
            out.append((int(w[wp]), int(w[wp + 1]) >> 31, locs, bytes(cg[cp:cp + ln])))
            wp += 2 + n
            cp += ln
        return out



class Server:
    """Request loop over a resident index (swm_serve_*): continuous batching of
    requests into block slots, slots admitted by free device memory."""

    def __init__(self, index: Index, block_reads: int = 65536, max_slots: int = 4, stride: int = 256,
                 max_queued_reads: int | None = None, device_mem_limit: int = 0, device_mem_reserve: int = 1 << 30):
        self.index = index
        self.stride = stride
        cfg = ServeConfig(block_reads, max_slots, stride, max_queued_reads or 4 * block_reads * max_slots,
                          device_mem_limit, device_mem_reserve)
        h = C.c_void_p()
        _check(lib().swm_serve_open(index._h, C.byref(cfg), C.byref(h)), "swm_serve_open")
        self._h = h
        self.block_reads = block_reads

    def submit(self, reads: np.ndarray, lens: np.ndarray, errors: int, errors_per_read=None) -> int:
        """Admit one request; returns its id (raises SwmError with .rc on refusal)."""
        reads = np.ascontiguousarray(reads, np.uint8)
        lens = np.ascontiguousarray(lens, np.uint32)
        n, stride = reads.shape
        epr = None if errors_per_read is None else np.ascontiguousarray(errors_per_read, np.uint8)
        b = Batch(reads.ctypes.data, lens.ctypes.data, stride, n, errors, epr.ctypes.data if epr is not None else None)
        rid = C.c_uint64()
        _check(lib().swm_serve_submit(self._h, C.byref(b), C.byref(rid)), "swm_serve_submit")
        return int(rid.value)

    def poll(self, timeout_ms: int = -1, out: "PackedBuffers | None" = None, records: bool = True):
        """(id, records, info dict) of the next finished request, or None when
        none finished within timeout_ms; records=False leaves the records in
        the buffers (self.last) instead of decoding them."""
        rid = C.c_uint64()
        info = RequestInfo()
        if out is None:
            out = self._buf = getattr(self, "_buf", None) or PackedBuffers(self.block_reads)
        while True:
            rc = lib().swm_serve_poll(self._h, timeout_ms, C.byref(rid), C.byref(out.c), C.byref(info))
            if rc == -6:
                return None
            if rc == -5:   # grow the buffers to the sizes reported and take it again
                c = out.c
                out = PackedBuffers(self.block_reads, words_per_read=1 + int(c.n_words) // max(1, self.block_reads),
                                    cigar_per_read=1 + int(c.n_cigar) // max(1, self.block_reads),
                                    records_per_read=1 + int(c.n_records) // max(1, self.block_reads))
                self._buf = out
                continue
            _check(rc, "swm_serve_poll")
            self.last = out
            return int(rid.value), out.records() if records else None, {
                "reads": int(info.reads), "block_reads": int(info.block_reads), "latency_ms": float(info.latency_ms)}

    def stats(self) -> dict:
        s = ServeCounters()
        _check(lib().swm_serve_stats(self._h, C.byref(s)), "swm_serve_stats")
        return {f: int(getattr(s, f)) for f in SERVE_FIELDS}

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().swm_serve_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

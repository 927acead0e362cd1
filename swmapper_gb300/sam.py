"""SAM output and FASTA/FASTQ read blocks (swm_sam.h) from Python.

    refs = load_refs(prefix)                 # <prefix>.ref_info
    blk = ReadBlock(n_cap, seq_stride)       # fixed-stride reads for the mapper
    with FastxReader(path) as fx:
        while fx.read(blk):
            m.submit(blk.seqs_2d(), blk.lens(), e); m.wait_packed(buf)
            text = sam_block(refs, blk, buf)

The text is the reference's sam_header / sam_format_2 (mapper_mpe.c:315-687)
for the same records.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import PackedBuffers, PackedResult, SwmError, lib

_u32, _u64, _vp = C.c_uint32, C.c_uint64, C.c_void_p


class Refs(C.Structure):
    _fields_ = [("n", _u32), ("name", C.POINTER(C.c_char_p)), ("name_len", C.POINTER(_u32)),
                ("start", C.POINTER(_u32))]


class _Block(C.Structure):
    _fields_ = [("names", _vp), ("name_len", _vp), ("seqs", _vp), ("quals", _vp), ("seq_len", _vp),
                ("name_stride", _u64), ("seq_stride", _u64), ("n_cap", _u64), ("n", _u64), ("have_qual", C.c_int)]


_ready = False


def _lib():
    global _ready
    L = lib()
    if not _ready:
        L.swm_refs_load.argtypes = [C.c_char_p, C.POINTER(Refs)]
        L.swm_refs_free.argtypes = [C.POINTER(Refs)]
        L.swm_sam_header.argtypes = [C.POINTER(Refs), _vp, C.c_size_t, C.POINTER(C.c_size_t)]
        L.swm_sam_block.argtypes = [C.POINTER(Refs), C.POINTER(_Block), C.POINTER(PackedResult), _vp,
                                    C.c_size_t, C.POINTER(C.c_size_t)]
        L.swm_fastx_open.argtypes = [C.c_char_p, C.POINTER(_vp)]
        L.swm_fastx_read_block.argtypes = [_vp, C.POINTER(_Block)]
        L.swm_fastx_close.argtypes = [_vp]
        _ready = True
    return L


class RefSet:
    """Chromosomes of an index (owned by the library; freed with the object)."""

    def __init__(self, prefix: str):
        self.c = Refs()
        rc = _lib().swm_refs_load(prefix.encode(), C.byref(self.c))
        if rc != 0:
            raise SwmError(f"swm_refs_load({prefix}): status {rc}")

    def __del__(self):
        try:
            _lib().swm_refs_free(C.byref(self.c))
        except Exception:
            pass


def load_refs(prefix: str) -> RefSet:
    return RefSet(prefix)


class ReadBlock:
    """A block of reads in the mapper's fixed-stride layout."""

    def __init__(self, n_cap: int, seq_stride: int, name_stride: int = 128):
        self.names = np.zeros((n_cap, name_stride), np.uint8)
        self.name_len = np.zeros(n_cap, np.uint32)
        self.seqs = np.zeros((n_cap, seq_stride), np.uint8)
        self.quals = np.zeros((n_cap, seq_stride), np.uint8)
        self.seq_len = np.zeros(n_cap, np.uint32)
        self.c = _Block(self.names.ctypes.data, self.name_len.ctypes.data, self.seqs.ctypes.data,
                        self.quals.ctypes.data, self.seq_len.ctypes.data, name_stride, seq_stride, n_cap, 0, 0)

    @property
    def n(self) -> int:
        return int(self.c.n)

    def set(self, names, seqs, quals=None):
        """Fill from Python lists of bytes (for tests and small inputs)."""
        self.c.n = len(seqs)
        self.c.have_qual = 1 if quals is not None else 0
        for i, (nm, sq) in enumerate(zip(names, seqs)):
            self.names[i, :len(nm)] = np.frombuffer(nm, np.uint8)
            self.name_len[i] = len(nm)
            self.seqs[i, :len(sq)] = np.frombuffer(sq, np.uint8)
            self.seq_len[i] = len(sq)
            if quals is not None:
                self.quals[i, :len(sq)] = np.frombuffer(quals[i], np.uint8)


class FastxReader:
    """Blocks of reads from a FASTA / FASTQ file (swm_fastx_*)."""

    def __init__(self, path: str):
        self.h = _vp()
        rc = _lib().swm_fastx_open(path.encode(), C.byref(self.h))
        if rc != 0:
            raise SwmError(f"swm_fastx_open({path}): status {rc}")

    def read(self, blk: ReadBlock) -> int:
        rc = _lib().swm_fastx_read_block(self.h, C.byref(blk.c))
        if rc != 0:
            raise SwmError(f"swm_fastx_read_block: status {rc}")
        return blk.n

    def close(self):
        if self.h:
            _lib().swm_fastx_close(self.h)
            self.h = _vp()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _text(call) -> bytes:
    n = C.c_size_t(0)
    call(None, 0, C.byref(n))
    buf = C.create_string_buffer(max(1, n.value))
    rc = call(buf, n.value, C.byref(n))
    if rc != 0:
        raise SwmError(f"SAM writer: status {rc}")
    return buf.raw[:n.value]


def sam_header(refs: RefSet) -> bytes:
    return _text(lambda b, cap, n: _lib().swm_sam_header(C.byref(refs.c), b, cap, n))


def sam_block(refs: RefSet, blk: ReadBlock, res: PackedBuffers) -> bytes:
    return _text(lambda b, cap, n: _lib().swm_sam_block(C.byref(refs.c), C.byref(blk.c), C.byref(res.c), b, cap, n))

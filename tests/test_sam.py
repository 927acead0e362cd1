"""SAM writer and FASTA/FASTQ block reader of the library (host code, CPU):
the SAM text equals the reference's own sam_header / sam_format_2
(mapper_mpe.c:315-687, compiled here by oracle/build_ref.sh) on the same
records."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import build as obuild
from oracle import pyoracle as po
from swmapper_gb300 import PackedBuffers, synth
from tests.helpers import oracle_index

REF_SAM = os.path.join(obuild.REF_DIR, "libswref_sam.so")


@pytest.fixture(scope="module")
def swsam():
    from swmapper_gb300 import _build
    _build.build_cuda()
    from swmapper_gb300 import sam
    return sam


def _packed(res, nreads):
    """The oracle's strided records (reference layout) as packed results."""
    words, cig, rlen = [], [], []
    for r in range(res.ref_pos.shape[0]):
        rec = res.ref_pos[r]
        n = int(rec[1] & 0x0FFFFFFF)
        words.extend(int(x) for x in rec[:2 + n])
        c = res.cigar[r]
        p = 0
        for _ in range(n):
            p += 2 + int(c[p + 1])
        cig.extend(int(x) for x in c[:p])
        rlen.append(p)
    pk = PackedBuffers(nreads)
    pk.words[:len(words)] = words
    pk.cigar[:len(cig)] = cig
    pk.rlen[:len(rlen)] = rlen
    pk.unmapped[:res.unmapped.size] = res.unmapped
    pk.c.n_words, pk.c.n_cigar = len(words), len(cig)
    pk.c.n_records, pk.c.n_unmapped = res.ref_pos.shape[0], res.unmapped.size
    return pk


def _reference_sam(chroms, names, seqs, quals, lens, res, name_stride, stride):
    if not os.path.exists(REF_SAM):
        pytest.skip("reference SAM writer not built (no reference tree)")
    L = C.CDLL(REF_SAM)
    L.swref_sam.restype = C.c_size_t
    vp, u32, u64 = C.c_void_p, C.c_uint32, C.c_uint64
    L.swref_sam.argtypes = [u32, vp, vp, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, u64, u64, u64, u32, u32, vp,
                            C.c_size_t]
    clen = np.array([c[1] for c in chroms], np.uint32)
    cname = np.zeros((len(chroms), 25), np.uint8)
    cnl = np.array([len(c[0]) for c in chroms], np.uint32)
    for i, (nm, _) in enumerate(chroms):
        cname[i, :len(nm)] = np.frombuffer(nm, np.uint8)
    n = len(seqs)
    rn = np.zeros((n, name_stride), np.uint8)
    rs = np.zeros((n, stride), np.uint8)
    rq = np.zeros((n, stride), np.uint8)
    for i in range(n):
        rn[i, :len(names[i])] = np.frombuffer(names[i], np.uint8)
        rs[i, :len(seqs[i])] = np.frombuffer(seqs[i], np.uint8)
        rq[i, :len(quals[i])] = np.frombuffer(quals[i], np.uint8)
    rnl = np.array([len(x) for x in names], np.uint32)
    ref_pos = np.ascontiguousarray(res.ref_pos)
    cigar = np.ascontiguousarray(res.cigar)
    unm = np.ascontiguousarray(res.unmapped.astype(np.uint32))
    out = np.zeros(64 << 20, np.uint8)
    m = L.swref_sam(len(chroms), clen.ctypes.data, cname.ctypes.data, 25, cnl.ctypes.data, rn.ctypes.data,
                    rs.ctypes.data, rq.ctypes.data, cigar.ctypes.data, ref_pos.ctypes.data, rnl.ctypes.data,
                    lens.ctypes.data, unm.ctypes.data, unm.size, ref_pos.shape[0], n, name_stride, stride,
                    out.ctypes.data, out.size)
    assert m <= out.size
    return out[:m].tobytes()


def test_sam_equals_reference_sam_format(swsam, tmp_path):
    g = synth.reference(600_000, seed=41, kind="repeats100m")
    chroms = [(b"chr1", 250_000), (b"chrX_random", 200_000), (b"c3", 150_000)]
    prefix = str(tmp_path / "ix")
    with open(prefix + ".ref_info", "wb") as f:
        for nm, ln in chroms:
            f.write(b"%d\n%d\n%s\n" % (ln, len(nm), nm))
    _, mix = oracle_index(g)
    reads, lens, _, _ = synth.reads(g, 1500, 60, 200, 0.03, seed=42)
    res = po.map_reads(mix, reads, lens, 7, nthreads=4)
    assert res.unmapped.size > 0 and res.ref_pos.shape[0] > 0
    rng = np.random.default_rng(5)
    names = [b"read%05d/1" % i for i in range(reads.shape[0])]
    seqs = [reads[i, :lens[i]].tobytes() for i in range(reads.shape[0])]
    quals = [rng.integers(33, 75, int(lens[i]), dtype=np.uint8).tobytes() for i in range(reads.shape[0])]
    want = _reference_sam(chroms, names, seqs, quals, lens, res, 20, reads.shape[1])
    refs = swsam.load_refs(prefix)
    blk = swsam.ReadBlock(reads.shape[0], reads.shape[1], name_stride=20)
    blk.set(names, seqs, quals)
    got = swsam.sam_header(refs) + swsam.sam_block(refs, blk, _packed(res, reads.shape[0]))
    assert got.count(b"\n") == want.count(b"\n")
    assert got == want
    lines = got.split(b"\n")
    assert any(l.split(b"\t")[1] == b"16" for l in lines if l and not l.startswith(b"@"))
    assert any(l.split(b"\t")[2] == b"chrX_random" for l in lines if l and not l.startswith(b"@"))


def test_fastx_reader_fastq_and_fasta(swsam, tmp_path):
    fq = tmp_path / "r.fq"
    fq.write_bytes(b"@a1 comment\nACGTN\n+\nIIIII\n@b2\nACG\nTTA\n+b2\nII@\nIII\n\n@c\n\n+\n\n")
    blk = swsam.ReadBlock(8, 16, name_stride=8)
    with swsam.FastxReader(str(fq)) as fx:
        assert fx.read(blk) == 3
        assert blk.c.have_qual == 1
        assert [blk.names[i, :blk.name_len[i]].tobytes() for i in range(3)] == [b"a1", b"b2", b"c"]
        assert [blk.seqs[i, :blk.seq_len[i]].tobytes() for i in range(3)] == [b"ACGTN", b"ACGTTA", b""]
        assert blk.quals[1, :6].tobytes() == b"II@III"
        assert fx.read(blk) == 0
    fa = tmp_path / "r.fa"
    fa.write_bytes(b">x one\nACGT\nAC\n>y\nGG\n")
    blk2 = swsam.ReadBlock(1, 16)
    with swsam.FastxReader(str(fa)) as fx:
        assert fx.read(blk2) == 1
        assert blk2.seqs[0, :blk2.seq_len[0]].tobytes() == b"ACGTAC"
        assert blk2.c.have_qual == 0
        assert fx.read(blk2) == 1
        assert blk2.names[0, :blk2.name_len[0]].tobytes() == b"y"
        assert fx.read(blk2) == 0
    long = tmp_path / "long.fa"
    long.write_bytes(b">z\n" + b"A" * 40 + b"\n")
    with swsam.FastxReader(str(long)) as fx:
        with pytest.raises(Exception):
            fx.read(swsam.ReadBlock(1, 16))

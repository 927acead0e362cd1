"""Error paths through the public C ABI (gpu).

The reference has no error returns: its functions are void, a failed malloc
only prints (mapper_mpe.c:142-148) and a missing reads file aborts
(mapper_mpe.c:185-188). Here each failure is a status code and the handles
stay usable afterwards. None of these tests makes the device fault: every
failure is detected by a size check on the host or by a device counter that
the host reads.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po
from swmapper_gb300 import synth
from tests.helpers import first_diff, genome, oracle_index

pytestmark = pytest.mark.gpu

SWM_ERR_IO = -2
SWM_ERR_OVERFLOW = -5


def test_counts_that_do_not_add_up(cuda_lib, tmp_path):
    """.hash_count whose sum differs from the number of positions (sizes all
    consistent): SWM_ERR_IO once the counts have been read."""
    g = genome(60_000, 5)
    hix = po.build_index(g, 12)
    prefix = str(tmp_path / "ix")
    files = hix.files()
    cnt = hix.hash_count.copy()
    cnt[int(np.argmax(cnt))] += 1
    files[".hash_count"] = cnt.tobytes()
    for ext, data in files.items():
        with open(prefix + ext, "wb") as f:
            f.write(data)
    L = cuda_lib.lib()
    h = C.c_void_p()
    assert L.swm_index_open(prefix.encode(), 12, 0, C.byref(h)) == SWM_ERR_IO
    assert b"adds up to" in L.swm_last_error()


def test_open_equals_build(cuda_lib, tmp_path):
    """The chunked loader gives the arrays of the index that wrote the files
    (files larger than one 32 MiB load chunk: 4^12 counts = 64 MiB)."""
    g = genome(3_000_000, 6, "human", nrun_min=2000, nrun_max=20000, copies_per_family=300)
    ix = cuda_lib.Index.build(g)
    prefix = str(tmp_path / "ix")
    ix.save(prefix, b"3000000\n4\nchrS\n")
    got = cuda_lib.Index.open(prefix).download()
    want = ix.download()
    for key in want:
        assert np.array_equal(got[key], want[key]), key
    assert cuda_lib.Index.open(prefix).info().n == 3_000_000


def _result(nrec, nreads):
    ref_pos = np.zeros((max(1, nrec), cuda_lib_record_words()), np.uint32)
    cig = np.zeros((max(1, nrec), 4096), np.uint8)
    unm = np.zeros(max(1, nreads), np.uint32)
    return ref_pos, cig, unm


def cuda_lib_record_words():
    import swmapper_gb300 as swm
    return swm.RECORD_WORDS


def test_small_result_buffer_reports_overflow_and_the_count(cuda_lib):
    """records_cap below the block's record count: SWM_ERR_OVERFLOW, the
    records that fit are written, n_records holds the count needed."""
    g = genome(1_000_000, 7, "repeats100m")
    reads, lens, _, _ = synth.reads(g, 500, 150, 150, 0.03, seed=8)
    ix = cuda_lib.Index.build(g)
    m = cuda_lib.Mapper(ix, max_reads=500)
    full = m.map(reads, lens, 7)
    need = full.ref_pos.shape[0]
    assert need > 20
    L = cuda_lib.lib()
    ref_pos, cig, unm = _result(20, 500)
    b = cuda_lib.Batch(reads.ctypes.data, lens.ctypes.data, reads.shape[1], 500, 7, None)
    r = cuda_lib.Result(ref_pos.ctypes.data, cig.ctypes.data, unm.ctypes.data, 20, unm.size, 0, 0)
    assert L.swm_map_batch(m._h, C.byref(b), C.byref(r)) == SWM_ERR_OVERFLOW
    assert r.n_records == need
    assert np.array_equal(ref_pos[:20], full.ref_pos[:20])
    # unmapped list too small as well
    ref_pos2, cig2, _ = _result(need, 500)
    unm1 = np.zeros(1, np.uint32)
    r2 = cuda_lib.Result(ref_pos2.ctypes.data, cig2.ctypes.data, unm1.ctypes.data, need, 0, 0, 0)
    assert L.swm_map_batch(m._h, C.byref(b), C.byref(r2)) == SWM_ERR_OVERFLOW
    assert r2.n_unmapped == full.unmapped.size
    # the mapper is still usable
    assert m.map(reads, lens, 7).records() == full.records()


def test_small_packed_buffers_report_overflow(cuda_lib):
    g = genome(1_000_000, 9, "repeats100m")
    reads, lens, _, _ = synth.reads(g, 400, 150, 150, 0.03, seed=10)
    ix = cuda_lib.Index.build(g)
    m = cuda_lib.Mapper(ix, max_reads=400)
    buf = cuda_lib.PackedBuffers(400, words_per_read=1, cigar_per_read=1, records_per_read=1)
    m.submit(reads, lens, 7)
    with pytest.raises(cuda_lib.SwmError, match=r"\(-5\)"):
        m.wait_packed(buf)
    big = cuda_lib.PackedBuffers(400)
    m.submit(reads, lens, 7)
    m.wait_packed(big)
    assert big.records() == m.map(reads, lens, 7).records()


def test_buffer_growth_retry_gives_oracle_records(cuda_lib):
    """A mapper sized for 16 reads on a genome of close repeat copies (items
    fetch thousands of positions): the first pass outgrows its work buffers,
    the host grows them and re-runs the block, and the records equal the
    oracle's."""
    g = genome(3_000_000, 11, "human", copies_per_family=1000, div_min=0.005, div_max=0.03, repeat_frac=0.6,
               rep_len_max=3000)
    reads, lens, _, _ = synth.reads(g, 16, 150, 150, 0.03, seed=12)
    _, mix = oracle_index(g)
    ref = po.map_reads(mix, reads, lens, 7, nthreads=8)
    ix = cuda_lib.Index.build(g)
    m = cuda_lib.Mapper(ix, max_reads=16)
    out = m.map(reads, lens, 7)
    assert m.stats()["retries"] > 0
    d = first_diff(out.records(), ref.records())
    assert d is None, d
    assert [int(x) for x in out.unmapped] == [int(x) for x in ref.unmapped]
    # the grown buffers serve the next block without another retry
    out2 = m.map(reads, lens, 7)
    assert m.stats()["retries"] == 0 and out2.records() == out.records()


def test_block_totals_past_32_bits_are_an_error(cuda_lib):
    """A genome that repeats ACGT: every sampled 12-mer falls in one bucket of
    2.5 M positions, and every long seed of a read from it selects that
    bucket. 64 reads of 250 bp at e = 15 (16 long seeds per strand) ask for
    64 x 2 x 16 x 2.5 M = 5.1 G fetched positions in one block, past the
    32-bit offsets of the work buffers: the block is refused with
    SWM_ERR_OVERFLOW instead of wrapping, and the mapper stays usable."""
    n = 10_000_000
    g = np.frombuffer(b"ACGT" * (n // 4), np.uint8).copy()
    ix = cuda_lib.Index.build(g)
    assert ix.download()["hash_count"].max() == (n - 12) // 4 + 1
    reads = np.tile(g[:250], (64, 1))
    lens = np.full(64, 250, np.uint32)
    m = cuda_lib.Mapper(ix, max_reads=64)
    with pytest.raises(cuda_lib.SwmError, match=r"\(-5\).*2\^32"):
        m.map(reads, lens, 15)
    rng = np.random.default_rng(13)
    rnd = rng.choice(np.frombuffer(b"ACGT", np.uint8), size=(8, 150))
    out = m.map(rnd, np.full(8, 150, np.uint32), 5)
    assert out.unmapped.size == 8

"""GPU index build against the oracle and the reference's own files (gpu)."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from tests.helpers import genome

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_outputs.json")))


def _same_as_oracle(swm, g, k=12):
    ix = swm.Index.build(g, k=k)
    got = ix.download()
    want = po.build_index(g, k)
    assert np.array_equal(got["hash_count"], want.hash_count)
    assert np.array_equal(got["hash_offset"], want.hash_offset_end)
    assert np.array_equal(got["positions"], want.positions)
    assert np.array_equal(got["pos_lseeds"], want.pos_lseeds)
    assert np.array_equal(got["base_2bits"], want.base_2bits)
    assert np.array_equal(got["base_3bits"], want.base_3bits)
    return ix


@pytest.mark.parametrize("n,kind,nruns", [(65536, "uniform", []), (1_000_003, "uniform", [(5, 70), (999_000, 999_100)]),
                                          (2_000_000, "repeats100m", [(100, 1100)]), (31, "uniform", []),
                                          (12, "uniform", []), (11, "uniform", [])])
def test_gpu_index_equals_oracle(cuda_lib, n, kind, nruns):
    over = {"copies_per_family": 40, "rep_len_max": 3000} if kind == "repeats100m" else {}
    _same_as_oracle(cuda_lib, genome(n, 3, kind, nruns, **over))


def test_gpu_index_large_buckets(cuda_lib):
    """Poly-A and a tandem repeat give buckets far above the shared-memory sort size."""
    g = genome(600_000, 4)
    g[10_000:60_000] = ord("A")
    unit = np.frombuffer(b"ACGTTGCAGGCA", np.uint8)
    g[100_000:100_000 + 36_000] = np.tile(unit, 3000)
    g[300_000:300_020] = ord("a")
    _same_as_oracle(cuda_lib, g)


@pytest.mark.parametrize("k", [8, 10, 13])
def test_gpu_index_other_k(cuda_lib, k):
    _same_as_oracle(cuda_lib, genome(200_003, 5, "repeats100m", copies_per_family=10, rep_len_max=2000), k=k)


@pytest.mark.parametrize("case", GOLD["cases"]["index"], ids=lambda c: c[0])
def test_gpu_fasta_build_equals_reference_files(cuda_lib, case, tmp_path):
    from tests.test_oracle_golden import _fasta, _genome
    name, n, seed, kind, over, nruns, splits = case
    g = _genome(n, seed, kind, over, nruns, lower=(name == "lower_iupac"))
    fa = str(tmp_path / "x.fa")
    _fasta(fa, g, splits)
    prefix = str(tmp_path / "idx")
    cuda_lib.Index.build_fasta(fa, prefix)
    for ext in po.FILE_EXTS:
        with open(prefix + ext, "rb") as f:
            assert hashlib.sha256(f.read()).hexdigest() == GOLD["index"][name][ext], ext


def test_gpu_index_save_open_roundtrip(cuda_lib, tmp_path):
    g = genome(300_001, 6, "repeats100m", copies_per_family=20, rep_len_max=2000)
    ix = cuda_lib.Index.build(g)
    prefix = str(tmp_path / "rt")
    ix.save(prefix, b"300001\n3\nchr\n")
    ix2 = cuda_lib.Index.open(prefix)
    a, b = ix.download(), ix2.download()
    for key in a:
        assert np.array_equal(a[key], b[key]), key
    assert ix2.info().n == 300001
    assert ix2.info().ref_length == ix.info().ref_length

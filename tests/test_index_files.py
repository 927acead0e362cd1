"""Index files that are missing or cut short are rejected with SWM_ERR_IO
before any device work (CPU: swm_index_open checks every file's size first).

The reference's load_ref_info freads whatever is there (mapper_mpe.c:198-314)
and the mapper aborts only when the reads file is missing
(mapper_mpe.c:185-188); here every such case is a status code.
"""
import ctypes as C
import os

import numpy as np
import pytest

from tests.helpers import genome

SWM_ERR_IO = -2
SWM_ERR_ARG = -1


@pytest.fixture(scope="module")
def lib():
    from swmapper_gb300 import _build
    _build.build_cuda()
    import swmapper_gb300 as swm
    return swm.lib()


@pytest.fixture()
def index_files(tmp_path):
    from oracle import pyoracle as po
    g = genome(50_000, 3)
    hix = po.build_index(g, 12)
    prefix = str(tmp_path / "ix")
    for ext, data in hix.files().items():
        with open(prefix + ext, "wb") as f:
            f.write(data)
    with open(prefix + ".ref_info", "wb") as f:
        f.write(b"50000\n4\nchrS\n")
    return prefix


def _open(lib, prefix, k=12):
    h = C.c_void_p()
    rc = lib.swm_index_open(prefix.encode(), k, 0, C.byref(h))
    return rc, lib.swm_last_error().decode()


@pytest.mark.parametrize("ext", [".hash_count", ".positions", ".pos_lseeds", ".base_2bits", ".base_3bits"])
def test_missing_index_file(lib, index_files, ext):
    os.remove(index_files + ext)
    rc, msg = _open(lib, index_files)
    assert rc == SWM_ERR_IO
    assert ext in msg and "missing" in msg


@pytest.mark.parametrize("ext,cut", [(".hash_count", 4), (".positions", 4), (".positions", 1),
                                     (".pos_lseeds", 2), (".base_2bits", 8), (".base_3bits", 4)])
def test_truncated_index_file(lib, index_files, ext, cut):
    path = index_files + ext
    size = os.path.getsize(path)
    with open(path, "r+b") as f:
        f.truncate(size - cut)
    rc, msg = _open(lib, index_files)
    assert rc == SWM_ERR_IO
    assert "inconsistent sizes" in msg


def test_wrong_k_for_the_files(lib, index_files):
    rc, msg = _open(lib, index_files, k=11)
    assert rc == SWM_ERR_IO and "k=11" in msg


def test_bad_arguments(lib):
    rc, _ = _open(lib, "/nonexistent/prefix", k=0)
    assert rc == SWM_ERR_ARG
    rc, _ = _open(lib, "/nonexistent/prefix", k=15)
    assert rc == SWM_ERR_ARG
    h = C.c_void_p()
    assert lib.swm_index_open(None, 12, 0, C.byref(h)) == SWM_ERR_ARG
    # entry points that take a handle reject a null one before any device work
    assert lib.swm_index_serialize_mappers(None, 1) == SWM_ERR_ARG
    assert lib.swm_index_candidate_table(None, -1, None) == SWM_ERR_ARG
    assert lib.swm_mapper_tuning(None, None, None) == SWM_ERR_ARG


def test_oracle_files_are_consistent(index_files):
    """The fixture's files satisfy every size rule the loader checks (so the
    failures above come from the damage alone)."""
    sz = {e: os.path.getsize(index_files + e) for e in (".hash_count", ".positions", ".pos_lseeds",
                                                        ".base_2bits", ".base_3bits")}
    S = sz[".positions"] // 4
    assert sz[".hash_count"] == 4 << 24
    assert sz[".pos_lseeds"] == 2 * S and sz[".base_2bits"] == 2 * sz[".base_3bits"]
    counts = np.fromfile(index_files + ".hash_count", np.uint32)
    assert int(counts.sum(dtype=np.uint64)) == S

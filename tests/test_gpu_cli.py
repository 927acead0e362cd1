"""The command-line drop-ins on the GPU (gpu): swm_index writes the same seven
files as the reference's serial_index, and swm_mapper writes the SAM the
reference's own sam_format_2 prints for the oracle's records of the same
reads (mapper_mpe.c:697-1125)."""
import gzip
import os
import subprocess

import numpy as np
import pytest

from oracle import pyoracle as po
from swmapper_gb300 import _build, synth
from tests.test_sam import _reference_sam

pytestmark = pytest.mark.gpu


def _write_fasta(path, chroms):
    with open(path, "wb") as f:
        for nm, seq in chroms:
            f.write(b">" + nm + b" test chromosome\n")
            for i in range(0, seq.size, 70):
                f.write(seq[i:i + 70].tobytes() + b"\n")


@pytest.fixture(scope="module")
def cli(cuda_lib):
    _build.build_cli()
    assert os.path.exists(_build.BIN_INDEX) and os.path.exists(_build.BIN_MAP)
    return _build.BIN_INDEX, _build.BIN_MAP


def test_cli_index_and_map_equal_reference(cli, tmp_path):
    bin_index, bin_map = cli
    g = synth.reference(900_000, seed=51, kind="repeats100m")
    chroms = [(b"chr1", g[:500_000]), (b"chr2", g[500_000:])]
    fa = str(tmp_path / "ref.fa")
    _write_fasta(fa, chroms)
    prefix = str(tmp_path / "ix")
    subprocess.run([bin_index, "-i", fa, "-p", prefix, "-s12"], check=True, capture_output=True)
    if po.have_ref():  # byte-identical index files
        want = po.ref_index_files(fa, str(tmp_path / "refix"))
        for ext, data in want.items():
            assert open(prefix + ext, "rb").read() == data, ext
    # reads as FASTQ, mapped by the CLI in blocks of 1,000
    reads, lens, _, _ = synth.reads(g, 2500, 80, 150, 0.03, seed=52)
    rng = np.random.default_rng(9)
    names = [b"r%05d" % i for i in range(reads.shape[0])]
    seqs = [reads[i, :lens[i]].tobytes() for i in range(reads.shape[0])]
    quals = [rng.integers(33, 75, int(lens[i]), dtype=np.uint8).tobytes() for i in range(reads.shape[0])]
    fq = str(tmp_path / "reads.fq")
    with open(fq, "wb") as f:
        for nm, sq, qu in zip(names, seqs, quals):
            f.write(b"@" + nm + b"\n" + sq + b"\n+\n" + qu + b"\n")
    out = str(tmp_path / "out")
    env = dict(os.environ, SWM_BLOCK_READS="1000")
    subprocess.run([bin_map, "-l150", "-e", "7", "-p", prefix, "-i" + fq, "-o" + out], check=True,
                   capture_output=True, env=env)
    path = out + ".sam.gz" if os.path.exists(out + ".sam.gz") else out + ".sam"
    got = gzip.open(path).read() if path.endswith(".gz") else open(path, "rb").read()
    # the reference's SAM of the oracle's records, block by block
    hix = po.build_index(g, 12)
    mix = po.MapIndex(hix)
    ref_chroms = [(nm, s.size) for nm, s in chroms]
    want = b""
    for b0 in range(0, reads.shape[0], 1000):
        sl = slice(b0, b0 + 1000)
        res = po.map_reads(mix, reads[sl], lens[sl], 7, nthreads=4)
        text = _reference_sam(ref_chroms, names[sl], seqs[sl], quals[sl], lens[sl], res, 20, reads.shape[1])
        want += text if b0 == 0 else text[text.index(b'CL:"CMDLINE"\n') + len(b'CL:"CMDLINE"\n'):]
    assert got.count(b"\n") == want.count(b"\n")
    assert got == want


def test_cli_help_exits_zero(cli):
    for b in cli:
        r = subprocess.run([b, "-h"], capture_output=True, text=True)
        assert r.returncode == 0 and "-p" in r.stdout

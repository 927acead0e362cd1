"""Block plans of the autotuner (host logic, no GPU)."""
import numpy as np

from swmapper_gb300 import tune


def _buckets(sizes, forms):
    out, first = [], 0
    for n, f in zip(sizes, forms):
        out.append({"first": first, "reads": n, "verify": f})
        first += n
    return out


def test_merged_plan_covers_every_read_once_in_order():
    bk = _buckets([148_982, 318_117, 318_059, 400_000], ["stream8", "head32", "head32", "head64"])
    n = sum(b["reads"] for b in bk)
    plan = tune.merged_plan(bk, n, 524_288)
    assert [b0 for b0, _, _ in plan] == list(range(0, n, 524_288))
    assert sum(nb for _, nb, _ in plan) == n
    assert all(nb <= 524_288 for _, nb, _ in plan)


def test_merged_plan_takes_the_form_of_the_largest_share():
    bk = _buckets([100, 300, 50], ["head64", "stream16", "head32"])
    # block 0 = reads 0..255: 100 of head64, 156 of stream16 -> stream16
    # block 1 = reads 256..449: 144 of stream16, 50 of head32 -> stream16
    assert tune.merged_plan(bk, 450, 256) == [(0, 256, "stream16"), (256, 194, "stream16")]
    # two buckets with the same form add up against a larger third one
    bk = _buckets([60, 50, 60], ["head32", "pair16", "head32"])
    assert tune.merged_plan(bk, 170, 170) == [(0, 170, "head32")]


def test_length_buckets_partition_reads_by_32bp():
    lens = np.array([50, 64, 65, 250, 96, 97, 33, 32], np.uint32)
    got = {b: sorted(ix.tolist()) for b, ix in tune.length_buckets(lens)}
    assert got == {0: [7], 1: [0, 1, 6], 2: [2, 4], 3: [5], 7: [3]}

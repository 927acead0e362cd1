"""The single-batch rule the GPU refill planner relies on (CPU, against the oracle).

The planner skips the seed heap of alignment_rmdup (mapper_cpe.c:2194-2419)
for an item whose selected buckets hold at most 2048 - 32 + 1 = 2017
positions: refills continue while npos + 32 <= 2048 and 1 + 2 runs < 256,
both only grow, so such an item is refilled until its heap is empty and forms
one batch of every chunk, whatever order the heap takes the refills in. This
checks that claim item by item on the oracle, which follows the reference's
schedule, on a repeat-rich genome where many items need refills.
"""
import numpy as np

from oracle import pyoracle as po
from swmapper_gb300 import synth
from tests.helpers import genome, oracle_index

LIMIT = 2048 - 32 + 1


def _items(n_reads, e):
    # many close copies: buckets of tens to hundreds of positions, items on
    # both sides of the limit
    g = genome(3_000_000, 7, "human", copies_per_family=1000, div_min=0.005, div_max=0.03, repeat_frac=0.6,
               rep_len_max=3000)
    reads, lens, _, _ = synth.reads(g, n_reads, 150, 150, 0.03, seed=21)
    _, mix = oracle_index(g)
    for r in range(n_reads):
        s = bytes(reads[r, :lens[r]])
        for strand in (0, 1):
            seq = s if strand == 0 else s[::-1].translate(bytes.maketrans(b"ACGT", b"TGCA"))
            yield po.trace_item(mix, seq, e)


def test_items_within_the_limit_form_one_batch():
    refilled_single = refilled_multi = 0
    near = 0
    for e in (7, 12):
        for tr in _items(600, e):
            cnt = tr["sel_count"].astype(np.int64)
            nel = int(cnt.sum())
            refills = bool((cnt > 32).any())
            if nel == 0:
                continue
            if not refills or nel <= LIMIT:
                assert tr["nbatches"] == 1, (e, nel, refills, tr["nbatches"])
                refilled_single += refills
                near = max(near, nel if refills else 0)
            else:
                refilled_multi += tr["nbatches"] > 1
    # the workload exercises both sides of the rule, and items close to it
    assert refilled_single > 50
    assert refilled_multi > 50
    assert near > 1900

"""Autotuner for the batched form: reads per block, mappers, length buckets
and, per 32-bp length bucket, the form of the verification stage and the
block size.

Verification runs the lanes of a warp over their candidates' read lengths,
so reads of very different lengths side by side waste lanes. The autotuner

* groups reads into length buckets of 32 bp (`length_buckets`), so a block
  holds reads of similar length,
* times a sample of resident reads under every (reads per block, mappers)
  candidate and keeps the fastest (`tune`), with an optional cache key
  (for example GPU, k, length bucket, e), and
* for each length bucket, times that bucket's reads under every
  (verification form, reads per block) pair and keeps the fastest
  (`tune_buckets`), then times that per-bucket plan against the
  length-sorted reads cut into blocks of the globally tuned size, each
  block with its main bucket's form (`merged_plan`, `tune_plan`): small
  buckets in blocks of their own pay each block's fixed cost more often.
  The forms: a first pass over 64 or 32 bases of every candidate with an
  exact stop test, then the rest ("head64", "head32"), or
  lanes that each run their own candidate and test a stop bound every 8 or
  16 bases, taking the next candidate as soon as theirs stops ("stream8",
  "stream16"), or two such candidates per lane when every threshold is <= 7
  ("pair16"). Which is faster depends on how early the candidates of that
  read length can be ruled out, against the per-chunk cost of the test.

Results do not depend on any choice: every read maps the same in any block
and under every form.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

BUCKET_BP = 32
BLOCKS = (65536, 131072, 262144, 524288)
MAPPERS = (1, 2, 3)
VERIFY = ("head64", "head32", "stream8", "stream16", "pair16")  # forms of the verification stage
BUCKET_BLOCKS = (131072, 524288)  # reads per block tried for each length bucket

_cache: dict = {}


def length_buckets(lens: np.ndarray, bucket_bp: int = BUCKET_BP) -> list[tuple[int, np.ndarray]]:
    """(bucket, read indices in input order) for every non-empty 32-bp length bucket."""
    b = (lens.astype(np.int64) - 1) // bucket_bp
    order = np.argsort(b, kind="stable")
    keys = b[order]
    out = []
    if order.size:
        cuts = np.flatnonzero(np.diff(keys)) + 1
        for part in np.split(order, cuts):
            out.append((int(b[part[0]]), part))
    return out


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            rt = C.CDLL(name)
            rt.cudaDeviceSynchronize.argtypes = []
            return rt
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


def run_blocks(mappers, d_reads: int, d_lens: int, stride: int, nreads: int, e: int, d_e: int | None, block: int,
               on_done=None, verify: str | None = None):
    """Map nreads device-resident reads in blocks taken by the mappers in turn
    (swm_map_device_submit / swm_map_device_wait); on_done(mapper) after each.
    verify: form of the verification stage for every block (None: keep)."""
    pend = []
    for i, b0 in enumerate(range(0, nreads, block)):
        nb = min(block, nreads - b0)
        if len(pend) == len(mappers):
            pm = pend.pop(0)
            pm.wait_device()
            if on_done:
                on_done(pm)
        m = mappers[i % len(mappers)]
        if verify is not None:
            m.set_verify(verify)
        m.submit_device(d_reads + b0 * stride, d_lens + b0 * 4, stride, nb, e,
                        None if d_e is None else d_e + b0)
        pend.append(m)
    while pend:
        pm = pend.pop(0)
        pm.wait_device()
        if on_done:
            on_done(pm)


def run_plan(mappers, d_reads: int, d_lens: int, stride: int, e: int, d_e: int | None, plan) -> None:
    """Map the blocks of plan -- (first read, reads, verification form) each --
    with the mappers in turn (swm_map_device_submit / swm_map_device_wait)."""
    pend = []
    for i, (b0, nb, form) in enumerate(plan):
        if len(pend) == len(mappers):
            pend.pop(0).wait_device()
        m = mappers[i % len(mappers)]
        m.set_verify(form)
        m.submit_device(d_reads + b0 * stride, d_lens + b0 * 4, stride, nb, e, None if d_e is None else d_e + b0)
        pend.append(m)
    while pend:
        pend.pop(0).wait_device()


def merged_plan(buckets: list[dict], nreads: int, block: int) -> list[tuple[int, int, str]]:
    """The length-sorted reads in blocks of `block` reads across bucket
    boundaries, each block with the form its largest share of reads' bucket
    chose: fewer, fuller blocks than one set per bucket, with the reads of a
    block still of similar length."""
    plan = []
    for b0 in range(0, nreads, block):
        nb = min(block, nreads - b0)
        share = {}
        for bk in buckets:
            ov = min(b0 + nb, bk["first"] + bk["reads"]) - max(b0, bk["first"])
            if ov > 0:
                share[bk["verify"]] = share.get(bk["verify"], 0) + ov
        plan.append((b0, nb, max(share, key=share.get) if share else "stream16"))
    return plan


def tune_plan(index, d_reads: int, d_lens: int, stride: int, e: int, d_e: int | None, plans: dict,
              nmappers: int) -> tuple[str, dict]:
    """The fastest of the named block plans over all the reads (a warm-up
    pass, then a timed one each); returns its name and every plan's rate."""
    import swmapper_gb300 as swm
    rt = _cudart()
    rates = {}
    for name, plan in plans.items():
        ms = [swm.Mapper(index, max_reads=max(nb for _, nb, _ in plan)) for _ in range(nmappers)]
        run_plan(ms, d_reads, d_lens, stride, e, d_e, plan)
        rt.cudaDeviceSynchronize()
        t0 = time.perf_counter()
        run_plan(ms, d_reads, d_lens, stride, e, d_e, plan)
        rt.cudaDeviceSynchronize()
        rates[name] = round(sum(nb for _, nb, _ in plan) / (time.perf_counter() - t0), 1)
        del ms
    return max(rates, key=rates.get), rates


def tune(index, d_reads: int, d_lens: int, stride: int, nreads: int, e: int, d_e: int | None = None,
         key=None, blocks=BLOCKS, mappers=MAPPERS, min_sample: int = 1 << 20) -> dict:
    """Fastest (reads per block, mappers) for these device-resident reads, timed
    on at least min_sample reads, so every mapper gets blocks (two passes, the
    second timed)."""
    import swmapper_gb300 as swm
    if key is not None and key in _cache:
        return _cache[key]
    rt = _cudart()
    best = None
    trials = []
    for nm in mappers:
        for blk in blocks:
            n = min(nreads, max(min_sample, 2 * nm * blk))
            if blk > n and blk != blocks[0]:
                continue
            ms = [swm.Mapper(index, max_reads=min(blk, n)) for _ in range(nm)]
            run_blocks(ms, d_reads, d_lens, stride, n, e, d_e, min(blk, n))  # warm-up (graphs, buffers)
            rt.cudaDeviceSynchronize()
            t0 = time.perf_counter()
            run_blocks(ms, d_reads, d_lens, stride, n, e, d_e, min(blk, n))
            rt.cudaDeviceSynchronize()
            rate = n / (time.perf_counter() - t0)
            del ms
            trials.append({"block": blk, "mappers": nm, "reads_per_s": round(rate, 1)})
            if best is None or rate > best["reads_per_s"]:
                best = trials[-1]
    res = {"block": best["block"], "mappers": best["mappers"], "trials": trials}
    if key is not None:
        _cache[key] = res
    return res


def tune_buckets(index, d_reads: int, d_lens: int, stride: int, lens: np.ndarray, e: int, d_e: int | None,
                 nmappers: int, forms=VERIFY, blocks=BUCKET_BLOCKS, sample: int = 524288) -> list[dict]:
    """For every 32-bp length bucket of device-resident reads already grouped
    by bucket (contiguous, in `length_buckets` order), the fastest
    (verification form, block) pair, timed on up to `sample` reads of the bucket with nmappers
    mappers (a warm-up pass, then a timed one)."""
    import swmapper_gb300 as swm
    rt = _cudart()
    out = []
    b0 = 0
    for bucket, idx in length_buckets(lens):
        n_b = idx.size
        n = min(n_b, sample)
        o = b0 + (n_b - n) // 2  # a window from the middle of the bucket
        trials = []
        for blk in blocks:
            bs = min(blk, n)
            if blk != blocks[0] and blk > n:
                continue
            ms = [swm.Mapper(index, max_reads=bs) for _ in range(nmappers)]
            for vf in forms:
                args = (d_reads + o * stride, d_lens + o * 4, stride, n, e, None if d_e is None else d_e + o, bs)
                run_blocks(ms, *args, verify=vf)
                rt.cudaDeviceSynchronize()
                t0 = time.perf_counter()
                run_blocks(ms, *args, verify=vf)
                rt.cudaDeviceSynchronize()
                trials.append({"verify": vf, "block": blk, "reads_per_s": round(n / (time.perf_counter() - t0), 1)})
            del ms
        best = max(trials, key=lambda t: t["reads_per_s"])
        lo = bucket * BUCKET_BP + 1
        out.append({"bucket": int(bucket), "lengths": [lo, lo + BUCKET_BP - 1], "reads": int(n_b), "first": int(b0),
                    "verify": best["verify"], "block": best["block"], "trials": trials})
        b0 += n_b
    return out

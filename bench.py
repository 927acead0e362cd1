#!/usr/bin/env python3
"""Mapped reads/s of SWMapper's hot path on GB300.

Workload (default, the human-scale configuration): a 3.1 Gbp synthetic genome
(41% GC, 5% N in runs of 10 kb-1 Mb, 50% of it repeat families at 2-15%
divergence), k=12 index built on the GPU, 10,000,000 reads of 150 bp at 3%
error (70% substitutions, 15% 1-bp insertions, 15% 1-bp deletions) from both
strands, error threshold e=7. `--workload batched | plain | uneven | serving`
selects the other configurations.

A step maps every read of the workload (both strands, in blocks) with the
index and the reads resident in HBM; several mappers take the blocks in turn
(swm_map_device_submit / swm_map_device_wait), so one block's gather-bound
stages overlap another's ALU-bound ones. Reads per block and the number of
mappers come from the autotuner (swmapper_gb300/tune.py), run before the timed
region. `value` is mapped reads per second over the K timed steps (CUDA events
spanning the mappers' streams). `e2e` runs the same reads through the public
host API (H2D from page-locked memory, mapping, D2H of the packed records)
with two mappers in turn over a continuous stream of blocks (the reference's
double buffering), timed on the host clock. The stage breakdown and the
roofline views come from one extra untimed pass with one mapper, so each
kernel runs alone: `roofline` (the dominant
kernel's algorithmic bytes against the measured HBM copy bandwidth),
`gather_roofline` (the seed and candidate kernels' 32-byte sector requests
against the random-read rate a probe kernel measures at their footprint) and
`int_pipe` (the Myers steps the device counted x 21 ops against the ALU pipe).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's own CPU code for the same workload
(the scalar mapper of mapper_cpe.c and serial_index.c compiled for the host,
all host threads) on a bounded sample of the reads per step.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

# The reference's benchmark configurations (synthetic stand-ins with the same
# shapes). "batched" is the headline line; the others are parity-test shapes
# that bench.py can also time with --workload.
WORKLOADS = {
    "batched": dict(workload="batched: 100 Mbp genome (41% GC, 10% repeat copies 300 bp-6 kb at 1% divergence), "
                             "1,000,000 x 150 bp reads at 3% error, e=7, k=12",
                    genome_bp=100_000_000, genome_kind="repeats100m", genome_seed=20261203,
                    reads=1_000_000, len_min=150, len_max=150, error_rate=0.03, e=7, k=12, read_seed=7,
                    block=262144),
    "plain": dict(workload="plain: 1 Mbp uniform genome, 10,000 x 100 bp reads at 2% error, e=5, k=12, "
                           "blocks of 4,096 reads",
                  genome_bp=1_000_000, genome_kind="uniform", genome_seed=1,
                  reads=10_000, len_min=100, len_max=100, error_rate=0.02, e=5, k=12, read_seed=2, block=4096),
    "uneven": dict(workload="uneven: 100 Mbp genome as batched, 2,000,000 reads of 50-250 bp at 4% error, "
                            "per-read e=ceil(0.05 L), k=12",
                   genome_bp=100_000_000, genome_kind="repeats100m", genome_seed=20261203,
                   reads=2_000_000, len_min=50, len_max=250, error_rate=0.04, e=None, e_frac=0.05, k=12,
                   read_seed=11, block=262144),
    "human": dict(workload="human-scale: 3.1 Gbp genome (41% GC, 5% N in runs of 10 kb-1 Mb, 50% repeat families "
                           "at 2-15% divergence), 10,000,000 x 150 bp reads at 3% error, e=7, k=12",
                  genome_bp=3_100_000_000, genome_kind="human", genome_seed=31,
                  reads=10_000_000, len_min=150, len_max=150, error_rate=0.03, e=7, k=12, read_seed=13,
                  block=262144),
}
WORKLOADS["serving"] = dict(
    workload="serving: index of the human-scale genome resident; Poisson arrivals of requests of log-uniform "
             "[1, 4096] reads, 50-250 bp at 3% error, e=ceil(0.05 L); offered load 25/50/90% of the measured peak",
    genome_bp=3_100_000_000, genome_kind="human", genome_seed=31, reads=1_000_000, len_min=50, len_max=250,
    error_rate=0.03, e=None, e_frac=0.05, k=12, read_seed=17, block=65536, requests=3000)
WORKLOAD = dict(WORKLOADS["human"])
METRIC = "mapped reads/s"
L2_FLUSH_BYTES = 512 << 20   # > the 129 MB L2
UNIT = "reads/s"


# ------------------------------------------------------------ plumbing

def cudart():
    for name in ("libcudart.so.13", "libcudart.so", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            L = C.CDLL(name)
            L.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
            L.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
            L.cudaFree.argtypes = [C.c_void_p]
            L.cudaEventCreate.argtypes = [C.POINTER(C.c_void_p)]
            L.cudaEventRecord.argtypes = [C.c_void_p, C.c_void_p]
            L.cudaEventSynchronize.argtypes = [C.c_void_p]
            L.cudaEventElapsedTime.argtypes = [C.POINTER(C.c_float), C.c_void_p, C.c_void_p]
            L.cudaSetDevice.argtypes = [C.c_int]
            return L
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max/sum over ranks (gloo on the host; no data-path collective)."""

    def __init__(self, ws):
        self.ws = ws
        self.pg = None
        if ws > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def reduce(self, values, op):
        if self.ws == 1:
            return values
        import torch
        t = torch.tensor(values, dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX if op == "max" else self.dist.ReduceOp.SUM)
        return t.tolist()

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


def aggregate(dist, elapsed, counts):
    """Whole-job view of one timed region: the slowest rank's time and the sum of
    each per-rank count over all ranks."""
    t, = dist.reduce([float(elapsed)], "max")
    sums = dist.reduce([float(c) for c in counts], "sum")
    return (t, *sums)


def shard_seed(rank):
    """Read seed of a rank's shard: every rank maps its own reads against a full
    index replica (reads are independent; nothing is exchanged)."""
    return WORKLOAD["read_seed"] + 1000 * rank


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 100 ms, time-stamped. The
    sampler starts before the warm-up (nvidia-smi takes a moment to come up)
    and stop(t0, t1) keeps the samples taken inside the timed window [t0, t1]
    (wall clock); a window shorter than the interval keeps the first sample
    after t0 and the last before it instead ("window": "nearest")."""

    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    @staticmethod
    def _stamp(text):
        import datetime
        for fmt in ("%Y/%m/%d %H:%M:%S.%f", "%Y/%m/%d %H:%M:%S"):
            try:
                return datetime.datetime.strptime(text, fmt).timestamp()
            except ValueError:
                continue
        return None

    def stop(self, t0=None, t1=None):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = []
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                rows.append((self._stamp(f[0]), float(f[1]), float(f[2]),
                             {nm for nm, v in zip(names, f[4:8]) if v.lower().startswith("active")}))
            except ValueError:
                continue
        window = "all"
        if t0 is not None and rows and all(r[0] is not None for r in rows):
            inside = [r for r in rows if t0 <= r[0] <= t1]
            if inside:
                rows, window = inside, "timed region"
            else:
                before = [r for r in rows if r[0] < t0][-1:]
                after = [r for r in rows if r[0] > t1][:1]
                rows, window = before + after, "nearest"
        sm = [r[1] for r in rows]
        mx = [r[2] for r in rows]
        reasons = set().union(*[r[3] for r in rows]) if rows else set()
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "window": window, "reasons": sorted(reasons)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured", d
    return 6800.0, "fallback", {}


def profile_traffic(kernel):
    """Per-launch DRAM traffic per unit of work from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_traffic.txt")
    if not os.path.exists(p):
        return None
    vals = {}
    for line in open(p):
        if ":" in line and not line.startswith("#"):
            k, v = line.split(":", 1)
            try:
                vals[k.strip()] = float(v.split()[0])
            except (ValueError, IndexError):
                pass
    return vals


def make_workload(rank=0):
    """Genome, reads, lengths and per-read thresholds (None: one e for all)."""
    from swmapper_gb300 import synth
    w = WORKLOAD
    g = synth.reference(w["genome_bp"], seed=w["genome_seed"], kind=w["genome_kind"])
    reads, lens, _, _ = synth.reads(g, w["reads"], w["len_min"], w["len_max"], w["error_rate"],
                                    seed=shard_seed(rank))
    eper = None
    if w.get("e") is None: # e = ceil(frac * L), at most the envelope's 15
        eper = np.minimum(np.ceil(w["e_frac"] * lens.astype(np.float64) - 1e-9), 15).astype(np.uint8)
    return g, reads, lens, eper


def e_arg(eper):
    """Scalar threshold passed with per-read ones (their maximum)."""
    return int(eper.max()) if eper is not None and eper.size else int(WORKLOAD.get("e") or 0)


# ------------------------------------------------------------ CPU legs

def host_map_index(arrays, k):
    """Mapper view of index arrays for the CPU legs (start offsets, padded words)."""
    from oracle import pyoracle as po
    hix = po.HostIndex(k, 0, arrays["hash_count"], arrays["hash_offset"], arrays["positions"],
                       arrays["pos_lseeds"], arrays["base_2bits"], arrays["base_3bits"])
    return po.MapIndex(hix)


CPU_BLOCK = 10_000   # reads per block of the reference's host loop (mapper_mpe.c:727)
REF_WINDOW_BASES = 224  # 7 x 32 bases: the 16-word window slot of the reference verifier
_cpu_bufs = {}


def cpu_map(mix, reads, lens, e, threads, eper=None):
    """Map on the host in blocks of 10,000 reads: the reference's own
    get_positions() when it was compiled here (kind 'reference'), else the
    oracle restatement (kind 'port'). Per-read thresholds map each e group
    on its own (the reference takes one e per call). Returns (mapped reads,
    kind)."""
    from oracle import pyoracle as po
    if eper is not None:
        mapped, kinds = 0, set()
        for ev in np.unique(eper):
            idx = np.nonzero(eper == ev)[0]
            mg, kd = cpu_map(mix, reads[idx], lens[idx], int(ev), threads)
            mapped += mg
            kinds.add(kd)
        return mapped, "reference" if kinds == {"reference"} else "port"
    if "out" not in _cpu_bufs:
        _cpu_bufs["out"] = po.out_buffers(CPU_BLOCK)
    mapped = 0
    # the reference's 16-word window slot holds L + 2e <= 224 (mapper_cpe.c:1600,1613); longer
    # windows overflow it, so such reads run on the oracle restatement
    in_env = reads.shape[0] == 0 or int(lens.max()) + 2 * e <= REF_WINDOW_BASES
    kind = "reference" if po.have_ref() and in_env else "port"
    for b0 in range(0, reads.shape[0], CPU_BLOCK):
        r, ln = reads[b0:b0 + CPU_BLOCK], lens[b0:b0 + CPU_BLOCK]
        if kind == "reference":
            res = po.ref_map_reads(mix, r, ln, e, nthreads=threads, out=_cpu_bufs["out"])
            mapped += r.shape[0] - res.unmapped.size
        else:
            res = po.map_reads(mix, r, ln, e, nthreads=threads)
            mapped += res.stats["mapped_reads"]
    return mapped, kind


def timed_cpu_sample(mix, reads, lens, e, threads, target_s, eper=None):
    """Time a bounded sample sized to take about target_s seconds."""
    n = min(2048, reads.shape[0])
    t0 = time.perf_counter()
    cpu_map(mix, reads[:n], lens[:n], e, threads, None if eper is None else eper[:n])
    dt = max(time.perf_counter() - t0, 1e-3)
    n = int(min(reads.shape[0], max(n, n * target_s / dt)))
    t0 = time.perf_counter()
    mapped, kind = cpu_map(mix, reads[:n], lens[:n], e, threads, None if eper is None else eper[:n])
    dt = time.perf_counter() - t0
    return mapped / dt, n, dt, kind


# ------------------------------------------------------------ GPU arm

STAGES = ["seed", "plan", "candidates", "compact", "verify", "traceback", "records"]


def stage_bytes(stage, st, L, e, table=False):
    """Algorithmic DRAM bytes of one stage over a whole step: what the stage must
    read and write once. Candidates without the candidate table: the 2-byte
    flank code of every fetched entry and the 4-byte position of each kept
    one; with it: two 4-byte offsets per selected seed and the 4-byte position
    of each kept entry (plus, in both, the seed records, refill chunks and the
    candidates written)."""
    nl = L // 15
    items = st["items"]
    ns = min(e + 1, nl) * 4
    if stage == "seed":
        return items * (L + nl * 4 * 8 + 128 + ns * 12 + 16)
    if stage == "plan":   # items with refills only: seed table, refill chunks, batch records
        return st["chunks"] * (8 + 8) + st["batches"] * 12 + items * 8
    if stage == "candidates":
        kept = st.get("kept", st["candidates"])
        common = items * ns * 9 + st["chunks"] * 8 + st["candidates"] * 4
        if table:  # seed records with their table keys (13 B), table offsets, kept positions
            return items * ns * (4 + 8) + kept * 4 + common
        return st["fetched"] * 2 + kept * 4 + common
    if stage == "compact":
        return st["candidates"] * 12 + st["batches"] * 12
    if stage == "verify":
        win = ((L + 2 * e + 31) // 32 + 1) * 8
        return st["candidates"] * (win + 64 + 8 + 16)
    if stage == "traceback":  # flags of every candidate, window + read + CIGAR of the passing ones
        win = ((L + 2 * e + 31) // 32 + 1) * 8
        return st["candidates"] * 1 + st["passed"] * (win + 128 + 32)
    if stage == "records":
        return st["candidates"] * 10 + st["locations"] * 12 + items * 24
    return 0


def block_plan(nreads, block, tuned, verify="stream16"):
    """(first read, reads, verification form) of every block: blocks of
    `block` reads with the given form, or, with per-bucket tuning, each
    length bucket's reads in blocks of its own size with its own form."""
    if not tuned or not tuned.get("buckets"):
        return [(b0, min(block, nreads - b0), verify) for b0 in range(0, nreads, block)]
    out = []
    for bk in tuned["buckets"]:
        lo, n, bs = bk["first"], bk["reads"], min(bk["block"], bk["reads"])
        out += [(b0, min(bs, lo + n - b0), bk["verify"]) for b0 in range(lo, lo + n, bs)]
    return out


def run_gpu(args):
    import swmapper_gb300 as swm
    ws, rank, local = dist_env()
    dist = Dist(ws)
    rt = cudart()
    rt.cudaSetDevice(local)
    w = WORKLOAD
    g, reads, lens, eper = make_workload(rank)
    E = e_arg(eper)
    bucketed = False
    if args.buckets and int(lens.min()) != int(lens.max()):
        # reads of similar length share a block (autotuner length buckets of 32 bp)
        from swmapper_gb300 import tune as swtune
        order = np.concatenate([ix_ for _, ix_ in swtune.length_buckets(lens)])
        reads, lens = np.ascontiguousarray(reads[order]), np.ascontiguousarray(lens[order])
        eper = None if eper is None else np.ascontiguousarray(eper[order])
        bucketed = True
    # index build on bases already in device memory (the copy of the genome
    # is not part of the build), host clock around the synchronous call
    d_g = C.c_void_p()
    assert rt.cudaMalloc(C.byref(d_g), g.nbytes) == 0
    rt.cudaMemcpy(d_g, g.ctypes.data, g.nbytes, 1)
    rt.cudaDeviceSynchronize()
    t0 = time.perf_counter()
    ix = swm.Index.build_device(d_g.value, g.size, k=w["k"], device=local)
    index_build_s = time.perf_counter() - t0
    rt.cudaFree(d_g)
    if args.table >= 0:  # else the library decides (large genomes only)
        ix.candidate_table(bool(args.table))
    nreads, stride = reads.shape
    block = min(args.block, nreads)
    # inputs resident in HBM
    d_reads, d_lens = C.c_void_p(), C.c_void_p()
    assert rt.cudaMalloc(C.byref(d_reads), reads.nbytes) == 0
    assert rt.cudaMalloc(C.byref(d_lens), lens.nbytes) == 0
    rt.cudaMemcpy(d_reads, reads.ctypes.data, reads.nbytes, 1)
    rt.cudaMemcpy(d_lens, lens.ctypes.data, lens.nbytes, 1)
    d_e = C.c_void_p()
    if eper is not None:
        assert rt.cudaMalloc(C.byref(d_e), eper.nbytes) == 0
        rt.cudaMemcpy(d_e, eper.ctypes.data, eper.nbytes, 1)
    # NMAP mappers (own stream and buffers each) take the blocks in turn, so
    # one block's gather-bound stages overlap another's ALU-bound ones
    tuned = None
    if args.tune:  # reads per block and mappers from timed trials on the resident reads
        from swmapper_gb300 import tune as swtune
        # a window from the middle of the reads (with length buckets: reads of middling length)
        n_t = min(nreads, 2_000_000)
        o_t = (nreads - n_t) // 2
        tuned = swtune.tune(ix, d_reads.value + o_t * stride, d_lens.value + o_t * 4, stride, n_t, E,
                            d_e.value + o_t if eper is not None else None)
        block, args.mappers = min(tuned["block"], nreads), tuned["mappers"]
        # per 32-bp length bucket (reads grouped by bucket): verification form
        # and reads per block
        if bucketed or int(lens.min()) == int(lens.max()):
            tuned["buckets"] = swtune.tune_buckets(ix, d_reads.value, d_lens.value, stride, lens, E,
                                                   d_e.value if eper is not None else None, args.mappers)
    blocks = block_plan(nreads, block, tuned, args.verify)
    if tuned and tuned.get("buckets"):
        # the per-bucket plan against the sorted reads in blocks of the tuned
        # size (each with its main bucket's form), over all the reads
        from swmapper_gb300 import tune as swtune
        merged = swtune.merged_plan(tuned["buckets"], nreads, block)
        best, rates = swtune.tune_plan(ix, d_reads.value, d_lens.value, stride, E,
                                       d_e.value if eper is not None else None,
                                       {"per_bucket": blocks, "merged": merged}, args.mappers)
        tuned["plan"] = {"chosen": best, "reads_per_s": rates}
        if best == "merged":
            blocks = merged
    block = max(nb for _, nb, _ in blocks)
    mappers = [swm.Mapper(ix, max_reads=block) for _ in range(args.mappers)]
    if args.serialize:  # the mappers' blocks take the GPU one at a time
        ix.serialize_mappers(True)
    m = mappers[0]
    streams = [C.c_void_p(mm.stream()) for mm in mappers]
    ev0, ev1, evq = C.c_void_p(), C.c_void_p(), C.c_void_p()
    for ev in (ev0, ev1, evq):
        rt.cudaEventCreate(C.byref(ev))
    rt.cudaStreamWaitEvent.argtypes = [C.c_void_p, C.c_void_p, C.c_uint]
    COUNTERS = ("mapped_reads", "candidates", "cells", "passed", "fetched", "chunks", "batches", "items",
                "locations", "records", "retries", "myers_steps", "kept")

    def run_steps(nsteps, acc):
        """nsteps passes over the reads as one continuous stream of blocks."""
        pend = []

        def drain():
            pm = pend.pop(0)
            pm.wait_device()
            if acc is not None:
                st = pm.stats()
                for f in COUNTERS:
                    acc[f] = acc.get(f, 0) + st[f]
                acc["launches"] = acc.get("launches", 0) + pm.launches()
                acc["blocks"] = acc.get("blocks", 0) + 1

        for i in range(nsteps * len(blocks)):
            b0, nb, hd = blocks[i % len(blocks)]
            if len(pend) == len(mappers):
                drain()
            mm = mappers[i % len(mappers)]
            mm.set_verify(hd)
            mm.submit_device(d_reads.value + b0 * stride, d_lens.value + b0 * 4, stride, nb, E,
                             d_e.value + b0 if eper is not None else None)
            pend.append(mm)
        while pend:
            drain()

    inf = ix.info()
    index_bytes = (2 * (4 << (2 * inf.k)) + 6 * inf.n_seeds + 4 * (inf.n_words2 + inf.n_words3))
    input_bytes = reads.nbytes + lens.nbytes + index_bytes
    flush = input_bytes < L2_FLUSH_BYTES  # small inputs: flush L2 between timed steps
    d_flush = C.c_void_p()
    if flush:
        assert rt.cudaMalloc(C.byref(d_flush), L2_FLUSH_BYTES) == 0
    rt.cudaMemsetAsync.argtypes = [C.c_void_p, C.c_int, C.c_size_t, C.c_void_p]

    def timed(nsteps, acc):
        """Device time of nsteps passes: ev0 on the first stream, which every
        other stream waits for; ev1 after every stream's last block."""
        rt.cudaDeviceSynchronize()
        rt.cudaEventRecord(ev0, streams[0])
        for sm in streams[1:]:
            rt.cudaStreamWaitEvent(sm, ev0, 0)
        run_steps(nsteps, acc)
        for sm in streams[1:]:
            rt.cudaEventRecord(evq, sm)
            rt.cudaStreamWaitEvent(streams[0], evq, 0)
        rt.cudaEventRecord(ev1, streams[0])
        rt.cudaEventSynchronize(ev1)
        rt.cudaDeviceSynchronize()
        ms = C.c_float()
        rt.cudaEventElapsedTime(C.byref(ms), ev0, ev1)
        return ms.value / 1000.0

    clocks = ClockSampler(local)
    clocks.start()
    run_steps(args.warmup, None)
    acc = {}
    dist.barrier()
    t_wall0 = time.time()
    if flush: # one step at a time, L2 flushed (outside the events) before each
        elapsed = 0.0
        for _ in range(args.steps):
            rt.cudaMemsetAsync(d_flush, 1, L2_FLUSH_BYTES, streams[0])
            elapsed += timed(1, acc)
    else:
        elapsed = timed(args.steps, acc)
    dist.barrier()
    clk = clocks.stop(t_wall0, time.time())
    tot_elapsed, tot_mapped, tot_cells = aggregate(dist, elapsed, [acc["mapped_reads"], acc["cells"]])
    value = tot_mapped / tot_elapsed
    # kernel times in isolation (one mapper, one block at a time) for the
    # stage breakdown and the roofline: one untimed pass over the reads
    for b0, nb, hd in blocks:
        m.set_verify(hd)
        m.map_device(d_reads.value + b0 * stride, d_lens.value + b0 * 4, stride, nb, E,
                     d_e.value + b0 if eper is not None else None)
        for sname in STAGES:
            acc["ms_" + sname] = acc.get("ms_" + sname, 0.0) + m.stage_ms(sname) * args.steps
    gcups = tot_cells / tot_elapsed / 1e9
    # cells the recurrence executed: read bases run x band width (the head
    # pass stops hopeless candidates early, so this is below the algorithmic
    # L x (2e + 1) per candidate)
    e_mean = E if eper is None else float(eper.mean())
    gcups_exec = acc["myers_steps"] * (2 * e_mean + 1) / elapsed / 1e9

    # the plain per-batch launch for comparison: one mapper, blocks of 4,096
    # reads (the plain configuration's batch), each mapped and waited for in turn
    plain_block = min(4096, nreads)
    mp = swm.Mapper(ix, max_reads=plain_block) if args.plain else None
    for b0 in range(0, min(nreads, 4 * plain_block) if mp else 0, plain_block):  # warm-up
        mp.map_device(d_reads.value + b0 * stride, d_lens.value + b0 * 4, stride, min(plain_block, nreads - b0), E,
                      d_e.value + b0 if eper is not None else None)
    rt.cudaDeviceSynchronize()
    t0 = time.perf_counter()
    plain_mapped = 0
    for b0 in range(0, nreads if mp else 0, plain_block):
        mp.map_device(d_reads.value + b0 * stride, d_lens.value + b0 * 4, stride, min(plain_block, nreads - b0), E,
                      d_e.value + b0 if eper is not None else None)
        plain_mapped += mp.stats()["mapped_reads"]
    rt.cudaDeviceSynchronize()
    plain_t = time.perf_counter() - t0
    del mp
    plain = {"value": round(plain_mapped / plain_t, 1), "unit": UNIT, "block_reads": plain_block, "mappers": 1,
             "path": "swm_map_device per block of 4,096 reads, synchronous; host clock over one pass"} if args.plain \
        else None

    # end to end through the host API: two mappers in ping-pong, packed
    # results; the reads and the result buffers are page-locked host memory;
    # the blocks' kernels run one block at a time while the other mapper's
    # copies overlap them (swm_index_serialize_mappers)
    ix.serialize_mappers(bool(args.e2e_serialize))
    ne = max(2, args.e2e_mappers)
    mappers = (mappers + [swm.Mapper(ix, max_reads=block) for _ in range(ne)])[:ne]
    bufs = [swm.PackedBuffers(block) for _ in range(ne)]
    rt.cudaHostRegister.argtypes = [C.c_void_p, C.c_size_t, C.c_uint]
    pinned = [reads, lens] + [a for bf in bufs for a in (bf.words, bf.cigar, bf.rlen)]
    for a in pinned:
        rt.cudaHostRegister(a.ctypes.data, a.nbytes, 0)

    def e2e_run(nsteps, acc2):
        """nsteps passes over the reads as one continuous stream of blocks:
        block i + ne is submitted as soon as block i's results are back."""
        pend = []

        def drain():
            j, pm = pend.pop(0)
            pm.wait_packed(bufs[j % ne])
            acc2["mapped"] += count_mapped(bufs[j % ne], blocks[j % len(blocks)][1])
            st = pm.stats()
            acc2["h2d"] += st["h2d_bytes"]
            acc2["d2h"] += st["d2h_bytes"]

        for i in range(nsteps * len(blocks)):
            b0, nb, hd = blocks[i % len(blocks)]
            if len(pend) == ne:
                drain()
            mappers[i % ne].set_verify(hd)
            mappers[i % ne].submit(reads[b0:b0 + nb], lens[b0:b0 + nb], E,
                                  None if eper is None else eper[b0:b0 + nb])
            pend.append((i, mappers[i % ne]))
        while pend:
            drain()

    e2e_clocks = ClockSampler(local)
    e2e_clocks.start()
    e2e_run(min(args.warmup, 2), {"mapped": 0, "h2d": 0, "d2h": 0})
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    acc2 = {"mapped": 0, "h2d": 0, "d2h": 0}
    dist.barrier()
    t_e2e0 = time.time()
    t0 = time.perf_counter()
    e2e_run(e2e_steps, acc2)
    e2e_t = time.perf_counter() - t0
    e2e_clk = e2e_clocks.stop(t_e2e0, time.time())
    e2e_t, e2e_mapped = aggregate(dist, e2e_t, [acc2["mapped"]])
    ix.serialize_mappers(bool(args.serialize))
    rt.cudaHostUnregister.argtypes = [C.c_void_p]
    for a in pinned:
        rt.cudaHostUnregister(a.ctypes.data)
    e2e = {"value": e2e_mapped / e2e_t, "unit": UNIT,
           "h2d_bytes_per_step": int(acc2["h2d"] / e2e_steps), "d2h_bytes_per_step": int(acc2["d2h"] / e2e_steps),
           "serialized": bool(args.e2e_serialize), "clocks": e2e_clk,
           "steps": e2e_steps, "path": f"swm_map_submit + swm_map_wait_packed, {ne} mappers in turn over a continuous stream of "
                   "blocks, page-locked host buffers"}

    # roofline of the dominant kernel
    peak, peak_kind, peaks = measured_peaks()
    table = ix.candidate_table(None) > 0
    # index build against the bytes it must move once: the bases read (1 B
    # each), the bit planes + N mask written and read back (2 x 3 bits per
    # base), the count and offset tables written and read (2 x 2 x 4^k x 4 B)
    # and every entry's position and flank code written (6 B)
    ib_bytes = g.size + 2 * (3 * g.size / 8) + 4 * (4 << (2 * inf.k)) + 6 * inf.n_seeds
    index_build = {"seconds": round(index_build_s, 4), "bytes": int(ib_bytes),
                   "gbs": round(ib_bytes / index_build_s / 1e9, 1), "peak": peak,
                   "frac": round(ib_bytes / index_build_s / 1e9 / peak, 4),
                   "model": "bases 1 B + bit planes and N mask written and read 2 x 3/8 B per base + count/offset "
                            "tables 2 x 2 x 4^k x 4 B + positions and flank codes 6 B per entry; bases already on "
                            "the device, host clock around swm_index_build_device"}
    L = float(lens.mean())
    e = E if eper is None else float(eper.mean())
    per_step = {k: v / args.steps for k, v in acc.items()}
    stage_rows = {}
    for sname in STAGES:
        t_ms = per_step["ms_" + sname]
        byts = stage_bytes(sname, per_step, L, e, table)
        stage_rows[sname] = {"ms_per_step": round(t_ms, 3),
                             "gbs": round(byts / (t_ms / 1e3) / 1e9, 1) if t_ms > 0 else None,
                             "bytes_per_step": int(byts)}
    dom = max(STAGES, key=lambda s: per_step["ms_" + s])
    # the verification kernels the blocks ran: streaming (k_verify_stream, then
    # k_verify_finish) or the two passes of k_verify
    streaming = all(hd.startswith(("stream", "pair")) for _, _, hd in blocks)
    vkern = ("k_verify_pair" if all(hd == "pair16" for _, _, hd in blocks) and eper is None and E <= 7
             else "k_verify_stream") if streaming else "k_verify"
    kern = {"seed": "k_seed12" if w["k"] == 12 else "k_seed", "plan": "k_plan",
            "candidates": "k_cand_table" if table else "k_cand", "compact": "k_compact",
            "verify": vkern, "traceback": "k_traceback", "records": "k_records"}[dom]
    launches_per_step = per_step["blocks"]
    avg_launch_s = per_step["ms_" + dom] / 1e3 / launches_per_step
    alg_bytes_launch = stage_bytes(dom, per_step, L, e, table) / launches_per_step
    achieved = alg_bytes_launch / avg_launch_s / 1e9
    tr = profile_traffic(kern)
    traffic = None
    if tr:
        unit_key = {"k_verify": "candidates", "k_verify_stream": "candidates", "k_cand": "fetched", "k_cand_table": "items", "k_seed": "items",
                    "k_seed12": "items",
                    "k_plan": "chunks", "k_traceback": "passed"}.get(kern)
        for key, val in tr.items():
            if key.startswith("dram_bytes_per_") and unit_key and key.endswith(unit_key):
                traffic = int(val * per_step[unit_key] / launches_per_step)
    roofline = {"bound": "hbm", "kernel": kern, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else
                "fallback 6.8 TB/s"}
    # the candidate stage against the HBM peak by the DRAM bytes it moves (ncu
    # bytes per unit from its committed capture x this step's units): its
    # scattered 4-byte reads each move a whole DRAM burst, so its algorithmic
    # bytes understate what bounds it
    cand_dram = None
    ckern = "k_cand_table" if table else "k_cand"
    ctr = profile_traffic(ckern) or {}
    cper = ctr.get("dram_bytes_per_item_human" if table and w["genome_kind"] == "human" else "")
    t_cand = per_step["ms_candidates"] / 1e3
    if cper and t_cand > 0:
        cgbs = cper * per_step["items"] / t_cand / 1e9
        cand_dram = {"kernel": ckern, "dram_gbs": round(cgbs, 1), "peak": peak, "frac": round(cgbs / peak, 4),
                     "algorithmic_gbs": stage_rows["candidates"]["gbs"],
                     "model": f"{cper:.0f} B of DRAM per item (ncu, profiles/{ckern}_traffic.txt) x items / "
                              "candidate-stage time"}
    # gather view of the seed and candidate kernels: they read scattered 32-byte
    # sectors (bucket offsets; flank codes and positions), so their ceiling is
    # the rate at which the device serves random sector reads from an array of
    # their footprint (L2 and DRAM in the proportion that footprint gives),
    # measured here by a probe kernel
    gather = None
    if rank == 0 and ws == 1 and args.workload == "batched":  # per-unit sector counts: batched genome
        kernels = {}
        for kern, stage, unit_key, foot in (("k_cand", "candidates", "fetched", 6 * inf.n_seeds),
                                            ("k_seed12", "seed", "items", 4 << (2 * inf.k))):
            tr = profile_traffic(kern) or {}
            spu = tr.get(f"l2_sectors_per_{unit_key}")
            t_s = per_step["ms_" + stage] / 1e3
            if not spu or t_s <= 0 or (kern == "k_seed12" and w["k"] != 12):
                continue
            foot = max(int(foot), 1 << 20)
            pk = swm.probe_random_reads(foot, local)
            ach = spu * per_step[unit_key] / t_s
            kernels[kern] = {"achieved": round(ach / 1e9, 1), "peak": round(pk / 1e9, 1), "frac": round(ach / pk, 3),
                             "footprint_bytes": foot, "sectors_per_unit": spu, "unit_of_work": unit_key}
        gather = {"unit": "G sectors/s",
                  "peak_model": "swm_probe_random_reads in this run: 4-byte reads from random 32-byte sectors of a "
                                "buffer of the kernel's gathered footprint (positions + flank codes; bucket "
                                "offsets), 8 in flight per thread, best of 5 launches",
                  "achieved_model": "32-byte sectors the kernel requests from L2 per unit of work (ncu "
                                    "lts__t_sectors_srcunit_tex_op_read, profiles/<kernel>_traffic.txt) x units / "
                                    "kernel time", "kernels": kernels}

    # integer-pipe view of the Myers kernel: its hot loop is LOP3 / SHF / IADD
    # work on the ALU pipe, which takes one warp instruction every second cycle
    # per SM sub-partition (ncu: sm__pipe_alu_cycles_active exceeds the issue
    # rate on this kernel), so 16 lanes x 4 sub-partitions per SM
    sm_mhz = clk.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    int_peak = 152 * 64 * sm_mhz * 1e6 / 1e12
    myers_ops = per_step["myers_steps"] * 21
    t_verify = per_step["ms_verify"] / 1e3
    int_pipe = {"kernel": vkern, "ops_per_step": int(myers_ops), "achieved_tops": round(myers_ops / t_verify / 1e12, 2)
                if t_verify > 0 else None, "peak_tops": round(int_peak, 2),
                "frac": round(myers_ops / t_verify / 1e12 / int_peak, 4) if t_verify > 0 else None,
                "ops_model": "21 int ops per executed Myers step (17 recurrence + 4 pattern word), steps counted "
                             "on the device over all verification kernels ("
                             + ("streaming: each lane stops its candidate at the first 16-base chunk whose band bound "
                                "exceeds e; the finishing kernel runs the last bases and reruns tracebacks"
                                if streaming else
                                "two passes: the head stops hopeless candidates after 64 bases") + ")",
                "peak_model": "152 SMs x 64 ALU-pipe lanes (16 per sub-partition) x median SM clock under load"}

    line = {"metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(tot_elapsed / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded genome and reads of the workload's shapes; no public dataset)",
            "config": {**WORKLOAD, "block_reads": block, "mappers": args.mappers,
                       "serialized_mappers": bool(args.serialize), "candidate_table": table,
                       "autotune": tuned, "length_buckets": bucketed,
                       "parallelism": f"replicas x{ws} (reads sharded by rank)",
                       "l2": (f"inputs {input_bytes / 1e6:.0f} MB (under {L2_FLUSH_BYTES >> 20} MiB, so treated as "
                              f"possibly cache-resident): L2 flushed ({L2_FLUSH_BYTES >> 20} MiB write) before each "
                              f"timed step" if flush else
                              f"inputs larger than L2 (reads {reads.nbytes / 1e6:.0f} MB, index "
                              f"{index_bytes / 1e9:.2f} GB); no flush")},
            "gcups": round(gcups, 2), "gcups_executed": round(gcups_exec, 2),
            "gcups_model": "gcups: algorithmic (reference-equivalent) cells, L x (2e + 1) per verified candidate; "
                           "gcups_executed: Myers steps the device ran x (2e + 1)",
            "index_build_s": round(index_build_s, 3), "index_build": index_build,
            "per_step": {k: int(v) if not k.startswith("ms_") else round(v, 3) for k, v in per_step.items()},
            "stages": stage_rows, "stage_timing": "kernel times of one mapper alone (untimed pass)",
            "clocks": clk, "e2e": e2e,
            "gpu_launches": int(acc["launches"]), "roofline": roofline, "int_pipe": int_pipe,
            "candidates_dram": cand_dram, "gather_roofline": gather,
            "plain_per_batch": plain}
    if rank == 0 and ws == 1 and (not args.no_cpu_baseline or args.parity_reads):
        arrays = ix.download()
        mix = host_map_index(arrays, w["k"])
        threads = os.cpu_count() or 1
        if args.parity_reads:
            line["parity"] = parity_sample(m, mix, reads, lens, E, eper, args.parity_reads, threads)
        if not args.no_cpu_baseline:
            v, n, dt, kind = timed_cpu_sample(mix, reads, lens, E, threads, args.cpu_seconds, eper)
            line["cpu_baseline"] = {"value": round(v, 1), "unit": UNIT, "cores": threads, "kind": kind,
                                    "sample": f"first {n} reads of the workload, {dt:.1f} s, {threads} threads"}
    if rank == 0 and ws == 1 and args.serving and w["genome_kind"] == "human":
        line["serving"] = serving_loads(swm, ix, g, args)
    if rank == 0 and ws == 1 and args.index_load:
        line["index_load"] = index_load(swm, rt, ix, w["k"], local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


def index_load(swm, rt, ix, k, device):
    """After the timing: the resident index written as the reference's seven
    files (swm_index_save) and read back by swm_index_open (sizes checked,
    one thread per file streaming chunks through page-locked buffers to the
    device), host clock around each call. The files were just written, so the
    load reads them from the page cache: it measures the loader and the H2D
    copies, not the disk. Skipped when the temporary directory lacks room."""
    import shutil
    inf = ix.info()
    nb = 1 << (2 * k)  # .hash_count and .hash_offset, then the entries and the bit planes
    need = 4 * nb + 4 * (nb + 1) + 6 * inf.n_seeds + 4 * (inf.n_words2 + inf.n_words3)
    tmp = tempfile.gettempdir()
    free = shutil.disk_usage(tmp).free
    if free < 2 * need:
        return {"skipped": f"{free / 1e9:.1f} GB free in {tmp}, {need / 1e9:.1f} GB of files"}
    d = tempfile.mkdtemp(prefix="swm_index_", dir=tmp)
    try:
        return _index_load(swm, rt, ix, k, device, inf, d)
    except (OSError, RuntimeError) as ex:  # a full disk or a loader error is reported, not fatal
        return {"skipped": f"{type(ex).__name__}: {ex}"}
    finally:
        shutil.rmtree(d, ignore_errors=True)


def _index_load(swm, rt, ix, k, device, inf, d):
    """Save the index as files in directory d, then time swm_index_open on them."""
    prefix = os.path.join(d, "genome")
    t0 = time.perf_counter()
    ix.save(prefix)
    t_save = time.perf_counter() - t0
    nbytes = sum(os.path.getsize(os.path.join(d, f)) for f in os.listdir(d))
    rt.cudaDeviceSynchronize()
    t0 = time.perf_counter()
    ix2 = swm.Index.open(prefix, k=k, device=device)
    rt.cudaDeviceSynchronize()
    t_load = time.perf_counter() - t0
    same = ix2.info().n_seeds == inf.n_seeds
    ix2.close()
    return {"load_s": round(t_load, 3), "save_s": round(t_save, 3), "file_bytes": int(nbytes),
            "load_gbs": round(nbytes / t_load / 1e9, 2), "entries_equal": bool(same),
            "path": "swm_index_open on the files swm_index_save just wrote (page cache warm): size checks, "
                    "one thread per file, 32 MiB chunks through two page-locked buffers, async H2D"}


def parity_sample(m, mix, reads, lens, E, eper, nsample, threads):
    """After the timing: the first nsample reads of the timed workload mapped
    by the GPU path (swm_map_batch, blocks of the timed mapper's size) and by
    the reference's own get_positions() compiled for the host (the oracle
    restatement where the reference cannot take the reads), on the index the
    GPU built; records, CIGARs and unmapped ids must be identical."""
    from oracle import pyoracle as po
    n = min(nsample, reads.shape[0])
    got, got_unm = [], []
    for b0 in range(0, n, m.max_reads):
        b1 = min(n, b0 + m.max_reads)
        out = m.map(reads[b0:b1], lens[b0:b1], E, None if eper is None else eper[b0:b1])
        got.extend((r[0] + 2 * b0,) + r[1:] for r in out.records())
        got_unm.extend(int(u) + 2 * b0 for u in out.unmapped)
    in_env = int(lens[:n].max()) + 2 * E <= REF_WINDOW_BASES
    against = "reference (oracle/_ref/libswref.so: the reference's get_positions compiled for the host)"
    if eper is None and po.have_ref() and in_env:
        want, want_unm = [], []
        for b0 in range(0, n, CPU_BLOCK):
            b1 = min(n, b0 + CPU_BLOCK)
            res = po.ref_map_reads(mix, reads[b0:b1], lens[b0:b1], E, nthreads=threads)
            want.extend((r[0] + 2 * b0,) + r[1:] for r in res.records())
            want_unm.extend(int(u) + 2 * b0 for u in res.unmapped)
    else:
        against = "oracle (oracle/swm_oracle.c restatement; reads outside the reference's window slot)"
        want, want_unm = [], []
        groups = [(E, np.arange(n))] if eper is None else [(int(ev), np.nonzero(eper[:n] == ev)[0])
                                                           for ev in np.unique(eper[:n])]
        per = {}
        for ev, idx in groups:
            res = po.map_reads(mix, reads[idx], lens[idx], ev, nthreads=threads)
            for rec in res.records():
                r = int(idx[rec[0] >> 1])
                per.setdefault(r, []).append((2 * r + (rec[0] & 1),) + rec[1:])
            for u in res.unmapped:
                per.setdefault(int(idx[u >> 1]), [])
        for r in sorted(per):
            if not per[r]:
                want_unm.append(2 * r + 1)
            want.extend(per[r])
    equal = got == want and got_unm == want_unm
    return {"reads": int(n), "equal": bool(equal), "records": len(got), "unmapped": len(got_unm),
            "against": against}


def count_mapped(buf, nreads):
    return nreads - int(buf.c.n_unmapped)


# ------------------------------------------------------------ serving

SERVE = dict(requests=4000, size_max=4096, len_min=50, len_max=250, error_rate=0.03, e_frac=0.05, read_seed=17,
             block_reads=65536, max_slots=4, loads=(0.25, 0.5, 0.9), runs=3)


def serving_loads(swm, ix, g, args):
    """Serving through the library's request loop (swm_serve_*): requests of
    log-uniform [1, 4096] reads of 50-250 bp at 3% error, e = ceil(0.05 L),
    arrive as a Poisson stream; the server coalesces the waiting ones into
    the next free block slot, admitting slots by free device memory. The peak
    is all requests submitted at once; then each offered load (a fraction of
    the peak) runs SERVE['runs'] times. A request's latency runs from its
    scheduled arrival to the return of the poll that hands over its records
    (host clock); p50 / p99 per run, and the spread of p99 over the runs."""
    import threading
    cfg = SERVE
    rng = np.random.default_rng(cfg["read_seed"])
    nreq = args.requests or cfg["requests"]
    sizes = np.minimum(np.exp(rng.uniform(0.0, math.log(cfg["size_max"]), nreq)).astype(np.int64), cfg["size_max"])
    sizes = np.maximum(sizes, 1)
    total = int(sizes.sum())
    reads, lens = synth_reads(g, total, cfg["len_min"], cfg["len_max"], cfg["error_rate"], cfg["read_seed"])
    eper = np.minimum(np.ceil(cfg["e_frac"] * lens.astype(np.float64) - 1e-9), 15).astype(np.uint8)
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    reqs = [(reads[o:o + n], lens[o:o + n], eper[o:o + n], int(eper[o:o + n].max())) for o, n in zip(offs, sizes)]
    srv = swm.Server(ix, block_reads=cfg["block_reads"], max_slots=cfg["max_slots"], stride=256,
                     max_queued_reads=total + cfg["block_reads"])

    def run(arrivals):
        nq = len(arrivals)
        lat = np.zeros(nq)
        done_t = [0.0]
        id2q = {}
        lock = threading.Lock()

        def collector():
            got = 0
            while got < nq:
                res = srv.poll(timeout_ms=120_000, records=False)
                if res is None:
                    raise RuntimeError("serving: no request finished within two minutes")
                t = time.perf_counter()
                with lock:
                    q = id2q.get(res[0])
                while q is None:  # the submitting thread has not recorded the id yet
                    time.sleep(0)
                    with lock:
                        q = id2q.get(res[0])
                lat[q] = t - (t_start + arrivals[q])
                done_t[0] = t
                got += 1

        th = threading.Thread(target=collector)
        t_start = time.perf_counter()
        th.start()
        for q in range(nq):
            while True:
                wait = t_start + arrivals[q] - time.perf_counter()
                if wait <= 0:
                    break
                time.sleep(wait if wait > 0.0005 else 0)
            r, ln, ep, emax = reqs[q]
            rid = srv.submit(r, ln, emax, errors_per_read=ep)
            with lock:
                id2q[rid] = q
        th.join()
        return lat, done_t[0] - t_start

    run(np.zeros(min(nreq, 200)))  # warm-up: slots made, graphs captured
    _, span = run(np.zeros(nreq))  # everything at once: the peak
    peak = total / span
    rows = []
    for load in cfg["loads"]:
        rate = load * peak / float(sizes.mean())   # requests per second
        per_run = []
        for _ in range(cfg["runs"]):
            arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
            lat, span = run(arrivals)
            per_run.append({"sustained_reads_per_s": round(total / span, 1),
                            "p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 3),
                            "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 3)})
        p99s = [x["p99_ms"] for x in per_run]
        rows.append({"load": load, "offered_reads_per_s": round(load * peak, 1),
                     "sustained_reads_per_s": round(statistics.median(x["sustained_reads_per_s"] for x in per_run), 1),
                     "p50_ms": round(statistics.median(x["p50_ms"] for x in per_run), 3),
                     "p99_ms": round(statistics.median(p99s), 3),
                     "p99_spread_ms": [min(p99s), max(p99s)], "runs": per_run})
    st = srv.stats()
    srv.close()
    return {"peak_reads_per_s": round(peak, 1), "loads": rows, "requests": nreq,
            "reads_per_request_mean": round(float(sizes.mean()), 1),
            "path": "swm_serve_submit / swm_serve_poll (library request loop: continuous batching into block "
                    "slots admitted by free device memory)",
            "server": {"block_reads": cfg["block_reads"], "max_slots": cfg["max_slots"], "slots_made": st["slots"],
                       "slot_bytes": st["slot_bytes"], "blocks": st["blocks"],
                       "max_blocks_in_flight": st["max_blocks_in_flight"]}}


def synth_reads(g, n, lmin, lmax, err, seed):
    from swmapper_gb300 import synth
    reads, lens, _, _ = synth.reads(g, n, lmin, lmax, err, seed=seed, stride=256)
    return reads, lens


def run_serving(args):
    """The serving configuration alone: the human-scale index resident, the
    request loop under Poisson arrivals (serving_loads)."""
    import swmapper_gb300 as swm
    ws, rank, local = dist_env()
    rt = cudart()
    rt.cudaSetDevice(local)
    w = WORKLOAD
    from swmapper_gb300 import synth
    g = synth.reference(w["genome_bp"], seed=w["genome_seed"], kind=w["genome_kind"])
    t0 = time.perf_counter()
    ix = swm.Index.build(g, k=w["k"], device=local)
    index_build_s = time.perf_counter() - t0
    res = serving_loads(swm, ix, g, args)
    line = {"metric": "batch latency p99 (serving)", "value": res["loads"][-1]["p99_ms"], "unit": "ms",
            "n_gpus": 1, "higher_is_better": False, "index_build_s": round(index_build_s, 3), "data": "synthetic",
            "config": {**WORKLOAD}, "serving": res}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ reference arm

def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import build as obuild
    from oracle import pyoracle as po
    w = WORKLOAD
    g, reads, lens, eper = make_workload(0)
    E = e_arg(eper)
    kind = "reference"
    t0 = time.perf_counter()
    exe = os.path.join(obuild.REF_DIR, "serial_index")
    with tempfile.TemporaryDirectory() as td:
        if po.have_ref() and os.path.exists(exe):
            fa = os.path.join(td, "g.fa")
            # records of at most 100 Mbp: serial_index reads each record with
            # kseq_read, whose int return value turns negative past 2^31 - 1
            # bases (kseq.h), and the builder then stops before indexing
            # anything. It indexes the concatenation of the records as one
            # stream, so the files equal those of a single record.
            rec = 100_000_000
            with open(fa, "wb") as f:
                for r0 in range(0, g.size, rec):
                    f.write(b">chr%d synthetic\n" % (r0 // rec + 1))
                    for i in range(r0, min(g.size, r0 + rec), 100_000):
                        f.write(g[i:min(i + 100_000, r0 + rec)].tobytes() + b"\n")
            prefix = os.path.join(td, "ix")
            subprocess.run([exe, "-i" + fa, "-p" + prefix, f"-s{w['k']}"], check=True, capture_output=True)
            arrays = {}
            for ext, dt in ((".hash_count", np.uint32), (".hash_offset", np.uint32), (".positions", np.uint32),
                            (".pos_lseeds", np.uint16), (".base_2bits", np.uint32), (".base_3bits", np.uint32)):
                arrays[ext[1:]] = np.fromfile(prefix + ext, dtype=dt)
        else:
            kind = "port"
            hix = po.build_index(g, w["k"])
            arrays = dict(hash_count=hix.hash_count, hash_offset=hix.hash_offset_end, positions=hix.positions,
                          pos_lseeds=hix.pos_lseeds, base_2bits=hix.base_2bits, base_3bits=hix.base_3bits)
    index_build_s = time.perf_counter() - t0
    mix = host_map_index(arrays, w["k"])
    threads = os.cpu_count() or 1
    # size one step to ~args.ref_step_seconds
    rate, n, _, kind2 = timed_cpu_sample(mix, reads, lens, E, threads, 1.0, eper)
    kind = kind if kind2 == "reference" else "port"
    per_step = int(min(reads.shape[0], max(1024, rate * args.ref_step_seconds)))
    total_mapped = 0
    tsum = 0.0
    off = 0
    for s in range(args.warmup + args.steps):
        lo = off % reads.shape[0]
        hi = min(reads.shape[0], lo + per_step)
        t0 = time.perf_counter()
        mapped, _ = cpu_map(mix, reads[lo:hi], lens[lo:hi], E, threads, None if eper is None else eper[lo:hi])
        dt = time.perf_counter() - t0
        off = hi
        if s >= args.warmup:
            total_mapped += mapped
            tsum += dt
    value = total_mapped / tsum
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(tsum / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded genome and reads of the workload's shapes; no public dataset)",
            "config": {**WORKLOAD, "parallelism": "host threads"},
            "index_build_s": round(index_build_s, 3),
            "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": f"{per_step} reads per step of the workload, {threads} threads"},
            "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="human",
                    help="benchmark configuration (default: human, the 3.1 Gbp headline line)")
    ap.add_argument("--block", type=int, default=None, help="reads per mapping block (default: the workload's)")
    ap.add_argument("--mappers", type=int, default=2, help="mappers taking the blocks in turn")
    ap.add_argument("--tune", type=int, default=1, help="autotune reads per block and mappers (1) or not (0)")
    ap.add_argument("--buckets", type=int, default=1,
                    help="group reads of different lengths into 32-bp length buckets (1) or not (0)")
    ap.add_argument("--e2e-steps", type=int, default=10,
                    help="passes over the reads in the end-to-end stream (pipeline fill and drain amortised over them)")
    ap.add_argument("--e2e-mappers", type=int, default=2, help="mappers in the end-to-end pipeline (>= 2)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-step-seconds", type=float, default=2.0)
    ap.add_argument("--parity-reads", type=int, default=20000,
                    help="reads of the timed workload compared with the reference's own mapper after the timing")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--requests", type=int, default=None, help="requests of the serving workload")
    ap.add_argument("--verify", choices=["head64", "head32", "stream8", "stream16", "pair16"], default="stream16",
                    help="form of the verification stage when the autotuner does not choose it per length bucket")
    ap.add_argument("--table", type=int, default=-1,
                    help="candidate table for k = 12: the library's choice (-1: built for genomes whose buckets "
                         "average 8 or more entries, when the device has room), always (1) or never (0)")
    ap.add_argument("--serving", type=int, default=1,
                    help="with the human-scale workload, also run the serving loads on its index (1) or not (0)")
    ap.add_argument("--serialize", type=int, default=0,
                    help="resident passes: the mappers' blocks run their kernels one block at a time (1) or side by side (0)")
    ap.add_argument("--e2e-serialize", type=int, default=1,
                    help="end-to-end pass: kernels one block at a time, copies overlapping (1), or side by side (0)")
    ap.add_argument("--index-load", type=int, default=1,
                    help="after the timing, save the index as files and time swm_index_open (1) or not (0)")
    ap.add_argument("--plain", type=int, default=1, help="also time the plain per-batch launch (1) or not (0)")
    ap.add_argument("--genome-bp", type=int, default=None, help="smaller genome for quick checks")
    ap.add_argument("--nreads", type=int, default=None, help="fewer reads for quick checks")
    args = ap.parse_args()
    WORKLOAD.clear()
    WORKLOAD.update(WORKLOADS[args.workload])
    if args.block is None:
        args.block = WORKLOAD["block"]
    if args.genome_bp is not None or args.nreads is not None:
        WORKLOAD.update(genome_bp=args.genome_bp or WORKLOAD["genome_bp"], reads=args.nreads or WORKLOAD["reads"])
        WORKLOAD["workload"] = (f"reduced check of {args.workload}: {WORKLOAD['genome_bp']} bp genome, "
                                f"{WORKLOAD['reads']} reads")
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "serving":
        run_serving(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

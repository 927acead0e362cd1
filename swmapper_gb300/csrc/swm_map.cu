// swm_map.cu -- GB300 mapping pipeline for one block of reads.
//
// The reference maps one read at a time on each of 64 CPEs
// (find_positions -> get_positions -> choose_seed / alignment_rmdup /
// banded_myers / align_reads / put_cigar, mapper_cpe.c:2592-229). Here the
// same per-(read, strand) semantics run as a sequence of data-parallel kernels
// over a whole block, each sized to its natural unit of work:
//
//   k_seed12   thread / item   read encodings, seed lookups, long-seed order,
//   (k_seed)                   flank codes            (mapper_cpe.c:1246-1401,
//                                                      2451-2499)
//   scan       chunk and element offsets per item
//   k_plan*    lane or warp /  the fetch schedule: 32-position chunks,
//              item            heap-ordered refills, batch boundaries
//                                                     (mapper_cpe.c:2124-2419)
//   k_cand /   warp / item     gather + position adjust + flank filter (or
//   k_cand_table               the candidate table's survivors) + per-batch
//                              sort-unique            (mapper_cpe.c:1893-2123)
//   scan       candidate offsets
//   k_compact  thread or warp  dense candidate list
//              / item
//   k_verify_stream   lane /   window, banded Myers 16 bases at a time with a
//   + k_verify_finish  cand    stop bound; last bases, final scan, Hamming
//   (or k_verify, two passes)  check               (mapper_cpe.c:229-660,
//                                                      1403-1435,1509-1586)
//   k_traceback thread / cand  traceback + CIGAR text (align_reads, mapper_cpe.c:229-517)
//   k_records  thread or warp  groups of 8, record flushes, dedup, primary
//              / item          flag (count pass, scan, write pass)
//                                                     (mapper_cpe.c:1437-1507,
//                                                      1753-1860)
//
// All sizes flow through device memory, so the host queues the whole block
// without synchronising; capacities are checked on the device and a block
// whose work outgrew a buffer is re-run with larger buffers.
#include <mutex>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "swm_common.cuh"

// item = 2 * read + strand (cur_read, mapper_cpe.c:2628)

enum { VR_FAIL = 0, VR_HAM = 1, VR_TB = 2, VR_INVALID = 3, VR_NEEDTB = 4 };
enum { OV_CHUNKS = 1, OV_ELEMS = 2, OV_CANDS = 4, OV_RECS = 8, OV_ARENA = 16, OV_BAD = 32 };
enum {
    ST_BATCHES = 0,
    ST_CELLS,
    ST_PASSED,
    ST_LOCS,
    ST_MAPPED,
    ST_STEPS, // Myers steps (read bases) run by k_verify
    ST_KEPT,  // positions the flank filter kept, before each batch's merge
    ST_N
};
// device totals (u32), written by the scans
enum {
    TOT_CHUNKS = 0, TOT_ELEMS, TOT_CANDS, TOT_RECS, TOT_WORDS, TOT_BYTES, TOT_ARENA, TOT_FLAGS, TOT_TB, TOT_SLOW,
    TOT_VQ, TOT_TBQ, // work-queue heads of k_verify and k_traceback
    TOT_VT, TOT_VTQ, // candidates alive after the head of verification, and their queue head
    TOT_PLN, TOT_PLQ,  // items with refills and at most 32 selected seeds, queue head of k_plan_lanes
    TOT_PLW, TOT_PLWQ, // items with refills and more selected seeds, queue head of k_plan
    TOT_CQ,            // queue head of the candidate stage (items)
    TOT_RQC, TOT_RQW,  // queue heads of the records count and write passes (groups of 32 items)
    TOT_N
};

// Next CAND_TAKE items of a warp in the candidate stage (head *q): items differ
// by a factor of a hundred in work (kept positions, batches), so warps take
// them from a queue in small groups instead of a fixed stride.
#define CAND_TAKE 4
__device__ __forceinline__ uint32_t warp_take_items(uint32_t *q) {
    uint32_t b = 0;
    if ((threadIdx.x & 31) == 0) b = atomicAdd(q, (uint32_t)CAND_TAKE);
    return __shfl_sync(0xffffffffu, b, 0);
}

// Next 32 work units of a warp from a device work queue (head *q): every lane
// gets the same base; the warp is done when it reaches n.
__device__ __forceinline__ uint32_t warp_take(uint32_t *q) {
    uint32_t b = 0;
    if ((threadIdx.x & 31) == 0) b = atomicAdd(q, 32u);
    return __shfl_sync(0xffffffffu, b, 0);
}

// 1 when the item's selected buckets form one batch whatever the refill
// order: no refills, or at most SWM_BATCH_POSITIONS - SWM_PER_FETCH + 1
// positions. alignment_rmdup refills while npos + 32 <= 2048 and
// 1 + 2 runs < 256 and flushes once either fails or the seed heap is empty;
// both only grow, and before the last refill npos <= nel - 1 and, with at
// most 64 seeds, runs <= nel / 32 + 64 - 1 < 127, so it refills until the
// heap is empty. That batch holds every chunk, its element 0 is the first
// seed's first position, and its candidates come out sorted and unique, so
// the heap's order changes nothing. 0 otherwise (k_plan counts the batches).
__device__ __forceinline__ uint32_t single_batch(uint32_t nref, uint32_t nel) {
    return nel > 0 && (nref == 0 || nel + SWM_PER_FETCH - 1 <= SWM_BATCH_POSITIONS) ? 1u : 0u;
}

#define ARENA_CAP_DEFAULT (1u << 20)

// The inputs of one block, in device memory so that the captured launch
// sequence of a mapper does not depend on them.
struct BlockParams {
    const char *reads;     // reads_num reads at a fixed stride
    const uint32_t *lens;  // their lengths
    const uint8_t *e;      // per-read thresholds, or null
    uint64_t stride;
    uint32_t nreads, nitems, errors, pad;
};

struct MapBufs {
    BlockParams *par;      // the block's inputs (device copy)
    // per item
    uint32_t *it_w;        // items * 32: [0..15] Myers planes, [16..31] Hamming planes
    uint2 *sel;            // items * 64: (bucket start, count) of the seed of long seed l, shift t at 4 l + t
    uint8_t *sel_fl;       // items * 64: its read flank bits rl | rh << 3 (rl, rh: 3 bits each)
    uint32_t *sel_key;     // items * 64: its candidate-table key (k = 12)
    unsigned long long *it_perm; // items: selected slot i is record 4 * nibble(i / 4) + i % 4
    uint8_t *it_nsel, *it_e;
    uint32_t *it_nch, *it_nel, *it_nbat;
    uint32_t *it_choff, *it_eloff; // items + 1
    uint32_t *it_nrec, *it_nw, *it_nb;
    uint32_t *it_recoff, *it_woff, *it_boff; // items + 1
    uint32_t *it_ncand, *it_coff;            // candidates per item, dense offsets (items + 1)
    uint32_t *plan_list; // items with refills: k_plan_lanes' from the front, k_plan's from the back (items)
    // per chunk / batch slot (cap_chunks; batch b of an item sits at slot it_choff + b)
    uint32_t *ch_g, *ch_meta;
    uint32_t *bt_c0, *bt_c1, *bt_e0, *bt_cnt; // cap_chunks + cap_items slots
    uint32_t *sort_scratch; // SWM_BATCH_POSITIONS words per resident k_cand warp
    // upper-bound candidates (cap_elems)
    uint32_t *cand_ub;
    // dense candidates (cap_cands)
    uint32_t *cc_pos, *cc_item;
    uint8_t *vr_flag;
    uint32_t *vr_loc;
    int32_t *vr_err, *vr_mloc;
    uint16_t *vr_tlen;
    uint8_t *vr_cig;  // cap_cands * SWM_CIGAR_SLOT
    uint32_t *vr_aoff;
    uint8_t *arena;   // long CIGAR texts
    uint16_t *unm;       // bit j of halfword w: read 16 w + j has no location (cap_items / 32 + 1)
    uint2 *vt_x;         // candidates alive after the head of verification: (candidate, ones) (cap_cands)
    uint4 *vt_st;        // and their Myers state (VP, VN, checkpoint before base 16) (cap_cands)
    uint4 *vt_cp;        // and the checkpoints before bases 32 and 48 (cap_cands)
    uint32_t *tb_list;   // candidates that need a traceback (cap_cands)
    uint32_t *tb_cp;     // (VP, VN) before every 16th read base of each of them (cap_cands * 32)
    uint32_t *plan_keys; // heap keys of items with more than PLAN_KEYS of them (cap_chunks)
    uint32_t *slow_list; // tracebacks whose route outgrew the fast path (cap_cands)
    // records
    uint32_t *out_w;  // cap_words
    uint8_t *out_c;   // cap_bytes
    uint32_t *rec_woff, *rec_boff, *rec_blen; // cap_recs
    // bookkeeping
    uint32_t *tot;    // TOT_N
    unsigned long long *stat; // ST_N
    uint32_t *scan_tmp;
};

// Forms of the verification stage (swm_mapper_tuning); all give the same
// results. HEAD32 / HEAD64: a head pass over the first 32 / 64 bases of every
// candidate, then a tail pass over the ones still alive. STREAM8 / STREAM16:
// k_verify_stream with its stop test every 8 / 16 bases, then the finishing
// pass. PAIR16: k_verify_pair (two candidates per lane, stop test every 16
// bases), then the finishing pass; a block that may hold a threshold above 7
// (per-read thresholds, or e > 7) runs STREAM16 instead.
enum { VMODE_HEAD32 = 0, VMODE_HEAD64, VMODE_STREAM8, VMODE_STREAM16, VMODE_PAIR16, VMODE_N };

struct swm_mapper {
    swm_index *ix;
    int device;
    cudaStream_t st;
    uint64_t max_reads;
    uint64_t cap_items, cap_chunks, cap_elems, cap_cands, cap_recs, cap_words, cap_bytes, cap_arena;
    uint64_t stride_cap;
    MapBufs b;
    // inputs (device) and pinned staging
    char *d_reads;
    uint32_t *d_lens;
    uint8_t *d_e;
    char *h_reads;
    uint32_t *h_lens;
    uint8_t *h_e;
    // pinned result staging
    uint32_t *h_w, *h_rw, *h_rb, *h_rl;
    uint16_t *h_unm;
    uint8_t *h_c;
    uint64_t h_cap_w, h_cap_c, h_cap_rw, h_cap_rb, h_cap_rl, h_cap_items;
    uint32_t *h_tot;           // pinned copy of B.tot
    unsigned long long *h_stat; // pinned copy of B.stat
    // state of the block in flight / last block
    const char *cur_reads;
    const uint32_t *cur_lens;
    const uint8_t *cur_e;
    uint64_t cur_stride, cur_n;
    uint32_t cur_errors;
    int pending; // submitted, not yet waited: 1 host inputs, 2 device inputs
    const char *dev_reads;     // device inputs of a pending swm_map_device_submit
    const uint32_t *dev_lens;
    const uint8_t *dev_e;
    uint64_t h2d_pending; // bytes copied in for the block being mapped
    int have_result;
    uint32_t tot[TOT_N];
    swm_map_stats stats;
    cudaEvent_t ev[9];
    float stage_ms[8];
    uint64_t launches;
    // the block's launch sequence, captured once per buffer set and read
    // length class; the block's inputs reach it through B.par
    BlockParams *h_par;        // pinned
    // one captured graph per (seed-kernel class, verification head length),
    // with the buffer and candidate-table generations it was captured with
    cudaGraphExec_t gx[3][VMODE_N];
    uint32_t gx_gen[3][VMODE_N], gx_tab[3][VMODE_N];
    uint32_t gen;              // buffer generation now
    int vmode;                 // verification form (VMODE_*)
};

// ======================================================================
// device helpers
// ======================================================================

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ uint32_t lanemask_lt() { // lanes below this one
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ void warp_add_u64(unsigned long long *dst, unsigned long long v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
    if (lane_id() == 0 && v) atomicAdd(dst, v);
}

__device__ __forceinline__ uint32_t base_code_c(char ch) {
    return ch == 'A' ? 0u : ch == 'C' ? 1u : ch == 'G' ? 2u : ch == 'T' ? 3u : 1u;
}

__device__ __forceinline__ bool is_acgt(char ch) { return ch == 'A' || ch == 'C' || ch == 'G' || ch == 'T'; }

__device__ __forceinline__ char comp_base(char c) {
    return c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : c == 'T' ? 'A' : c;
}

// compress the even bits of x (16 of them) into the low half
__device__ __forceinline__ uint32_t even_bits(uint32_t x) {
    x &= 0x55555555u;
    x = (x | (x >> 1)) & 0x33333333u;
    x = (x | (x >> 2)) & 0x0f0f0f0fu;
    x = (x | (x >> 4)) & 0x00ff00ffu;
    x = (x | (x >> 8)) & 0x0000ffffu;
    return x;
}

// spread the low 16 bits of x to the even bit positions
__device__ __forceinline__ uint32_t spread_bits(uint32_t x) {
    x &= 0x0000ffffu;
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

struct ReadView { // base i of the strand being mapped (reverse_read, mapper_cpe.c:2429-2450)
    const char *src;
    uint32_t L, strand;
    __device__ __forceinline__ char operator()(uint32_t i) const {
        return strand ? comp_base(src[L - 1 - i]) : src[i];
    }
};

// The rolling seed of long seed l at shift s in closed form: base p of the
// window enters with its code, or, when it is not A/C/G/T, with d % 4 where
// d = p - l (k + 3) if d < k (built at shift 0, mapper_cpe.c:1294 with i = d)
// and (k - 1) % 4 otherwise (added at a later shift with i = k - 1).
__device__ __forceinline__ uint32_t seed_closed(const ReadView &rv, uint32_t k, uint32_t l, uint32_t s) {
    const uint32_t p0 = l * (k + SWM_SEED_STEP - 1);
    uint32_t seed = 0;
    for (uint32_t t = 0; t < k; t++) {
        const uint32_t d = s + t;
        const char ch = rv(p0 + d);
        const uint32_t c = is_acgt(ch) ? base_code_c(ch) : (d < k ? d % 4 : (k - 1) % 4);
        seed |= c << (2 * t);
    }
    return seed;
}

// True once any earlier stage of this block ran out of a buffer or met an
// input outside the envelope: later stages then skip their work (their
// inputs may be partial) and the host re-runs or rejects the block.
__device__ __forceinline__ bool block_failed(const MapBufs &B, uint64_t cap_chunks, uint64_t cap_elems,
                                             uint64_t cap_cands) {
    return B.tot[TOT_FLAGS] != 0 || B.tot[TOT_CHUNKS] > cap_chunks || B.tot[TOT_ELEMS] > cap_elems ||
           B.tot[TOT_CANDS] > cap_cands;
}

// ======================================================================
// k_seed: one warp per (read, strand)
// ======================================================================
//
// choose_seed / get_seed_from_reads (mapper_cpe.c:1246-1401) encode the read
// with a state machine whose main loop visits positions 0, 1, ..., P in
// order (P = 15 nl - 1, or the last base of the first call whose tail test
// L - rp < k fires; only calls of the last long seed can fire it). Up to P
// the bit planes hold the bases' codes and every complete 2-bit word is the
// interleave of the planes; the partial word is not yet written. The lanes
// compute that state with ballots; one lane then replays the rest of the
// state machine literally (the tail encoder re-runs and rewrites the last
// 2-bit words, mapper_cpe.c:1312-1362) -- at most four tails of < k bases.

#define SEED_WARPS 4

// Shared state of one warp: 32 items, word w of item t at [w][(t + w) % 32].
// The skew keeps both access patterns free of bank conflicts: all lanes on
// one item reading different words (phases A and C), and each lane on its
// own item (phase B).
struct SeedSmem {
    uint32_t pl[16][32];   // [2b] lo / [2b + 1] hi plane of bases 32b .. 32b + 31
    uint32_t w2[16][32];   // 2-bit words, 16 bases each
    uint32_t cnt[16][32];  // bucket counts summed per long seed
    uint32_t idx[16][32];  // long seed order (exchange sort)
};
#define SK(arr, w, t) S.arr[(w)][((t) + (w)) & 31]

__global__ void __launch_bounds__(SEED_WARPS * 32) k_seed(const uint32_t *__restrict__ off, uint32_t k, MapBufs B) {
    __shared__ SeedSmem sm_all[SEED_WARPS];
    const BlockParams P = *B.par;
    const char *__restrict__ reads = P.reads;
    const uint32_t *__restrict__ lens = P.lens;
    const uint8_t *__restrict__ e_arr = P.e;
    const uint64_t stride = P.stride;
    const uint32_t nreads = P.nreads, e_glob = P.errors;
    const uint32_t lane = lane_id(), wib = threadIdx.x >> 5;
    SeedSmem &S = sm_all[wib];
    uint2 *__restrict__ sel = B.sel;
    const uint32_t nitems = 2 * nreads;
    const uint32_t klong = k + SWM_SEED_STEP - 1;
    const uint32_t kmask = (1u << k) - 1, lmask = (1u << klong) - 1, rmask = (1u << (SWM_SEED_STEP - 1)) - 1;
    for (uint32_t g0 = (blockIdx.x * SEED_WARPS + wib) * 32; g0 < nitems; g0 += gridDim.x * SEED_WARPS * 32) {
        // ---- phase A, item by item, lanes in parallel: planes, clean 2-bit
        // words, bucket counts per long seed
        uint32_t my_P = 0, my_jt = 0xffffffffu, my_nl = 0, my_L = 0, my_ok = 0, my_hasn = 0;
        for (uint32_t t = 0; t < 32; t++) {
            const uint32_t item = g0 + t;
            if (item >= nitems) break;
            const uint32_t r = item >> 1, strand = item & 1;
            const uint32_t L = lens[r];
            const uint32_t e = e_arr ? e_arr[r] : e_glob;
            const bool ok = !(L > SWM_MAX_READ_LEN || L > stride || L / klong > 16 || e > SWM_MAX_ERRORS);
            if (!ok) {
                if (lane == t) my_ok = 0;
                continue;
            }
            const ReadView rv{reads + (uint64_t)r * stride, L, strand};
            const uint32_t nl = L / klong;
            // first tail trigger (only calls of the last long seed can fire it)
            uint32_t jt = 0xffffffffu, P = nl ? nl * klong - 1 : 0u;
            if (nl) {
                for (uint32_t sft = 0; sft < SWM_SEED_STEP; sft++) {
                    const uint32_t rp = (nl - 1) * klong + sft + k - 1;
                    if (L - rp < k) {
                        jt = (nl - 1) * SWM_SEED_STEP + sft;
                        P = rp;
                        break;
                    }
                }
            }
            const uint32_t vis = nl ? (jt != 0xffffffffu ? L : nl * klong) : 0u;
            const uint32_t seedspan = nl * klong;
            bool has_n = false;
#pragma unroll
            for (uint32_t b = 0; b < 8; b++) {
                const uint32_t p = 32 * b + lane;
                uint32_t code = 0;
                bool n = false;
                if (p < vis) {
                    const char ch = rv(p);
                    code = base_code_c(ch);
                    n = !is_acgt(ch) && p < seedspan;
                }
                const uint32_t lo = __ballot_sync(0xffffffffu, code & 1u), hi = __ballot_sync(0xffffffffu, code >> 1);
                has_n |= __any_sync(0xffffffffu, n);
                if (lane == 2 * b) SK(pl, 2 * b, t) = lo;
                if (lane == 2 * b + 1) SK(pl, 2 * b + 1, t) = hi;
            }
            __syncwarp();
            if (lane < 16) { // complete words up to P from the planes, the rest 0
                uint32_t wv = 0;
                if (nl && 16 * lane + 15 <= P) {
                    const uint32_t sh = (lane & 1) * 16;
                    const uint32_t lo = (SK(pl, 2 * (lane >> 1), t) >> sh) & 0xffffu;
                    const uint32_t hi = (SK(pl, 2 * (lane >> 1) + 1, t) >> sh) & 0xffffu;
                    wv = spread_bits(lo) | (spread_bits(hi) << 1);
                }
                SK(w2, lane, t) = wv;
            }
            // bucket counts of every seed, summed per long seed (choose_seed, 1372-1390)
            const uint32_t ns_all = nl * SWM_SEED_STEP;
            for (uint32_t j0 = 0; j0 < ns_all; j0 += 32) {
                const uint32_t j = j0 + lane;
                uint32_t c = 0;
                if (j < ns_all) {
                    const uint32_t l = j / SWM_SEED_STEP, sft = j % SWM_SEED_STEP;
                    uint32_t sd;
                    if (!has_n) {
                        const uint32_t o = l * klong, wj = o >> 5, sh = o & 31;
                        const uint32_t nlo = wj + 1 < 8 ? SK(pl, 2 * (wj + 1), t) : 0u;
                        const uint32_t nhi = wj + 1 < 8 ? SK(pl, 2 * (wj + 1) + 1, t) : 0u;
                        const uint32_t lo = (swm_fsr(SK(pl, 2 * wj, t), nlo, sh) >> sft) & kmask;
                        const uint32_t hi = (swm_fsr(SK(pl, 2 * wj + 1, t), nhi, sh) >> sft) & kmask;
                        sd = spread_bits(lo) | (spread_bits(hi) << 1);
                    } else {
                        sd = seed_closed(rv, k, l, sft);
                    }
                    c = off[sd + 1] - off[sd];
                }
                c += __shfl_xor_sync(0xffffffffu, c, 1);
                c += __shfl_xor_sync(0xffffffffu, c, 2);
                if (j < ns_all && (j % SWM_SEED_STEP) == 0) SK(cnt, j / SWM_SEED_STEP, t) = c;
            }
            if (lane == t) {
                my_P = P;
                my_jt = jt;
                my_nl = nl;
                my_L = L;
                my_ok = 1;
                my_hasn = has_n ? 1u : 0u;
            }
        }
        __syncwarp();
        // ---- phase B, lane t works on item t: exchange sort of the long
        // seeds (1391-1399) and the literal replay of the tail encoder
        // (1312-1362) from the first call whose tail test fires
        if (g0 + lane < nitems && my_ok) {
            const uint32_t t = lane, nl = my_nl, L = my_L, P = my_P;
            for (uint32_t a = 0; a < 16; a++) SK(idx, a, t) = a;
            for (uint32_t a = 0; a < nl; a++)
                for (uint32_t m = a + 1; m < nl; m++)
                    if (SK(cnt, a, t) > SK(cnt, m, t)) {
                        uint32_t x = SK(cnt, a, t);
                        SK(cnt, a, t) = SK(cnt, m, t);
                        SK(cnt, m, t) = x;
                        x = SK(idx, a, t);
                        SK(idx, a, t) = SK(idx, m, t);
                        SK(idx, m, t) = x;
                    }
            if (my_jt != 0xffffffffu) {
                auto code_at = [&](uint32_t q) -> uint32_t {
                    return ((SK(pl, 2 * (q >> 5), t) >> (q & 31)) & 1u) |
                           (((SK(pl, 2 * (q >> 5) + 1, t) >> (q & 31)) & 1u) << 1);
                };
                uint32_t acc = 0;
                if (P % 16 != 15)
                    for (uint32_t q = P & ~15u; q <= P; q++) acc |= code_at(q) << ((q % 16) * 2);
                for (uint32_t j = my_jt; j < nl * SWM_SEED_STEP; j++) {
                    const uint32_t rp = (j / SWM_SEED_STEP) * klong + j % SWM_SEED_STEP + k - 1;
                    if (j > my_jt) { // the one base this call's main loop adds
                        acc |= code_at(rp) << ((rp % 16) * 2);
                        if (rp % 16 == 15) {
                            SK(w2, rp / 16, t) = acc;
                            acc = 0;
                        }
                    }
                    for (uint32_t q = rp; q < L; q++) { // tail encoder, re-run from rp
                        acc |= code_at(q) << ((q % 16) * 2);
                        if (q % 16 == 15) {
                            SK(w2, q / 16, t) = acc;
                            acc = 0;
                        }
                    }
                    SK(w2, (L - 1) / 16, t) = acc;
                }
            }
        }
        __syncwarp();
        // ---- phase C, item by item, lanes in parallel: selected slots (the
        // (e + 1) rarest long seeds x 4 shifts, alignment_rmdup 2194-2196;
        // slots past nl read count 0), bucket ranges, flank codes, read words
        for (uint32_t t = 0; t < 32; t++) {
            const uint32_t item = g0 + t;
            if (item >= nitems) break;
            const uint32_t ok = __shfl_sync(0xffffffffu, my_ok, t);
            const uint32_t r = item >> 1, strand = item & 1;
            const uint32_t e = e_arr ? e_arr[r] : e_glob;
            if (!ok) {
                if (lane == 0) {
                    atomicOr(&B.tot[TOT_FLAGS], OV_BAD);
                    B.it_nsel[item] = 0;
                    B.it_e[item] = 0;
                    B.it_nch[item] = 0;
                    B.it_nel[item] = 0;
                    B.it_nbat[item] = 0;
                }
                continue;
            }
            const uint32_t nl = __shfl_sync(0xffffffffu, my_nl, t);
            const uint32_t L = __shfl_sync(0xffffffffu, my_L, t);
            const bool has_n = __shfl_sync(0xffffffffu, my_hasn, t) != 0;
            const ReadView rv{reads + (uint64_t)r * stride, L, strand};
            const uint32_t nsl = (e + 1 < nl) ? e + 1 : nl;
            const uint32_t ns = nsl * SWM_SEED_STEP;
            const uint64_t sb = (uint64_t)item * SWM_MAX_SEL;
            uint32_t nref = 0;
            uint64_t nel = 0; // saturated below: sums past 32 bits are reported, not wrapped
            for (uint32_t i0 = 0; i0 < ns; i0 += 32) {
                const uint32_t i = i0 + lane;
                if (i < ns) {
                    const uint32_t l = SK(idx, i / SWM_SEED_STEP, t), sft = i % SWM_SEED_STEP;
                    const uint32_t o = l * klong, wj = o >> 5, sh = o & 31;
                    const uint32_t nlo = wj + 1 < 8 ? SK(pl, 2 * (wj + 1), t) : 0u;
                    const uint32_t nhi = wj + 1 < 8 ? SK(pl, 2 * (wj + 1) + 1, t) : 0u;
                    const uint32_t lr = swm_fsr(SK(pl, 2 * wj, t), nlo, sh) & lmask; // set_read_long_seeds, 2474-2478
                    const uint32_t hr = swm_fsr(SK(pl, 2 * wj + 1, t), nhi, sh) & lmask;
                    const uint32_t sd = has_n ? seed_closed(rv, k, l, sft)
                                              : (spread_bits((lr >> sft) & kmask) | (spread_bits((hr >> sft) & kmask) << 1));
                    const uint32_t o0 = off[sd], c = off[sd + 1] - o0;
                    const uint32_t m = (1u << sft) - 1, kk = k + sft;
                    const uint32_t rl = ((lr & m) | ((lr >> kk) << sft)) & rmask; // 2483-2495
                    const uint32_t rh = ((hr & m) | ((hr >> kk) << sft)) & rmask;
                    sel[sb + SWM_SEED_STEP * l + sft] = make_uint2(o0, c);
                    B.sel_fl[sb + SWM_SEED_STEP * l + sft] = (uint8_t)(rl | (rh << 3));
                    nref += c > SWM_PER_FETCH ? (c - 1) / SWM_PER_FETCH : 0u;
                    nel += c;
                }
            }
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
                nref += __shfl_xor_sync(0xffffffffu, nref, d);
                nel += __shfl_xor_sync(0xffffffffu, nel, d);
            }
            if (nel > SWM_SCAN_SATURATED) nel = SWM_SCAN_SATURATED;
            // read words: [0..15] Myers planes from the 2-bit words, [16..31] Hamming planes
            uint32_t ow;
            if (lane < 16) {
                const uint32_t b = lane >> 1, hi = lane & 1;
                ow = even_bits(SK(w2, 2 * b, t) >> hi) | (even_bits(SK(w2, 2 * b + 1, t) >> hi) << 16);
            } else {
                ow = SK(pl, lane - 16, t);
            }
            B.it_w[(uint64_t)item * 32 + lane] = ow;
            if (lane == 0) {
                B.it_nsel[item] = (uint8_t)ns;
                unsigned long long perm = 0;
                for (uint32_t a = 0; a < nsl; a++) perm |= (unsigned long long)SK(idx, a, t) << (4 * a);
                B.it_perm[item] = perm;
                B.it_e[item] = (uint8_t)e;
                B.it_nch[item] = nref;                  // refill chunks (beyond the first chunk of each seed)
                B.it_nel[item] = (uint32_t)nel;
                B.it_nbat[item] = single_batch(nref, (uint32_t)nel); // k_plan sets it for the other items with refills
            }
        }
        __syncwarp();
    }
}

// ======================================================================
// k_seed12: one thread per (read, strand), k = 12
// ======================================================================
//
// The same outputs as k_seed with every register array indexed at compile
// time. The two threads of a read (strands 0 and 1 are adjacent lanes) decode
// alternate words of it and exchange the halves; the reverse strand is the
// bit reverse of the forward planes. Seed codes come from interleaved 2-bit
// words of the strand (one funnel shift per seed), so every bucket lookup of
// a read issues back to back. Every seed's record (bucket start, count,
// flank bits) is written at slot 4 l + shift as soon as its lookup returns;
// the selection is then only the rank order of the long seeds, stored as a
// permutation (sel_slot), so no lookup is repeated and no shared memory
// limits the occupancy. The literal tail replay touches at most two 2-bit
// words (P >= L - 11), kept in registers.

#define K12 12u
#define KL12 15u
#define SEED12_THREADS 64
// resident blocks per SM the register budget of each k_seed12 is sized for
// (0: the compiler's choice). The short-read kernel is latency-bound on its
// bucket-offset lookups: 16 blocks (64 registers, a few spills) keep twice as
// many lookups in flight as its natural 80 registers and run 20-25% faster;
// the 16-long-seed kernel loses more to spills than it gains.
#ifndef SEED12_MIN_BLOCKS_10
#define SEED12_MIN_BLOCKS_10 16
#endif
#ifndef SEED12_MIN_BLOCKS_16
#define SEED12_MIN_BLOCKS_16 0
#endif
#define SEED12_BOUNDS __launch_bounds__(SEED12_THREADS, NL == 10 ? SEED12_MIN_BLOCKS_10 : SEED12_MIN_BLOCKS_16)

// 4 read bytes -> 4 lo bits, 4 hi bits, 4 "is A/C/G/T" bits (base j of the
// word at bit j). Code ((c >> 1) ^ (c >> 2)) & 3 maps A C G T to 0 1 2 3;
// anything else encodes as C (lo 1, hi 0), mapper_cpe.c:1293-1300.
__device__ __forceinline__ void decode4(uint32_t w, uint32_t &lo, uint32_t &hi, uint32_t &ok) {
    const uint32_t t = (w >> 1) ^ (w >> 2);
    const uint32_t acgt = __vcmpeq4(w, 0x41414141u) | __vcmpeq4(w, 0x43434343u) | __vcmpeq4(w, 0x47474747u) |
                          __vcmpeq4(w, 0x54545454u);
    const uint32_t okb = acgt & 0x01010101u;
    const uint32_t lob = (t & okb) | (~acgt & 0x01010101u);
    const uint32_t hib = (t >> 1) & okb;
    lo = (lob * 0x10204080u) >> 28;
    hi = (hib * 0x10204080u) >> 28;
    ok = (okb * 0x10204080u) >> 28;
}

// 2-bit codes an N takes at each position of the seed at shift sft: d % 4
// for d = sft + t inside the first k bases, (k - 1) % 4 past them
// (mapper_cpe.c:1294).
__host__ __device__ constexpr uint32_t nfill12(uint32_t sft) {
    uint32_t w = 0;
    for (uint32_t t = 0; t < K12; t++) {
        const uint32_t d = sft + t;
        w |= (d < K12 ? d % 4u : (K12 - 1u) % 4u) << (2u * t);
    }
    return w;
}

// Bucket offsets are read through an L2 evict-last policy: the 64 MB table
// stays in L2 while reads and records stream past it.
__device__ __forceinline__ uint64_t l2_keep_policy() {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ uint32_t ld_keep(const uint32_t *p, uint64_t pol) {
    uint32_t v;
    asm("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ uint2 ld_keep2(const uint32_t *p, uint64_t pol) { // p 8-byte aligned
    uint2 v;
    asm("ld.global.nc.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;" : "=r"(v.x), "=r"(v.y) : "l"(p), "l"(pol));
    return v;
}

// Start and count of bucket sd: one 8-byte load holds off[sd] and off[sd + 1]
// when sd is even; an odd sd takes off[sd + 1] from a second load.
__device__ __forceinline__ void bucket_range(const uint32_t *__restrict__ off, uint32_t sd, uint64_t pol,
                                             uint32_t &o0, uint32_t &c) {
    const bool odd = sd & 1u;
    const uint2 v = ld_keep2(off + (sd & ~1u), pol);
    const uint32_t w = odd ? ld_keep(off + sd + 1, pol) : 0u;
    o0 = odd ? v.y : v.x;
    c = (odd ? w : v.y) - o0;
}

// Seed code of the seed at read offset o (12 bases from o) from the
// interleaved words w0 = word o / 16 and w1 = the next one; with N bases
// (nk = the "not A/C/G/T" bits of bases o .. o + 11) the N positions take
// their code nfill12(sft).
__device__ __forceinline__ uint32_t seed12_code(uint32_t w0, uint32_t w1, uint32_t o) {
    const uint32_t sh = 2 * (o & 15);
    return (sh ? __funnelshift_r(w0, w1, sh) : w0) & 0xffffffu;
}
__device__ __forceinline__ uint32_t seed12_nfix(uint32_t sd, uint32_t nk, uint32_t sft) {
    const uint32_t M = spread_bits(nk & 0xfffu) * 3u;
    return (sd & ~M) | (nfill12(sft) & M);
}

// Record of every seed of long seeds 0 .. NL-1 at slot 4 l + shift: (bucket
// start, count) in rec and the flank byte rl | rh << 3 in byte 4 l + shift of
// flw, where rl / rh are the lo / hi bits of the 3 long-seed bases outside
// the 12-mer (set_read_long_seeds, 2474-2478). cnt gets the bucket counts summed per
// long seed (choose_seed, 1372-1390), nref the refill chunks. Every lookup is
// independent, so they all issue back to back.
template <int NL, bool HASN, bool KEYS>
__device__ __forceinline__ void seed12_records(const uint32_t (&iw)[NL], const uint32_t (&plo)[8],
                                               const uint32_t (&phi)[8], const uint32_t (&pok)[8], uint32_t nl,
                                               const uint32_t *__restrict__ off, uint64_t pol,
                                               uint2 *__restrict__ rec, uint32_t *__restrict__ flw,
                                               uint32_t *__restrict__ keys, uint32_t (&cnt)[NL],
                                               uint32_t (&nref)[NL]) {
    static_assert(NL % 2 == 0, "flank words are stored in pairs");
    uint32_t pf = 0;
#pragma unroll
    for (int l = 0; l < NL; l++) {
        const bool act = (uint32_t)l < nl;
        const uint32_t ob = KL12 * l, wj0 = ob >> 5, sh0 = ob & 31;
        const uint32_t nlo = wj0 + 1 < 8 ? plo[wj0 + 1] : 0u, nhi = wj0 + 1 < 8 ? phi[wj0 + 1] : 0u;
        const uint32_t lr = (sh0 ? __funnelshift_r(plo[wj0], nlo, sh0) : plo[wj0]) & 0x7fffu;
        const uint32_t hr = (sh0 ? __funnelshift_r(phi[wj0], nhi, sh0) : phi[wj0]) & 0x7fffu;
        uint32_t csum = 0, rsum = 0, f = 0, po = 0, pc = 0, kk4[SWM_SEED_STEP];
#pragma unroll
        for (uint32_t sft = 0; sft < SWM_SEED_STEP; sft++) {
            const uint32_t o = ob + sft, w = o >> 4;
            uint32_t sd = seed12_code(iw[w], (w + 1 < (uint32_t)NL) ? iw[w + 1] : 0u, o);
            if (HASN) {
                const uint32_t wj = o >> 5, s5 = o & 31;
                const uint32_t nx = wj + 1 < 8 ? pok[wj + 1] : 0xffffffffu;
                sd = seed12_nfix(sd, ~(s5 ? __funnelshift_r(pok[wj], nx, s5) : pok[wj]), sft);
            }
            sd = act ? sd : 0u;
            uint32_t o0, c;
            bucket_range(off, sd, pol, o0, c);
            const uint32_t m = (1u << sft) - 1, kk = K12 + sft;
            const uint32_t rl = ((lr & m) | ((lr >> kk) << sft)) & 7u;
            const uint32_t rh = ((hr & m) | ((hr >> kk) << sft)) & 7u;
            if (sft & 1) // two records per 16-byte store
                __stcs(reinterpret_cast<uint4 *>(rec) + ((SWM_SEED_STEP * l + sft) >> 1), make_uint4(po, pc, o0, c));
            po = o0;
            pc = c;
            f |= (rl | (rh << 3)) << (8 * sft);
            if (KEYS) kk4[sft] = swm_ctab_key(sd, sft, rl | (rh << 3));
            csum += c;
            rsum += c > SWM_PER_FETCH ? (c - 1) / SWM_PER_FETCH : 0u;
        }
        if (l & 1) __stcs(reinterpret_cast<uint2 *>(flw) + (l >> 1), make_uint2(pf, f)); // two long seeds per store
        if (KEYS) __stcs(reinterpret_cast<uint4 *>(keys) + l, make_uint4(kk4[0], kk4[1], kk4[2], kk4[3]));
        pf = f;
        cnt[l] = act ? csum : 0u;
        nref[l] = act ? rsum : 0u;
    }
}

template <int NL, bool TABLE>
// Items whose read length is outside [lo_len, hi_len] belong to the other
// instantiation launched beside this one (reads of up to 164 bases take the
// 10-long-seed kernel, longer ones the 16-long-seed kernel). TABLE: the
// candidate table is in use, so each seed's table key is stored too.
__global__ void SEED12_BOUNDS k_seed12(const uint32_t *__restrict__ off, MapBufs B,
                                                           uint32_t lo_len, uint32_t hi_len) {
    const BlockParams P = *B.par;
    const char *__restrict__ reads = P.reads;
    const uint32_t *__restrict__ lens = P.lens;
    const uint8_t *__restrict__ e_arr = P.e;
    const uint64_t stride = P.stride;
    const uint32_t nreads = P.nreads, e_glob = P.errors;
    uint2 *__restrict__ sel = B.sel;
    uint32_t *__restrict__ it_w = B.it_w;
    const uint32_t tid = threadIdx.x;
    const uint32_t nitems = 2 * nreads;
    const char *const limit = reads + (uint64_t)nreads * stride;
    const uint64_t pol = l2_keep_policy();
    for (uint32_t item = blockIdx.x * blockDim.x + tid; item < nitems; item += gridDim.x * blockDim.x) {
        // items 2r and 2r + 1 sit in adjacent lanes (even block size and stride)
        const uint32_t pair = 3u << (lane_id() & ~1u);
        const uint32_t r = item >> 1, strand = item & 1;
        const uint32_t L = lens[r];
        if (L < lo_len || L > hi_len) continue; // both lanes of the read skip it
        const uint32_t e = e_arr ? e_arr[r] : e_glob;
        if (L > SWM_MAX_READ_LEN || L > stride || e > SWM_MAX_ERRORS || L > NL * KL12 + KL12 - 1) {
            atomicOr(&B.tot[TOT_FLAGS], OV_BAD);
            B.it_nsel[item] = 0;
            B.it_e[item] = 0;
            B.it_nch[item] = 0;
            B.it_nel[item] = 0;
            B.it_nbat[item] = 0;
            continue;
        }
        // ---- forward planes of the read bytes: this lane decodes words
        // 2 jj + strand, the other lane of the pair the rest
        uint32_t flo[8], fhi[8], fok[8];
#pragma unroll
        for (int b = 0; b < 8; b++) flo[b] = fhi[b] = fok[b] = 0;
        {
            const char *a = reads + (uint64_t)r * stride;
            const uintptr_t ua = (uintptr_t)a;
            const uint32_t *a0 = (const uint32_t *)(ua & ~(uintptr_t)3);
            const uint32_t sh = (uint32_t)(ua & 3) * 8;
            const char *end = a + L;
#pragma unroll
            for (int b = 0; b < 8; b++) {
                if (32 * b < (int)L) {
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const uint32_t j = 8 * b + 2 * q + strand; // word j: bytes 4j .. 4j + 3 of the read
                        const char *p0 = (const char *)(a0 + j), *p1 = (const char *)(a0 + j + 1);
                        const uint32_t w0 = (p0 < end && p0 < limit) ? __ldcs(a0 + j) : 0u;
                        const uint32_t w1 = (p1 < end && p1 < limit) ? __ldcs(a0 + j + 1) : 0u;
                        const uint32_t w = sh ? __funnelshift_r(w0, w1, sh) : w0;
                        uint32_t lo, hi, ok;
                        decode4(w, lo, hi, ok);
                        const uint32_t s = 4 * (2 * q + strand);
                        flo[b] |= lo << s;
                        fhi[b] |= hi << s;
                        fok[b] |= ok << s;
                    }
                }
            }
#pragma unroll
            for (int b = 0; b < 8; b++) {
                flo[b] |= __shfl_xor_sync(pair, flo[b], 1);
                fhi[b] |= __shfl_xor_sync(pair, fhi[b], 1);
                fok[b] |= __shfl_xor_sync(pair, fok[b], 1);
                // bases at or past L are not part of the read
                const int rem = (int)L - 32 * b;
                const uint32_t m = rem >= 32 ? 0xffffffffu : rem <= 0 ? 0u : ((1u << rem) - 1u);
                flo[b] &= m;
                fhi[b] &= m;
                fok[b] &= m;
            }
        }
        // ---- planes of the strand: reverse complement for strand 1
        // (reverse_read, 2429-2450: A<->T, C<->G, anything else kept)
        uint32_t plo[8], phi[8], pok[8];
        if (strand == 0) {
#pragma unroll
            for (int b = 0; b < 8; b++) {
                plo[b] = flo[b];
                phi[b] = fhi[b];
                pok[b] = fok[b];
            }
        } else {
            // base i of the strand = base L - 1 - i of the read: bit reverse the
            // 256-bit planes, then shift right by 256 - L (word steps of 4, 2,
            // 1 words as selects, then a funnel shift)
            const uint32_t sr = 256u - L, ws = sr >> 5, bs = sr & 31;
#pragma unroll
            for (int b = 0; b < 8; b++) {
                plo[b] = __brev(flo[7 - b]);
                phi[b] = __brev(fhi[7 - b]);
                pok[b] = __brev(fok[7 - b]);
            }
#pragma unroll
            for (int step = 4; step >= 1; step >>= 1) {
                const bool mv = (ws & step) != 0;
#pragma unroll
                for (int b = 0; b < 8; b++) {
                    const uint32_t nlo = b + step < 8 ? plo[b + step] : 0u;
                    const uint32_t nhi = b + step < 8 ? phi[b + step] : 0u;
                    const uint32_t nok = b + step < 8 ? pok[b + step] : 0u;
                    plo[b] = mv ? nlo : plo[b];
                    phi[b] = mv ? nhi : phi[b];
                    pok[b] = mv ? nok : pok[b];
                }
            }
#pragma unroll
            for (int b = 0; b < 8; b++) {
                const uint32_t nlo = b + 1 < 8 ? plo[b + 1] : 0u;
                const uint32_t nhi = b + 1 < 8 ? phi[b + 1] : 0u;
                const uint32_t nok = b + 1 < 8 ? pok[b + 1] : 0u;
                const uint32_t lo = bs ? __funnelshift_r(plo[b], nlo, bs) : plo[b];
                const uint32_t hi = bs ? __funnelshift_r(phi[b], nhi, bs) : phi[b];
                const uint32_t ok = bs ? __funnelshift_r(pok[b], nok, bs) : pok[b];
                plo[b] = lo ^ ok; // complement flips both bits of A/C/G/T only
                phi[b] = hi ^ ok;
                pok[b] = ok;
            }
        }
        const uint32_t nl = L / KL12;
        uint32_t jt = 0xffffffffu, P = nl ? nl * KL12 - 1 : 0u;
        if (nl) {
#pragma unroll
            for (uint32_t sft = 0; sft < SWM_SEED_STEP; sft++) {
                const uint32_t rp = (nl - 1) * KL12 + sft + K12 - 1;
                if (jt == 0xffffffffu && L - rp < K12) {
                    jt = (nl - 1) * SWM_SEED_STEP + sft;
                    P = rp;
                }
            }
        }
        const uint32_t vis = nl ? (jt != 0xffffffffu ? L : nl * KL12) : 0u;
        const uint32_t span = nl * KL12;
        bool has_n = false;
#pragma unroll
        for (int b = 0; b < 8; b++) { // planes hold the visited bases only; N flag over seed windows
            const int rem = (int)vis - 32 * b;
            const uint32_t m = rem >= 32 ? 0xffffffffu : rem <= 0 ? 0u : ((1u << rem) - 1u);
            const int rs = (int)span - 32 * b;
            const uint32_t ms = rs >= 32 ? 0xffffffffu : rs <= 0 ? 0u : ((1u << rs) - 1u);
            has_n |= ((~pok[b]) & ms) != 0;
            plo[b] &= m;
            phi[b] &= m;
            pok[b] |= ~m; // positions outside the visit are not N
        }
        // ---- interleaved 2-bit words of the strand (base 16 w + i at bits
        // 2i, 2i + 1)
        uint32_t iw[NL];
#pragma unroll
        for (int w = 0; w < NL; w++) {
            const uint32_t l16 = (w & 1) ? (plo[w >> 1] >> 16) : plo[w >> 1];
            const uint32_t h16 = (w & 1) ? (phi[w >> 1] >> 16) : phi[w >> 1];
            iw[w] = spread_bits(l16) | (spread_bits(h16) << 1);
        }
        // ---- Myers planes: complete 2-bit words up to P are the planes, the
        // partial word is unwritten; the tail replay rewrites words P/16 and
        // P/16 + 1 (the only ones it can touch)
        uint32_t mlo[8], mhi[8];
#pragma unroll
        for (int b = 0; b < 8; b++) {
            uint32_t m = 0;
            if (nl) {
                if (32 * b + 15 <= (int)P) m |= 0x0000ffffu;
                if (32 * b + 31 <= (int)P) m |= 0xffff0000u;
            }
            mlo[b] = plo[b] & m;
            mhi[b] = phi[b] & m;
        }
        if (jt != 0xffffffffu) {
            const uint32_t w0 = P >> 4;
            uint32_t wa = 0, wb = 0; // 2-bit words w0 and w0 + 1
            // the planes of bases 16 w0 .. 16 w0 + 31 (they cover L - 1)
            uint32_t pl0 = 0, pl1 = 0, ph0 = 0, ph1 = 0;
#pragma unroll
            for (int q = 0; q < 8; q++) { // masks, not indexing by w0
                const uint32_t m0 = ((uint32_t)q == (w0 >> 1)) ? 0xffffffffu : 0u;
                const uint32_t m1 = ((uint32_t)q == (w0 >> 1) + 1) ? 0xffffffffu : 0u;
                pl0 |= plo[q] & m0;
                ph0 |= phi[q] & m0;
                pl1 |= plo[q] & m1;
                ph1 |= phi[q] & m1;
            }
            const uint32_t base0 = 16 * w0, sh0 = (w0 & 1) * 16;
            const uint32_t lwin = __funnelshift_r(pl0, pl1, sh0), hwin = __funnelshift_r(ph0, ph1, sh0);
            auto code_at = [&](uint32_t q) -> uint32_t { // base q in [16 w0, 16 w0 + 31]
                const uint32_t t = q - base0;
                return ((lwin >> t) & 1u) | (((hwin >> t) & 1u) << 1);
            };
            auto put = [&](uint32_t q, uint32_t v) {
                if ((q >> 4) == w0) wa = v;
                else wb = v;
            };
            if (P % 16 == 15) {
                wa = spread_bits(lwin & 0xffffu) | (spread_bits(hwin & 0xffffu) << 1);
            }
            uint32_t acc = 0;
            if (P % 16 != 15)
                for (uint32_t q = base0; q <= P; q++) acc |= code_at(q) << ((q % 16) * 2);
            for (uint32_t j = jt; j < nl * SWM_SEED_STEP; j++) {
                const uint32_t rp = (j / SWM_SEED_STEP) * KL12 + j % SWM_SEED_STEP + K12 - 1;
                if (j > jt) { // the one base this call's main loop adds
                    acc |= code_at(rp) << ((rp % 16) * 2);
                    if (rp % 16 == 15) {
                        put(rp, acc);
                        acc = 0;
                    }
                }
                for (uint32_t q = rp; q < L; q++) { // tail encoder, re-run from rp
                    acc |= code_at(q) << ((q % 16) * 2);
                    if (q % 16 == 15) {
                        put(q, acc);
                        acc = 0;
                    }
                }
                put(L - 1, acc);
            }
            // write words w0 and w0 + 1 back into the Myers planes
            const uint32_t lo_a = even_bits(wa), hi_a = even_bits(wa >> 1);
            const uint32_t lo_b = even_bits(wb), hi_b = even_bits(wb >> 1);
#pragma unroll
            for (int b = 0; b < 8; b++) { // blend, no indexing by w0
                const uint32_t q0 = 2 * b, q1 = 2 * b + 1;
                const uint32_t ma = ((q0 == w0) ? 0x0000ffffu : 0u) | ((q1 == w0) ? 0xffff0000u : 0u);
                const uint32_t mb = ((q0 == w0 + 1) ? 0x0000ffffu : 0u) | ((q1 == w0 + 1) ? 0xffff0000u : 0u);
                const uint32_t la = lo_a | (lo_a << 16), ha = hi_a | (hi_a << 16);
                const uint32_t lb = lo_b | (lo_b << 16), hb = hi_b | (hi_b << 16);
                mlo[b] = (mlo[b] & ~(ma | mb)) | (la & ma) | (lb & mb);
                mhi[b] = (mhi[b] & ~(ma | mb)) | (ha & ma) | (hb & mb);
            }
        }
        uint4 *ow = reinterpret_cast<uint4 *>(it_w + (uint64_t)item * 32);
        // the seed records and read words stream out with an evict-first hint
        // (a block's are far larger than L2), keeping the bucket-offset table
        // the lookups hit in L2
        __stcs(ow + 0, make_uint4(mlo[0], mhi[0], mlo[1], mhi[1]));
        __stcs(ow + 1, make_uint4(mlo[2], mhi[2], mlo[3], mhi[3]));
        __stcs(ow + 2, make_uint4(mlo[4], mhi[4], mlo[5], mhi[5]));
        __stcs(ow + 3, make_uint4(mlo[6], mhi[6], mlo[7], mhi[7]));
        __stcs(ow + 4, make_uint4(plo[0], phi[0], plo[1], phi[1]));
        __stcs(ow + 5, make_uint4(plo[2], phi[2], plo[3], phi[3]));
        __stcs(ow + 6, make_uint4(plo[4], phi[4], plo[5], phi[5]));
        __stcs(ow + 7, make_uint4(plo[6], phi[6], plo[7], phi[7]));
        // ---- every seed's record, all lookups in flight together
        const uint64_t sb = (uint64_t)item * SWM_MAX_SEL;
        uint32_t CNT[NL], IDX[NL], REF[NL];
        uint32_t *flw = reinterpret_cast<uint32_t *>(B.sel_fl + sb);
        uint32_t *keys = B.sel_key + sb;
        if (has_n) seed12_records<NL, true, TABLE>(iw, plo, phi, pok, nl, off, pol, sel + sb, flw, keys, CNT, REF);
        else seed12_records<NL, false, TABLE>(iw, plo, phi, pok, nl, off, pol, sel + sb, flw, keys, CNT, REF);
#pragma unroll
        for (int l = 0; l < NL; l++) IDX[l] = l;
        // exchange sort (1391-1399), unrolled
#pragma unroll
        for (int a = 0; a < NL; a++) {
#pragma unroll
            for (int m2 = a + 1; m2 < NL; m2++) {
                const bool sw = ((uint32_t)m2 < nl) & (CNT[a] > CNT[m2]);
                const uint32_t ca = CNT[a], cm = CNT[m2], ia = IDX[a], im = IDX[m2], ra = REF[a], rm = REF[m2];
                CNT[a] = sw ? cm : ca;
                CNT[m2] = sw ? ca : cm;
                IDX[a] = sw ? im : ia;
                IDX[m2] = sw ? ia : im;
                REF[a] = sw ? rm : ra;
                REF[m2] = sw ? ra : rm;
            }
        }
        // ---- the (e + 1) rarest long seeds x 4 shifts (alignment_rmdup
        // 2194-2196): ranks 0 .. nsl - 1 of the sorted order
        const uint32_t nsl = (e + 1 < nl) ? e + 1 : nl;
        const uint32_t ns = nsl * SWM_SEED_STEP;
        uint32_t nref = 0;
        uint64_t nel = 0; // saturated below: sums past 32 bits are reported, not wrapped
        unsigned long long perm = 0;
#pragma unroll
        for (int a = 0; a < NL; a++) {
            nref += (uint32_t)a < nsl ? REF[a] : 0u;
            nel += (uint32_t)a < nsl ? CNT[a] : 0u;
            perm |= (unsigned long long)IDX[a] << (4 * a);
        }
        if (nel > SWM_SCAN_SATURATED) nel = SWM_SCAN_SATURATED;
        B.it_perm[item] = perm;
        B.it_nsel[item] = (uint8_t)ns;
        B.it_e[item] = (uint8_t)e;
        B.it_nch[item] = nref;
        B.it_nel[item] = (uint32_t)nel;
        B.it_nbat[item] = single_batch(nref, (uint32_t)nel); // k_plan sets it for the other items with refills
    }
}


// Record of selected slot i (rank i / 4, shift i % 4) in the item's sel
// records: k_seed12 writes every seed at 4 l + shift and the ranks as a
// permutation of the long seeds l.
__device__ __forceinline__ uint32_t sel_slot(unsigned long long perm, uint32_t i) {
    return (uint32_t)((perm >> (4 * (i >> 2))) & 15u) * SWM_SEED_STEP + (i & 3u);
}

// ======================================================================
// k_plan: the refill schedule of alignment_rmdup, one thread per item whose
// buckets need refills (some selected seed has more than 32 positions)
// ======================================================================

__device__ __forceinline__ uint32_t warp_scan_incl(uint32_t v) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, d);
        if ((int)lane_id() >= d) v += t;
    }
    return v;
}

// The items whose selected buckets need refills, compacted into the planners'
// work lists (warp-aggregated appends; order does not matter, items are
// independent): items with at most PLAN_LANE_SEEDS selected seeds from the
// front for k_plan_lanes, the others from the back for k_plan.
#define PLAN_LANE_SEEDS 32
// chunks: write the refill chunks of the single-batch items (the candidate
// kernel without the candidate table gathers from them; k_cand_table reads
// chunks only of items with several batches).
__global__ void __launch_bounds__(256) k_plan_list(MapBufs B, uint64_t cap_chunks, bool chunks) {
    const uint32_t nitems = B.par->nitems;
    const uint32_t lane = lane_id();
    for (uint32_t base = blockIdx.x * 256 + (threadIdx.x & ~31u); base < nitems; base += gridDim.x * 256) {
        const uint32_t item = base + lane;
        const bool has = item < nitems && B.it_nch[item] != 0 && B.it_nbat[item] == 0;
        const bool few = has && B.it_nsel[item] <= PLAN_LANE_SEEDS;
        const uint32_t mf = __ballot_sync(0xffffffffu, few), mm = __ballot_sync(0xffffffffu, has && !few);
        uint32_t af = 0, am = 0;
        if (lane == 0 && mf) af = atomicAdd(&B.tot[TOT_PLN], (uint32_t)__popc(mf));
        if (lane == 0 && mm) am = atomicAdd(&B.tot[TOT_PLW], (uint32_t)__popc(mm));
        af = __shfl_sync(0xffffffffu, af, 0);
        am = __shfl_sync(0xffffffffu, am, 0);
        if (few) B.plan_list[af + __popc(mf & lanemask_lt())] = item;
        if (has && !few) B.plan_list[nitems - 1 - (am + __popc(mm & lanemask_lt()))] = item;
        // items whose refills all fit in one batch (single_batch) need no heap:
        // the warp writes their refill chunks seed by seed and the batch record
        uint32_t one = __ballot_sync(0xffffffffu, item < nitems && B.it_nch[item] != 0 && B.it_nbat[item] == 1);
        while (one) {
            const uint32_t it = base + __ffs(one) - 1;
            one &= one - 1;
            const uint32_t ns = B.it_nsel[it], nref = B.it_nch[it], rb = B.it_choff[it];
            if ((uint64_t)rb + nref > cap_chunks) {
                if (lane == 0) {
                    atomicOr(&B.tot[TOT_FLAGS], OV_CHUNKS);
                    B.it_nbat[it] = 0;
                }
                continue;
            }
            const unsigned long long perm = B.it_perm[it];
            const uint64_t sb = (uint64_t)it * SWM_MAX_SEL;
            uint32_t q = 0;
            for (uint32_t i0 = 0; chunks && i0 < ns; i0 += 32) {
                const uint32_t i = i0 + lane;
                const uint2 sv = i < ns ? B.sel[sb + sel_slot(perm, i)] : make_uint2(0u, 0u);
                const uint32_t r = sv.y > SWM_PER_FETCH ? (sv.y - 1) / SWM_PER_FETCH : 0u;
                const uint32_t rinc = warp_scan_incl(r);
                const uint32_t q0 = rb + q + rinc - r;
                for (uint32_t j = 0; j < r; j++) {
                    const uint32_t at = SWM_PER_FETCH * (j + 1), left = sv.y - at;
                    B.ch_g[q0 + j] = sv.x + at;
                    B.ch_meta[q0 + j] = (left > SWM_PER_FETCH ? SWM_PER_FETCH : left) | (i << 8);
                }
                q += __shfl_sync(0xffffffffu, rinc, 31);
            }
            if (lane == 0) {
                const uint32_t sbase = rb + it;
                B.bt_c0[sbase] = rb; // batch 0 also holds every initial chunk
                B.bt_c1[sbase] = rb + nref;
                B.bt_e0[sbase] = B.it_eloff[it];
            }
        }
    }
}

#define PLAN_WARPS 4
#define PLAN_KEYS 512 // heap keys of an item held in shared memory; more go to global scratch

struct PlanSmem {
    uint32_t sst[SWM_MAX_SEL], scn[SWM_MAX_SEL], pc[SWM_MAX_SEL], koff[SWM_MAX_SEL + 1];
    uint32_t hloc[SWM_MAX_SEL + 8], hidx[SWM_MAX_SEL + 8];
    uint32_t key[PLAN_KEYS];
};

// One warp per item whose buckets need refills (a warp looks at 32 items at
// a time and takes those with refills one by one). The heap keys (the raw
// position of the last element of every chunk that leaves a seed with
// positions to fetch: pos[start + 32 (j + 1) - 1] for refill j) are all
// known up front, so the lanes load them in parallel; lane 0 then runs the
// seed heap of alignment_rmdup (2194-2419) on shared memory only.
__global__ void __launch_bounds__(PLAN_WARPS * 32) k_plan(const uint32_t *__restrict__ pos, MapBufs B,
                                                          uint64_t cap_chunks, uint64_t cap_elems) {
    __shared__ PlanSmem sm_all[PLAN_WARPS];
    const uint32_t lane = lane_id(), wib = threadIdx.x >> 5;
    PlanSmem &S = sm_all[wib];
    // warps take the items with refills one at a time from the list k_plan_list
    // built: a heavy item (a read in a large repeat family has thousands of
    // refills) keeps one warp, and the others move on
    const uint32_t nlist = B.tot[TOT_PLW], nitems = B.par->nitems;
    for (;;) {
        uint32_t idx = 0;
        if (lane == 0) idx = atomicAdd(&B.tot[TOT_PLWQ], 1u);
        idx = __shfl_sync(0xffffffffu, idx, 0);
        if (idx >= nlist) break;
        const uint32_t item = B.plan_list[nitems - 1 - idx];
        const uint32_t nref = B.it_nch[item];
        const uint32_t rb = B.it_choff[item], eb = B.it_eloff[item];
        const uint32_t sbase = rb + item;
        if ((uint64_t)rb + nref > cap_chunks || (uint64_t)eb + B.it_nel[item] > cap_elems) {
            if (lane == 0) {
                atomicOr(&B.tot[TOT_FLAGS], (uint64_t)rb + nref > cap_chunks ? OV_CHUNKS : OV_ELEMS);
                B.it_nbat[item] = 0;
            }
            continue;
        }
        const uint32_t ns = B.it_nsel[item];
        const uint64_t sb = (uint64_t)item * SWM_MAX_SEL;
        const unsigned long long perm = B.it_perm[item];
        // seed records in rank order and the offsets of their keys
        uint32_t carry = 0;
        for (uint32_t i0 = 0; i0 < ns; i0 += 32) {
            const uint32_t i = i0 + lane;
            uint32_t r = 0;
            if (i < ns) {
                const uint2 sv = B.sel[sb + sel_slot(perm, i)];
                S.sst[i] = sv.x;
                S.scn[i] = sv.y;
                S.pc[i] = sv.y > SWM_PER_FETCH ? SWM_PER_FETCH : sv.y; // initial fetch, 2194-2236
                r = sv.y > SWM_PER_FETCH ? (sv.y - 1) / SWM_PER_FETCH : 0u;
            }
            const uint32_t inc = warp_scan_incl(r);
            if (i < ns) S.koff[i] = carry + inc - r;
            carry += __shfl_sync(0xffffffffu, inc, 31);
        }
        if (lane == 0) S.koff[ns] = carry; // == nref
        __syncwarp();
        uint32_t *keys = nref <= PLAN_KEYS ? S.key : B.plan_keys + rb;
        for (uint32_t c = lane; c < nref; c += 32) {
            uint32_t lo = 0, hi = ns; // seed with koff <= c < koff of the next
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (S.koff[mid] <= c) lo = mid;
                else hi = mid;
            }
            const uint32_t j = c - S.koff[lo];
            keys[c] = pos[S.sst[lo] + SWM_PER_FETCH * (j + 1) - 1];
        }
        __syncwarp();
        if (lane == 0) {
            uint32_t hs = 0, rc = 0, e = 0, b = 0, br0 = 0, be0 = 0, npos = 0, runs = 0;
            for (uint32_t i = 0; i < ns; i++) {
                e += S.pc[i];
                npos += S.pc[i];
                runs += S.pc[i] ? 1u : 0u;
            }
            auto key_of = [&](uint32_t i) { return keys[S.koff[i] + S.pc[i] / SWM_PER_FETCH - 1]; };
            for (uint32_t i = 0; i < ns; i++) { // seeds_heap_insert, 1919-1935 (keys: raw positions)
                if (S.pc[i] != S.scn[i]) {
                    hs++;
                    S.hloc[hs] = key_of(i);
                    S.hidx[hs] = i;
                    uint32_t q = hs;
                    while (q > 1) {
                        const uint32_t t = q / 2;
                        if (S.hloc[t] > S.hloc[q]) {
                            uint32_t a = S.hloc[t];
                            S.hloc[t] = S.hloc[q];
                            S.hloc[q] = a;
                            a = S.hidx[t];
                            S.hidx[t] = S.hidx[q];
                            S.hidx[q] = a;
                        } else break;
                        q = t;
                    }
                }
            }
            for (;;) { // 2261-2419
                if (hs > 0 && npos + SWM_PER_FETCH <= SWM_BATCH_POSITIONS && 1 + 2 * runs < SWM_MAX_RUNS_BLOCK) {
                    const uint32_t i = S.hidx[1];
                    const uint32_t left = S.scn[i] - S.pc[i];
                    const uint32_t get = left > SWM_PER_FETCH ? SWM_PER_FETCH : left;
                    B.ch_g[rb + rc] = S.sst[i] + S.pc[i];
                    B.ch_meta[rb + rc] = get | (i << 8);
                    rc++;
                    S.pc[i] += get;
                    e += get;
                    npos += get;
                    runs++;
                    // seeds_heap_pop_and_insert, 1936-1962 (loop bound i * 2 < size)
                    if (S.pc[i] == S.scn[i]) {
                        S.hloc[1] = S.hloc[hs];
                        S.hidx[1] = S.hidx[hs];
                        hs--;
                    } else {
                        S.hloc[1] = key_of(i);
                    }
                    uint32_t q = 1;
                    while (q * 2 < hs) {
                        uint32_t t = q * 2;
                        if (q * 2 + 1 <= hs && S.hloc[q * 2] > S.hloc[q * 2 + 1]) t = q * 2 + 1;
                        if (S.hloc[t] < S.hloc[q]) {
                            uint32_t a = S.hloc[t];
                            S.hloc[t] = S.hloc[q];
                            S.hloc[q] = a;
                            a = S.hidx[t];
                            S.hidx[t] = S.hidx[q];
                            S.hidx[q] = a;
                        } else break;
                        q = t;
                    }
                }
                if (npos + SWM_PER_FETCH > SWM_BATCH_POSITIONS || hs == 0 || 1 + 2 * runs >= SWM_MAX_RUNS_BLOCK) {
                    if (npos > 0) {
                        B.bt_c0[sbase + b] = rb + br0; // refill chunks of the batch; batch 0 also
                        B.bt_c1[sbase + b] = rb + rc;  // holds every initial chunk
                        B.bt_e0[sbase + b] = eb + be0;
                        b++;
                    }
                    br0 = rc;
                    be0 = e;
                    npos = 0;
                    runs = 0;
                    if (hs == 0) break;
                }
            }
            B.it_nbat[item] = b;
        }
        __syncwarp();
    }
}

// Lane-per-item refill planning for the items with at most PLAN_LANE_SEEDS
// selected seeds: each lane runs one item's seed heap, the same schedule as
// k_plan (alignment_rmdup 2194-2419 with the heap of 1919-1962 and its sift
// bound), and a lane whose item is planned takes the next item from the list.
// The heap key of seed i is the raw position of the last entry fetched from
// it, pos[start + fetched - 1], loaded when the seed goes back into the heap.
// Per-lane state sits in shared memory as [slot][lane], so the lanes' accesses
// never share a bank.
#define PLAN_LANE_WARPS 2
#ifndef PLAN_LANE_REFILL
#define PLAN_LANE_REFILL 16
#endif

// Per lane (one item each): every selected seed's next position index and
// the end of its bucket (global indices into the position array), and the
// seed heap (keys and seed indices). Two words per seed, not three, keep the
// block at 26.5 KB: 8 resident blocks per SM instead of 6 -- the kernel waits
// on one position-array key per refill, so resident lanes are what it runs on.
struct PlanLaneSmem {
    uint32_t cur[PLAN_LANE_SEEDS][32], end[PLAN_LANE_SEEDS][32];
    uint32_t hloc[PLAN_LANE_SEEDS + 1][32];
    uint8_t hidx[PLAN_LANE_SEEDS + 1][32];
};

__global__ void __launch_bounds__(PLAN_LANE_WARPS * 32) k_plan_lanes(const uint32_t *__restrict__ pos, MapBufs B,
                                                                     uint64_t cap_chunks, uint64_t cap_elems) {
    __shared__ PlanLaneSmem sm_all[PLAN_LANE_WARPS];
    const uint32_t lane = lane_id();
    PlanLaneSmem &S = sm_all[threadIdx.x >> 5];
    const uint32_t nlist = B.tot[TOT_PLN];
    bool active = false, drained = false;
    uint32_t item = 0, hs = 0, rc = 0, rb = 0, eb = 0, sbase = 0, e = 0, b = 0, br0 = 0, be0 = 0, npos = 0, runs = 0;
    for (;;) {
        // lanes without an item take the next ones from the list (one atomic per
        // warp), once PLAN_LANE_REFILL of them wait or none is busy: the warp
        // stands still while a lane sets up an item, so set-ups go in groups
        const bool need = !active && !drained;
        const uint32_t m = __ballot_sync(0xffffffffu, need);
        if (m && (__popc(m) >= PLAN_LANE_REFILL || !__any_sync(0xffffffffu, active))) {
            const uint32_t leader = __ffs(m) - 1;
            uint32_t first = 0;
            if (lane == leader) first = atomicAdd(&B.tot[TOT_PLQ], (uint32_t)__popc(m));
            first = __shfl_sync(0xffffffffu, first, leader);
            if (need) {
                const uint32_t idx = first + __popc(m & lanemask_lt());
                if (idx >= nlist) {
                    drained = true;
                } else {
                    item = B.plan_list[idx];
                    const uint32_t nref = B.it_nch[item];
                    rb = B.it_choff[item];
                    eb = B.it_eloff[item];
                    sbase = rb + item;
                    if ((uint64_t)rb + nref > cap_chunks || (uint64_t)eb + B.it_nel[item] > cap_elems) {
                        atomicOr(&B.tot[TOT_FLAGS], (uint64_t)rb + nref > cap_chunks ? OV_CHUNKS : OV_ELEMS);
                        B.it_nbat[item] = 0;
                    } else {
                        const uint32_t ns = B.it_nsel[item];
                        const uint64_t sb = (uint64_t)item * SWM_MAX_SEL;
                        const unsigned long long perm = B.it_perm[item];
                        e = npos = runs = hs = rc = b = br0 = be0 = 0;
                        // seed records in rank order and the initial fetch (2194-2236), 8 loads in flight
                        for (uint32_t i0 = 0; i0 < ns; i0 += 8) {
                            uint2 sv[8];
#pragma unroll
                            for (uint32_t j = 0; j < 8; j++)
                                sv[j] = i0 + j < ns ? B.sel[sb + sel_slot(perm, i0 + j)] : make_uint2(0u, 0u);
#pragma unroll
                            for (uint32_t j = 0; j < 8; j++) {
                                if (i0 + j >= ns) break;
                                const uint32_t pc0 = sv[j].y > SWM_PER_FETCH ? SWM_PER_FETCH : sv[j].y;
                                S.cur[i0 + j][lane] = sv[j].x + pc0;
                                S.end[i0 + j][lane] = sv[j].x + sv[j].y;
                                e += pc0;
                                npos += pc0;
                                runs += pc0 ? 1u : 0u;
                            }
                        }
                        // seeds_heap_insert (1919-1935) of the seeds with entries left, in
                        // seed order; their keys loaded 8 at a time
                        for (uint32_t i0 = 0; i0 < ns; i0 += 8) {
                            uint32_t key[8];
                            bool ins[8];
#pragma unroll
                            for (uint32_t j = 0; j < 8; j++) {
                                const uint32_t i = i0 + j;
                                ins[j] = i < ns && S.cur[i][lane] != S.end[i][lane];
                                key[j] = pos[ins[j] ? S.cur[i][lane] - 1 : 0u];
                            }
#pragma unroll
                            for (uint32_t j = 0; j < 8; j++) {
                                if (!ins[j]) continue;
                                uint32_t q = ++hs;
                                while (q > 1) {
                                    const uint32_t t = q / 2, pk = S.hloc[t][lane];
                                    if (pk > key[j]) {
                                        S.hloc[q][lane] = pk;
                                        S.hidx[q][lane] = S.hidx[t][lane];
                                        q = t;
                                    } else {
                                        break;
                                    }
                                }
                                S.hloc[q][lane] = key[j];
                                S.hidx[q][lane] = (uint8_t)(i0 + j);
                            }
                        }
                        active = true;
                    }
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (__all_sync(0xffffffffu, drained)) break;
            continue;
        }
        if (!active) continue;
        // one refill (2261-2419), then the batch bounds
        if (hs > 0 && npos + SWM_PER_FETCH <= SWM_BATCH_POSITIONS && 1 + 2 * runs < SWM_MAX_RUNS_BLOCK) {
            const uint32_t i = S.hidx[1][lane];
            const uint32_t en = S.end[i][lane];
            uint32_t cu = S.cur[i][lane];
            const uint32_t left = en - cu;
            const uint32_t get = left > SWM_PER_FETCH ? SWM_PER_FETCH : left;
            B.ch_g[rb + rc] = cu;
            B.ch_meta[rb + rc] = get | (i << 8);
            rc++;
            cu += get;
            S.cur[i][lane] = cu;
            e += get;
            npos += get;
            runs++;
            // seeds_heap_pop_and_insert (1936-1962): the root leaves or takes
            // the seed's next key, then sinks while q * 2 < size
            uint32_t xk, xi;
            if (cu == en) {
                xk = S.hloc[hs][lane];
                xi = S.hidx[hs][lane];
                hs--;
            } else {
                xk = pos[cu - 1];
                xi = i;
            }
            uint32_t q = 1;
            while (q * 2 < hs) {
                uint32_t t = q * 2, kt = S.hloc[t][lane];
                if (t + 1 <= hs) {
                    const uint32_t k2 = S.hloc[t + 1][lane];
                    if (kt > k2) {
                        t++;
                        kt = k2;
                    }
                }
                if (kt < xk) {
                    S.hloc[q][lane] = kt;
                    S.hidx[q][lane] = S.hidx[t][lane];
                    q = t;
                } else {
                    break;
                }
            }
            S.hloc[q][lane] = xk;
            S.hidx[q][lane] = (uint8_t)xi;
        }
        if (npos + SWM_PER_FETCH > SWM_BATCH_POSITIONS || hs == 0 || 1 + 2 * runs >= SWM_MAX_RUNS_BLOCK) {
            if (npos > 0) {
                B.bt_c0[sbase + b] = rb + br0; // refill chunks of the batch; batch 0 also
                B.bt_c1[sbase + b] = rb + rc;  // holds every initial chunk
                B.bt_e0[sbase + b] = eb + be0;
                b++;
            }
            br0 = rc;
            be0 = e;
            npos = 0;
            runs = 0;
            if (hs == 0) {
                B.it_nbat[item] = b;
                active = false;
            }
        }
    }
}

// ======================================================================
// k_cand: one warp per batch slot -- gather, adjust, filter, sort-unique
// ======================================================================

// Bitonic sort of the first K lanes' values (K = 2..32, lanes >= K hold
// 0xffffffff): the network's first group of K lanes ends ascending.
template <int K>
__device__ __forceinline__ void warp_sort_k(uint32_t &v) {
    const uint32_t lane = lane_id();
#pragma unroll
    for (int size = 2; size <= K; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            uint32_t w = __shfl_xor_sync(0xffffffffu, v, stride);
            bool up = ((lane & size) == 0);
            bool lower = ((lane & stride) == 0);
            v = (lower == up) ? min(v, w) : max(v, w);
        }
    }
}

// Ascending sort of the first n <= 32 K values of buf, held in registers as
// element k * 32 + lane (bitonic network: strides >= 32 within a lane,
// smaller ones across lanes by shuffles), then the distinct values written to
// dst in order. Returns how many were written. 0xffffffff pads and never
// occurs as a position.
template <int K>
__device__ __forceinline__ uint32_t warp_sort_unique(const uint32_t *buf, uint32_t n, uint32_t *dst) {
    const uint32_t lane = lane_id();
    uint32_t v[K];
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = k * 32 + lane < n ? buf[k * 32 + lane] : 0xffffffffu;
#pragma unroll
    for (uint32_t size = 2; size <= 32 * K; size <<= 1) {
#pragma unroll
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= 32) { // partner k ^ (stride / 32) of the same lane; size >= 64
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const int ks = (int)(stride / 32);
                    if (k & ks) continue;
                    const bool up = ((k * 32) & size) == 0;
                    const uint32_t a = v[k], d = v[k | ks];
                    v[k] = up ? min(a, d) : max(a, d);
                    v[k | ks] = up ? max(a, d) : min(a, d);
                }
            } else {
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const uint32_t w = __shfl_xor_sync(0xffffffffu, v[k], stride);
                    const bool up = ((k * 32 + lane) & size) == 0, lower = (lane & stride) == 0;
                    v[k] = (lower == up) ? min(v[k], w) : max(v[k], w);
                }
            }
        }
    }
    uint32_t u = 0;
#pragma unroll
    for (int k = 0; k < K; k++) {
        const uint32_t above = __shfl_up_sync(0xffffffffu, v[k], 1);
        const uint32_t last = __shfl_sync(0xffffffffu, k ? v[k ? k - 1 : 0] : 0u, 31);
        const uint32_t prev = lane ? above : last;
        const bool keep = v[k] != 0xffffffffu && ((k == 0 && lane == 0) || v[k] != prev);
        const uint32_t m = __ballot_sync(0xffffffffu, keep);
        if (keep) dst[u + __popc(m & lanemask_lt())] = v[k];
        u += __popc(m);
    }
    return u;
}

// The kept (adjusted) positions of one batch, sorted ascending and unique,
// written to dst (merge + unique of block_heap_sort, mapper_cpe.c:1999-2089);
// returns how many. They sit in sc (shared memory) or, when spilled, in the
// warp's global scratch gs (room for SWM_BATCH_POSITIONS).
__device__ __forceinline__ uint32_t batch_sort_unique(uint32_t *sc, uint32_t *gs, bool spilled, uint32_t kept,
                                                      uint32_t *dst) {
    const uint32_t lane = lane_id();
    uint32_t u = 0;
    if (kept <= 8) {
        // at most 8 values: take the distinct ones smallest first
        uint32_t v = lane < kept ? sc[lane] : 0xffffffffu, res = 0;
        for (;;) {
            const uint32_t m = __reduce_min_sync(0xffffffffu, v);
            if (m == 0xffffffffu) break;
            res = lane == u ? m : res;
            v = v == m ? 0xffffffffu : v;
            u++;
        }
        if (lane < u) dst[lane] = res;
    } else if (kept <= 32) {
        uint32_t v = lane < kept ? sc[lane] : 0xffffffffu;
        if (kept <= 16) warp_sort_k<16>(v); // lanes 16.. hold the pad, already in order
        else warp_sort_k<32>(v);
        const uint32_t prev = __shfl_up_sync(0xffffffffu, v, 1);
        const bool keep = v != 0xffffffffu && (lane == 0 || prev != v);
        const uint32_t m = __ballot_sync(0xffffffffu, keep);
        if (keep) dst[__popc(m & lanemask_lt())] = v;
        u = __popc(m);
    } else if (kept <= 64) {
        u = warp_sort_unique<2>(sc, kept, dst);
    } else if (kept <= 128) {
        u = warp_sort_unique<4>(spilled ? gs : sc, kept, dst);
    } else if (kept <= 256) {
        u = warp_sort_unique<8>(gs, kept, dst);
    } else { // bitonic sort in the warp's global scratch
        uint32_t n2 = 512;
        while (n2 < kept) n2 <<= 1;
        uint32_t *buf = spilled ? gs : sc;
        for (uint32_t i = kept + lane; i < n2; i += 32) buf[i] = 0xffffffffu;
        __syncwarp();
        for (uint32_t size = 2; size <= n2; size <<= 1) {
            for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
                for (uint32_t i = lane; i < n2 / 2; i += 32) {
                    const uint32_t lo = 2 * i - (i & (stride - 1)), hi = lo + stride;
                    const bool up = ((lo & size) == 0);
                    const uint32_t a = buf[lo], d = buf[hi];
                    if ((a > d) == up) {
                        buf[lo] = d;
                        buf[hi] = a;
                    }
                }
                __syncwarp();
            }
        }
        for (uint32_t i0 = 0; i0 < kept; i0 += 32) {
            const uint32_t i = i0 + lane;
            const bool keep = i < kept && (i == 0 || buf[i - 1] != buf[i]);
            const uint32_t m = __ballot_sync(0xffffffffu, keep);
            if (keep) dst[u + __popc(m & lanemask_lt())] = buf[i];
            u += __popc(m);
        }
    }
    return u;
}

#define CAND_MAXCH 128 // chunks (runs) per batch: block_size < 256 allows at most 128

#define CAND_SMEM_KEEP 128 // survivors of a batch held in shared memory (more go to global scratch)

struct CandSmem {
    uint32_t gs[CAND_MAXCH];     // first global index of each chunk minus its start in the batch
    uint32_t cm[CAND_MAXCH];     // descriptor (sel[]) of the chunk's seed
    uint16_t start[CAND_MAXCH + 1];
    uint32_t sel[SWM_MAX_SEL];   // base | shift << 16 | rl << 20 | rh << 24
    uint32_t st[SWM_MAX_SEL];    // bucket start of each selected seed
    uint32_t cn[SWM_MAX_SEL];    // bucket count of each selected seed
    uint32_t sc[CAND_SMEM_KEEP]; // kept positions of a batch, while they fit
};

#define CAND_WARPS 8
#ifndef CAND_MIN_BLOCKS
#define CAND_MIN_BLOCKS 8 // resident blocks per SM the register budget is sized for
#endif

// One warp per item, every batch of the item: element-parallel gather of
// (position, flank code) pairs, position adjust, flank filter, sort-unique.
__global__ void __launch_bounds__(CAND_WARPS * 32, CAND_MIN_BLOCKS) k_cand(const uint32_t *__restrict__ pos,
                                                             const uint16_t *__restrict__ lsd, MapBufs B,
                                                             uint64_t cap_chunks, uint64_t cap_elems, uint32_t klong) {
    const uint32_t nitems = B.par->nitems;
    __shared__ CandSmem sm_all[CAND_WARPS];
    if (B.tot[TOT_FLAGS] != 0 || B.tot[TOT_CHUNKS] > cap_chunks || B.tot[TOT_ELEMS] > cap_elems) return;
    const uint32_t lane = lane_id(), wib = threadIdx.x >> 5;
    CandSmem &S = sm_all[wib];
    // a warp's survivors past CAND_SMEM_KEEP go to its slice of global scratch
    auto gscratch = [&]() { return B.sort_scratch + (uint64_t)(blockIdx.x * CAND_WARPS + wib) * SWM_BATCH_POSITIONS; };
    unsigned long long kept_all = 0; // this warp's kept positions, added to the block's count once
    for (uint32_t g0 = warp_take_items(&B.tot[TOT_CQ]), gi = 0; g0 < nitems;) {
        const uint32_t item = g0 + gi;
        if (++gi == CAND_TAKE || item + 1 >= nitems) {
            gi = 0;
            g0 = warp_take_items(&B.tot[TOT_CQ]);
        }
        if (item >= nitems) break;
        const uint32_t nb = B.it_nbat[item];
        uint32_t total = 0;
        if (nb) {
            const uint64_t sb = (uint64_t)item * SWM_MAX_SEL;
            const uint32_t ns = B.it_nsel[item], nref = B.it_nch[item];
            const unsigned long long perm = B.it_perm[item];
            const uint32_t sbase = B.it_choff[item] + item;
            for (uint32_t i = lane; i < ns; i += 32) {
                const uint32_t rs = sel_slot(perm, i), l = rs / SWM_SEED_STEP, sft = rs % SWM_SEED_STEP;
                const uint2 sv = B.sel[sb + rs];
                const uint32_t fb = B.sel_fl[sb + rs];
                // base | shift << 16 | rl << 20 | rh << 24
                S.sel[i] = (l * klong + sft) | ((SWM_SEED_STEP - 1 - sft) << 16) | ((fb & 7u) << 20) | ((fb >> 3) << 24);
                S.st[i] = sv.x;
                S.cn[i] = sv.y;
            }
            __syncwarp();
            for (uint32_t b = 0; b < nb; b++) {
                uint32_t c0 = 0, c1 = 0, e0;
                if (nref == 0) {
                    e0 = B.it_eloff[item];
                } else {
                    c0 = B.bt_c0[sbase + b];
                    c1 = B.bt_c1[sbase + b];
                    e0 = B.bt_e0[sbase + b];
                }
                // chunk table: the first chunk of every seed (batch 0), then refills
                uint32_t nchk = 0, carry = 0;
                if (b == 0) {
                    for (uint32_t i0 = 0; i0 < ns; i0 += 32) {
                        const uint32_t i = i0 + lane;
                        const uint32_t cnt = i < ns ? S.cn[i] : 0u;
                        const uint32_t len = cnt > SWM_PER_FETCH ? SWM_PER_FETCH : cnt;
                        const uint32_t m = __ballot_sync(0xffffffffu, len != 0);
                        const uint32_t inc = warp_scan_incl(len);
                        if (len) {
                            const uint32_t q = nchk + __popc(m & lanemask_lt()), st0 = carry + inc - len;
                            S.gs[q] = S.st[i] - st0;
                            S.cm[q] = S.sel[i];
                            S.start[q] = (uint16_t)st0;
                        }
                        nchk += __popc(m);
                        carry += __shfl_sync(0xffffffffu, inc, 31);
                    }
                }
                for (uint32_t q0 = c0; q0 < c1; q0 += 32) {
                    const uint32_t c = q0 + lane;
                    uint32_t len = 0, meta = 0;
                    if (c < c1) {
                        meta = B.ch_meta[c];
                        len = meta & 0xffu;
                    }
                    const uint32_t inc = warp_scan_incl(len);
                    if (c < c1) {
                        const uint32_t st0 = carry + inc - len;
                        S.gs[nchk + (c - q0)] = B.ch_g[c] - st0;
                        S.cm[nchk + (c - q0)] = S.sel[meta >> 8];
                        S.start[nchk + (c - q0)] = (uint16_t)st0;
                    }
                    nchk += min(32u, c1 - q0);
                    carry += __shfl_sync(0xffffffffu, inc, 31);
                }
                const uint32_t E = carry;
                if (lane == 0) S.start[nchk] = (uint16_t)E;
                __syncwarp();
                bool spilled = false; // survivors in S.sc, or in global scratch once they outgrow it
                uint32_t kept = 0, cdone = 0; // cdone: chunks that start before eb
                for (uint32_t eb = 0; eb < E; eb += 32) {
                    const uint32_t el = eb + lane;
                    // chunks are non-empty, so at most 32 start in [eb, eb + 32):
                    // lane j looks at chunk cdone + j and the starts become a bit mask
                    const uint32_t cs = cdone + lane < nchk ? S.start[cdone + lane] : eb + 32;
                    const uint32_t bits = __reduce_or_sync(0xffffffffu, cs < eb + 32 ? 1u << (cs - eb) : 0u);
                    const uint32_t q = cdone + __popc(bits & (0xffffffffu >> (31 - lane))) - 1; // chunk of el
                    cdone += __popc(bits);
                    bool ok = false;
                    uint32_t p = 0;
                    if (el < E) {
                        const uint32_t g = S.gs[q] + el;
                        const uint32_t sm = S.cm[q];
                        const uint32_t base = sm & 0xffffu, shift = (sm >> 16) & 0xfu, rl = (sm >> 20) & 0xfu,
                                       rh = (sm >> 24) & 0xfu;
                        const uint32_t ls = lsd[g];
                        const uint32_t rs = (((ls >> shift) ^ rl) | ((ls >> (6 + shift)) ^ rh)) & 7u; // 2107-2112
                        ok = (rs == 0) && (el != 0); // element 0 of the batch is dropped (2113)
                        if (ok) { // positions only for the entries the flank filter keeps
                            const uint32_t raw = pos[g];
                            p = raw > base ? raw - base : 0u; // adjust_ref_pos_rmdup, 1893-1917
                        }
                    }
                    const uint32_t m = __ballot_sync(0xffffffffu, ok);
                    if (!spilled && kept + __popc(m) > CAND_SMEM_KEEP) {
                        uint32_t *gs = gscratch();
                        for (uint32_t i = lane; i < kept; i += 32) gs[i] = S.sc[i];
                        spilled = true;
                        __syncwarp();
                    }
                    if (ok) {
                        const uint32_t at = kept + __popc(m & lanemask_lt());
                        if (spilled) gscratch()[at] = p;
                        else S.sc[at] = p;
                    }
                    kept += __popc(m);
                }
                __syncwarp();
                const uint32_t u = batch_sort_unique(S.sc, gscratch(), spilled, kept, B.cand_ub + e0);
                if (lane == 0) B.bt_cnt[sbase + b] = u;
                total += u;
                kept_all += kept;
                __syncwarp();
            }
        }
        if (lane == 0) B.it_ncand[item] = total;
    }
    if (lane == 0 && kept_all) atomicAdd(&B.stat[ST_KEPT], kept_all);
}

// ======================================================================
// k_cand_table: the same batches from the candidate table (k = 12)
// ======================================================================
//
// With the candidate table, the entries a seed's flank filter keeps are one
// position-ordered range of the table (key: seed code, shift, read flank), so
// a batch reads only its survivors instead of every entry of its chunks. A
// batch's survivors of seed i are the range's entries whose bucket rank is
// among the ranks the batch fetched for that seed: all of them when the item
// has one batch; otherwise those after the previous batches' and at or below
// the position of the last rank fetched so far (positions are unique and
// ascending in a bucket, so position bounds are rank bounds). Element 0 of a
// batch (the first entry of its first chunk, mapper_cpe.c:2113) is dropped
// when it passes the filter; it is then the first survivor of its seed in that
// batch.

struct CandTabSmem {
    uint32_t st[SWM_MAX_SEL];        // bucket start of each selected seed
    uint32_t cn[SWM_MAX_SEL];        // bucket count
    uint32_t sel[SWM_MAX_SEL];       // base | shift << 16 | rl << 20 | rh << 24
    uint32_t cur[SWM_MAX_SEL];       // next table index of the seed's range
    uint32_t end[SWM_MAX_SEL];       // end of the seed's range
    uint32_t r1[SWM_MAX_SEL];        // bucket ranks fetched through this batch
    uint32_t rst[SWM_MAX_SEL + 1];   // first element of each run of this batch
    uint32_t ri[SWM_MAX_SEL];        // its first table index
    uint32_t rb[SWM_MAX_SEL];        // its seed's base (position adjust)
    uint32_t sc[CAND_SMEM_KEEP];     // kept positions of a batch, while they fit
};

// First index in [a, z) whose position is above p1 (positions ascending).
__device__ __forceinline__ uint32_t upper_pos(const uint32_t *__restrict__ tp, uint32_t a, uint32_t z, uint32_t p1) {
    while (a < z) {
        const uint32_t mid = a + ((z - a) >> 1);
        if (tp[mid] <= p1) a = mid + 1;
        else z = mid;
    }
    return a;
}

__global__ void __launch_bounds__(CAND_WARPS * 32, CAND_MIN_BLOCKS)
    k_cand_table(const uint32_t *__restrict__ pos, const uint16_t *__restrict__ lsd,
                 const uint32_t *__restrict__ ctab_off, const uint32_t *__restrict__ ctab_pos, MapBufs B,
                 uint64_t cap_chunks, uint64_t cap_elems, uint32_t klong) {
    const uint32_t nitems = B.par->nitems;
    __shared__ CandTabSmem sm_all[CAND_WARPS];
    if (B.tot[TOT_FLAGS] != 0 || B.tot[TOT_CHUNKS] > cap_chunks || B.tot[TOT_ELEMS] > cap_elems) return;
    const uint32_t lane = lane_id(), wib = threadIdx.x >> 5;
    CandTabSmem &S = sm_all[wib];
    auto gscratch = [&]() { return B.sort_scratch + (uint64_t)(blockIdx.x * CAND_WARPS + wib) * SWM_BATCH_POSITIONS; };
    unsigned long long kept_all = 0; // this warp's kept positions, added to the block's count once
    for (uint32_t g0 = warp_take_items(&B.tot[TOT_CQ]), gi = 0; g0 < nitems;) {
        const uint32_t item = g0 + gi;
        if (++gi == CAND_TAKE || item + 1 >= nitems) {
            gi = 0;
            g0 = warp_take_items(&B.tot[TOT_CQ]);
        }
        if (item >= nitems) break;
        const uint32_t nb = B.it_nbat[item];
        uint32_t total = 0;
        if (nb) {
            const uint64_t sb = (uint64_t)item * SWM_MAX_SEL;
            const uint32_t ns = B.it_nsel[item], nref = B.it_nch[item];
            const unsigned long long perm = B.it_perm[item];
            const uint32_t sbase = B.it_choff[item] + item;
            for (uint32_t i = lane; i < ns; i += 32) {
                const uint32_t rs = sel_slot(perm, i), l = rs / SWM_SEED_STEP, sft = rs % SWM_SEED_STEP;
                const uint2 sv = B.sel[sb + rs];
                const uint32_t fb = B.sel_fl[sb + rs];
                const uint32_t key = B.sel_key[sb + rs];
                S.sel[i] = (l * klong + sft) | ((SWM_SEED_STEP - 1 - sft) << 16) | ((fb & 7u) << 20) | ((fb >> 3) << 24);
                S.st[i] = sv.x;
                S.cn[i] = sv.y;
                uint32_t d0 = 0, d1 = 0;
                if (sv.y) {
                    d0 = ctab_off[key];
                    d1 = ctab_off[(uint64_t)key + 1];
                }
                S.cur[i] = d0;
                S.end[i] = d1;
                S.r1[i] = sv.y < SWM_PER_FETCH ? sv.y : SWM_PER_FETCH; // batch 0 holds every seed's first chunk
            }
            __syncwarp();
            // element 0 of batch 0: the first entry of the first seed (rank order) with positions
            uint32_t s0 = 0xffffffffu;
            for (uint32_t i0 = 0; i0 < ns && s0 == 0xffffffffu; i0 += 32) {
                const uint32_t m = __ballot_sync(0xffffffffu, i0 + lane < ns && S.cn[i0 + lane] != 0);
                if (m) s0 = i0 + __ffs(m) - 1;
            }
            uint32_t g0 = s0 != 0xffffffffu ? S.st[s0] : 0u;
            for (uint32_t b = 0; b < nb; b++) {
                uint32_t c0 = 0, c1 = 0, e0;
                if (nref == 0) {
                    e0 = B.it_eloff[item];
                } else {
                    c0 = B.bt_c0[sbase + b];
                    c1 = B.bt_c1[sbase + b];
                    e0 = B.bt_e0[sbase + b];
                }
                if (nb > 1) {
                    // the batch's refill chunks raise their seed's fetched rank
                    for (uint32_t q0 = c0; q0 < c1; q0 += 32) {
                        const uint32_t c = q0 + lane;
                        if (c < c1) {
                            const uint32_t meta = B.ch_meta[c], si = meta >> 8;
                            atomicMax(&S.r1[si], B.ch_g[c] - S.st[si] + (meta & 0xffu));
                        }
                    }
                    if (b > 0) { // element 0: the first entry of the batch's first chunk
                        uint32_t gg = 0, ss = 0;
                        if (lane == 0 && c0 < c1) {
                            gg = B.ch_g[c0];
                            ss = B.ch_meta[c0] >> 8;
                        }
                        g0 = __shfl_sync(0xffffffffu, gg, 0);
                        s0 = c0 < c1 ? __shfl_sync(0xffffffffu, ss, 0) : 0xffffffffu;
                    }
                    __syncwarp();
                }
                // each seed's survivors in this batch, as runs of the table
                uint32_t nruns = 0, carry = 0;
                for (uint32_t i0 = 0; i0 < ns; i0 += 32) {
                    const uint32_t i = i0 + lane;
                    uint32_t a = 0, z = 0;
                    if (i < ns) {
                        a = S.cur[i];
                        z = S.end[i];
                        const uint32_t r1 = S.r1[i], cn = S.cn[i];
                        if (nb > 1 && r1 < cn && a < z) z = upper_pos(ctab_pos, a, z, pos[S.st[i] + r1 - 1]);
                        S.cur[i] = z;
                        if (i == s0 && a < z) { // element 0 passes the filter: then it is this run's first entry
                            const uint32_t sm = S.sel[i], shift = (sm >> 16) & 0xfu, rl = (sm >> 20) & 0xfu,
                                           rh = (sm >> 24) & 0xfu;
                            const uint32_t ls = lsd[g0];
                            if (((((ls >> shift) ^ rl) | ((ls >> (6 + shift)) ^ rh)) & 7u) == 0) a++; // 2107-2113
                        }
                    }
                    const uint32_t len = z - a;
                    const uint32_t m = __ballot_sync(0xffffffffu, len != 0);
                    const uint32_t inc = warp_scan_incl(len);
                    if (len) {
                        const uint32_t q = nruns + __popc(m & lanemask_lt());
                        S.rst[q] = carry + inc - len;
                        S.ri[q] = a;
                        S.rb[q] = S.sel[i] & 0xffffu;
                    }
                    nruns += __popc(m);
                    carry += __shfl_sync(0xffffffffu, inc, 31);
                }
                const uint32_t K = carry;
                if (lane == 0) S.rst[nruns] = K;
                __syncwarp();
                // gather the survivors' positions, adjusted (adjust_ref_pos_rmdup, 1893-1917)
                bool spilled = false;
                uint32_t kept = 0, rdone = 0;
                for (uint32_t eb = 0; eb < K; eb += 32) {
                    const uint32_t el = eb + lane;
                    // runs are non-empty: at most 32 start in [eb, eb + 32)
                    const uint32_t cs = rdone + lane < nruns ? S.rst[rdone + lane] : eb + 32;
                    const uint32_t bits = __reduce_or_sync(0xffffffffu, cs < eb + 32 ? 1u << (cs - eb) : 0u);
                    const uint32_t q = rdone + __popc(bits & (0xffffffffu >> (31 - lane))) - 1; // run of el
                    rdone += __popc(bits);
                    const bool ok = el < K;
                    uint32_t p = 0;
                    if (ok) {
                        const uint32_t raw = ctab_pos[S.ri[q] + (el - S.rst[q])];
                        const uint32_t base = S.rb[q];
                        p = raw > base ? raw - base : 0u;
                    }
                    const uint32_t m = __ballot_sync(0xffffffffu, ok);
                    if (!spilled && kept + __popc(m) > CAND_SMEM_KEEP) {
                        uint32_t *gs = gscratch();
                        for (uint32_t i = lane; i < kept; i += 32) gs[i] = S.sc[i];
                        spilled = true;
                        __syncwarp();
                    }
                    if (ok) {
                        const uint32_t at = kept + __popc(m & lanemask_lt());
                        if (spilled) gscratch()[at] = p;
                        else S.sc[at] = p;
                    }
                    kept += __popc(m);
                }
                __syncwarp();
                const uint32_t u = batch_sort_unique(S.sc, gscratch(), spilled, kept, B.cand_ub + e0);
                if (lane == 0) B.bt_cnt[sbase + b] = u;
                total += u;
                kept_all += kept;
                __syncwarp();
            }
        }
        if (lane == 0) B.it_ncand[item] = total;
    }
    if (lane == 0 && kept_all) atomicAdd(&B.stat[ST_KEPT], kept_all);
}

// Dense candidate list: item by item, batch by batch, in verification order.
#define COMPACT_HEAVY 16 // candidates above which an item is copied by its whole warp

__global__ void __launch_bounds__(256) k_compact(MapBufs B, uint64_t cap_chunks, uint64_t cap_elems,
                                                 uint64_t cap_cands) {
    const uint32_t nitems = B.par->nitems;
    if (B.tot[TOT_FLAGS] != 0 || B.tot[TOT_CHUNKS] > cap_chunks || B.tot[TOT_ELEMS] > cap_elems) return;
    const uint32_t lane = lane_id();
    // warp-uniform loop over groups of 32 items
    for (uint32_t item0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); item0 < nitems;
         item0 += gridDim.x * blockDim.x) {
        const uint32_t item = item0 + lane;
        // one thread per item: its scalars in one round trip, then its few
        // candidates batch by batch; items with many candidates are left to
        // the whole warp below
        uint32_t nb = 0, nref = 0, o0 = 0, nc = 0, sbase = 0, eloff = 0;
        bool heavy = false;
        if (item < nitems) {
            nb = B.it_nbat[item];
            nref = B.it_nch[item];
            o0 = B.it_coff[item];
            nc = B.it_ncand[item];
            sbase = B.it_choff[item] + item;
            eloff = B.it_eloff[item];
            if (nb && (uint64_t)o0 + nc > cap_cands) {
                atomicOr(&B.tot[TOT_FLAGS], OV_CANDS);
                nb = 0;
            }
            heavy = nb && nc > COMPACT_HEAVY;
            if (nb && !heavy) {
                uint32_t o = o0;
                for (uint32_t b = 0; b < nb; b++) {
                    const uint32_t n = nref ? B.bt_cnt[sbase + b] : nc; // one batch when there are no refills
                    const uint32_t e0 = nref ? B.bt_e0[sbase + b] : eloff;
                    for (uint32_t j = 0; j < n; j++) {
                        B.cc_pos[o + j] = B.cand_ub[e0 + j];
                        B.cc_item[o + j] = item;
                    }
                    o += n;
                }
            }
        }
        uint32_t hm = __ballot_sync(0xffffffffu, heavy);
        while (hm) { // the warp copies each heavy item of the group, lanes over its candidates
            const uint32_t src = __ffs(hm) - 1;
            hm &= hm - 1;
            const uint32_t hnb = __shfl_sync(0xffffffffu, nb, src), hnref = __shfl_sync(0xffffffffu, nref, src);
            const uint32_t hnc = __shfl_sync(0xffffffffu, nc, src), hsb = __shfl_sync(0xffffffffu, sbase, src);
            const uint32_t hel = __shfl_sync(0xffffffffu, eloff, src);
            uint32_t o = __shfl_sync(0xffffffffu, o0, src);
            for (uint32_t b = 0; b < hnb; b++) {
                const uint32_t n = hnref ? B.bt_cnt[hsb + b] : hnc;
                const uint32_t e0 = hnref ? B.bt_e0[hsb + b] : hel;
                for (uint32_t j = lane; j < n; j += 32) {
                    B.cc_pos[o + j] = B.cand_ub[e0 + j];
                    B.cc_item[o + j] = item0 + src;
                }
                o += n;
            }
        }
    }
}

// ======================================================================
// k_verify: one thread per candidate
// ======================================================================

// adjust_ref_len + pos_start (mapper_cpe.c:1403-1435) with the reference's
// integer types; returns 0xffffffff when the window is rejected.
__device__ __forceinline__ uint32_t window_start(uint32_t base_pos, uint32_t L, uint32_t e, uint64_t ref_length,
                                                 uint32_t *rl_out) {
    // the window base_pos - e .. base_pos + L + e - 1 inside the genome (and
    // base_pos + L inside 32 bits): front > 0 > back below, so ref_len stays
    // L + 2e and the shift e
    if (base_pos > e && (uint64_t)base_pos + L + e < ref_length && (uint64_t)base_pos + L <= 0xffffffffull) {
        *rl_out = L + 2 * e;
        return base_pos - e;
    }
    const uint64_t dist_error = e;
    uint64_t shift_tmp = e;
    uint64_t ref_len = (uint64_t)L + 2 * shift_tmp;
    if (base_pos <= shift_tmp) {
        shift_tmp = base_pos;
        ref_len -= (dist_error - base_pos);
    }
    int64_t front = (int64_t)ref_length - (int64_t)((uint64_t)base_pos - dist_error);
    int64_t back = (int64_t)((uint64_t)(uint32_t)(base_pos + L) + dist_error) - (int64_t)ref_length;
    if (front > back) {
        if (back >= 0) ref_len -= (uint64_t)(back + 1);
    } else {
        shift_tmp = dist_error - (uint64_t)front - 1;
        ref_len -= (uint64_t)front;
    }
    uint32_t rl = (uint32_t)ref_len;
    *rl_out = rl;
    if ((uint64_t)rl < (uint64_t)L - dist_error) return 0xffffffffu;
    return (uint32_t)((uint64_t)base_pos - shift_tmp);
}

// Banded Myers / Hyyro recurrence of banded_myers_simd (mapper_cpe.c:519-660)
// with the pattern-match word built from window bit planes: at read base i
// bit j of eq is [window[i + j] == read[i]] for j <= 2e, the same word the
// reference keeps in peq[read[i]]. myers_blocks runs the 32-base blocks
// b0 .. b1 - 1 (the last one may be partial) from the state (VP, VN, ones =
// steps whose D0 bit 0 was set); cp gets (VP, VN) at the start of each.
__device__ __forceinline__ void myers_blocks(const uint32_t *WL, const uint32_t *WH, const uint32_t *RW, uint32_t L,
                                             uint32_t MASK, uint32_t b0, uint32_t b1, uint32_t &vp, uint32_t &vn,
                                             uint32_t &ones, uint32_t *cp) {
    for (uint32_t b = b0; b < b1; b++) {
        const uint32_t wl0 = WL[b], wl1 = WL[b + 1], wh0 = WH[b], wh1 = WH[b + 1];
        const uint32_t rlw = RW[2 * b], rhw = RW[2 * b + 1];
        const uint32_t steps = min(32u, L - 32 * b);
        cp[4 * b] = vp; // (VP, VN) before bases 32 b and 32 b + 16, for the traceback
        cp[4 * b + 1] = vn;
        uint32_t acc = 0;
        if (steps == 32) {
#pragma unroll
            for (uint32_t t = 0; t < 32; t++) {
                if (t == 16) {
                    cp[4 * b + 2] = vp;
                    cp[4 * b + 3] = vn;
                }
                const uint32_t wls = __funnelshift_r(wl0, wl1, t), whs = __funnelshift_r(wh0, wh1, t);
                const uint32_t mL = (uint32_t)((int32_t)(rlw << (31 - t)) >> 31);
                const uint32_t mH = (uint32_t)((int32_t)(rhw << (31 - t)) >> 31);
                const uint32_t eq = ~((wls ^ mL) | (whs ^ mH)) & MASK;
                uint32_t x = eq | vn;
                const uint32_t d0 = ((vp + (x & vp)) ^ vp) | x;
                const uint32_t hn = vp & d0;
                const uint32_t hp = vn | ~(vp | d0);
                x = d0 >> 1;
                vn = x & hp;
                vp = hn | ~(x | hp);
                acc = __funnelshift_r(acc, d0, 1);
            }
        } else {
            for (uint32_t t = 0; t < steps; t++) {
                if (t == 16) {
                    cp[4 * b + 2] = vp;
                    cp[4 * b + 3] = vn;
                }
                const uint32_t wls = __funnelshift_r(wl0, wl1, t), whs = __funnelshift_r(wh0, wh1, t);
                const uint32_t mL = 0u - ((rlw >> t) & 1u), mH = 0u - ((rhw >> t) & 1u);
                const uint32_t eq = ~((wls ^ mL) | (whs ^ mH)) & MASK;
                uint32_t x = eq | vn;
                const uint32_t d0 = ((vp + (x & vp)) ^ vp) | x;
                const uint32_t hn = vp & d0;
                const uint32_t hp = vn | ~(vp | d0);
                x = d0 >> 1;
                vn = x & hp;
                vp = hn | ~(x | hp);
                acc = __funnelshift_r(acc, d0, 1);
            }
        }
        ones += __popc(acc);
    }
}

// The reference's final scan (634-650) after all L steps: (error, location)
// of the first strict minimum with error <= e, or (SWM_MAXERROR, -1).
__device__ __forceinline__ int myers_final(uint32_t vp, uint32_t vn, uint32_t ones, uint32_t L, uint32_t e,
                                           uint32_t rl, int *loc_out) {
    int err = (int)L - (int)ones;
    const int last_high = (int)rl - (int)L;
    const int site = (int)L - 1;
    int location = -1, error = SWM_MAXERROR;
    if (err <= (int)e && err < error) {
        error = err;
        location = site;
    }
    for (int i = 0; i < last_high; i++) {
        err += (int)((vp >> i) & 1u);
        err -= (int)((vn >> i) & 1u);
        if (err <= (int)e && err < error) {
            error = err;
            location = site + i + 1;
        }
    }
    *loc_out = location;
    return error;
}

// Same recurrence keeping D0 / HP per read base for the traceback
// (align_reads, mapper_cpe.c:288-362).
__device__ void myers_history(const uint32_t *WL, const uint32_t *WH, const uint32_t *RW, uint32_t L, uint32_t e,
                              uint32_t *d0h, uint32_t *hph) {
    const uint32_t MASK = (1u << (2 * e + 1)) - 1u;
    uint32_t vp = 0, vn = 0;
    for (uint32_t i = 0; i < L; i++) {
        const uint32_t b = i >> 5, t = i & 31;
        const uint32_t wls = __funnelshift_r(WL[b], WL[b + 1], t), whs = __funnelshift_r(WH[b], WH[b + 1], t);
        const uint32_t mL = 0u - ((RW[2 * b] >> t) & 1u), mH = 0u - ((RW[2 * b + 1] >> t) & 1u);
        const uint32_t eq = ~((wls ^ mL) | (whs ^ mH)) & MASK;
        uint32_t x = eq | vn;
        const uint32_t d0 = ((vp + (x & vp)) ^ vp) | x;
        const uint32_t hn = vp & d0;
        const uint32_t hp = vn | ~(vp | d0);
        x = d0 >> 1;
        vn = x & hp;
        vp = hn | ~(x | hp);
        d0h[i] = d0;
        hph[i] = hp;
    }
}

// sprint_length (mapper_cpe.c:214-228) including its signed-char digit:
// '0' + (char)v % 10 with the cast binding first.
__device__ __forceinline__ int put_len(uint8_t *p, uint32_t v) {
    int n = 0;
    for (uint32_t t = v; t; t /= 10) n++;
    for (int i = n - 1; i >= 0; i--) {
        int b = (int)(v & 0xffu);
        if (b >= 128) b -= 256;
        p[i] = (uint8_t)('0' + b % 10);
        v /= 10;
    }
    return n;
}

// Aligned window bit planes of [ws, ws + 32 * SWM_WIN_WORDS): bit b of
// WL[j] / WH[j] is the lo / hi bit of genome base ws + 32j + b
// (shift_ref_pos_v, mapper_cpe.c:1509-1586); zero past the index padding.
__device__ __forceinline__ void load_window(const uint32_t *__restrict__ b2, uint64_t b2_words, uint32_t ws,
                                            uint32_t L, uint32_t e, uint32_t *WL, uint32_t *WH) {
    const uint64_t w0 = (uint64_t)(ws >> 5) * 2;
    const uint32_t sh = ws & 31;
    const uint32_t nw = (L + 2 * e + 31) / 32 + 2;
    uint32_t plo = (w0 < b2_words) ? b2[w0] : 0u, phi = (w0 + 1 < b2_words) ? b2[w0 + 1] : 0u;
#pragma unroll
    for (uint32_t j = 0; j < SWM_WIN_WORDS; j++) {
        uint32_t nlo = 0, nhi = 0;
        if (j < nw) {
            const uint64_t q = w0 + 2 * j + 2;
            nlo = q < b2_words ? b2[q] : 0u;
            nhi = q + 1 < b2_words ? b2[q + 1] : 0u;
        }
        WL[j] = swm_fsr(plo, nlo, sh);
        WH[j] = swm_fsr(phi, nhi, sh);
        plo = nlo;
        phi = nhi;
    }
}

#define TB_TEXT_MAX 2304 // >= 4 bytes x every route entry a bounded walk can make

// Verification in two passes. The head runs the first HB (1 or 2) 32-base
// blocks of every candidate, the tail finishes the ones that can
// still end at or below e, queued with their state.
//
// The band of step i holds the edit-distance cells of read prefix i against
// window positions i .. i + 31: cell 0 is the site error, and bit k of VP /
// VN says that cell k + 1 is one above / below cell k. The final scan
// (mapper_cpe.c:634-650) reports the first of cells 0 .. last_high of the
// last step that is <= e. No cell of a later step is below the minimum of
// cells 0 .. last_high of this step: every cell is a diagonal (+0 or +1), an
// up (+1) or a left (+1) move from cells of the previous step or its own, and
// a path into the scan range from cell k > last_high needs k - last_high up
// moves while (cell k) + k never decreases as k grows. So when that minimum is
// already above e after the head, the full run would return
// (SWM_MAXERROR, -1), and the head writes that result at once. On the
// human-scale genome most candidates stop there.
// Minimum over cells 0 .. lh of a band: site error err, vertical steps VP /
// VN (the reference's final scan, taking the minimum instead of the first
// hit). A fixed-length loop: early exits measured slower.
__device__ __forceinline__ int band_scan_min(int err, uint32_t vp, uint32_t vn, int lh) {
    int m = err;
    for (int k = 0; k < lh; k++) {
        err += (int)((vp >> k) & 1u) - (int)((vn >> k) & 1u);
        m = min(m, err);
    }
    return m;
}

// HB: 32-base blocks the head pass runs (1 or 2; the autotuner picks it per
// read-length bucket). Any HB gives the same results: the stop is exact.
template <bool HEAD, int HB>
__global__ void __launch_bounds__(128, HEAD ? 10 : 0) k_verify(const uint32_t *__restrict__ b2,
                                                uint64_t b2_words, uint64_t ref_length, MapBufs B,
                                                uint64_t cap_chunks, uint64_t cap_elems, uint64_t cap_cands,
                                                uint64_t cap_arena) {
    if (block_failed(B, cap_chunks, cap_elems, cap_cands)) return;
    const uint32_t *__restrict__ lens = B.par->lens;
    uint64_t n;
    if (HEAD) {
        const uint64_t nc_all = B.tot[TOT_CANDS];
        n = nc_all < cap_cands ? nc_all : cap_cands;
    } else {
        n = B.tot[TOT_VT];
    }
    unsigned long long cells = 0, passed = 0, steps = 0;
    for (;;) { // persistent warps take work 32 at a time from the queue
        const uint32_t jb = warp_take(&B.tot[HEAD ? TOT_VQ : TOT_VTQ]);
        if (jb >= n) break;
        const uint64_t j = jb + (threadIdx.x & 31);
        if (j >= n) continue;
        uint64_t c;
        uint32_t vp = 0, vn = 0, ones = 0;
        uint32_t cp[32];
        cp[0] = cp[1] = 0;
        if (HEAD) {
            c = j;
        } else {
            const uint2 x = B.vt_x[j];
            const uint4 st = B.vt_st[j], st2 = HB >= 2 ? B.vt_cp[j] : make_uint4(0u, 0u, 0u, 0u);
            c = x.x;
            ones = x.y;
            vp = st.x;
            vn = st.y;
            cp[2] = st.z;
            cp[3] = st.w;
            if (HB >= 2) {
                cp[4] = st2.x;
                cp[5] = st2.y;
                cp[6] = st2.z;
                cp[7] = st2.w;
            }
        }
        const uint32_t item = B.cc_item[c], p = B.cc_pos[c];
        const uint32_t L = lens[item >> 1], e = B.it_e[item];
        uint32_t rl;
        const uint32_t ws = window_start(p, L, e, ref_length, &rl);
        if (HEAD && ws == 0xffffffffu) {
            B.vr_flag[c] = VR_INVALID;
            B.vr_err[c] = SWM_MAXERROR;
            B.vr_mloc[c] = -1;
            continue;
        }
        const uint32_t nblk = (L + 31) >> 5;
        const bool head_only = HEAD && nblk > HB;
        uint32_t WL[SWM_WIN_WORDS], WH[SWM_WIN_WORDS];
        // the head reads window words 0 .. HB only
        load_window(b2, b2_words, ws, head_only ? 32 * HB - 2 * e : L, e, WL, WH);
        const uint32_t *RW = B.it_w + (uint64_t)item * 32;
        uint32_t rw[16];
#pragma unroll
        for (int i = 0; i < 16; i++) rw[i] = (HEAD && i >= 2 * HB) ? 0u : RW[i];
        const uint32_t MASK = (1u << (2 * e + 1)) - 1u;
        const uint32_t b0 = HEAD ? 0u : HB, b1 = HEAD ? min(nblk, (uint32_t)HB) : nblk;
        steps += min(L, 32 * b1) - 32 * b0;
        myers_blocks(WL, WH, rw, L, MASK, b0, b1, vp, vn, ones, cp);
        if (head_only) {
            if (band_scan_min(32 * HB - (int)ones, vp, vn, (int)rl - (int)L) > (int)e) {
                cells += (unsigned long long)L * (2 * e + 1);
                B.vr_err[c] = SWM_MAXERROR;
                B.vr_mloc[c] = -1;
                B.vr_flag[c] = VR_FAIL;
            } else {
                const uint32_t at = atomicAdd(&B.tot[TOT_VT], 1u);
                B.vt_x[at] = make_uint2((uint32_t)c, ones);
                B.vt_st[at] = make_uint4(vp, vn, cp[2], cp[3]);
                if (HB >= 2) B.vt_cp[at] = make_uint4(cp[4], cp[5], cp[6], cp[7]);
            }
            continue;
        }
        int loc;
        const int err = myers_final(vp, vn, ones, L, e, rl, &loc);
        cells += (unsigned long long)L * (2 * e + 1);
        B.vr_err[c] = err;
        B.vr_mloc[c] = loc;
        if (err > (int)e) {
            B.vr_flag[c] = VR_FAIL;
            continue;
        }
        passed++;
        // Hamming shortcut (align_reads, 252-287)
        int start = loc - (int)L + 1;
        int ham = 0;
        for (uint32_t ii = 0; ii * 32 < L; ii++) {
            uint32_t mask = 0xffffffffu;
            if ((ii + 1) * 32 > L) mask >>= (32 - (L - ii * 32));
            const uint32_t lref = swm_fsr(WL[ii], WL[ii + 1], (uint32_t)start);
            const uint32_t href = swm_fsr(WH[ii], WH[ii + 1], (uint32_t)start);
            const uint32_t x = ((RW[16 + 2 * ii + 1] ^ href) | (RW[16 + 2 * ii] ^ lref)) & mask;
            ham += __popc(x);
        }
        uint8_t *slot = B.vr_cig + c * SWM_CIGAR_SLOT;
        if (ham == err) {
            uint8_t txt[8];
            int n = put_len(txt, L);
            txt[n++] = 'M';
            slot[0] = (uint8_t)ham;
            slot[1] = (uint8_t)n;
            for (int i = 0; i < n; i++) slot[2 + i] = txt[i];
            B.vr_tlen[c] = (uint16_t)n;
            B.vr_loc[c] = ws + (uint32_t)start + 1;
            B.vr_flag[c] = VR_HAM;
            continue;
        }
        B.vr_loc[c] = ws; // window start, used by the traceback
        B.vr_flag[c] = VR_NEEDTB;
        const uint32_t at = atomicAdd(&B.tot[TOT_TB], 1u);
        B.tb_list[at] = (uint32_t)c;
        uint4 *cpo = reinterpret_cast<uint4 *>(B.tb_cp + (uint64_t)at * 32);
#pragma unroll
        for (uint32_t k = 0; k < 8; k++)
            if (k < nblk) cpo[k] = make_uint4(cp[4 * k], cp[4 * k + 1], cp[4 * k + 2], cp[4 * k + 3]);
    }
    warp_add_u64(&B.stat[ST_CELLS], cells);
    warp_add_u64(&B.stat[ST_PASSED], passed);
    warp_add_u64(&B.stat[ST_STEPS], steps);
}


// Streaming verification. Every lane runs its own candidate, CH read bases at
// a time, and after each chunk tests whether the band can still end at or
// below e: cell 0 of the band is i - ones after i steps and each of the cells
// 1 .. last_high is at least cell 0 minus the down steps (VN bits) below it,
// so when (i - ones) - popc(VN & cells 0 .. last_high - 1) > e every cell of
// the band, and by the argument above every cell of every later step, is
// above e: the full run would return (SWM_MAXERROR, -1) and the lane writes
// that at once. A lane whose candidate stopped or reached its last base takes
// the next one from the warp's share of the queue (ranges of 32 taken with one
// atomic), so lanes are not held by the slowest candidate of a group. The
// candidates with fewer than CH bases left (about 2% on the human-scale
// genome) are queued with their state for the finishing pass k_verify_finish.
//
// Each lane keeps a sliding window of the packed genome in registers: the
// (lo, hi) word pairs k .. k + 2 that hold window bases i .. i + 95, where k
// is the pair of the chunk's first base, and pair k + 3 loaded ahead; the
// read's word pair of the current 32-base block and the next one likewise.
// A chunk of 16 bases moves k by at most one, so every genome and read word
// is loaded once per candidate, a chunk before it is needed. The per-candidate
// set-up (item, length, threshold, window start) runs for the 32 candidates of
// a range at once with every lane busy, not in the few lanes that happen to
// need a new candidate (on the human-scale genome that cut the kernel's time
// by 6%: 65.6 -> 61.5 ms per 10M reads).
//
// Resident blocks of 128 threads per SM of the streaming verification kernels
// (48 registers: the register file of every SM is full). Launching them with
// fewer so that another mapper's candidate and seed kernels share the SMs was
// slower at every count tried (4-6 blocks, 2-3 mappers).
#define VERIFY_BLOCKS_PER_SM 10
template <int CH>
__global__ void __launch_bounds__(128, VERIFY_BLOCKS_PER_SM)
    k_verify_stream(const uint32_t *__restrict__ b2, uint64_t b2_words, uint64_t ref_length, MapBufs B,
                    uint64_t cap_chunks, uint64_t cap_elems, uint64_t cap_cands) {
    static_assert(CH == 8 || CH == 16, "a chunk moves the window by at most one word pair");
    if (block_failed(B, cap_chunks, cap_elems, cap_cands)) return;
    const uint2 *__restrict__ b2p = reinterpret_cast<const uint2 *>(b2); // (lo, hi) word pairs
    const uint64_t npairs = b2_words / 2;
    auto pair_at = [&](uint64_t q) { return q < npairs ? b2p[q] : make_uint2(0u, 0u); };
    const uint64_t nc_all = B.tot[TOT_CANDS];
    const uint32_t n = (uint32_t)(nc_all < cap_cands ? nc_all : cap_cands);
    const uint32_t lane = lane_id();
    // per-lane counts fit 32 bits: a lane runs at most ceil(cap_cands / lanes of
    // the grid) candidates of at most 254 x 31 cells
    uint32_t cells = 0, nsteps = 0;
    bool drained = false;    // the queue has no more ranges
    bool act = false;
    // meta: read length | e << 8 | (last_high + 1, 0 when last_high < 0) << 16
    uint32_t c = 0, meta = 0, i = 0, vp = 0, vn = 0, ones = 0, ws = 0;
    uint2 a0 = {0, 0}, a1 = {0, 0}, a2 = {0, 0}, nx = {0, 0}, rr = {0, 0}, nrr = {0, 0};
    const uint2 *rwp = nullptr; // the item's read word pairs (lo, hi) per 32-base block
    // A warp sets up the 32 candidates of each range it takes with all
    // lanes at once -- item, length, threshold, window start; rejected windows
    // written, candidates shorter than a chunk queued for the finishing pass --
    // and keeps the rest in a ring of 64 slots {candidate, meta, window start,
    // item}; a lane whose candidate stopped takes the next slot and loads only
    // its window and read words. Fewer than 32 slots are waiting when a range
    // is taken, so the ring never overwrites a slot not yet handed out.
    __shared__ uint4 ring_s[4][64]; // 128 threads: 4 warps
    uint4 *ring = ring_s[threadIdx.x >> 5];
    uint32_t rh = 0, rt = 0; // slots handed out / staged (counts; slot = count & 63)
    for (;;) {
        const unsigned need = __ballot_sync(0xffffffffu, !act);
        if (need) {
            const uint32_t k = __popc(need), r = __popc(need & lanemask_lt());
            while (rt - rh < k && !drained) {
                const uint32_t t = warp_take(&B.tot[TOT_VQ]);
                if (t >= n) {
                    drained = true;
                    break;
                }
                const uint32_t cj = t + lane;
                bool keep = false, shortc = false;
                uint4 rec = make_uint4(0u, 0u, 0u, 0u);
                if (cj < n) {
                    const uint32_t item = B.cc_item[cj], p = B.cc_pos[cj];
                    const uint32_t L = B.par->lens[item >> 1], e = B.it_e[item];
                    uint32_t rl;
                    const uint32_t w0 = window_start(p, L, e, ref_length, &rl);
                    const int lh = (int)rl - (int)L; // last_high: cells 0 .. lh of the final scan
                    if (w0 == 0xffffffffu) {
                        B.vr_flag[cj] = VR_INVALID;
                        B.vr_err[cj] = SWM_MAXERROR;
                        B.vr_mloc[cj] = -1;
                    } else if (L < CH) { // shorter than a chunk: straight to the finishing pass
                        shortc = true;
                    } else {
                        keep = true;
                        rec = make_uint4(cj, L | e << 8 | (uint32_t)(lh > 0 ? lh : 0) << 16, w0, item);
                    }
                }
                const unsigned sm = __ballot_sync(0xffffffffu, shortc);
                if (sm) {
                    const uint32_t leader = __ffs(sm) - 1;
                    uint32_t at = 0;
                    if (lane == leader) at = atomicAdd(&B.tot[TOT_VT], (uint32_t)__popc(sm));
                    at = __shfl_sync(0xffffffffu, at, leader);
                    if (shortc) {
                        const uint32_t q = at + __popc(sm & lanemask_lt());
                        B.vt_x[q] = make_uint2(cj, 0u);
                        B.vt_st[q] = make_uint4(0u, 0u, 0u, 0u);
                    }
                }
                const unsigned km = __ballot_sync(0xffffffffu, keep);
                if (keep) ring[(rt + __popc(km & lanemask_lt())) & 63u] = rec;
                rt += __popc(km);
                __syncwarp();
            }
            const uint32_t got = min(k, rt - rh);
            if (!act && r < got) {
                const uint4 sl = ring[(rh + r) & 63u];
                c = sl.x;
                meta = sl.y;
                ws = sl.z;
                act = true;
                i = vp = vn = ones = 0;
                const uint64_t q = ws >> 5;
                a0 = pair_at(q);
                a1 = pair_at(q + 1);
                a2 = pair_at(q + 2);
                nx = pair_at(q + 3);
                rwp = reinterpret_cast<const uint2 *>(B.it_w + (uint64_t)sl.w * 32);
                rr = rwp[0];
                nrr = (meta & 0xffu) > 32 ? rwp[1] : make_uint2(0u, 0u);
            }
            rh += got;
            __syncwarp(); // slots read before a later range overwrites them
        }
        bool fin = false, dead = false;
        if (act) {
            const uint32_t L = meta & 0xffu, e = (meta >> 8) & 0xffu;
            const uint32_t MASK = (1u << (2 * e + 1)) - 1u, lhm = (1u << (meta >> 16)) - 1u;
            const uint32_t sh = (ws + i) & 31; // window bit of the chunk's first step within pair k
            const uint32_t xl0 = __funnelshift_r(a0.x, a1.x, sh), xl1 = __funnelshift_r(a1.x, a2.x, sh);
            const uint32_t xh0 = __funnelshift_r(a0.y, a1.y, sh), xh1 = __funnelshift_r(a1.y, a2.y, sh);
            const uint32_t rlw = rr.x >> (i & 31), rhw = rr.y >> (i & 31);
            uint32_t acc = 0;
#define SWM_STREAM_STEP(t)                                                                                        \
    {                                                                                                             \
        const uint32_t wls = __funnelshift_r(xl0, xl1, (t)), whs = __funnelshift_r(xh0, xh1, (t));              \
        const uint32_t mL = (uint32_t)((int32_t)(rlw << (31 - (t))) >> 31);                                      \
        const uint32_t mH = (uint32_t)((int32_t)(rhw << (31 - (t))) >> 31);                                      \
        const uint32_t eq = ~((wls ^ mL) | (whs ^ mH)) & MASK;                                                   \
        uint32_t x = eq | vn;                                                                                     \
        const uint32_t d0 = ((vp + (x & vp)) ^ vp) | x;                                                          \
        const uint32_t hn = vp & d0;                                                                              \
        const uint32_t hp = vn | ~(vp | d0);                                                                      \
        x = d0 >> 1;                                                                                              \
        vn = x & hp;                                                                                              \
        vp = hn | ~(x | hp);                                                                                      \
        acc = __funnelshift_r(acc, d0, 1);                                                                        \
    }
#pragma unroll
            for (uint32_t t = 0; t < CH; t++) SWM_STREAM_STEP(t)
#undef SWM_STREAM_STEP
            ones += __popc(acc);
            i += CH;
            nsteps += CH;
            // a candidate with fewer than CH bases left goes to the finishing
            // pass, which runs it from the first base: every chunk is whole
            if (i + CH > L) {
                fin = true;
            } else if ((int)(i - ones) - (int)__popc(vn & lhm) > (int)e) {
                dead = true;
            } else {
                if (sh + CH >= 32) { // the next chunk starts in pair k + 1
                    a0 = a1;
                    a1 = a2;
                    a2 = nx;
                    nx = pair_at((uint64_t)((ws + i) >> 5) + 3);
                }
                if ((i & 31) == 0) { // the next chunk starts a new 32-base block of the read
                    rr = nrr;
                    nrr = (i >> 5) + 1 < 8 ? rwp[(i >> 5) + 1] : make_uint2(0u, 0u);
                }
            }
        }
        const unsigned fm = __ballot_sync(0xffffffffu, fin);
        if (fm) {
            const uint32_t leader = __ffs(fm) - 1;
            uint32_t at = 0;
            if (lane == leader) at = atomicAdd(&B.tot[TOT_VT], (uint32_t)__popc(fm));
            at = __shfl_sync(0xffffffffu, at, leader);
            if (fin) { // the finishing pass resumes from this state
                const uint32_t q = at + __popc(fm & lanemask_lt());
                B.vt_x[q] = make_uint2(c, ones);
                B.vt_st[q] = make_uint4(vp, vn, i, 0u);
                act = false;
            }
        }
        if (dead) {
            cells += (meta & 0xffu) * (2 * ((meta >> 8) & 0xffu) + 1);
            B.vr_err[c] = SWM_MAXERROR;
            B.vr_mloc[c] = -1;
            B.vr_flag[c] = VR_FAIL;
            act = false;
        }
        if (drained && rh >= rt && !__any_sync(0xffffffffu, act)) break;
    }
    warp_add_u64(&B.stat[ST_CELLS], (unsigned long long)cells);
    warp_add_u64(&B.stat[ST_STEPS], (unsigned long long)nsteps);
}

// Streaming verification with two candidates per lane (every e <= 7). The
// band of e <= 7 is at most 15 bits, and the recurrence run in a 15-bit lane
// gives the same band, D0 bit 0 and state as in a 32-bit one, so a lane packs
// candidate A in bits 0..14 and B in bits 16..30 of one word. Bits 15 and 31
// are guards kept at 0 in VP, VN and X & VP, so the carry of VP + (X & VP)
// out of a half stops in its guard; D0 is masked to the halves (the carry
// would otherwise enter the top bit of X through D0 >> 1) and VN after the
// shift (bit 15 gets B's bit 0); VP's guards then stay 0 by themselves. The
// step costs 10 logic ops for both candidates plus their pattern words: each
// half's window bits by funnel shift and one byte permute, the read bases as
// all-ones / all-zeros per half by the permute's sign replication. Each half
// stops, finishes and refills on its own exactly as in k_verify_stream, and
// its state goes to k_verify_finish as a 32-bit lane (the same continuation).
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel) {
    uint32_t d;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(sel));
    return d;
}

template <int CH>
__global__ void __launch_bounds__(128, VERIFY_BLOCKS_PER_SM)
    k_verify_pair(const uint32_t *__restrict__ b2, uint64_t b2_words, uint64_t ref_length, MapBufs B,
                  uint64_t cap_chunks, uint64_t cap_elems, uint64_t cap_cands) {
    static_assert(CH == 16, "a chunk is 16 read bases: one halfword of read bits per half");
    if (block_failed(B, cap_chunks, cap_elems, cap_cands)) return;
    const uint2 *__restrict__ b2p = reinterpret_cast<const uint2 *>(b2);
    const uint64_t npairs = b2_words / 2;
    auto pair_at = [&](uint64_t q) { return q < npairs ? b2p[q] : make_uint2(0u, 0u); };
    const uint64_t nc_all = B.tot[TOT_CANDS];
    const uint32_t n = (uint32_t)(nc_all < cap_cands ? nc_all : cap_cands);
    const uint32_t lane = lane_id();
    uint32_t cells = 0, nsteps = 0; // per lane, both halves
    bool drained = false;
    bool act[2] = {false, false};
    // per half: candidate, L | e << 8 | max(last_high, 0) << 16, bases done, window start, item, D0 bit-0 count
    uint32_t c[2] = {0, 0}, meta[2] = {0, 0}, i[2] = {0, 0}, ws[2] = {0, 0}, item[2] = {0, 0}, ones[2] = {0, 0};
    uint32_t vp = 0, vn = 0, PM = 0; // packed state and band masks
    // Candidates are set up 32 at a time with every lane (as in
    // k_verify_stream) into a ring of 128 slots per warp; up to 64 halves can
    // ask at once, so fewer than 64 slots are waiting when a range is taken.
    __shared__ uint4 ring_s[4][128]; // 128 threads: 4 warps
    uint4 *ring = ring_s[threadIdx.x >> 5];
    uint32_t rh = 0, rt = 0; // slots handed out / staged (counts; slot = count & 127)
    for (;;) {
        const unsigned needA = __ballot_sync(0xffffffffu, !act[0]), needB = __ballot_sync(0xffffffffu, !act[1]);
        bool fin[2] = {false, false}, dead[2] = {false, false};
        if (needA | needB) {
            const uint32_t na = __popc(needA), k = na + __popc(needB);
            while (rt - rh < k && !drained) {
                const uint32_t t = warp_take(&B.tot[TOT_VQ]);
                if (t >= n) {
                    drained = true;
                    break;
                }
                const uint32_t cj = t + lane;
                bool keep = false, shortc = false;
                uint4 rec = make_uint4(0u, 0u, 0u, 0u);
                if (cj < n) {
                    const uint32_t it = B.cc_item[cj], p = B.cc_pos[cj];
                    const uint32_t L = B.par->lens[it >> 1], e = B.it_e[it];
                    uint32_t rl;
                    const uint32_t w0 = window_start(p, L, e, ref_length, &rl);
                    const int lh = (int)rl - (int)L;
                    if (w0 == 0xffffffffu) {
                        B.vr_flag[cj] = VR_INVALID;
                        B.vr_err[cj] = SWM_MAXERROR;
                        B.vr_mloc[cj] = -1;
                    } else if (L < CH) { // shorter than a chunk: straight to the finishing pass
                        shortc = true;
                    } else {
                        keep = true;
                        rec = make_uint4(cj, L | e << 8 | (uint32_t)(lh > 0 ? lh : 0) << 16, w0, it);
                    }
                }
                const unsigned sm = __ballot_sync(0xffffffffu, shortc);
                if (sm) {
                    const uint32_t leader = __ffs(sm) - 1;
                    uint32_t at = 0;
                    if (lane == leader) at = atomicAdd(&B.tot[TOT_VT], (uint32_t)__popc(sm));
                    at = __shfl_sync(0xffffffffu, at, leader);
                    if (shortc) {
                        const uint32_t q = at + __popc(sm & lanemask_lt());
                        B.vt_x[q] = make_uint2(cj, 0u);
                        B.vt_st[q] = make_uint4(0u, 0u, 0u, 0u);
                    }
                }
                const unsigned km = __ballot_sync(0xffffffffu, keep);
                if (keep) ring[(rt + __popc(km & lanemask_lt())) & 127u] = rec;
                rt += __popc(km);
                __syncwarp();
            }
            const uint32_t got = min(k, rt - rh);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const uint32_t r = h == 0 ? __popc(needA & lanemask_lt()) : na + __popc(needB & lanemask_lt());
                if (act[h] || r >= got) continue;
                const uint4 sl = ring[(rh + r) & 127u];
                const uint32_t hm = h ? 0xffff0000u : 0x0000ffffu, e = (sl.y >> 8) & 0xffu;
                c[h] = sl.x;
                meta[h] = sl.y;
                ws[h] = sl.z;
                item[h] = sl.w;
                vp &= ~hm;
                vn &= ~hm;
                PM = (PM & ~hm) | (((1u << (2 * e + 1)) - 1u) << (16 * h));
                ones[h] = 0;
                i[h] = 0;
                act[h] = true;
            }
            rh += got;
            __syncwarp(); // slots read before a later range overwrites them
        }
        if (act[0] || act[1]) {
            uint32_t xl0[2], xh0[2], rb[2][2];
#pragma unroll
            for (int h = 0; h < 2; h++) { // window bits and read bits of the chunk (inactive half: zeros)
                const uint32_t pos = ws[h] + i[h], sh = pos & 31;
                uint2 a0 = make_uint2(0u, 0u), a1 = a0, rr = a0;
                if (act[h]) {
                    const uint64_t q = pos >> 5;
                    a0 = pair_at(q);
                    a1 = pair_at(q + 1);
                    rr = reinterpret_cast<const uint2 *>(B.it_w + (uint64_t)item[h] * 32)[i[h] >> 5];
                }
                // window bits 0 .. 29 from the chunk's first base: a 16-base chunk and
                // a band of <= 15 bits
                xl0[h] = __funnelshift_r(a0.x, a1.x, sh);
                xh0[h] = __funnelshift_r(a0.y, a1.y, sh);
                // read base t of the chunk at bit 15 - t of the half (bit reverse of the low halfword)
                rb[h][0] = __brev((rr.x >> (i[h] & 31)) & 0xffffu);
                rb[h][1] = __brev((rr.y >> (i[h] & 31)) & 0xffffu);
            }
            // A's reversed bits in 15..0, B's in 31..16
            const uint32_t RL = prmt(rb[0][0], rb[1][0], 0x7632u), RH = prmt(rb[0][1], rb[1][1], 0x7632u);
            uint32_t acc = 0;
#pragma unroll
            for (uint32_t t = 0; t < CH; t++) {
                // window bits t .. t + 14 of each half (t + 14 <= 29: one word)
                const uint32_t wl = prmt(xl0[0] >> t, xl0[1] >> t, 0x5410u);
                const uint32_t wh = prmt(xh0[0] >> t, xh0[1] >> t, 0x5410u);
                // read base t of each half as all-ones / all-zeros: the sign of bytes 1 and 3
                const uint32_t mL = prmt(RL << t, 0u, 0xbb99u), mH = prmt(RH << t, 0u, 0xbb99u);
                const uint32_t eq = ~((wl ^ mL) | (wh ^ mH)) & PM;
                uint32_t x = eq | vn;
                const uint32_t d0 = (((vp + (x & vp)) ^ vp) | x) & 0x7fff7fffu;
                const uint32_t hn = vp & d0;
                const uint32_t hp = vn | ~(vp | d0);
                x = d0 >> 1;
                vn = x & hp & 0x7fff7fffu;
                vp = hn | ~(x | hp);
                acc += d0 & 0x00010001u;
            }
#pragma unroll
            for (int h = 0; h < 2; h++) {
                if (!act[h]) continue;
                ones[h] += h ? acc >> 16 : acc & 0xffffu;
                i[h] += CH;
                nsteps += CH;
                const uint32_t L = meta[h] & 0xffu, e = (meta[h] >> 8) & 0xffu;
                const uint32_t vnh = (vn >> (16 * h)) & 0x7fffu, lhm = (1u << (meta[h] >> 16)) - 1u;
                if (i[h] + CH > L) fin[h] = true;
                else if ((int)(i[h] - ones[h]) - (int)__popc(vnh & lhm) > (int)e) dead[h] = true;
            }
        }
        const unsigned fA = __ballot_sync(0xffffffffu, fin[0]), fB = __ballot_sync(0xffffffffu, fin[1]);
        if (fA | fB) {
            const uint32_t leader = __ffs(fA | fB) - 1;
            uint32_t at = 0;
            if (lane == leader) at = atomicAdd(&B.tot[TOT_VT], (uint32_t)(__popc(fA) + __popc(fB)));
            at = __shfl_sync(0xffffffffu, at, leader);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                if (!fin[h]) continue;
                const uint32_t q = at + (h == 0 ? __popc(fA & lanemask_lt()) : __popc(fA) + __popc(fB & lanemask_lt()));
                B.vt_x[q] = make_uint2(c[h], ones[h]);
                B.vt_st[q] = make_uint4((vp >> (16 * h)) & 0x7fffu, (vn >> (16 * h)) & 0x7fffu, i[h], 0u);
                act[h] = false;
            }
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
            if (!dead[h]) continue;
            cells += (meta[h] & 0xffu) * (2 * ((meta[h] >> 8) & 0xffu) + 1);
            B.vr_err[c[h]] = SWM_MAXERROR;
            B.vr_mloc[c[h]] = -1;
            B.vr_flag[c[h]] = VR_FAIL;
            act[h] = false;
        }
        if (drained && rh >= rt && !__any_sync(0xffffffffu, act[0] || act[1])) break;
    }
    warp_add_u64(&B.stat[ST_CELLS], (unsigned long long)cells);
    warp_add_u64(&B.stat[ST_STEPS], (unsigned long long)nsteps);
}

// Finishing pass of the streaming form. Each queued candidate resumes from
// the state k_verify_stream left (at most CH - 1 bases to go), then the final
// scan (634-650); a passing candidate gets the Hamming check (252-287) and,
// when that does not resolve it, a rerun from the first base that leaves the
// traceback its (VP, VN) checkpoints, as the two-pass tail does.
__global__ void __launch_bounds__(128, 8) k_verify_finish(const uint32_t *__restrict__ b2, uint64_t b2_words,
                                                       uint64_t ref_length, MapBufs B, uint64_t cap_chunks,
                                                       uint64_t cap_elems, uint64_t cap_cands, uint64_t cap_arena) {
    if (block_failed(B, cap_chunks, cap_elems, cap_cands)) return;
    const uint2 *__restrict__ b2p = reinterpret_cast<const uint2 *>(b2);
    const uint64_t npairs = b2_words / 2;
    auto pair_at = [&](uint64_t q) { return q < npairs ? b2p[q] : make_uint2(0u, 0u); };
    const uint64_t n = B.tot[TOT_VT];
    unsigned long long cells = 0, passed = 0, steps = 0;
    for (;;) {
        const uint32_t jb = warp_take(&B.tot[TOT_VTQ]);
        if (jb >= n) break;
        const uint64_t j = jb + (threadIdx.x & 31);
        if (j >= n) continue;
        const uint2 x = B.vt_x[j];
        const uint4 st = B.vt_st[j];
        const uint32_t c = x.x, i0 = st.z;
        uint32_t ones = x.y, vp = st.x, vn = st.y;
        const uint32_t item = B.cc_item[c], L = B.par->lens[item >> 1], e = B.it_e[item];
        uint32_t rl;
        const uint32_t ws = window_start(B.cc_pos[c], L, e, ref_length, &rl);
        const uint32_t MASK = (1u << (2 * e + 1)) - 1u;
        const uint32_t *RW = B.it_w + (uint64_t)item * 32;
        {   // the last L - i0 < 32 bases
            const uint32_t pos = ws + i0, sh = pos & 31;
            const uint64_t q = pos >> 5;
            const uint2 a0 = pair_at(q), a1 = pair_at(q + 1), a2 = pair_at(q + 2);
            const uint32_t xl0 = __funnelshift_r(a0.x, a1.x, sh), xl1 = __funnelshift_r(a1.x, a2.x, sh);
            const uint32_t xh0 = __funnelshift_r(a0.y, a1.y, sh), xh1 = __funnelshift_r(a1.y, a2.y, sh);
            const uint32_t rb = i0 >> 5, rs = i0 & 31;
            const uint32_t rlw = __funnelshift_r(RW[2 * rb], rb + 1 < 8 ? RW[2 * rb + 2] : 0u, rs);
            const uint32_t rhw = __funnelshift_r(RW[2 * rb + 1], rb + 1 < 8 ? RW[2 * rb + 3] : 0u, rs);
            uint32_t acc = 0;
            for (uint32_t t = 0; t < L - i0; t++) {
                const uint32_t wls = __funnelshift_r(xl0, xl1, t), whs = __funnelshift_r(xh0, xh1, t);
                const uint32_t mL = 0u - ((rlw >> t) & 1u), mH = 0u - ((rhw >> t) & 1u);
                const uint32_t eq = ~((wls ^ mL) | (whs ^ mH)) & MASK;
                uint32_t xx = eq | vn;
                const uint32_t d0 = ((vp + (xx & vp)) ^ vp) | xx;
                const uint32_t hn = vp & d0;
                const uint32_t hp = vn | ~(vp | d0);
                xx = d0 >> 1;
                vn = xx & hp;
                vp = hn | ~(xx | hp);
                acc = __funnelshift_r(acc, d0, 1);
            }
            ones += __popc(acc);
            steps += L - i0;
        }
        int loc;
        const int err = myers_final(vp, vn, ones, L, e, rl, &loc);
        cells += (unsigned long long)L * (2 * e + 1);
        B.vr_err[c] = err;
        B.vr_mloc[c] = loc;
        if (err > (int)e) {
            B.vr_flag[c] = VR_FAIL;
            continue;
        }
        passed++;
        uint32_t WL[SWM_WIN_WORDS], WH[SWM_WIN_WORDS];
        load_window(b2, b2_words, ws, L, e, WL, WH);
        // Hamming shortcut (align_reads, 252-287)
        const int start = loc - (int)L + 1;
        int ham = 0;
        for (uint32_t ii = 0; ii * 32 < L; ii++) {
            uint32_t mask = 0xffffffffu;
            if ((ii + 1) * 32 > L) mask >>= (32 - (L - ii * 32));
            const uint32_t lref = swm_fsr(WL[ii], WL[ii + 1], (uint32_t)start);
            const uint32_t href = swm_fsr(WH[ii], WH[ii + 1], (uint32_t)start);
            const uint32_t xm = ((RW[16 + 2 * ii + 1] ^ href) | (RW[16 + 2 * ii] ^ lref)) & mask;
            ham += __popc(xm);
        }
        uint8_t *slot = B.vr_cig + c * SWM_CIGAR_SLOT;
        if (ham == err) {
            uint8_t txt[8];
            int nt = put_len(txt, L);
            txt[nt++] = 'M';
            slot[0] = (uint8_t)ham;
            slot[1] = (uint8_t)nt;
            for (int t = 0; t < nt; t++) slot[2 + t] = txt[t];
            B.vr_tlen[c] = (uint16_t)nt;
            B.vr_loc[c] = ws + (uint32_t)start + 1;
            B.vr_flag[c] = VR_HAM;
            continue;
        }
        // checkpoints for the traceback: the recurrence again from the first base
        uint32_t rw[16];
#pragma unroll
        for (int t = 0; t < 16; t++) rw[t] = RW[t];
        uint32_t cp[32];
        uint32_t vp2 = 0, vn2 = 0, ones2 = 0;
        const uint32_t nblk = (L + 31) >> 5;
        myers_blocks(WL, WH, rw, L, MASK, 0, nblk, vp2, vn2, ones2, cp);
        steps += L;
        B.vr_loc[c] = ws; // window start, used by the traceback
        B.vr_flag[c] = VR_NEEDTB;
        const uint32_t at = atomicAdd(&B.tot[TOT_TB], 1u);
        B.tb_list[at] = c;
        uint4 *cpo = reinterpret_cast<uint4 *>(B.tb_cp + (uint64_t)at * 32);
#pragma unroll
        for (uint32_t kq = 0; kq < 8; kq++)
            if (kq < nblk) cpo[kq] = make_uint4(cp[4 * kq], cp[4 * kq + 1], cp[4 * kq + 2], cp[4 * kq + 3]);
    }
    warp_add_u64(&B.stat[ST_CELLS], cells);
    warp_add_u64(&B.stat[ST_PASSED], passed);
    warp_add_u64(&B.stat[ST_STEPS], steps);
}

// Traceback of the passing candidates that the Hamming check did not resolve
// (align_reads, mapper_cpe.c:288-509): walk back from (L - 1, location)
// through the D0 / HP words of the Myers run and emit the start position and
// the CIGAR.
//
// The walk keeps match_site = i + search_site. While 0 <= search_site <= 2e
// the pattern bit of step i at search_site is [ref(match_site) == read(i)]
// and D0 contains it, so a step whose bases agree is always an M step: runs
// of agreeing bases along the diagonal are taken 32 at a time from the bit
// planes. Only the other steps (errors, or walks outside the band) need D0 /
// HP, which are recomputed from the (VP, VN) checkpoint k_verify left at the
// start of their 32-base block. The run-length route stays in shared memory;
// a walk with more than TB_ROUTE runs is handed to k_traceback_slow.
#define TB_THREADS 64
#define TB_ROUTE 48

struct TbSmem {
    uint16_t route[TB_ROUTE][TB_THREADS]; // size | kind << 12 (M S I D)
};

// D0 and HP of read base i: Myers steps from the checkpoint before the
// 16-base half block that holds it (at most 16 steps).
__device__ __forceinline__ void myers_at(const uint32_t *WL, const uint32_t *WH, const uint32_t *rw,
                                         const uint32_t *cp, int i, uint32_t MASK, uint32_t &d0o, uint32_t &hpo) {
    const uint32_t b = (uint32_t)i >> 5, h = ((uint32_t)i >> 4) & 1u, tend = (uint32_t)i & 31;
    uint32_t vp = cp[4 * b + 2 * h], vn = cp[4 * b + 2 * h + 1]; // checkpoint before base 16 (2 b + h)
    const uint32_t wl0 = WL[b], wl1 = WL[b + 1], wh0 = WH[b], wh1 = WH[b + 1];
    const uint32_t rlw = rw[2 * b], rhw = rw[2 * b + 1];
    uint32_t d0 = 0, hp = 0;
    for (uint32_t t = 16 * h; t <= tend; t++) {
        const uint32_t wls = __funnelshift_r(wl0, wl1, t), whs = __funnelshift_r(wh0, wh1, t);
        const uint32_t mL = 0u - ((rlw >> t) & 1u), mH = 0u - ((rhw >> t) & 1u);
        const uint32_t eq = ~((wls ^ mL) | (whs ^ mH)) & MASK;
        uint32_t x = eq | vn;
        d0 = ((vp + (x & vp)) ^ vp) | x;
        const uint32_t hn = vp & d0;
        hp = vn | ~(vp | d0);
        x = d0 >> 1;
        vn = x & hp;
        vp = hn | ~(x | hp);
    }
    d0o = d0;
    hpo = hp;
}

// Bits start .. start + 31 of a bit array held as words P[0], P[st], P[2 st]
// ...; positions below 0 read 0.
__device__ __forceinline__ uint32_t bits32(const uint32_t *P, int st, int start) {
    const int wi = start >> 5; // floor
    const uint32_t a = wi >= 0 ? P[wi * st] : 0u, b = wi + 1 >= 0 ? P[(wi + 1) * st] : 0u;
    return __funnelshift_r(a, b, (uint32_t)start & 31);
}

// Number of steps i, i - 1, ... (at most i + 1) whose read base equals the
// window base at the same offset s.
__device__ __forceinline__ int match_run(const uint32_t *WL, const uint32_t *WH, const uint32_t *rw, int i, int s) {
    int run = 0, pos = i;
    while (pos >= 0) {
        const int lo = pos - 31;
        const uint32_t x = (bits32(rw, 2, lo) ^ bits32(WL, 1, lo + s)) | (bits32(rw + 1, 2, lo) ^ bits32(WH, 1, lo + s));
        const int k = x ? __clz(x) : 32;
        if (k >= pos + 1) return run + pos + 1;
        run += k;
        if (k < 32) break;
        pos -= 32;
    }
    return run;
}

__global__ void __launch_bounds__(TB_THREADS) k_traceback(const uint32_t *__restrict__ b2, uint64_t b2_words,
                                                          uint64_t ref_length, MapBufs B, uint64_t cap_chunks,
                                                          uint64_t cap_elems, uint64_t cap_cands, uint64_t cap_arena) {
    __shared__ TbSmem T;
    if (block_failed(B, cap_chunks, cap_elems, cap_cands)) return;
    const uint32_t *__restrict__ lens = B.par->lens;
    const uint32_t tid = threadIdx.x;
    const uint64_t ntb = B.tot[TOT_TB];
    for (;;) { // persistent warps take tracebacks 32 at a time from the queue (walks vary in length)
        const uint32_t qb = warp_take(&B.tot[TOT_TBQ]);
        if (qb >= ntb) break;
        const uint64_t q = qb + (tid & 31);
        if (q >= ntb) continue;
        const uint32_t c = B.tb_list[q];
        const uint32_t item = B.cc_item[c];
        const uint32_t L = lens[item >> 1], e = B.it_e[item];
        const uint32_t ws = B.vr_loc[c];
        const int err = B.vr_err[c], loc = B.vr_mloc[c];
        uint32_t WL[SWM_WIN_WORDS], WH[SWM_WIN_WORDS];
        load_window(b2, b2_words, ws, L, e, WL, WH);
        const uint32_t *RW = B.it_w + (uint64_t)item * 32;
        uint32_t rw[16], cp[32];
        const uint4 *cps = reinterpret_cast<const uint4 *>(B.tb_cp + q * 32);
        const uint32_t nblk = (L + 31) >> 5;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint4 r4 = reinterpret_cast<const uint4 *>(RW)[k];
            rw[4 * k] = r4.x;
            rw[4 * k + 1] = r4.y;
            rw[4 * k + 2] = r4.z;
            rw[4 * k + 3] = r4.w;
        }
#pragma unroll
        for (uint32_t k = 0; k < 8; k++) { // (VP, VN) before bases 32 k and 32 k + 16
            const uint4 c4 = k < nblk ? cps[k] : make_uint4(0u, 0u, 0u, 0u);
            cp[4 * k] = c4.x;
            cp[4 * k + 1] = c4.y;
            cp[4 * k + 2] = c4.z;
            cp[4 * k + 3] = c4.w;
        }
        const uint32_t MASK = (1u << (2 * e + 1)) - 1u;
        auto bits = [&](int i, int ss, uint32_t *d0b, uint32_t *hpb) {
            uint32_t d0, hp;
            myers_at(WL, WH, rw, cp, i, MASK, d0, hp);
            const bool in = ss >= 0 && ss < 32; // defined read of bits outside 0..31: 0
            *d0b = in ? ((d0 >> ss) & 1u) : 0u;
            *hpb = in ? ((hp >> ss) & 1u) : 0u;
        };
#define TREF(m_) (((WL[(m_) >> 5] >> ((m_) & 31)) & 1u) | (((WH[(m_) >> 5] >> ((m_) & 31)) & 1u) << 1))
#define TREAD(r_) (((rw[2 * ((r_) >> 5)] >> ((r_) & 31)) & 1u) | (((rw[2 * ((r_) >> 5) + 1] >> ((r_) & 31)) & 1u) << 1))
        int start = loc - (int)L + 1;
        int match_site = loc;
        int search_site = match_site - ((int)L - 1);
        int i = (int)L - 1, sum_err = 0;
        uint32_t nr = 0; // route entries written (index 1 .. nr in the reference's numbering)
        bool overflow = false;
        int pre_size = 1;
        uint32_t pre = 0; // 0 M, 1 S, 2 I, 3 D
        auto flush_run = [&](uint32_t kind) { // a new run of `kind` starts
            if (nr < TB_ROUTE) T.route[nr][tid] = (uint16_t)(pre_size | (pre << 12));
            else overflow = true;
            nr++;
            pre_size = 1;
            pre = kind;
        };
        auto push = [&](uint32_t kind) {
            if (pre != kind) flush_run(kind);
            else pre_size++;
        };
        { // first step, mapper_cpe.c:380-410
            uint32_t d0b, hpb;
            bits(i, search_site, &d0b, &hpb);
            if (d0b && TREF(match_site) == TREAD(i)) {
                i--; pre = 0; match_site--;
            } else if (!d0b && TREF(match_site) != TREAD(i)) {
                i--; pre = 1; match_site--; sum_err++;
            } else if (hpb) {
                i--; search_site++; pre = 1; sum_err++; start++; // labelled S in the reference
            } else {
                search_site--; pre = 3; match_site--; sum_err++; start--;
            }
        }
        // mapper_cpe.c:412-466. One iteration = a run of matching steps (if
        // any) and the step after it: a run stops at a base that differs, so
        // the reference's next iteration would find no run and take that
        // step; doing both here keeps the lanes of a warp in step.
        while (i >= 0) {
            if (sum_err == err) break;
            if (match_site < 0) break; // defined stop below the window start
            if (search_site >= 0 && search_site <= 2 * (int)e) {
                const int run = match_run(WL, WH, rw, i, search_site);
                if (run > 0) { // run M steps
                    if (pre != 0) {
                        flush_run(0);
                        pre_size = run;
                    } else {
                        pre_size += run;
                    }
                    i -= run;
                    match_site -= run;
                    if (i < 0 || match_site < 0) break;
                }
            }
            uint32_t d0b, hpb;
            bits(i, search_site, &d0b, &hpb);
            if (d0b && TREF(match_site) == TREAD(i)) {
                i--; match_site--; push(0);
            } else if (!d0b && TREF(match_site) != TREAD(i)) {
                i--; match_site--; sum_err++; push(1);
            } else if (hpb) {
                i--; search_site++; sum_err++; push(2); start++;
            } else {
                search_site--; match_site--; sum_err++; push(3); start--;
            }
        }
#undef TREF
#undef TREAD
        if (nr < TB_ROUTE) T.route[nr][tid] = (uint16_t)(pre_size | (pre << 12));
        else overflow = true;
        nr++;
        if (i >= 0) {
            if (nr < TB_ROUTE) T.route[nr][tid] = (uint16_t)((i + 1) | (0u << 12));
            else overflow = true;
            nr++;
        }
        if (overflow) {
            const uint32_t at = atomicAdd(&B.tot[TOT_SLOW], 1u);
            B.slow_list[at] = c;
            continue;
        }
        // CIGAR text, read start first: consecutive M / S runs merge into M
        // (mapper_cpe.c:486-504). First its length, then the bytes.
        static const char KC[4] = {'M', 'S', 'I', 'D'};
        auto digits = [](uint32_t v) -> int {
            int d = 0;
            for (; v; v /= 10) d++;
            return d;
        };
        int n = 0;
        for (int j = (int)nr - 1; j >= 0;) {
            const uint32_t kind = T.route[j][tid] >> 12;
            if (kind <= 1) {
                uint32_t smv = 0;
                while (j >= 0 && (T.route[j][tid] >> 12) <= 1) {
                    smv += T.route[j][tid] & 0xfffu;
                    j--;
                }
                n += digits(smv) + 1;
            } else {
                n += digits(T.route[j][tid] & 0xfffu) + 1;
                j--;
            }
        }
        uint8_t *slot = B.vr_cig + (uint64_t)c * SWM_CIGAR_SLOT;
        uint8_t *dst = slot + 2;
        if (n > SWM_CIGAR_SLOT - 2) {
            const uint32_t at = atomicAdd(&B.tot[TOT_ARENA], (uint32_t)n);
            if ((uint64_t)at + n > cap_arena) {
                atomicOr(&B.tot[TOT_FLAGS], OV_ARENA);
                continue;
            }
            dst = B.arena + at;
            B.vr_aoff[c] = at;
        }
        int w = 0;
        for (int j = (int)nr - 1; j >= 0;) {
            const uint32_t kind = T.route[j][tid] >> 12;
            uint32_t v;
            char ch;
            if (kind <= 1) {
                v = 0;
                while (j >= 0 && (T.route[j][tid] >> 12) <= 1) {
                    v += T.route[j][tid] & 0xfffu;
                    j--;
                }
                ch = 'M';
            } else {
                v = T.route[j][tid] & 0xfffu;
                ch = KC[kind];
                j--;
            }
            w += put_len(dst + w, v);
            dst[w++] = (uint8_t)ch;
        }
        slot[0] = (uint8_t)err;
        slot[1] = (uint8_t)n;
        B.vr_tlen[c] = (uint16_t)n;
        B.vr_loc[c] = ws + (uint32_t)start + 1;
        B.vr_flag[c] = VR_TB;
    }
}

// Traceback with the whole D0 / HP history in local memory, for the rare walks
// whose route outgrows the shared-memory path of k_traceback (align_reads,
// mapper_cpe.c:288-509).
__global__ void __launch_bounds__(128) k_traceback_slow(const uint32_t *__restrict__ b2, uint64_t b2_words,
                                                        uint64_t ref_length, MapBufs B, uint64_t cap_chunks,
                                                        uint64_t cap_elems, uint64_t cap_cands, uint64_t cap_arena) {
    if (block_failed(B, cap_chunks, cap_elems, cap_cands)) return;
    const uint32_t *__restrict__ lens = B.par->lens;
    const uint64_t nslow = B.tot[TOT_SLOW];
    for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nslow; q += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t c = B.slow_list[q];
        const uint32_t item = B.cc_item[c];
        const uint32_t L = lens[item >> 1], e = B.it_e[item];
        const uint32_t ws = B.vr_loc[c];
        const int err = B.vr_err[c], loc = B.vr_mloc[c];
        uint32_t rl;
        window_start(B.cc_pos[c], L, e, ref_length, &rl);
        uint32_t WL[SWM_WIN_WORDS], WH[SWM_WIN_WORDS];
        load_window(b2, b2_words, ws, L, e, WL, WH);
        const uint32_t *RW = B.it_w + (uint64_t)item * 32;
        uint32_t rw[16];
#pragma unroll
        for (int i = 0; i < 16; i++) rw[i] = RW[i];
        int start = loc - (int)L + 1;
        uint8_t *slot = B.vr_cig + c * SWM_CIGAR_SLOT;
        uint32_t d0h[SWM_MAX_READ_LEN], hph[SWM_MAX_READ_LEN];
        myers_history(WL, WH, rw, L, e, d0h, hph);
        int match_site = loc;
        int search_site = match_site - ((int)L - 1);
        int i = (int)L - 1, sum_err = 0, jj = 1;
        int pre_size = 1;
        char pre_char = 'N';
        uint16_t rsz[3 * SWM_MAX_READ_LEN + 64];
        char rch[3 * SWM_MAX_READ_LEN + 64];
#define TBBIT(arr, ii_, s_) (((s_) >= 0 && (s_) < 32) ? (((arr)[ii_] >> (s_)) & 1u) : 0u)
#define TBREF(m_) (((WL[(m_) >> 5] >> ((m_) & 31)) & 1u) | (((WH[(m_) >> 5] >> ((m_) & 31)) & 1u) << 1))
#define TBREAD(r_) (((rw[2 * ((r_) >> 5)] >> ((r_) & 31)) & 1u) | (((rw[2 * ((r_) >> 5) + 1] >> ((r_) & 31)) & 1u) << 1))
        if (TBBIT(d0h, i, search_site) && TBREF(match_site) == TBREAD(i)) {
            i--; pre_size = 1; pre_char = 'M'; match_site--;
        } else if (!TBBIT(d0h, i, search_site) && TBREF(match_site) != TBREAD(i)) {
            i--; pre_size = 1; pre_char = 'S'; match_site--; sum_err++;
        } else if (TBBIT(hph, i, search_site)) {
            i--; search_site++; pre_size = 1; pre_char = 'S'; sum_err++; start++;
        } else {
            search_site--; pre_size = 1; pre_char = 'D'; match_site--; sum_err++; start--;
        }
        while (i >= 0) {
            if (sum_err == err) break;
            if (match_site < 0) break; // defined stop below the window start
            if (TBBIT(d0h, i, search_site) && TBREF(match_site) == TBREAD(i)) {
                i--; match_site--;
                if (pre_char != 'M') { rsz[jj] = (uint16_t)pre_size; rch[jj++] = pre_char; pre_size = 1; pre_char = 'M'; }
                else pre_size++;
            } else if (!TBBIT(d0h, i, search_site) && TBREF(match_site) != TBREAD(i)) {
                i--; match_site--; sum_err++;
                if (pre_char != 'S') { rsz[jj] = (uint16_t)pre_size; rch[jj++] = pre_char; pre_size = 1; pre_char = 'S'; }
                else pre_size++;
            } else if (TBBIT(hph, i, search_site)) {
                i--; search_site++; sum_err++;
                if (pre_char != 'I') { rsz[jj] = (uint16_t)pre_size; rch[jj++] = pre_char; pre_size = 1; pre_char = 'I'; }
                else pre_size++;
                start++;
            } else {
                search_site--; match_site--; sum_err++;
                if (pre_char != 'D') { rsz[jj] = (uint16_t)pre_size; rch[jj++] = pre_char; pre_size = 1; pre_char = 'D'; }
                else pre_size++;
                start--;
            }
        }
#undef TBBIT
#undef TBREF
#undef TBREAD
        rsz[jj] = (uint16_t)pre_size;
        rch[jj++] = pre_char;
        if (i >= 0) {
            rsz[jj] = (uint16_t)(i + 1);
            rch[jj++] = 'M';
        }
        uint8_t txt[TB_TEXT_MAX];
        int n = 0;
        for (jj = jj - 1; jj > 0; jj--) {
            if (n > TB_TEXT_MAX - 8) break;
            if (rch[jj] == 'M' || rch[jj] == 'S') {
                int smv = 0;
                while (jj > 0 && (rch[jj] == 'M' || rch[jj] == 'S')) {
                    smv += rsz[jj];
                    jj--;
                }
                jj++;
                n += put_len(txt + n, (uint32_t)smv);
                txt[n++] = 'M';
            } else {
                n += put_len(txt + n, rsz[jj]);
                txt[n++] = (uint8_t)rch[jj];
            }
        }
        slot[0] = (uint8_t)err;
        slot[1] = (uint8_t)n;
        if (n <= SWM_CIGAR_SLOT - 2) {
            for (int q = 0; q < n; q++) slot[2 + q] = txt[q];
        } else {
            uint32_t at = atomicAdd(&B.tot[TOT_ARENA], (uint32_t)n);
            if ((uint64_t)at + n <= cap_arena) {
                for (int q = 0; q < n; q++) B.arena[at + q] = txt[q];
                B.vr_aoff[c] = at;
            } else {
                atomicOr(&B.tot[TOT_FLAGS], OV_ARENA);
            }
        }
        B.vr_tlen[c] = (uint16_t)n;
        B.vr_loc[c] = ws + (uint32_t)start + 1;
        B.vr_flag[c] = VR_TB;
    }
}

// ======================================================================
// k_records: groups of 8, record flushes, dedup, primary flag
// ======================================================================

// One item's records by the reference's rules, one thread: candidates in
// batch order, groups of 8 with the flush test after each (1790) and after a
// batch's last partial group (1858), the traceback path's dedup against the
// previous location (475-477), the primary flag on the first record. The
// count pass (WRITE false) stores the item's record / word / byte counts, the
// write pass writes the records at the scanned offsets. Returns the records.
template <bool WRITE>
__device__ uint32_t records_seq(const MapBufs &B, uint32_t item, uint64_t cap_recs, uint64_t cap_words,
                                uint64_t cap_bytes, unsigned long long &locs_total) {
    const uint8_t *__restrict__ vflag = B.vr_flag;
    const uint32_t *__restrict__ vloc = B.vr_loc;
    const uint16_t *__restrict__ vtlen = B.vr_tlen;
    const uint8_t *__restrict__ vcig = B.vr_cig;
    uint8_t *__restrict__ out_c = B.out_c;
    uint32_t *__restrict__ out_w = B.out_w;
    const uint32_t s0 = B.it_choff[item] + item, nb = B.it_nbat[item];
    uint32_t cnext = B.it_coff[item];
    uint32_t num = 0, len = 0, last = 0, mainf = 1, nrec = 0, nw = 0, nby = 0;
    uint32_t recbase = 0, wbase = 0, bbase = 0;
    bool ok = true;
    if (WRITE) {
        recbase = B.it_recoff[item];
        wbase = B.it_woff[item];
        bbase = B.it_boff[item];
        ok = (uint64_t)recbase + B.it_nrec[item] <= cap_recs && (uint64_t)wbase + B.it_nw[item] <= cap_words &&
             (uint64_t)bbase + B.it_nb[item] <= cap_bytes;
        if (!ok) atomicOr(&B.tot[TOT_FLAGS], OV_RECS);
    }
    uint32_t wrec = wbase, bcur = bbase;
    auto put = [&]() { // put_cigar, 1437-1507
        if (num > 0) {
            if (WRITE && ok) {
                out_w[wrec] = item;
                out_w[wrec + 1] = num | (mainf ? (1u << 31) : 0u);
                B.rec_woff[recbase + nrec] = wrec;
                B.rec_boff[recbase + nrec] = bcur - len;
                B.rec_blen[recbase + nrec] = len;
            }
            mainf = 0;
            nrec++;
            nw += 2 + num;
            nby += len;
            wrec += 2 + num;
            locs_total += num;
        }
        num = 0;
        len = 0;
    };
    for (uint32_t s = s0; s < s0 + nb; s++) {
        const uint32_t cbeg = cnext, cn = B.bt_cnt[s];
        cnext += cn;
        uint32_t g = 0; // candidates of the batch's current group of 8 (failed and passing, not invalid)
        const uint32_t cend = cbeg + cn;
        for (uint32_t c = cbeg; c < cend; c++) {
            // Runs of failed candidates (flag 0: no location, one group
            // slot each) are taken 16 or 4 at a time. Between two
            // locations the flush test at a group boundary sees the same
            // (num, len) every time, and after a flush it is false, so a
            // run that crosses one or more boundaries needs one test.
            if ((c & 15) == 0 && c + 16 <= cend) {
                const uint4 w = *reinterpret_cast<const uint4 *>(vflag + c);
                if ((w.x | w.y | w.z | w.w) == 0) {
                    if (g + 16 >= 8 && (num + 8 > SWM_MAX_CIGAR || len + 16 * 16 > SWM_MAX_CIGAR * 16)) put();
                    g = (g + 16) & 7;
                    c += 15;
                    continue;
                }
            }
            if ((c & 3) == 0 && c + 4 <= cend && *reinterpret_cast<const uint32_t *>(vflag + c) == 0) {
                if (g + 4 >= 8 && (num + 8 > SWM_MAX_CIGAR || len + 16 * 16 > SWM_MAX_CIGAR * 16)) put();
                g = (g + 4) & 7;
                c += 3;
                continue;
            }
            const uint8_t f = vflag[c];
            if (f == VR_INVALID) continue;
            if (f == VR_HAM || f == VR_TB) {
                const uint32_t loc = vloc[c];
                if (f == VR_HAM || !(num > 0 && last == loc)) { // 475-477
                    const uint32_t tl = vtlen[c];
                    if (WRITE && ok) {
                        out_w[wrec + 2 + num] = loc;
                        // [NM, len, text]: the slot's first 16 bytes in one load
                        const uint4 h = *reinterpret_cast<const uint4 *>(vcig + (uint64_t)c * SWM_CIGAR_SLOT);
                        const uint32_t hw[4] = {h.x, h.y, h.z, h.w};
                        if (tl + 2 <= 16) {
#pragma unroll
                            for (uint32_t q = 0; q < 16; q++)
                                if (q < tl + 2) out_c[bcur + q] = (uint8_t)(hw[q >> 2] >> (8 * (q & 3)));
                        } else {
                            out_c[bcur] = (uint8_t)h.x;
                            out_c[bcur + 1] = (uint8_t)(h.x >> 8);
                            const uint8_t *tx = (tl <= SWM_CIGAR_SLOT - 2) ? vcig + (uint64_t)c * SWM_CIGAR_SLOT + 2
                                                                          : B.arena + B.vr_aoff[c];
                            for (uint32_t q = 0; q < tl; q++) out_c[bcur + 2 + q] = tx[q];
                        }
                    }
                    bcur += 2 + tl;
                    num++;
                    len += 2 + tl;
                    last = loc;
                }
            }
            if (++g == 8) {
                g = 0;
                if (num + 8 > SWM_MAX_CIGAR || len + 16 * 16 > SWM_MAX_CIGAR * 16) put(); // 1790
            }
        }
        if (g > 0 && (num + 8 > SWM_MAX_CIGAR || len + 16 * 16 > SWM_MAX_CIGAR * 16)) put(); // 1858
    }
    put();
    if (!WRITE) {
        B.it_nrec[item] = nrec;
        B.it_nw[item] = nw;
        B.it_nb[item] = nby;
    }
    return nrec;
}

// Items with at most this many candidates take the one-thread path of
// k_records (records_seq); the others the warp path.
#define RECORDS_LIGHT 16

// Records, groups of 32 consecutive items taken from a queue: items with few
// candidates one thread each (records_seq, all lanes at once), the others
// one warp each. Most of those need none of the sequential machinery: while
// num + 8 <= SWM_MAX_CIGAR and len + 256 <= 16 SWM_MAX_CIGAR the flush tests are false,
// so when the item's passing candidates (P of them, S bytes of [NM, len,
// text] before dedup) keep within those bounds, or (write pass) the count
// pass found at most one record, the item is one record of every passing
// candidate in order except a traceback hit whose location equals the
// previous passing candidate's (that previous one was then emitted or had
// the same location itself). The warp reads 32 verdict flags per load, and
// only the passing lanes read their location and CIGAR; the rest go through
// records_seq on lane 0. Count pass: the item's record / word / byte counts;
// write pass: the records, and the unmapped-read bits of the group.
template <bool WRITE>
__global__ void __launch_bounds__(128) k_records(MapBufs B, uint64_t cap_chunks, uint64_t cap_elems,
                                                 uint64_t cap_cands, uint64_t cap_recs, uint64_t cap_words,
                                                 uint64_t cap_bytes) {
    if (block_failed(B, cap_chunks, cap_elems, cap_cands)) return;
    const uint32_t nitems = B.par->nitems, lane = lane_id();
    const uint8_t *__restrict__ vflag = B.vr_flag;
    const uint32_t *__restrict__ vloc = B.vr_loc;
    const uint16_t *__restrict__ vtlen = B.vr_tlen;
    const uint8_t *__restrict__ vcig = B.vr_cig;
    uint8_t *__restrict__ out_c = B.out_c;
    uint32_t *__restrict__ out_w = B.out_w;
    unsigned long long locs_total = 0, mapped = 0;
    for (;;) {
        const uint32_t item0 = warp_take(&B.tot[WRITE ? TOT_RQW : TOT_RQC]);
        if (item0 >= nitems) break;
        // the group's scalars: lane j holds item item0 + j's
        const uint32_t mine = item0 + lane;
        uint32_t g_cb = 0, g_nc = 0, g_nrec = 0, g_wb = 0, g_bb = 0, g_rb = 0;
        bool g_ok = true;
        if (mine < nitems) {
            g_cb = B.it_coff[mine];
            g_nc = B.it_nbat[mine] ? B.it_ncand[mine] : 0u;
            if (WRITE) {
                g_nrec = B.it_nrec[mine];
                g_wb = B.it_woff[mine];
                g_bb = B.it_boff[mine];
                g_rb = B.it_recoff[mine];
                g_ok = (uint64_t)g_rb + g_nrec <= cap_recs && (uint64_t)g_wb + B.it_nw[mine] <= cap_words &&
                       (uint64_t)g_bb + B.it_nb[mine] <= cap_bytes;
            }
        }
        // items with few candidates: one lane each, all at once (the warp
        // path below would spend a pass of 32 lanes on a handful of flags)
        const bool light = mine < nitems && g_nc <= RECORDS_LIGHT;
        if (light && !(WRITE && g_nrec == 0))
            records_seq<WRITE>(B, mine, cap_recs, cap_words, cap_bytes, locs_total);
        const unsigned heavy = __ballot_sync(0xffffffffu, mine < nitems && !light);
        for (unsigned hm = heavy; hm; hm &= hm - 1) {
            const uint32_t j = __ffs(hm) - 1;
            const uint32_t item = item0 + j;
            const uint32_t cb = __shfl_sync(0xffffffffu, g_cb, j), nc = __shfl_sync(0xffffffffu, g_nc, j);
            const uint32_t nrec_c = __shfl_sync(0xffffffffu, g_nrec, j);
            if (WRITE && nrec_c == 0) continue; // nothing passed (or every location deduped)
            if (WRITE && nrec_c > 1) {          // flushes: the sequential rules
                if (lane == 0) records_seq<true>(B, item, cap_recs, cap_words, cap_bytes, locs_total);
                continue;
            }
            const uint32_t wbase = __shfl_sync(0xffffffffu, g_wb, j), bbase = __shfl_sync(0xffffffffu, g_bb, j);
            const bool ok = __shfl_sync(0xffffffffu, (uint32_t)g_ok, j) != 0;
            uint32_t num = 0, len = 0, P = 0, S = 0, last = 0;
            bool has = false;
            for (uint32_t c0 = cb; c0 < cb + nc; c0 += 32) {
                const uint32_t c = c0 + lane;
                const uint8_t f = c < cb + nc ? vflag[c] : (uint8_t)VR_FAIL;
                const bool pass = f == VR_HAM || f == VR_TB;
                const unsigned pm = __ballot_sync(0xffffffffu, pass);
                if (!pm) continue;
                uint32_t loc = 0, tl = 0;
                if (pass) {
                    loc = vloc[c];
                    tl = vtlen[c];
                }
                const unsigned below = pm & lanemask_lt();
                const uint32_t ploc = __shfl_sync(0xffffffffu, loc, below ? 31 - __clz(below) : lane);
                const bool dup = f == VR_TB && (below ? ploc == loc : (has && last == loc));
                const bool keep = pass && !dup;
                const unsigned km = __ballot_sync(0xffffffffu, keep);
                const uint32_t by = keep ? 2 + tl : 0u;
                const uint32_t incl = warp_scan_incl(by);
                if (WRITE && keep && ok) {
                    out_w[wbase + 2 + num + __popc(km & lanemask_lt())] = loc;
                    const uint32_t bcur = bbase + len + incl - by;
                    const uint4 h = *reinterpret_cast<const uint4 *>(vcig + (uint64_t)c * SWM_CIGAR_SLOT);
                    const uint32_t hw[4] = {h.x, h.y, h.z, h.w};
                    if (tl + 2 <= 16) {
#pragma unroll
                        for (uint32_t q = 0; q < 16; q++)
                            if (q < tl + 2) out_c[bcur + q] = (uint8_t)(hw[q >> 2] >> (8 * (q & 3)));
                    } else {
                        out_c[bcur] = (uint8_t)h.x;
                        out_c[bcur + 1] = (uint8_t)(h.x >> 8);
                        const uint8_t *tx = (tl <= SWM_CIGAR_SLOT - 2) ? vcig + (uint64_t)c * SWM_CIGAR_SLOT + 2
                                                                      : B.arena + B.vr_aoff[c];
                        for (uint32_t q = 0; q < tl; q++) out_c[bcur + 2 + q] = tx[q];
                    }
                }
                num += __popc(km);
                len += __shfl_sync(0xffffffffu, incl, 31);
                if (!WRITE) {
                    P += __popc(pm);
                    S += __reduce_add_sync(0xffffffffu, pass ? 2 + tl : 0u);
                }
                last = __shfl_sync(0xffffffffu, loc, 31 - __clz(pm));
                has = true;
            }
            if (!WRITE) {
                if (P + 8 <= SWM_MAX_CIGAR && S + 16 * 16 <= SWM_MAX_CIGAR * 16) {
                    if (lane == 0) {
                        B.it_nrec[item] = num ? 1u : 0u;
                        B.it_nw[item] = num ? 2 + num : 0u;
                        B.it_nb[item] = len;
                    }
                } else if (lane == 0) {
                    records_seq<false>(B, item, cap_recs, cap_words, cap_bytes, locs_total);
                }
            } else {
                const uint32_t rb = __shfl_sync(0xffffffffu, g_rb, j);
                if (!ok && lane == 0) atomicOr(&B.tot[TOT_FLAGS], OV_RECS);
                if (lane == 0 && num) {
                    if (ok) {
                        out_w[wbase] = item;
                        out_w[wbase + 1] = num | (1u << 31);
                        B.rec_woff[rb] = wbase;
                        B.rec_boff[rb] = bbase;
                        B.rec_blen[rb] = len;
                    }
                    locs_total += num;
                }
            }
        }
        if (WRITE) {
            // unmapped reads as bits, 16 reads (the group's 32 items) per halfword
            const uint32_t prev = __shfl_up_sync(0xffffffffu, g_nrec, 1);
            const bool valid = mine < nitems;
            const bool mp = (lane & 1) && (g_nrec + prev) > 0;
            const unsigned bal = __ballot_sync(0xffffffffu, valid && (lane & 1) && !mp);
            const unsigned mb = __ballot_sync(0xffffffffu, valid && mp);
            if (lane == 0) {
                B.unm[item0 >> 5] = (uint16_t)even_bits(bal >> 1);
                mapped += __popc(mb);
            }
        }
    }
    if (WRITE) {
        warp_add_u64(&B.stat[ST_LOCS], locs_total);
        warp_add_u64(&B.stat[ST_MAPPED], mapped);
    }
}

__global__ void k_batches_stat(MapBufs B) {
    const uint32_t nitems = B.par->nitems;
    unsigned long long s = 0;
    for (uint32_t item = blockIdx.x * blockDim.x + threadIdx.x; item < nitems; item += gridDim.x * blockDim.x)
        s += B.it_nbat[item];
    warp_add_u64(&B.stat[ST_BATCHES], s);
}

// ======================================================================
// host side
// ======================================================================

// Work-buffer capacities stay below SWM_SCAN_SATURATED, so a block whose
// 32-bit totals saturated always exceeds them and its later stages skip.
#define CAP_MAX ((uint64_t)SWM_SCAN_SATURATED - 1)

static uint64_t cap_clamp(uint64_t c) { return c < CAP_MAX ? c : CAP_MAX; }

static int g_sms = 0;
static std::mutex g_chain_mu; // serialised mappers: wait, launch and record as one step

static unsigned grid_cap(uint64_t work, unsigned threads, int per_sm) {
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 1;
    }
    uint64_t g = (work + threads - 1) / threads;
    uint64_t cap = (uint64_t)g_sms * per_sm;
    if (g > cap) g = cap;
    return (unsigned)(g ? g : 1);
}

template <typename T>
static int dmalloc(T **p, uint64_t count) {
    cudaError_t e = cudaMalloc((void **)p, (count ? count : 1) * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        swm_set_error("cudaMalloc(%llu bytes): %s", (unsigned long long)(count * sizeof(T)), cudaGetErrorString(e));
        return SWM_ERR_OOM;
    }
    return SWM_OK;
}

static void free_bufs(MapBufs &B) {
    void *ps[] = {B.par, B.it_w, B.sel, B.sel_fl, B.sel_key, B.it_perm, B.unm, B.it_nsel, B.it_e, B.it_nch, B.it_nel, B.it_nbat,
                  B.it_choff, B.it_eloff, B.it_nrec, B.it_nw, B.it_nb, B.it_recoff, B.it_woff, B.it_boff, B.it_ncand, B.plan_list,
                  B.it_coff, B.ch_g, B.ch_meta, B.bt_c0, B.bt_c1, B.bt_e0, B.bt_cnt, B.sort_scratch, B.cand_ub, B.cc_pos,
                  B.cc_item, B.plan_keys, B.vr_flag, B.vr_loc, B.vr_err, B.vr_mloc, B.vr_tlen, B.vr_cig, B.vr_aoff, B.arena, B.tb_list,
                  B.tb_cp, B.slow_list, B.vt_x, B.vt_st, B.vt_cp,
                  B.out_w, B.out_c, B.rec_woff, B.rec_boff, B.rec_blen, B.tot, B.stat, B.scan_tmp};
    for (void *p : ps) cudaFree(p);
    memset(&B, 0, sizeof(B));
}

static uint64_t scan_cap(const swm_mapper *m) { return m->cap_items + 1; }

static unsigned cand_grid(const swm_mapper *m) { return grid_cap(m->cap_items * 32, CAND_WARPS * 32, 8); }

static int alloc_items(swm_mapper *m) {
    MapBufs &B = m->b;
    const uint64_t I = m->cap_items;
    int rc = SWM_OK;
    rc |= dmalloc(&B.it_w, I * 32);
    rc |= dmalloc(&B.sel, I * SWM_MAX_SEL);
    rc |= dmalloc(&B.sel_fl, I * SWM_MAX_SEL);
    rc |= dmalloc(&B.sel_key, I * SWM_MAX_SEL);
    rc |= dmalloc(&B.it_perm, I);
    rc |= dmalloc(&B.unm, I / 32 + 1);
    rc |= dmalloc(&B.it_nsel, I);
    rc |= dmalloc(&B.it_e, I);
    rc |= dmalloc(&B.it_nch, I);
    rc |= dmalloc(&B.it_nel, I);
    rc |= dmalloc(&B.it_nbat, I);
    rc |= dmalloc(&B.it_choff, I + 1);
    rc |= dmalloc(&B.it_eloff, I + 1);
    rc |= dmalloc(&B.it_nrec, I);
    rc |= dmalloc(&B.it_nw, I);
    rc |= dmalloc(&B.it_nb, I);
    rc |= dmalloc(&B.it_recoff, I + 1);
    rc |= dmalloc(&B.it_woff, I + 1);
    rc |= dmalloc(&B.it_boff, I + 1);
    rc |= dmalloc(&B.it_ncand, I);
    rc |= dmalloc(&B.plan_list, I);
    rc |= dmalloc(&B.it_coff, I + 1);
    rc |= dmalloc(&B.tot, TOT_N);
    rc |= dmalloc(&B.stat, ST_N);
    rc |= dmalloc(&B.par, 1);
    m->gen++;
    return rc ? SWM_ERR_OOM : SWM_OK;
}

static int alloc_work(swm_mapper *m) {
    MapBufs &B = m->b;
    int rc = SWM_OK;
    m->gen++; // the captured graph holds the old buffers
    cudaFree(B.ch_g); cudaFree(B.ch_meta); cudaFree(B.plan_keys); cudaFree(B.bt_c0); cudaFree(B.bt_c1); cudaFree(B.bt_e0);
    cudaFree(B.bt_cnt); cudaFree(B.sort_scratch); cudaFree(B.cand_ub); cudaFree(B.cc_pos);
    cudaFree(B.cc_item); cudaFree(B.vr_flag); cudaFree(B.vr_loc); cudaFree(B.vr_err); cudaFree(B.vr_mloc);
    cudaFree(B.vr_tlen); cudaFree(B.vr_cig); cudaFree(B.vr_aoff); cudaFree(B.arena); cudaFree(B.out_w);
    cudaFree(B.tb_list); cudaFree(B.tb_cp); cudaFree(B.slow_list); cudaFree(B.vt_x); cudaFree(B.vt_st); cudaFree(B.vt_cp);
    cudaFree(B.out_c); cudaFree(B.rec_woff); cudaFree(B.rec_boff); cudaFree(B.rec_blen); cudaFree(B.scan_tmp);
    rc |= dmalloc(&B.ch_g, m->cap_chunks);
    rc |= dmalloc(&B.ch_meta, m->cap_chunks);
    rc |= dmalloc(&B.plan_keys, m->cap_chunks);
    rc |= dmalloc(&B.bt_c0, m->cap_chunks + m->cap_items);
    rc |= dmalloc(&B.bt_c1, m->cap_chunks + m->cap_items);
    rc |= dmalloc(&B.bt_e0, m->cap_chunks + m->cap_items);
    rc |= dmalloc(&B.bt_cnt, m->cap_chunks + m->cap_items);
    rc |= dmalloc(&B.sort_scratch, (uint64_t)cand_grid(m) * CAND_WARPS * SWM_BATCH_POSITIONS);
    rc |= dmalloc(&B.cand_ub, m->cap_elems);
    rc |= dmalloc(&B.cc_pos, m->cap_cands);
    rc |= dmalloc(&B.cc_item, m->cap_cands);
    rc |= dmalloc(&B.vr_flag, m->cap_cands);
    rc |= dmalloc(&B.vr_loc, m->cap_cands);
    rc |= dmalloc(&B.vr_err, m->cap_cands);
    rc |= dmalloc(&B.vr_mloc, m->cap_cands);
    rc |= dmalloc(&B.vr_tlen, m->cap_cands);
    rc |= dmalloc(&B.vr_cig, m->cap_cands * SWM_CIGAR_SLOT);
    rc |= dmalloc(&B.vr_aoff, m->cap_cands);
    rc |= dmalloc(&B.arena, m->cap_arena);
    rc |= dmalloc(&B.tb_list, m->cap_cands);
    rc |= dmalloc(&B.tb_cp, m->cap_cands * 32);
    rc |= dmalloc(&B.slow_list, m->cap_cands);
    rc |= dmalloc(&B.vt_x, m->cap_cands);
    rc |= dmalloc(&B.vt_st, m->cap_cands);
    rc |= dmalloc(&B.vt_cp, m->cap_cands);
    rc |= dmalloc(&B.out_w, m->cap_words);
    rc |= dmalloc(&B.out_c, m->cap_bytes);
    rc |= dmalloc(&B.rec_woff, m->cap_recs);
    rc |= dmalloc(&B.rec_boff, m->cap_recs);
    rc |= dmalloc(&B.rec_blen, m->cap_recs);
    rc |= dmalloc(&B.scan_tmp, swm_scan_tmp_words(scan_cap(m)));
    return rc ? SWM_ERR_OOM : SWM_OK;
}

extern "C" int swm_mapper_create(swm_index *ix, uint64_t max_reads, swm_mapper **out) {
    if (!ix || !out || max_reads == 0 || max_reads > (1ull << 30)) return SWM_ERR_ARG;
    SWM_CUDA(cudaSetDevice(ix->device));
    // the index's candidate table (k = 12), built once when the device has room
    // and the buckets are large enough for it to pay
    const int trc = swm_ctab_build(ix, 0);
    if (trc) return trc;
    swm_mapper *m = (swm_mapper *)calloc(1, sizeof(swm_mapper));
    if (!m) return SWM_ERR_OOM;
    m->ix = ix;
    m->device = ix->device;
    m->max_reads = max_reads;
    m->cap_items = 2 * max_reads;
    m->cap_chunks = cap_clamp(m->cap_items * 16 + 1024);
    m->cap_elems = cap_clamp(m->cap_items * 128 + 4096);
    m->cap_cands = cap_clamp(m->cap_items * 8 + 4096);
    m->cap_recs = cap_clamp(m->cap_items + 1024);
    m->cap_words = cap_clamp(m->cap_items * 8 + 4096);
    m->cap_bytes = cap_clamp(m->cap_items * 32 + 4096);
    m->cap_arena = ARENA_CAP_DEFAULT;
    m->stride_cap = 0;
    m->vmode = VMODE_STREAM16;
    int rc = SWM_OK;
    if (cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) != cudaSuccess) rc = SWM_ERR_CUDA;
    for (int i = 0; i < 9 && rc == SWM_OK; i++)
        if (cudaEventCreate(&m->ev[i]) != cudaSuccess) rc = SWM_ERR_CUDA;
    if (rc == SWM_OK) rc = alloc_items(m);
    if (rc == SWM_OK) rc = alloc_work(m);
    if (rc == SWM_OK && (dmalloc(&m->d_lens, max_reads) || dmalloc(&m->d_e, max_reads))) rc = SWM_ERR_OOM;
    if (rc == SWM_OK && (cudaHostAlloc((void **)&m->h_lens, max_reads * 4, 0) != cudaSuccess ||
                         cudaHostAlloc((void **)&m->h_e, max_reads, 0) != cudaSuccess ||
                         cudaHostAlloc((void **)&m->h_unm, (m->cap_items / 32 + 1) * 2, 0) != cudaSuccess ||
                         cudaHostAlloc((void **)&m->h_tot, TOT_N * 4, 0) != cudaSuccess ||
                         cudaHostAlloc((void **)&m->h_stat, ST_N * 8, 0) != cudaSuccess ||
                         cudaHostAlloc((void **)&m->h_par, sizeof(BlockParams), 0) != cudaSuccess))
        rc = SWM_ERR_OOM;
    if (rc != SWM_OK) {
        swm_mapper_free(m);
        return rc;
    }
    m->h_cap_items = m->cap_items / 32 + 1;
    *out = m;
    return SWM_OK;
}

extern "C" void swm_mapper_free(swm_mapper *m) {
    if (!m) return;
    cudaSetDevice(m->device);
    if (m->st) cudaStreamSynchronize(m->st);
    for (int a = 0; a < 3; a++)
        for (int h = 0; h < VMODE_N; h++)
            if (m->gx[a][h]) cudaGraphExecDestroy(m->gx[a][h]);
    free_bufs(m->b);
    cudaFree(m->d_reads);
    cudaFree(m->d_lens);
    cudaFree(m->d_e);
    cudaFreeHost(m->h_reads);
    cudaFreeHost(m->h_lens);
    cudaFreeHost(m->h_e);
    cudaFreeHost(m->h_w);
    cudaFreeHost(m->h_c);
    cudaFreeHost(m->h_rw);
    cudaFreeHost(m->h_rb);
    cudaFreeHost(m->h_rl);
    cudaFreeHost(m->h_unm);
    cudaFreeHost(m->h_tot);
    cudaFreeHost(m->h_stat);
    cudaFreeHost(m->h_par);
    for (int i = 0; i < 9; i++)
        if (m->ev[i]) cudaEventDestroy(m->ev[i]);
    if (m->st) cudaStreamDestroy(m->st);
    free(m);
}

#define LAUNCH_CHECK()                                                                              \
    do {                                                                                            \
        cudaError_t e_ = cudaGetLastError();                                                        \
        if (e_ != cudaSuccess) {                                                                    \
            swm_set_error("kernel launch: %s", cudaGetErrorString(e_));                             \
            return SWM_ERR_CUDA;                                                                    \
        }                                                                                           \
    } while (0)

// The whole pipeline of one block on st, every size read on the device (the
// grids cover the buffers' capacity; kernels loop over what the block has).
// Captured into the mapper's graph; gclass picks the seed kernel.
static int enqueue_ops(swm_mapper *m, cudaStream_t st, int gclass, int vmode) {
    MapBufs &B = m->b;
    const uint32_t *d_n = &B.par->nitems;
    const uint64_t ci = m->cap_items;
    const swm_index *ix = m->ix;
    m->launches = 0;
    SWM_CUDA(cudaMemcpyAsync(B.par, m->h_par, sizeof(BlockParams), cudaMemcpyHostToDevice, st));
    SWM_CUDA(cudaMemsetAsync(B.tot, 0, TOT_N * 4, st));
    SWM_CUDA(cudaMemsetAsync(B.stat, 0, ST_N * 8, st));
    // stage events: external records become event nodes of the captured graph
    SWM_CUDA(cudaEventRecordWithFlags(m->ev[0], st, cudaEventRecordExternal));
    const uint32_t short_max = 10 * KL12 + KL12 - 1; // 164: longest read with <= 10 long seeds
    const bool table = ix->d_ctab_off && ix->k == K12;
    auto seed10 = table ? k_seed12<10, true> : k_seed12<10, false>;
    auto seed16 = table ? k_seed12<16, true> : k_seed12<16, false>;
    if (gclass == 1) {
        seed10<<<grid_cap(ci, SEED12_THREADS, 16), SEED12_THREADS, 0, st>>>(ix->d_off, B, 0u, 0xffffffffu);
    } else if (gclass == 2) { // each read to the instantiation of its length
        seed10<<<grid_cap(ci, SEED12_THREADS, 16), SEED12_THREADS, 0, st>>>(ix->d_off, B, 0u, short_max);
        seed16<<<grid_cap(ci, SEED12_THREADS, 8), SEED12_THREADS, 0, st>>>(ix->d_off, B, short_max + 1, 0xffffffffu);
        m->launches++;
    } else
        k_seed<<<grid_cap(ci, SEED_WARPS * 32, 8), SEED_WARPS * 32, 0, st>>>(ix->d_off, ix->k, B);
    m->launches++;
    LAUNCH_CHECK();
    SWM_CUDA(cudaEventRecordWithFlags(m->ev[1], st, cudaEventRecordExternal));
    int rc = swm_exclusive_scan(B.it_nch, B.it_choff, d_n, 0, ci, B.scan_tmp, B.tot + TOT_CHUNKS, st);
    if (rc) return rc;
    rc = swm_exclusive_scan(B.it_nel, B.it_eloff, d_n, 0, ci, B.scan_tmp, B.tot + TOT_ELEMS, st);
    if (rc) return rc;
    m->launches += 6;
    k_plan_list<<<grid_cap(ci, 256, 8), 256, 0, st>>>(B, m->cap_chunks, !table);
    k_plan_lanes<<<grid_cap(ci, PLAN_LANE_WARPS * 32, 8), PLAN_LANE_WARPS * 32, 0, st>>>(ix->d_pos, B, m->cap_chunks,
                                                                                         m->cap_elems);
    k_plan<<<grid_cap(ci, PLAN_WARPS * 32, 16), PLAN_WARPS * 32, 0, st>>>(ix->d_pos, B, m->cap_chunks,
                                                                          m->cap_elems);
    m->launches += 3;
    LAUNCH_CHECK();
    SWM_CUDA(cudaEventRecordWithFlags(m->ev[2], st, cudaEventRecordExternal));
    if (table)
        k_cand_table<<<cand_grid(m), CAND_WARPS * 32, 0, st>>>(ix->d_pos, ix->d_ls, ix->d_ctab_off, ix->d_ctab_pos, B,
                                                               m->cap_chunks, m->cap_elems, ix->k + SWM_SEED_STEP - 1);
    else
        k_cand<<<cand_grid(m), CAND_WARPS * 32, 0, st>>>(ix->d_pos, ix->d_ls, B, m->cap_chunks, m->cap_elems,
                                                         ix->k + SWM_SEED_STEP - 1);
    m->launches++;
    LAUNCH_CHECK();
    SWM_CUDA(cudaEventRecordWithFlags(m->ev[3], st, cudaEventRecordExternal));
    rc = swm_exclusive_scan(B.it_ncand, B.it_coff, d_n, 0, ci, B.scan_tmp, B.tot + TOT_CANDS, st);
    if (rc) return rc;
    m->launches += 3;
    k_compact<<<grid_cap(ci, 256, 8), 256, 0, st>>>(B, m->cap_chunks, m->cap_elems, m->cap_cands);
    m->launches++;
    LAUNCH_CHECK();
    SWM_CUDA(cudaEventRecordWithFlags(m->ev[4], st, cudaEventRecordExternal));
    {
        const unsigned vg = grid_cap(m->cap_cands, 128, 16);
        const uint64_t nw = ix->n_words2 + SWM_PAD_WORDS;
        if (vmode == VMODE_STREAM8 || vmode == VMODE_STREAM16 || vmode == VMODE_PAIR16) {
            auto stream = vmode == VMODE_STREAM8 ? k_verify_stream<8>
                          : vmode == VMODE_STREAM16 ? k_verify_stream<16> : k_verify_pair<16>;
            stream<<<grid_cap(m->cap_cands, 128, VERIFY_BLOCKS_PER_SM), 128, 0, st>>>(ix->d_b2, nw, ix->ref_length, B, m->cap_chunks,
                                                                     m->cap_elems, m->cap_cands);
            k_verify_finish<<<vg, 128, 0, st>>>(ix->d_b2, nw, ix->ref_length, B, m->cap_chunks, m->cap_elems,
                                                m->cap_cands, m->cap_arena);
        } else {
            auto head = vmode == VMODE_HEAD32 ? k_verify<true, 1> : k_verify<true, 2>;
            auto tail = vmode == VMODE_HEAD32 ? k_verify<false, 1> : k_verify<false, 2>;
            head<<<vg, 128, 0, st>>>(ix->d_b2, nw, ix->ref_length, B, m->cap_chunks, m->cap_elems, m->cap_cands,
                                     m->cap_arena);
            tail<<<vg, 128, 0, st>>>(ix->d_b2, nw, ix->ref_length, B, m->cap_chunks, m->cap_elems, m->cap_cands,
                                     m->cap_arena);
        }
    }
    m->launches += 2;
    LAUNCH_CHECK();
    SWM_CUDA(cudaEventRecordWithFlags(m->ev[5], st, cudaEventRecordExternal));
    k_traceback<<<grid_cap(m->cap_cands, TB_THREADS, 16), TB_THREADS, 0, st>>>(
        ix->d_b2, ix->n_words2 + SWM_PAD_WORDS, ix->ref_length, B, m->cap_chunks, m->cap_elems, m->cap_cands,
        m->cap_arena);
    k_traceback_slow<<<grid_cap(m->cap_cands, 128, 4), 128, 0, st>>>(
        ix->d_b2, ix->n_words2 + SWM_PAD_WORDS, ix->ref_length, B, m->cap_chunks, m->cap_elems, m->cap_cands,
        m->cap_arena);
    m->launches += 2;
    LAUNCH_CHECK();
    SWM_CUDA(cudaEventRecordWithFlags(m->ev[6], st, cudaEventRecordExternal));
    k_records<false><<<grid_cap(ci, 128, 32), 128, 0, st>>>(B, m->cap_chunks, m->cap_elems, m->cap_cands,
                                                             m->cap_recs, m->cap_words, m->cap_bytes);
    rc = swm_exclusive_scan(B.it_nrec, B.it_recoff, d_n, 0, ci, B.scan_tmp, B.tot + TOT_RECS, st);
    if (rc) return rc;
    rc = swm_exclusive_scan(B.it_nw, B.it_woff, d_n, 0, ci, B.scan_tmp, B.tot + TOT_WORDS, st);
    if (rc) return rc;
    rc = swm_exclusive_scan(B.it_nb, B.it_boff, d_n, 0, ci, B.scan_tmp, B.tot + TOT_BYTES, st);
    if (rc) return rc;
    k_records<true><<<grid_cap(ci, 128, 32), 128, 0, st>>>(B, m->cap_chunks, m->cap_elems, m->cap_cands,
                                                            m->cap_recs, m->cap_words, m->cap_bytes);
    k_batches_stat<<<grid_cap(ci, 256, 8), 256, 0, st>>>(B);
    m->launches += 12;
    LAUNCH_CHECK();
    SWM_CUDA(cudaEventRecordWithFlags(m->ev[7], st, cudaEventRecordExternal));
    SWM_CUDA(cudaMemcpyAsync(m->h_tot, B.tot, TOT_N * 4, cudaMemcpyDeviceToHost, st));
    SWM_CUDA(cudaMemcpyAsync(m->h_stat, B.stat, ST_N * 8, cudaMemcpyDeviceToHost, st));
    return SWM_OK;
}

static void drop_graph(swm_mapper *m, int gclass, int h) {
    if (m->gx[gclass][h]) cudaGraphExecDestroy(m->gx[gclass][h]);
    m->gx[gclass][h] = nullptr;
}

// Queue one block on m->st: its inputs into the pinned parameter block, then
// the mapper's graph (captured again after its buffers changed). No host
// synchronisation.
static int enqueue(swm_mapper *m, const char *d_reads, const uint32_t *d_lens, uint64_t stride, uint32_t nreads,
                   uint32_t errors, const uint8_t *d_e) {
    const int gclass = m->ix->k != K12 ? 0 : (stride <= 10 * KL12 + KL12 - 1 ? 1 : 2);
    BlockParams *P = m->h_par;
    P->reads = d_reads;
    P->lens = d_lens;
    P->e = d_e;
    P->stride = stride;
    P->nreads = nreads;
    P->nitems = 2 * nreads;
    P->errors = errors;
    P->pad = 0;
    const int h = m->vmode == VMODE_PAIR16 && (d_e || errors > 7) ? VMODE_STREAM16 : m->vmode;
    if (!m->gx[gclass][h] || m->gx_gen[gclass][h] != m->gen || m->gx_tab[gclass][h] != m->ix->ctab_gen) {
        drop_graph(m, gclass, h);
        cudaGraph_t g = nullptr;
        SWM_CUDA(cudaStreamBeginCapture(m->st, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_ops(m, m->st, gclass, h);
        const cudaError_t ce = cudaStreamEndCapture(m->st, &g);
        if (rc != SWM_OK || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            if (rc == SWM_OK) swm_set_error("capturing the block pipeline: %s", cudaGetErrorString(ce));
            cudaGetLastError();
            return rc != SWM_OK ? rc : SWM_ERR_CUDA;
        }
        const cudaError_t ie = cudaGraphInstantiate(&m->gx[gclass][h], g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            m->gx[gclass][h] = nullptr;
            swm_set_error("instantiating the block pipeline: %s", cudaGetErrorString(ie));
            return SWM_ERR_CUDA;
        }
        m->gx_gen[gclass][h] = m->gen;
        m->gx_tab[gclass][h] = m->ix->ctab_gen;
    }
    if (m->ix->chain) { // one block's kernels at a time across the index's mappers
        std::lock_guard<std::mutex> lk(g_chain_mu);
        SWM_CUDA(cudaStreamWaitEvent(m->st, m->ix->chain_ev, 0));
        SWM_CUDA(cudaGraphLaunch(m->gx[gclass][h], m->st));
        SWM_CUDA(cudaEventRecord(m->ix->chain_ev, m->st));
        return SWM_OK;
    }
    SWM_CUDA(cudaGraphLaunch(m->gx[gclass][h], m->st));
    return SWM_OK;
}

// Serialised mappers: a block's inputs are copied on its mapper's stream
// before the wait on chain_ev, and its results after the record, so the
// copies of one mapper overlap the kernels of another (the reference's
// double buffering, mapper_mpe.c:972-1106) while the kernels of two blocks
// never share the SMs.
extern "C" int swm_index_serialize_mappers(swm_index *ix, int on) {
    if (!ix) return SWM_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_chain_mu);
    if (on && !ix->chain_ev) {
        SWM_CUDA(cudaSetDevice(ix->device));
        SWM_CUDA(cudaEventCreateWithFlags(&ix->chain_ev, cudaEventDisableTiming));
    }
    ix->chain = on ? 1 : 0;
    return SWM_OK;
}

static void grow(uint64_t *cap, uint64_t need) {
    if (need <= *cap) return;
    uint64_t n = *cap;
    while (n < need) n *= 2;
    *cap = cap_clamp(n + n / 4);
}

// Queue the copy of the block's totals to pinned memory (after enqueue).

// Wait for the queued block and inspect its totals. *again is set when a
// work buffer was too small; the capacities are grown and the buffers
// reallocated, and the caller must queue the block again.
static int finish_block(swm_mapper *m, uint32_t nreads, uint64_t retries, int *again) {
    *again = 0;
    cudaError_t se = cudaStreamSynchronize(m->st);
    if (se != cudaSuccess) {
        swm_set_error("mapping block failed: %s", cudaGetErrorString(se));
        return SWM_ERR_CUDA;
    }
    memcpy(m->tot, m->h_tot, sizeof(m->tot));
    const uint32_t fl = m->tot[TOT_FLAGS];
    if (fl & OV_BAD) {
        swm_set_error("a read is outside the envelope (length <= %d and <= stride, threshold <= %d)",
                      SWM_MAX_READ_LEN, SWM_MAX_ERRORS);
        return SWM_ERR_ARG;
    }
    // A scan total that saturated means the block's work does not fit the
    // 32-bit offsets at all. Each total is checked once the stage that feeds
    // its scan is known to have run in full (a stage skips its work once an
    // earlier buffer overflowed, leaving its per-item counts stale).
    auto saturated = [&](int t, const char *what) {
        if (m->tot[t] != SWM_SCAN_SATURATED) return false;
        swm_set_error("the block's %s reach 2^32 - 1, past the 32-bit offsets of the work buffers: map it in "
                      "smaller blocks (%u reads here)", what, nreads);
        return true;
    };
    if (saturated(TOT_CHUNKS, "refill chunks") || saturated(TOT_ELEMS, "fetched positions")) return SWM_ERR_OVERFLOW;
    bool need = false;
    // totals from the item scans are exact even when a later buffer overflowed
    if (m->tot[TOT_CHUNKS] > m->cap_chunks) {
        grow(&m->cap_chunks, m->tot[TOT_CHUNKS]);
        need = true;
    }
    if (m->tot[TOT_ELEMS] > m->cap_elems) {
        grow(&m->cap_elems, m->tot[TOT_ELEMS]);
        need = true;
    }
    if (!need) { // the candidate stage ran in full
        if (saturated(TOT_CANDS, "candidates")) return SWM_ERR_OVERFLOW;
        if ((fl & OV_CANDS) || m->tot[TOT_CANDS] > m->cap_cands) {
            grow(&m->cap_cands, m->tot[TOT_CANDS]);
            need = true;
        }
        if (fl & OV_ARENA) {
            grow(&m->cap_arena, (uint64_t)m->tot[TOT_ARENA] + 1);
            need = true;
        }
        if (!need) { // so did the records' count pass
            if (saturated(TOT_RECS, "records") || saturated(TOT_WORDS, "record words") ||
                saturated(TOT_BYTES, "CIGAR bytes"))
                return SWM_ERR_OVERFLOW;
            if ((fl & OV_RECS) || m->tot[TOT_RECS] > m->cap_recs || m->tot[TOT_WORDS] > m->cap_words ||
                m->tot[TOT_BYTES] > m->cap_bytes) {
                grow(&m->cap_recs, m->tot[TOT_RECS]);
                grow(&m->cap_words, m->tot[TOT_WORDS]);
                grow(&m->cap_bytes, m->tot[TOT_BYTES]);
                need = true;
            }
        }
    }
    if (need) {
        *again = 1;
        return alloc_work(m);
    }
    float t;
    for (int i = 0; i < 8; i++) {
        const cudaError_t te = cudaEventElapsedTime(&t, m->ev[i < 7 ? i : 0], m->ev[i < 7 ? i + 1 : 7]);
        m->stage_ms[i] = te == cudaSuccess ? t : 0.0f;
        if (te != cudaSuccess) cudaGetLastError(); // timing only: no stale error for later calls
    }
    const unsigned long long *stat = m->h_stat;
    swm_map_stats &S = m->stats;
    memset(&S, 0, sizeof S);
    S.reads = nreads;
    S.items = 2ull * nreads;
    S.chunks = m->tot[TOT_CHUNKS];
    S.fetched = m->tot[TOT_ELEMS];
    S.batches = stat[ST_BATCHES];
    S.candidates = m->tot[TOT_CANDS];
    S.cells = stat[ST_CELLS];
    S.passed = stat[ST_PASSED];
    S.records = m->tot[TOT_RECS];
    S.locations = stat[ST_LOCS];
    S.mapped_reads = stat[ST_MAPPED];
    S.myers_steps = stat[ST_STEPS];
    S.kept = stat[ST_KEPT];
    S.retries = retries;
    S.h2d_bytes = m->h2d_pending;
    m->h2d_pending = 0;
    m->have_result = 1;
    m->cur_n = nreads;
    return SWM_OK;
}

// Run one block on device-resident inputs, re-running it with larger work
// buffers when a capacity was exceeded.
static int run_block(swm_mapper *m, const char *d_reads, const uint32_t *d_lens, uint64_t stride, uint32_t nreads,
                     uint32_t errors, const uint8_t *d_e, uint64_t retries) {
    for (int attempt = 0; attempt < 8; attempt++) {
        int rc = enqueue(m, d_reads, d_lens, stride, nreads, errors, d_e);
        if (rc) return rc;
        int again = 0;
        rc = finish_block(m, nreads, retries, &again);
        if (rc) return rc;
        if (!again) return SWM_OK;
        retries++;
    }
    swm_set_error("mapping block did not fit after repeated buffer growth");
    return SWM_ERR_OOM;
}

static int check_batch(const swm_mapper *m, uint64_t nreads, uint64_t stride, uint32_t errors) {
    if (nreads > m->max_reads) {
        swm_set_error("block of %llu reads exceeds max_reads %llu", (unsigned long long)nreads,
                      (unsigned long long)m->max_reads);
        return SWM_ERR_ARG;
    }
    if (errors > SWM_MAX_ERRORS || stride == 0) {
        swm_set_error("errors must be <= %d and stride > 0", SWM_MAX_ERRORS);
        return SWM_ERR_ARG;
    }
    return SWM_OK;
}

static int check_host_reads(const swm_mapper *m, const uint32_t *lens, const uint8_t *e_arr, uint64_t nreads,
                            uint64_t stride) {
    const uint32_t klong = m->ix->k + SWM_SEED_STEP - 1;
    for (uint64_t r = 0; r < nreads; r++) {
        if (lens[r] > SWM_MAX_READ_LEN || lens[r] > stride || lens[r] / klong > 16 ||
            (e_arr && e_arr[r] > SWM_MAX_ERRORS)) {
            swm_set_error("read %llu: length %u or threshold outside the envelope (L <= %d, L <= stride, e <= %d)",
                          (unsigned long long)r, lens[r], SWM_MAX_READ_LEN, SWM_MAX_ERRORS);
            return SWM_ERR_ARG;
        }
    }
    return SWM_OK;
}

extern "C" int swm_map_device(swm_mapper *m, const char *d_reads, const uint32_t *d_lens, uint64_t stride,
                              uint64_t reads_num, uint32_t errors, const uint8_t *d_errors) {
    if (!m || (!d_reads && reads_num) || (!d_lens && reads_num)) return SWM_ERR_ARG;
    int rc = check_batch(m, reads_num, stride, errors);
    if (rc) return rc;
    SWM_CUDA(cudaSetDevice(m->device));
    if (m->pending) return SWM_ERR_STATE;
    m->have_result = 0;
    return run_block(m, d_reads, d_lens, stride, (uint32_t)reads_num, errors, d_errors, 0);
}

extern "C" int swm_map_device_submit(swm_mapper *m, const char *d_reads, const uint32_t *d_lens, uint64_t stride,
                                     uint64_t reads_num, uint32_t errors, const uint8_t *d_errors) {
    if (!m || (!d_reads && reads_num) || (!d_lens && reads_num)) return SWM_ERR_ARG;
    int rc = check_batch(m, reads_num, stride, errors);
    if (rc) return rc;
    SWM_CUDA(cudaSetDevice(m->device));
    if (m->pending) return SWM_ERR_STATE;
    m->have_result = 0;
    m->dev_reads = d_reads;
    m->dev_lens = d_lens;
    m->dev_e = d_errors;
    m->cur_stride = stride;
    m->cur_n = reads_num;
    m->cur_errors = errors;
    rc = enqueue(m, d_reads, d_lens, stride, (uint32_t)reads_num, errors, d_errors);
    if (rc) return rc;
    m->pending = 2;
    return SWM_OK;
}

extern "C" int swm_map_device_wait(swm_mapper *m) {
    if (!m) return SWM_ERR_ARG;
    if (m->pending != 2) return SWM_ERR_STATE;
    SWM_CUDA(cudaSetDevice(m->device));
    m->pending = 0;
    int again = 0;
    int rc = finish_block(m, (uint32_t)m->cur_n, 0, &again);
    if (rc) return rc;
    if (again) // a work buffer was too small: repeat the block
        rc = run_block(m, m->dev_reads, m->dev_lens, m->cur_stride, (uint32_t)m->cur_n, m->cur_errors, m->dev_e, 1);
    return rc;
}

static int ensure_host(void **p, uint64_t *cap, uint64_t need, size_t elt) {
    if (need <= *cap && *p) return SWM_OK;
    uint64_t n = need + need / 4 + 1024;
    cudaFreeHost(*p);
    *p = nullptr;
    if (cudaHostAlloc(p, n * elt, 0) != cudaSuccess) {
        *p = nullptr;
        *cap = 0;
        swm_set_error("cudaHostAlloc(%llu bytes) failed", (unsigned long long)(n * elt));
        return SWM_ERR_OOM;
    }
    *cap = n;
    return SWM_OK;
}

static bool is_pinned(const void *p) {
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Copy the packed records of the last block to pinned staging.
// cur_read ids (2 * read + 1) of the reads without a location, in read
// order, from the device's bit list (mapper_cpe.c:1455-1458).
static uint64_t unmapped_list(const swm_mapper *m, uint32_t *out, uint64_t cap, int *status) {
    uint64_t nu = 0;
    const uint64_t nh = (m->cur_n + 15) / 16;
    for (uint64_t w = 0; w < nh; w++) {
        uint32_t bits = m->h_unm[w];
        while (bits) {
            const uint32_t j = (uint32_t)__builtin_ctz(bits);
            bits &= bits - 1;
            const uint64_t rd = 16 * w + j;
            if (rd >= m->cur_n) break;
            if (nu < cap && out) out[nu] = (uint32_t)(2 * rd + 1);
            else *status = SWM_ERR_OVERFLOW;
            nu++;
        }
    }
    return nu;
}

static int download_results(swm_mapper *m) {
    if (!m->have_result) return SWM_ERR_STATE;
    SWM_CUDA(cudaSetDevice(m->device));
    const uint64_t nitems = 2 * m->cur_n;
    const uint64_t nrec = m->tot[TOT_RECS], nw = m->tot[TOT_WORDS], nby = m->tot[TOT_BYTES];
    int rc = ensure_host((void **)&m->h_w, &m->h_cap_w, nw, 4);
    if (!rc) rc = ensure_host((void **)&m->h_c, &m->h_cap_c, nby, 1);
    if (!rc) rc = ensure_host((void **)&m->h_rw, &m->h_cap_rw, nrec, 4);
    if (!rc) rc = ensure_host((void **)&m->h_rb, &m->h_cap_rb, nrec, 4);
    if (!rc) rc = ensure_host((void **)&m->h_rl, &m->h_cap_rl, nrec, 4);
    if (!rc) rc = ensure_host((void **)&m->h_unm, &m->h_cap_items, nitems / 32 + 1, 2);
    if (rc) return rc;
    cudaStream_t st = m->st;
    if (nw) SWM_CUDA(cudaMemcpyAsync(m->h_w, m->b.out_w, nw * 4, cudaMemcpyDeviceToHost, st));
    if (nby) SWM_CUDA(cudaMemcpyAsync(m->h_c, m->b.out_c, nby, cudaMemcpyDeviceToHost, st));
    if (nrec) {
        SWM_CUDA(cudaMemcpyAsync(m->h_rw, m->b.rec_woff, nrec * 4, cudaMemcpyDeviceToHost, st));
        SWM_CUDA(cudaMemcpyAsync(m->h_rb, m->b.rec_boff, nrec * 4, cudaMemcpyDeviceToHost, st));
        SWM_CUDA(cudaMemcpyAsync(m->h_rl, m->b.rec_blen, nrec * 4, cudaMemcpyDeviceToHost, st));
    }
    const uint64_t nunm = (m->cur_n + 15) / 16;
    if (nunm) SWM_CUDA(cudaMemcpyAsync(m->h_unm, m->b.unm, nunm * 2, cudaMemcpyDeviceToHost, st));
    SWM_CUDA(cudaStreamSynchronize(st));
    m->stats.d2h_bytes = nw * 4 + nby + nrec * 12 + nunm * 2 + TOT_N * 4 + ST_N * 8;
    return SWM_OK;
}

// Expand the packed records of the last block into the reference layout
// (records at SWM_RECORD_WORDS, CIGARs at SWM_CIGAR_STRIDE, unmapped ids).
extern "C" int swm_map_fetch(swm_mapper *m, swm_result *r) {
    if (!m || !r) return SWM_ERR_ARG;
    int rc = download_results(m);
    if (rc) return rc;
    const uint64_t nrec = m->tot[TOT_RECS];
    int status = SWM_OK;
    r->n_records = nrec;
    for (uint64_t q = 0; q < nrec; q++) {
        const uint32_t *src = m->h_w + m->h_rw[q];
        const uint32_t n = src[1] & 0x7fffffffu;
        const uint32_t bl = m->h_rl[q];
        if (q < r->records_cap) {
            if (r->ref_pos_buffer) memcpy(r->ref_pos_buffer + q * SWM_RECORD_WORDS, src, (2 + n) * 4);
            if (r->cigar_buffer) {
                uint32_t cl = bl <= SWM_CIGAR_STRIDE ? bl : SWM_CIGAR_STRIDE;
                memcpy(r->cigar_buffer + q * SWM_CIGAR_STRIDE, m->h_c + m->h_rb[q], cl);
                if (bl > SWM_CIGAR_STRIDE) status = SWM_ERR_OVERFLOW;
            }
        } else {
            status = SWM_ERR_OVERFLOW;
        }
    }
    r->n_unmapped = unmapped_list(m, r->unmapped, r->unmapped_cap, &status);
    if (status) swm_set_error("result buffers too small (records %llu, unmapped %llu)", (unsigned long long)nrec,
                              (unsigned long long)r->n_unmapped);
    return status;
}

extern "C" int swm_map_fetch_packed(swm_mapper *m, swm_packed_result *r) {
    if (!m || !r) return SWM_ERR_ARG;
    if (!m->have_result) return SWM_ERR_STATE;
    const uint64_t nrec = m->tot[TOT_RECS], nw = m->tot[TOT_WORDS], nby = m->tot[TOT_BYTES];
    if (nw <= r->words_cap && nby <= r->cigar_cap && nrec <= r->records_cap && is_pinned(r->words) &&
        is_pinned(r->cigar) && (!r->record_cigar_len || is_pinned(r->record_cigar_len))) {
        // page-locked caller buffers: copy the packed results straight into them
        SWM_CUDA(cudaSetDevice(m->device));
        const uint64_t nitems = 2 * m->cur_n;
        int rc0 = ensure_host((void **)&m->h_unm, &m->h_cap_items, nitems / 32 + 1, 2);
        if (rc0) return rc0;
        cudaStream_t st = m->st;
        if (nw) SWM_CUDA(cudaMemcpyAsync(r->words, m->b.out_w, nw * 4, cudaMemcpyDeviceToHost, st));
        if (nby) SWM_CUDA(cudaMemcpyAsync(r->cigar, m->b.out_c, nby, cudaMemcpyDeviceToHost, st));
        if (nrec && r->record_cigar_len)
            SWM_CUDA(cudaMemcpyAsync(r->record_cigar_len, m->b.rec_blen, nrec * 4, cudaMemcpyDeviceToHost, st));
        const uint64_t nunm = (m->cur_n + 15) / 16;
        if (nunm) SWM_CUDA(cudaMemcpyAsync(m->h_unm, m->b.unm, nunm * 2, cudaMemcpyDeviceToHost, st));
        SWM_CUDA(cudaStreamSynchronize(st));
        m->stats.d2h_bytes = nw * 4 + nby + (r->record_cigar_len ? nrec * 4 : 0) + nunm * 2 + TOT_N * 4 + ST_N * 8;
        r->n_records = nrec;
        r->n_words = nw;
        r->n_cigar = nby;
        int status = SWM_OK;
        r->n_unmapped = unmapped_list(m, r->unmapped, r->unmapped_cap, &status);
        return status;
    }
    int rc = download_results(m);
    if (rc) return rc;
    r->n_records = nrec;
    r->n_words = nw;
    r->n_cigar = nby;
    int status = SWM_OK;
    if (nw > r->words_cap || nby > r->cigar_cap || nrec > r->records_cap) {
        status = SWM_ERR_OVERFLOW;
    } else {
        // records are laid out in order on the device, so the packed words and
        // bytes are already contiguous
        if (nw) memcpy(r->words, m->h_w, nw * 4);
        if (nby) memcpy(r->cigar, m->h_c, nby);
        if (r->record_cigar_len && nrec) memcpy(r->record_cigar_len, m->h_rl, nrec * 4);
    }
    r->n_unmapped = unmapped_list(m, r->unmapped, r->unmapped_cap, &status);
    if (status) swm_set_error("packed result buffers too small (words %llu, bytes %llu, records %llu)",
                              (unsigned long long)nw, (unsigned long long)nby, (unsigned long long)nrec);
    return status;
}

static int stage_inputs(swm_mapper *m, const swm_batch *b) {
    const uint64_t n = b->reads_num;
    int rc = check_batch(m, n, b->stride, b->errors);
    if (rc) return rc;
    rc = check_host_reads(m, b->reads_len, b->errors_per_read, n, b->stride);
    if (rc) return rc;
    const uint64_t bytes = n * b->stride;
    if (bytes > m->stride_cap) {
        cudaFree(m->d_reads);
        cudaFreeHost(m->h_reads);
        m->d_reads = nullptr;
        m->h_reads = nullptr;
        uint64_t cap = m->max_reads * (b->stride > 256 ? b->stride : 256);
        if (cap < bytes) cap = bytes;
        if (dmalloc(&m->d_reads, cap) || cudaHostAlloc((void **)&m->h_reads, cap, 0) != cudaSuccess) {
            m->stride_cap = 0;
            return SWM_ERR_OOM;
        }
        m->stride_cap = cap;
    }
    // page-locked caller buffers are copied directly; others go through the
    // mapper's pinned staging so that the copy can run asynchronously
    const void *src_reads = b->reads, *src_lens = b->reads_len, *src_e = b->errors_per_read;
    if (!is_pinned(b->reads)) {
        memcpy(m->h_reads, b->reads, bytes);
        src_reads = m->h_reads;
    }
    if (!is_pinned(b->reads_len)) {
        memcpy(m->h_lens, b->reads_len, n * 4);
        src_lens = m->h_lens;
    }
    if (b->errors_per_read && !is_pinned(b->errors_per_read)) {
        memcpy(m->h_e, b->errors_per_read, n);
        src_e = m->h_e;
    }
    SWM_CUDA(cudaMemcpyAsync(m->d_reads, src_reads, bytes, cudaMemcpyHostToDevice, m->st));
    SWM_CUDA(cudaMemcpyAsync(m->d_lens, src_lens, n * 4, cudaMemcpyHostToDevice, m->st));
    if (b->errors_per_read) SWM_CUDA(cudaMemcpyAsync(m->d_e, src_e, n, cudaMemcpyHostToDevice, m->st));
    m->h2d_pending = bytes + n * 4 + (b->errors_per_read ? n : 0);
    return SWM_OK;
}

extern "C" int swm_map_submit(swm_mapper *m, const swm_batch *b) {
    if (!m || !b || (!b->reads && b->reads_num) || (!b->reads_len && b->reads_num)) return SWM_ERR_ARG;
    if (m->pending) return SWM_ERR_STATE;
    SWM_CUDA(cudaSetDevice(m->device));
    int rc = stage_inputs(m, b);
    if (rc) return rc;
    m->cur_stride = b->stride;
    m->cur_n = b->reads_num;
    m->cur_errors = b->errors;
    m->cur_e = b->errors_per_read;
    m->have_result = 0;
    rc = enqueue(m, m->d_reads, m->d_lens, b->stride, (uint32_t)b->reads_num, b->errors,
                 b->errors_per_read ? m->d_e : nullptr);
    if (rc) return rc;
    m->pending = 1;
    return SWM_OK;
}

extern "C" int swm_map_wait(swm_mapper *m, swm_result *r) {
    if (!m || !r) return SWM_ERR_ARG;
    if (m->pending != 1) return SWM_ERR_STATE;
    SWM_CUDA(cudaSetDevice(m->device));
    m->pending = 0;
    int again = 0;
    int rc = finish_block(m, (uint32_t)m->cur_n, 0, &again);
    if (rc) return rc;
    if (again) {
        // a work buffer was too small: repeat the block from the staged inputs
        rc = run_block(m, m->d_reads, m->d_lens, m->cur_stride, (uint32_t)m->cur_n, m->cur_errors,
                       m->cur_e ? m->d_e : nullptr, 1);
        if (rc) return rc;
    }
    return swm_map_fetch(m, r);
}

extern "C" int swm_map_wait_packed(swm_mapper *m, swm_packed_result *r) {
    if (!m || !r) return SWM_ERR_ARG;
    if (m->pending != 1) return SWM_ERR_STATE;
    SWM_CUDA(cudaSetDevice(m->device));
    m->pending = 0;
    int again = 0;
    int rc = finish_block(m, (uint32_t)m->cur_n, 0, &again);
    if (rc) return rc;
    if (again) {
        rc = run_block(m, m->d_reads, m->d_lens, m->cur_stride, (uint32_t)m->cur_n, m->cur_errors,
                       m->cur_e ? m->d_e : nullptr, 1);
        if (rc) return rc;
    }
    return swm_map_fetch_packed(m, r);
}

extern "C" int swm_map_batch(swm_mapper *m, const swm_batch *b, swm_result *r) {
    int rc = swm_map_submit(m, b);
    if (rc) return rc;
    return swm_map_wait(m, r);
}

extern "C" int swm_mapper_stats(const swm_mapper *m, swm_map_stats *s) {
    if (!m || !s) return SWM_ERR_ARG;
    *s = m->stats;
    return SWM_OK;
}

extern "C" int swm_mapper_stage_ms(const swm_mapper *m, const char *stage, float *ms) {
    static const char *names[8] = {"seed", "plan", "candidates", "compact", "verify", "traceback", "records",
                                   "total"};
    if (!m || !stage || !ms) return SWM_ERR_ARG;
    for (int i = 0; i < 8; i++)
        if (!strcmp(stage, names[i])) {
            *ms = m->stage_ms[i];
            return SWM_OK;
        }
    return SWM_ERR_ARG;
}

extern "C" int swm_mapper_tuning(swm_mapper *m, const swm_tuning *set, swm_tuning *get) {
    if (!m) return SWM_ERR_ARG;
    if (set) {
        int mode;
        if (set->verify_pairs > 1 || (set->verify_pairs && set->verify_chunk != 16)) {
            swm_set_error("swm_mapper_tuning: verify_pairs must be 0, or 1 with verify_chunk 16 (got %u, %u)",
                          set->verify_pairs, set->verify_chunk);
            return SWM_ERR_ARG;
        }
        if (set->verify_pairs) mode = VMODE_PAIR16;
        else if (set->verify_chunk == 8) mode = VMODE_STREAM8;
        else if (set->verify_chunk == 16) mode = VMODE_STREAM16;
        else if (set->verify_chunk != 0) {
            swm_set_error("swm_mapper_tuning: verify_chunk must be 0, 8 or 16 (got %u)", set->verify_chunk);
            return SWM_ERR_ARG;
        } else if (set->verify_head_bases == 32 || set->verify_head_bases == 64) {
            mode = set->verify_head_bases == 32 ? VMODE_HEAD32 : VMODE_HEAD64;
        } else {
            swm_set_error("swm_mapper_tuning: verify_head_bases must be 32 or 64 (got %u)", set->verify_head_bases);
            return SWM_ERR_ARG;
        }
        if (m->pending) return SWM_ERR_STATE;
        m->vmode = mode;
    }
    if (get) {
        get->verify_head_bases = m->vmode == VMODE_HEAD32 ? 32u : 64u;
        get->verify_chunk = m->vmode == VMODE_STREAM8 ? 8u : m->vmode >= VMODE_STREAM16 ? 16u : 0u;
        get->verify_pairs = m->vmode == VMODE_PAIR16 ? 1u : 0u;
    }
    return SWM_OK;
}

extern "C" uint64_t swm_mapper_launches(const swm_mapper *m) { return m ? m->launches : 0; }

extern "C" void *swm_mapper_stream(const swm_mapper *m) { return m ? (void *)m->st : nullptr; }

extern "C" int swm_mapper_debug_candidates(const swm_mapper *m, uint32_t *item, uint32_t *pos, int32_t *err,
                                           int32_t *loc, uint64_t cap, uint64_t *n) {
    if (!m || !n) return SWM_ERR_ARG;
    if (!m->have_result) return SWM_ERR_STATE;
    SWM_CUDA(cudaSetDevice(m->device));
    const uint64_t tot = m->tot[TOT_CANDS];
    *n = tot;
    const uint64_t k = tot < cap ? tot : cap;
    if (k) {
        if (item) SWM_CUDA(cudaMemcpy(item, m->b.cc_item, k * 4, cudaMemcpyDeviceToHost));
        if (pos) SWM_CUDA(cudaMemcpy(pos, m->b.cc_pos, k * 4, cudaMemcpyDeviceToHost));
        if (err) SWM_CUDA(cudaMemcpy(err, m->b.vr_err, k * 4, cudaMemcpyDeviceToHost));
        if (loc) SWM_CUDA(cudaMemcpy(loc, m->b.vr_mloc, k * 4, cudaMemcpyDeviceToHost));
    }
    return SWM_OK;
}

extern "C" int swm_mapper_debug_read_words(const swm_mapper *m, uint32_t *words, uint64_t cap_items) {
    if (!m || !words) return SWM_ERR_ARG;
    if (!m->have_result) return SWM_ERR_STATE;
    SWM_CUDA(cudaSetDevice(m->device));
    uint64_t n = 2 * m->cur_n;
    if (n > cap_items) n = cap_items;
    if (n) SWM_CUDA(cudaMemcpy(words, m->b.it_w, n * 32 * 4, cudaMemcpyDeviceToHost));
    return SWM_OK;
}

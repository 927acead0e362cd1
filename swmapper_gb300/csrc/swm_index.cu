// swm_index.cu -- GPU k-mer index build, index files, device scan.
//
// Index build (serial_index.c:157-445, rebuilt for the GPU):
//   kb_encode   32 bases per thread -> lo/hi bit planes, N mask, 2-bit seed
//               words (get_seed, serial_index.c:157-232)
//   kb_count    one thread per sampled position p = 4t: k-mer and N test
//               from the packed words, atomic count (chromo_hash_index,
//               serial_index.c:253-269)
//   scan        start offsets (store_positions, serial_index.c:337-340)
//   kb_scatter  atomic slot per sampled position, key = position << 16 | lseed
//               (serial_index.c:343-352 without the serial order)
//   kb_sort_*   per-bucket sort of the keys: positions are unique, so sorting
//               each bucket restores the ascending order the reference's
//               serial scatter produces
//   kb_split    the sorted keys into the resident index: positions (u32) and
//               flank codes (u16), the layout of .positions / .pos_lseeds
#include <errno.h>
#include <fcntl.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "swm_common.cuh"
#include "swm_files.h"

// ----------------------------------------------------------------- errors

static thread_local char g_err[512] = "";

void swm_set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

extern "C" const char *swm_last_error(void) { return g_err; }

// ------------------------------------------------------------------- scan

#define SCAN_T 256
#define SCAN_V 8
#define SCAN_TILE (SCAN_T * SCAN_V)

uint64_t swm_scan_tmp_words(uint64_t n_cap) { return (n_cap + SCAN_TILE - 1) / SCAN_TILE + 64; }

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, d);
        if ((threadIdx.x & 31) >= d) v += t;
    }
    return v;
}

// exclusive block scan of one value per thread (blockDim.x == SCAN_T or 1024)
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *total) {
    __shared__ uint32_t wsum[33];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    uint32_t inc = warp_incl_scan(v);
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = lane < nw ? wsum[lane] : 0u;
        uint32_t si = warp_incl_scan(s);
        if (lane < nw) wsum[lane] = si - s;
        if (lane == nw - 1) wsum[32] = si;
    }
    __syncthreads();
    uint32_t r = inc - v + wsum[wid];
    if (total) *total = wsum[32];
    __syncthreads();
    return r;
}

__device__ __forceinline__ uint64_t scan_n(const uint32_t *d_n, uint64_t n_host, uint64_t n_cap) {
    uint64_t n = d_n ? (uint64_t)*d_n : n_host;
    return n < n_cap ? n : n_cap;
}

// Sum of one 64-bit value per thread over the block (every thread gets it).
__device__ __forceinline__ uint64_t block_sum_u64(uint64_t v) {
    __shared__ unsigned long long wsum64[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    if (lane == 0) wsum64[wid] = v;
    __syncthreads();
    uint64_t t = 0;
    for (int w = 0; w < nw; w++) t += wsum64[w];
    __syncthreads();
    return t;
}

// Totals are 32-bit: a sum that does not fit saturates to SWM_SCAN_SATURATED
// (each tile's partial, then the total), so callers see an overflow instead
// of a wrapped value.
__global__ void k_scan_reduce(const uint32_t *__restrict__ in, const uint32_t *d_n, uint64_t n_host, uint64_t n_cap,
                              uint32_t *__restrict__ part) {
    const uint64_t n = scan_n(d_n, n_host, n_cap);
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    uint64_t s = 0;
    if (base < n) {
#pragma unroll
        for (int v = 0; v < SCAN_V; v++) {
            uint64_t i = base + threadIdx.x + (uint64_t)v * SCAN_T;
            if (i < n) s += in[i];
        }
    }
    const uint64_t tot = block_sum_u64(s);
    if (threadIdx.x == 0)
        part[blockIdx.x] = (base < n) ? (tot < SWM_SCAN_SATURATED ? (uint32_t)tot : SWM_SCAN_SATURATED) : 0u;
}

__global__ void k_scan_top(uint32_t *part, const uint32_t *d_n, uint64_t n_host, uint64_t n_cap, uint32_t *out,
                           uint32_t *d_total) {
    const uint64_t n = scan_n(d_n, n_host, n_cap);
    const uint64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    const uint64_t per = (nb + blockDim.x - 1) / blockDim.x;
    const uint64_t b0 = threadIdx.x * per;
    uint32_t s = 0;
    uint64_t s64 = 0;
    for (uint64_t i = b0; i < b0 + per && i < nb; i++) {
        s += part[i];
        s64 += part[i];
    }
    const uint64_t tot64 = block_sum_u64(s64);
    uint32_t tot;
    uint32_t ex = block_excl_scan(s, &tot);
    for (uint64_t i = b0; i < b0 + per && i < nb; i++) {
        uint32_t v = part[i];
        part[i] = ex;
        ex += v;
    }
    if (threadIdx.x == 0) {
        if (tot64 >= SWM_SCAN_SATURATED) tot = SWM_SCAN_SATURATED;
        out[n] = tot;
        if (d_total) *d_total = tot;
    }
}

__global__ void k_scan_down(const uint32_t *__restrict__ in, const uint32_t *d_n, uint64_t n_host, uint64_t n_cap,
                            const uint32_t *__restrict__ part, uint32_t *__restrict__ out) {
    const uint64_t n = scan_n(d_n, n_host, n_cap);
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    if (base >= n) return;
    const uint64_t i0 = base + (uint64_t)threadIdx.x * SCAN_V;
    uint32_t v[SCAN_V];
#pragma unroll
    for (int j = 0; j < SCAN_V; j++) v[j] = (i0 + j < n) ? in[i0 + j] : 0u;
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_V; j++) s += v[j];
    uint32_t ex = block_excl_scan(s, nullptr) + part[blockIdx.x];
#pragma unroll
    for (int j = 0; j < SCAN_V; j++) {
        if (i0 + j < n) out[i0 + j] = ex;
        ex += v[j];
    }
}

int swm_exclusive_scan(const uint32_t *d_in, uint32_t *d_out, const uint32_t *d_n, uint64_t n_host, uint64_t n_cap,
                       uint32_t *d_tmp, uint32_t *d_total, cudaStream_t st) {
    const uint64_t nb = (n_cap + SCAN_TILE - 1) / SCAN_TILE;
    const unsigned grid = (unsigned)(nb ? nb : 1);
    k_scan_reduce<<<grid, SCAN_T, 0, st>>>(d_in, d_n, n_host, n_cap, d_tmp);
    k_scan_top<<<1, 1024, 0, st>>>(d_tmp, d_n, n_host, n_cap, d_out, d_total);
    k_scan_down<<<grid, SCAN_T, 0, st>>>(d_in, d_n, n_host, n_cap, d_tmp, d_out);
    SWM_CUDA(cudaGetLastError());
    return SWM_OK;
}

// ------------------------------------------------------------ index build

__global__ void kb_encode(const uint8_t *__restrict__ seq, uint64_t n, uint32_t *__restrict__ b2,
                          uint32_t *__restrict__ b3, uint32_t *__restrict__ s2) {
    __shared__ uint8_t tab[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        int u = i & 0xdf; // toupper for letters (serial_index.c:152)
        tab[i] = u == 'A' ? 0 : u == 'C' ? 1 : u == 'G' ? 2 : u == 'T' ? 3 : 4;
    }
    __syncthreads();
    const uint64_t W = (n + 31) / 32;
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < W; w += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t p0 = w * 32;
        const uint32_t cnt = (n - p0 >= 32) ? 32u : (uint32_t)(n - p0);
        uint8_t bytes[32];
        if (cnt == 32 && (((uintptr_t)(seq + p0)) & 15) == 0) {
            const uint4 *v = reinterpret_cast<const uint4 *>(seq + p0);
            uint4 a = v[0], b = v[1];
            memcpy(bytes, &a, 16);
            memcpy(bytes + 16, &b, 16);
        } else {
            for (uint32_t j = 0; j < cnt; j++) bytes[j] = seq[p0 + j];
        }
        uint32_t lo = 0, hi = 0, nm = 0, sa = 0, sb = 0;
#pragma unroll
        for (uint32_t j = 0; j < 32; j++) {
            if (j < cnt) {
                uint32_t c = tab[bytes[j]];
                if (c == 4) {
                    nm |= 1u << j;
                } else {
                    lo |= (c & 1u) << j;
                    hi |= (c >> 1) << j;
                    if (j < 16) sa |= c << (2 * j);
                    else sb |= c << (2 * (j - 16));
                }
            }
        }
        b2[2 * w] = lo;
        b2[2 * w + 1] = hi;
        b3[w] = nm;
        s2[2 * w] = sa;
        s2[2 * w + 1] = sb;
    }
}

// k-mer at sampled position i (get_seed_from_enc_bits, serial_index.c:280-331)
__device__ __forceinline__ bool sample_at(const uint32_t *__restrict__ b2, const uint32_t *__restrict__ b3,
                                          const uint32_t *__restrict__ s2, uint64_t i, uint32_t k, uint32_t *seed,
                                          uint32_t *lseed) {
    const uint32_t smask = (k >= 16) ? 0xffffffffu : ((1u << (2 * k)) - 1);
    const uint32_t nmask = (1u << k) - 1;
    uint32_t nf = swm_fsr(b3[i / 32], b3[i / 32 + 1], (uint32_t)(i % 32)) & nmask;
    if (nf) return false;
    *seed = swm_fsr(s2[i / 16], s2[i / 16 + 1], (uint32_t)(i % 16) * 2) & smask;
    const uint32_t res = SWM_SEED_STEP - 1, rmask = (1u << res) - 1;
    uint64_t sp = (i >= res) ? i - res : 0;
    uint32_t fl = swm_fsr(b2[(sp / 32) * 2], b2[(sp / 32 + 1) * 2], sp % 32) & rmask;
    uint32_t fh = swm_fsr(b2[(sp / 32) * 2 + 1], b2[(sp / 32 + 1) * 2 + 1], sp % 32) & rmask;
    sp = i + k;
    uint32_t bl = swm_fsr(b2[(sp / 32) * 2], b2[(sp / 32 + 1) * 2], sp % 32) & rmask;
    uint32_t bh = swm_fsr(b2[(sp / 32) * 2 + 1], b2[(sp / 32 + 1) * 2 + 1], sp % 32) & rmask;
    fl |= bl << res;
    fh |= bh << res;
    *lseed = (fl | (fh << (res * 2))) & 0xffffu;
    return true;
}

__global__ void kb_count(const uint32_t *__restrict__ b2, const uint32_t *__restrict__ b3,
                         const uint32_t *__restrict__ s2, uint64_t T, uint32_t k, uint32_t *__restrict__ count) {
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < T; t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t sd, ls;
        if (sample_at(b2, b3, s2, t * SWM_SEED_STEP, k, &sd, &ls)) atomicAdd(&count[sd], 1u);
    }
}

__global__ void kb_scatter(const uint32_t *__restrict__ b2, const uint32_t *__restrict__ b3,
                           const uint32_t *__restrict__ s2, uint64_t T, uint32_t k, uint32_t *__restrict__ cursor,
                           unsigned long long *__restrict__ keys) {
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < T; t += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t sd, ls;
        const uint64_t i = t * SWM_SEED_STEP;
        if (sample_at(b2, b3, s2, i, k, &sd, &ls)) {
            uint32_t slot = atomicAdd(&cursor[sd], 1u);
            keys[slot] = ((unsigned long long)i << 16) | ls;
        }
    }
}

#define SORT_SMALL 32
#define SORT_MED 2048

__global__ void kb_classify(const uint32_t *__restrict__ count, uint64_t nb, uint32_t *__restrict__ lists,
                            uint32_t *__restrict__ nlist, uint64_t list_cap) {
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t c = count[b];
        if (c <= 1) continue;
        int cls = c <= SORT_SMALL ? 0 : c <= SORT_MED ? 1 : 2;
        uint32_t at = atomicAdd(&nlist[cls], 1u);
        if (at < list_cap) lists[(uint64_t)cls * list_cap + at] = (uint32_t)b;
    }
}

__device__ __forceinline__ unsigned long long shfl_u64(unsigned long long v, int lane_mask) {
    uint32_t lo = (uint32_t)v, hi = (uint32_t)(v >> 32);
    lo = __shfl_xor_sync(0xffffffffu, lo, lane_mask);
    hi = __shfl_xor_sync(0xffffffffu, hi, lane_mask);
    return ((unsigned long long)hi << 32) | lo;
}

// one warp per bucket with <= 32 keys: bitonic sort across lanes
__global__ void kb_sort_small(const uint32_t *__restrict__ list, const uint32_t *__restrict__ nlist,
                              const uint32_t *__restrict__ off, const uint32_t *__restrict__ count,
                              unsigned long long *__restrict__ keys) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    const uint32_t total = *nlist;
    for (uint64_t wi = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; wi < total; wi += nwarps) {
        const uint32_t b = list[wi];
        const uint32_t o = off[b], c = count[b];
        unsigned long long v = lane < c ? keys[o + lane] : ~0ull;
#pragma unroll
        for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                unsigned long long w = shfl_u64(v, stride);
                bool up = ((lane & size) == 0);
                bool lower = ((lane & stride) == 0);
                bool take_min = (lower == up);
                v = take_min ? (w < v ? w : v) : (w > v ? w : v);
            }
        }
        if (lane < c) keys[o + lane] = v;
    }
}

// one block per bucket with <= SORT_MED keys: bitonic sort in shared memory
__global__ void kb_sort_med(const uint32_t *__restrict__ list, const uint32_t *__restrict__ nlist,
                            const uint32_t *__restrict__ off, const uint32_t *__restrict__ count,
                            unsigned long long *__restrict__ keys) {
    __shared__ unsigned long long sm[SORT_MED];
    const uint32_t total = *nlist;
    for (uint32_t bi = blockIdx.x; bi < total; bi += gridDim.x) {
        const uint32_t b = list[bi];
        const uint32_t o = off[b], c = count[b];
        uint32_t n2 = 1;
        while (n2 < c) n2 <<= 1;
        for (uint32_t i = threadIdx.x; i < n2; i += blockDim.x) sm[i] = i < c ? keys[o + i] : ~0ull;
        __syncthreads();
        for (uint32_t size = 2; size <= n2; size <<= 1) {
            for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
                for (uint32_t i = threadIdx.x; i < n2 / 2; i += blockDim.x) {
                    uint32_t lo = 2 * i - (i & (stride - 1));
                    uint32_t hi = lo + stride;
                    bool up = ((lo & size) == 0);
                    unsigned long long a = sm[lo], d = sm[hi];
                    if ((a > d) == up) {
                        sm[lo] = d;
                        sm[hi] = a;
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t i = threadIdx.x; i < c; i += blockDim.x) keys[o + i] = sm[i];
        __syncthreads();
    }
}

// one block per large bucket: bitonic sort in a padded global scratch region
__global__ void kb_sort_large(const uint32_t *__restrict__ list, const uint32_t *__restrict__ off,
                              const uint32_t *__restrict__ count, const uint64_t *__restrict__ scratch_off,
                              unsigned long long *__restrict__ scratch, unsigned long long *__restrict__ keys) {
    const uint32_t b = list[blockIdx.x];
    const uint32_t o = off[b], c = count[b];
    unsigned long long *sm = scratch + scratch_off[blockIdx.x];
    uint32_t n2 = 1;
    while (n2 < c) n2 <<= 1;
    for (uint32_t i = threadIdx.x; i < n2; i += blockDim.x) sm[i] = i < c ? keys[o + i] : ~0ull;
    __syncthreads();
    for (uint32_t size = 2; size <= n2; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (uint32_t i = threadIdx.x; i < n2 / 2; i += blockDim.x) {
                uint32_t lo = 2 * i - (i & (stride - 1));
                uint32_t hi = lo + stride;
                bool up = ((lo & size) == 0);
                unsigned long long a = sm[lo], d = sm[hi];
                if ((a > d) == up) {
                    sm[lo] = d;
                    sm[hi] = a;
                }
            }
            __syncthreads();
        }
    }
    for (uint32_t i = threadIdx.x; i < c; i += blockDim.x) keys[o + i] = sm[i];
}

__global__ void kb_split(const unsigned long long *__restrict__ keys, uint64_t S, uint32_t *__restrict__ pos,
                         uint16_t *__restrict__ lseed) {
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < S; j += (uint64_t)gridDim.x * blockDim.x) {
        unsigned long long v = keys[j];
        if (pos) pos[j] = (uint32_t)(v >> 16);
        if (lseed) lseed[j] = (uint16_t)(v & 0xffffu);
    }
}

// ---------------------------------------------------- candidate table
//
// long_seeds_filter (mapper_cpe.c:2090-2123) keeps an entry of a seed's
// bucket when the 3 flank bits of each plane at the seed's shift equal the
// read's, i.e. when the whole 15-base long seed matches. The table groups, for
// every bucket and every shift t, the bucket's entries by that 6-bit flank
// value (stable: ascending position inside a group), so that the entries one
// (seed, shift, read flank) keeps are one contiguous range of positions, found
// with a single offset lookup. Segment (bucket B, shift t) starts at
// 4 * off[B] + t * count[B]; ctab_off[key(B, t, v)] is where flank value v
// starts in it, and ctab_off[key + 1] where it ends (the next key's start,
// also across shifts and buckets; the last entry holds 4 * n_seeds).

#define CTAB_WARPS 8

// One warp per bucket: for each shift a 64-bin histogram of the flank values,
// its exclusive scan (the 64 offsets, written as one coalesced 256-byte row)
// and a stable scatter of the positions (rank among equal values from a
// match mask, chunk by chunk in position order).
__global__ void __launch_bounds__(CTAB_WARPS * 32) kb_ctab(const uint32_t *__restrict__ off, uint64_t nb,
                                                           const uint32_t *__restrict__ pos,
                                                           const uint16_t *__restrict__ ls,
                                                           uint32_t *__restrict__ ctab_off,
                                                           uint32_t *__restrict__ ctab_pos) {
    __shared__ uint32_t hist_all[CTAB_WARPS][64];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t *hist = hist_all[wib];
    uint32_t lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    const uint64_t nwarps = (uint64_t)gridDim.x * CTAB_WARPS;
    for (uint64_t b = (uint64_t)blockIdx.x * CTAB_WARPS + wib; b < nb; b += nwarps) {
        const uint32_t o = off[b], c = off[b + 1] - o;
        uint32_t *row = ctab_off + (b << 8);
        if (c == 0) { // every key of an empty bucket starts (and ends) at its segment
            const uint32_t v = 4u * o;
            reinterpret_cast<uint4 *>(row)[lane] = make_uint4(v, v, v, v);
            reinterpret_cast<uint4 *>(row)[lane + 32] = make_uint4(v, v, v, v);
            continue;
        }
        // small buckets keep their entries in registers across the 4 shifts
        const uint32_t l0 = lane < c ? ls[o + lane] : 0u;
        const uint32_t p0 = lane < c ? pos[o + lane] : 0u;
        for (uint32_t t = 0; t < SWM_SEED_STEP; t++) {
            const uint32_t base = 4u * o + t * c;
            hist[lane] = 0;
            hist[lane + 32] = 0;
            __syncwarp();
            for (uint32_t j0 = 0; j0 < c; j0 += 32) {
                const bool in = j0 + lane < c;
                const uint32_t l = c <= 32 ? l0 : (in ? (uint32_t)ls[o + j0 + lane] : 0u);
                const uint32_t v = in ? swm_ctab_flank(l, t) : 64u + lane; // out-of-range lanes match nobody
                const uint32_t mm = __match_any_sync(0xffffffffu, v);
                if (in && (mm & lt) == 0) hist[v] += __popc(mm); // one leader per value
                __syncwarp();
            }
            // exclusive scan of the 64 bins, two per lane
            const uint32_t a = hist[2 * lane], d = hist[2 * lane + 1];
            uint32_t inc = a + d;
#pragma unroll
            for (int k = 1; k < 32; k <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, inc, k);
                if ((int)lane >= k) inc += y;
            }
            const uint32_t s0 = base + inc - (a + d);
            reinterpret_cast<uint2 *>(row + (t << 6))[lane] = make_uint2(s0, s0 + a);
            __syncwarp();
            hist[2 * lane] = s0; // now the running cursor of each value
            hist[2 * lane + 1] = s0 + a;
            __syncwarp();
            for (uint32_t j0 = 0; j0 < c; j0 += 32) {
                const bool in = j0 + lane < c;
                const uint32_t l = c <= 32 ? l0 : (in ? (uint32_t)ls[o + j0 + lane] : 0u);
                const uint32_t p = c <= 32 ? p0 : (in ? pos[o + j0 + lane] : 0u);
                const uint32_t v = in ? swm_ctab_flank(l, t) : 64u + lane;
                const uint32_t mm = __match_any_sync(0xffffffffu, v);
                uint32_t at = 0;
                if (in) at = hist[v] + __popc(mm & lt);
                __syncwarp();
                if (in) {
                    ctab_pos[at] = p;
                    if ((mm & lt) == 0) hist[v] += __popc(mm);
                }
                __syncwarp();
            }
        }
    }
}

// ----------------------------------------------------------- host helpers
// ----------------------------------------------------------- host helpers

static int sm_count(int device) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
    return n > 0 ? n : 1;
}

static unsigned grid_for(uint64_t work, unsigned threads, int device, int per_sm = 8) {
    uint64_t g = (work + threads - 1) / threads;
    uint64_t cap = (uint64_t)sm_count(device) * per_sm;
    if (g > cap) g = cap;
    return (unsigned)(g ? g : 1);
}

static void index_release(swm_index *ix) {
    if (!ix) return;
    if (ix->chain_ev) cudaEventDestroy(ix->chain_ev);
    cudaFree(ix->d_ctab_off);
    cudaFree(ix->d_ctab_pos);
    cudaFree(ix->d_count);
    cudaFree(ix->d_off);
    cudaFree(ix->d_pos);
    cudaFree(ix->d_ls);
    cudaFree(ix->d_b2);
    cudaFree(ix->d_b3);
    free(ix);
}

template <typename T>
static int dalloc(T **p, uint64_t count) {
    *p = nullptr;
    cudaError_t e = cudaMalloc((void **)p, (count ? count : 1) * sizeof(T));
    if (e != cudaSuccess) {
        swm_set_error("cudaMalloc(%llu bytes): %s", (unsigned long long)(count * sizeof(T)), cudaGetErrorString(e));
        *p = nullptr;
        return SWM_ERR_OOM;
    }
    return SWM_OK;
}

static int build_on_device(const uint8_t *d_seq, uint64_t n, uint32_t k, int device, swm_index **out) {
    if (k < 1 || k > 14 || n >= 0xffffffffull) {
        swm_set_error("swm_index_build: k must be in [1, 14] and n < 2^32 (k=%u n=%llu)", k, (unsigned long long)n);
        return SWM_ERR_ARG;
    }
    SWM_CUDA(cudaSetDevice(device));
    swm_index *ix = (swm_index *)calloc(1, sizeof(swm_index));
    if (!ix) return SWM_ERR_OOM;
    ix->device = device;
    ix->k = k;
    ix->n = n;
    const uint64_t W = (n + 31) / 32;
    const uint64_t nb = 1ull << (2 * k);
    ix->n_words2 = 2 * W;
    ix->n_words3 = W;
    ix->ref_length = ix->n_words2 * 4 * 16;
    cudaStream_t st = 0;
    uint32_t *d_s2 = nullptr, *d_cursor = nullptr, *d_tmp = nullptr, *d_lists = nullptr, *d_nlist = nullptr;
    unsigned long long *d_keys = nullptr; // position << 16 | lseed: sorting these sorts positions in a bucket
    auto cleanup = [&]() {
        cudaFree(d_keys);
        d_keys = nullptr;
        cudaFree(d_s2);
        cudaFree(d_cursor);
        cudaFree(d_tmp);
        cudaFree(d_lists);
        cudaFree(d_nlist);
    };
#define TRYC(x)                  \
    do {                         \
        int rc_ = (x);           \
        if (rc_ != SWM_OK) {     \
            cleanup();           \
            index_release(ix);   \
            return rc_;          \
        }                        \
    } while (0)
#define CUC(x)                                                                                   \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess) {                                                                 \
            swm_set_error("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_));       \
            cleanup();                                                                           \
            index_release(ix);                                                                   \
            return SWM_ERR_CUDA;                                                                 \
        }                                                                                        \
    } while (0)
    TRYC(dalloc(&ix->d_b2, ix->n_words2 + SWM_PAD_WORDS));
    TRYC(dalloc(&ix->d_b3, ix->n_words3 + SWM_PAD_WORDS));
    TRYC(dalloc(&d_s2, 2 * W + SWM_PAD_WORDS));
    TRYC(dalloc(&ix->d_count, nb));
    TRYC(dalloc(&ix->d_off, nb + 1));
    TRYC(dalloc(&d_cursor, nb + 1));
    TRYC(dalloc(&d_tmp, swm_scan_tmp_words(nb)));
    CUC(cudaMemsetAsync(ix->d_b2 + ix->n_words2, 0, SWM_PAD_WORDS * 4, st));
    CUC(cudaMemsetAsync(ix->d_b3 + ix->n_words3, 0, SWM_PAD_WORDS * 4, st));
    CUC(cudaMemsetAsync(d_s2 + 2 * W, 0, SWM_PAD_WORDS * 4, st));
    CUC(cudaMemsetAsync(ix->d_count, 0, nb * 4, st));
    if (W) kb_encode<<<grid_for(W, 256, device, 16), 256, 0, st>>>(d_seq, n, ix->d_b2, ix->d_b3, d_s2);
    const uint64_t T = (n >= k) ? (n - k) / SWM_SEED_STEP + 1 : 0;
    if (T) kb_count<<<grid_for(T, 256, device, 16), 256, 0, st>>>(ix->d_b2, ix->d_b3, d_s2, T, k, ix->d_count);
    CUC(cudaGetLastError());
    TRYC(swm_exclusive_scan(ix->d_count, ix->d_off, nullptr, nb, nb, d_tmp, nullptr, st));
    uint32_t S32 = 0;
    CUC(cudaMemcpyAsync(&S32, ix->d_off + nb, 4, cudaMemcpyDeviceToHost, st));
    CUC(cudaStreamSynchronize(st));
    const uint64_t S = S32;
    ix->n_seeds = S;
    TRYC(dalloc(&d_keys, S + 8));
    if (S) {
        CUC(cudaMemcpyAsync(d_cursor, ix->d_off, nb * 4, cudaMemcpyDeviceToDevice, st));
        kb_scatter<<<grid_for(T, 256, device, 16), 256, 0, st>>>(ix->d_b2, ix->d_b3, d_s2, T, k, d_cursor, d_keys);
        // per-bucket sort, classified by bucket size
        const uint64_t list_cap = nb;
        TRYC(dalloc(&d_lists, 3 * list_cap));
        TRYC(dalloc(&d_nlist, 4));
        CUC(cudaMemsetAsync(d_nlist, 0, 16, st));
        kb_classify<<<grid_for(nb, 256, device, 16), 256, 0, st>>>(ix->d_count, nb, d_lists, d_nlist, list_cap);
        kb_sort_small<<<sm_count(device) * 8, 256, 0, st>>>(d_lists, d_nlist, ix->d_off, ix->d_count, d_keys);
        kb_sort_med<<<sm_count(device) * 4, 256, 0, st>>>(d_lists + list_cap, d_nlist + 1, ix->d_off, ix->d_count,
                                                          d_keys);
        CUC(cudaGetLastError());
        uint32_t nl[3];
        CUC(cudaMemcpyAsync(nl, d_nlist, 12, cudaMemcpyDeviceToHost, st));
        CUC(cudaStreamSynchronize(st));
        if (nl[2]) {
            std::vector<uint32_t> big(nl[2]);
            CUC(cudaMemcpy(big.data(), d_lists + 2 * list_cap, nl[2] * 4ull, cudaMemcpyDeviceToHost));
            std::vector<uint32_t> cnt(nl[2]);
            for (uint32_t i = 0; i < nl[2]; i++) CUC(cudaMemcpy(&cnt[i], ix->d_count + big[i], 4, cudaMemcpyDeviceToHost));
            // process in groups whose padded scratch fits a bounded buffer
            const uint64_t scratch_cap = 1ull << 27; // keys (1 GiB)
            uint64_t i0 = 0;
            while (i0 < nl[2]) {
                std::vector<uint64_t> soff;
                uint64_t tot = 0, i1 = i0;
                while (i1 < nl[2]) {
                    uint64_t n2 = 1;
                    while (n2 < cnt[i1]) n2 <<= 1;
                    if (tot && tot + n2 > scratch_cap) break;
                    soff.push_back(tot);
                    tot += n2;
                    i1++;
                }
                unsigned long long *d_scr = nullptr;
                uint64_t *d_soff = nullptr;
                TRYC(dalloc(&d_scr, tot));
                if (dalloc(&d_soff, soff.size()) != SWM_OK) {
                    cudaFree(d_scr);
                    cleanup();
                    index_release(ix);
                    return SWM_ERR_OOM;
                }
                cudaMemcpy(d_soff, soff.data(), soff.size() * 8, cudaMemcpyHostToDevice);
                kb_sort_large<<<(unsigned)(i1 - i0), 1024, 0, st>>>(d_lists + 2 * list_cap + i0, ix->d_off,
                                                                   ix->d_count, d_soff, d_scr, d_keys);
                cudaError_t e = cudaStreamSynchronize(st);
                cudaFree(d_scr);
                cudaFree(d_soff);
                CUC(e);
                i0 = i1;
            }
        }
        CUC(cudaGetLastError());
    }
    // the mapper reads the two halves separately: flank codes for every
    // fetched entry, positions only for the entries the flank filter keeps
    TRYC(dalloc(&ix->d_pos, S + 8));
    TRYC(dalloc(&ix->d_ls, S + 8));
    CUC(cudaMemsetAsync(ix->d_pos + S, 0, 8 * 4, st));
    CUC(cudaMemsetAsync(ix->d_ls + S, 0, 8 * 2, st));
    if (S) kb_split<<<grid_for(S, 256, device, 16), 256, 0, st>>>(d_keys, S, ix->d_pos, ix->d_ls);
    CUC(cudaGetLastError());
    CUC(cudaStreamSynchronize(st));
    cleanup();
    *out = ix;
    return SWM_OK;
#undef TRYC
#undef CUC
}

extern "C" int swm_index_build_device(const uint8_t *d_seq, uint64_t n, uint32_t k, int device, swm_index **out) {
    if (!out || (!d_seq && n)) return SWM_ERR_ARG;
    return build_on_device(d_seq, n, k, device, out);
}

extern "C" int swm_index_build(const uint8_t *seq, uint64_t n, uint32_t k, int device, swm_index **out) {
    if (!out || (!seq && n)) return SWM_ERR_ARG;
    SWM_CUDA(cudaSetDevice(device));
    uint8_t *d_seq = nullptr;
    if (n) {
        cudaError_t e = cudaMalloc(&d_seq, n);
        if (e != cudaSuccess) {
            swm_set_error("cudaMalloc(sequence %llu): %s", (unsigned long long)n, cudaGetErrorString(e));
            return SWM_ERR_OOM;
        }
        e = cudaMemcpy(d_seq, seq, n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(d_seq);
            swm_set_error("H2D sequence: %s", cudaGetErrorString(e));
            return SWM_ERR_CUDA;
        }
    }
    int rc = build_on_device(d_seq, n, k, device, out);
    cudaFree(d_seq);
    return rc;
}

extern "C" int swm_index_get_info(const swm_index *ix, swm_index_info *info) {
    if (!ix || !info) return SWM_ERR_ARG;
    info->k = ix->k;
    info->n = ix->n;
    info->n_seeds = ix->n_seeds;
    info->n_words2 = ix->n_words2;
    info->n_words3 = ix->n_words3;
    info->ref_length = ix->ref_length;
    info->device = ix->device;
    return SWM_OK;
}

extern "C" int swm_index_download(const swm_index *ix, uint32_t *hash_count, uint32_t *hash_offset_end,
                                  uint32_t *positions, uint16_t *pos_lseeds, uint32_t *base_2bits,
                                  uint32_t *base_3bits) {
    if (!ix) return SWM_ERR_ARG;
    SWM_CUDA(cudaSetDevice(ix->device));
    const uint64_t nb = 1ull << (2 * ix->k);
    if (hash_count) SWM_CUDA(cudaMemcpy(hash_count, ix->d_count, nb * 4, cudaMemcpyDeviceToHost));
    if (hash_offset_end) {
        // the reference's file holds the scatter cursors: start[i + 1] for
        // bucket i, and the total once more at [4^k] (serial_index.c:337-352)
        SWM_CUDA(cudaMemcpy(hash_offset_end, ix->d_off + 1, nb * 4, cudaMemcpyDeviceToHost));
        hash_offset_end[nb] = (uint32_t)ix->n_seeds;
    }
    if (positions && ix->n_seeds)
        SWM_CUDA(cudaMemcpy(positions, ix->d_pos, ix->n_seeds * 4, cudaMemcpyDeviceToHost));
    if (pos_lseeds && ix->n_seeds)
        SWM_CUDA(cudaMemcpy(pos_lseeds, ix->d_ls, ix->n_seeds * 2, cudaMemcpyDeviceToHost));
    if (base_2bits && ix->n_words2)
        SWM_CUDA(cudaMemcpy(base_2bits, ix->d_b2, ix->n_words2 * 4, cudaMemcpyDeviceToHost));
    if (base_3bits && ix->n_words3)
        SWM_CUDA(cudaMemcpy(base_3bits, ix->d_b3, ix->n_words3 * 4, cudaMemcpyDeviceToHost));
    return SWM_OK;
}

extern "C" int swm_index_save(const swm_index *ix, const char *prefix, const char *ref_info, size_t ref_info_len) {
    if (!ix || !prefix) return SWM_ERR_ARG;
    const uint64_t nb = 1ull << (2 * ix->k);
    std::vector<uint32_t> cnt(nb), off(nb + 1), pos(ix->n_seeds), b2(ix->n_words2), b3(ix->n_words3);
    std::vector<uint16_t> ls(ix->n_seeds);
    int rc = swm_index_download(ix, cnt.data(), off.data(), pos.data(), ls.data(), b2.data(), b3.data());
    if (rc) return rc;
    if (swmf_write(prefix, ".ref_info", ref_info ? ref_info : "", ref_info ? ref_info_len : 0) ||
        swmf_write(prefix, ".hash_count", cnt.data(), nb * 4) ||
        swmf_write(prefix, ".hash_offset", off.data(), (nb + 1) * 4) ||
        swmf_write(prefix, ".positions", pos.data(), ix->n_seeds * 4) ||
        swmf_write(prefix, ".pos_lseeds", ls.data(), ix->n_seeds * 2) ||
        swmf_write(prefix, ".base_2bits", b2.data(), ix->n_words2 * 4) ||
        swmf_write(prefix, ".base_3bits", b3.data(), ix->n_words3 * 4)) {
        swm_set_error("cannot write index files under %s", prefix);
        return SWM_ERR_IO;
    }
    return SWM_OK;
}

extern "C" int swm_index_build_fasta(const char *fasta_path, const char *prefix, uint32_t k, int device) {
    if (!fasta_path || !prefix) return SWM_ERR_ARG;
    uint8_t *seq = nullptr;
    uint64_t n = 0;
    char *info = nullptr;
    size_t info_len = 0;
    int rc = swmf_read_fasta(fasta_path, &seq, &n, &info, &info_len);
    if (rc) {
        swm_set_error("cannot read FASTA %s", fasta_path);
        return rc == -3 ? SWM_ERR_OOM : SWM_ERR_IO;
    }
    swm_index *ix = nullptr;
    rc = swm_index_build(seq, n, k, device, &ix);
    free(seq);
    if (rc == SWM_OK) {
        rc = swm_index_save(ix, prefix, info, info_len);
        swm_index_free(ix);
    }
    free(info);
    return rc;
}

// ------------------------------------------------------------ index load
//
// load_ref_info (mapper_mpe.c:198-314) freads each file whole into malloc'ed
// memory before the mapper uses it. Here each file streams into device
// memory: one host thread per file reads 32 MiB chunks with pread into two
// page-locked buffers in turn while the previous chunk's copy runs on the
// thread's own stream, so disk (or page cache) reads overlap the H2D copies
// and the five files load concurrently.

#define LOAD_CHUNK (32ull << 20)

static std::string index_path(const char *prefix, const char *ext) { return std::string(prefix) + ext; }

// Size of a regular file, or -1 when it cannot be stat'ed.
static int64_t file_bytes(const std::string &path) {
    struct stat sb;
    if (stat(path.c_str(), &sb) != 0 || !S_ISREG(sb.st_mode)) return -1;
    return (int64_t)sb.st_size;
}

struct FileLoad {
    std::string path;
    uint64_t bytes;
    void *d_dst;
    bool sum_words; // add up the file's u32 words (the bucket counts)
    uint64_t sum;
    int rc;
    char err[256];
};

static void load_file(FileLoad *L, int device) {
    L->rc = SWM_OK;
    L->sum = 0;
    if (cudaSetDevice(device) != cudaSuccess) {
        snprintf(L->err, sizeof L->err, "cudaSetDevice(%d) failed", device);
        L->rc = SWM_ERR_CUDA;
        return;
    }
    const int fd = open(L->path.c_str(), O_RDONLY);
    if (fd < 0) {
        snprintf(L->err, sizeof L->err, "cannot open %s", L->path.c_str());
        L->rc = SWM_ERR_IO;
        return;
    }
#ifdef POSIX_FADV_SEQUENTIAL
    posix_fadvise(fd, 0, 0, POSIX_FADV_SEQUENTIAL);
#endif
    cudaStream_t st = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    uint8_t *buf[2] = {nullptr, nullptr};
    const uint64_t chunk = L->bytes < LOAD_CHUNK ? (L->bytes ? L->bytes : 1) : LOAD_CHUNK;
    bool ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
    for (int i = 0; i < 2 && ok; i++)
        ok = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) == cudaSuccess &&
             cudaHostAlloc((void **)&buf[i], chunk, 0) == cudaSuccess;
    if (!ok) {
        snprintf(L->err, sizeof L->err, "staging buffers for %s", L->path.c_str());
        L->rc = SWM_ERR_OOM;
    }
    bool used[2] = {false, false};
    for (uint64_t off = 0, i = 0; L->rc == SWM_OK && off < L->bytes; i ^= 1) {
        const uint64_t len = L->bytes - off < chunk ? L->bytes - off : chunk;
        if (used[i] && cudaEventSynchronize(ev[i]) != cudaSuccess) { // buffer i's last copy is done
            snprintf(L->err, sizeof L->err, "H2D of %s failed", L->path.c_str());
            L->rc = SWM_ERR_CUDA;
            break;
        }
        uint64_t got = 0;
        while (got < len) {
            const ssize_t r = pread(fd, buf[i] + got, len - got, (off_t)(off + got));
            if (r < 0 && errno == EINTR) continue;
            if (r <= 0) break;
            got += (uint64_t)r;
        }
        if (got != len) {
            snprintf(L->err, sizeof L->err, "%s is shorter than its %llu bytes", L->path.c_str(),
                     (unsigned long long)L->bytes);
            L->rc = SWM_ERR_IO;
            break;
        }
        if (L->sum_words) {
            const uint32_t *w = (const uint32_t *)buf[i];
            for (uint64_t j = 0; j < len / 4; j++) L->sum += w[j];
        }
        if (cudaMemcpyAsync((uint8_t *)L->d_dst + off, buf[i], len, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaEventRecord(ev[i], st) != cudaSuccess) {
            snprintf(L->err, sizeof L->err, "H2D of %s failed", L->path.c_str());
            L->rc = SWM_ERR_CUDA;
            break;
        }
        used[i] = true;
        off += len;
    }
    if (st && cudaStreamSynchronize(st) != cudaSuccess && L->rc == SWM_OK) {
        snprintf(L->err, sizeof L->err, "H2D of %s failed", L->path.c_str());
        L->rc = SWM_ERR_CUDA;
    }
    for (int i = 0; i < 2; i++) {
        if (buf[i]) cudaFreeHost(buf[i]);
        if (ev[i]) cudaEventDestroy(ev[i]);
    }
    if (st) cudaStreamDestroy(st);
    close(fd);
}

extern "C" int swm_index_open(const char *prefix, uint32_t k, int device, swm_index **out) {
    if (!prefix || !out || k < 1 || k > 14) {
        swm_set_error("swm_index_open: null argument or k outside [1, 14]");
        return SWM_ERR_ARG;
    }
    // every file present and the sizes consistent before any device work
    static const char *exts[5] = {".hash_count", ".positions", ".pos_lseeds", ".base_2bits", ".base_3bits"};
    int64_t sz[5];
    for (int f = 0; f < 5; f++) {
        sz[f] = file_bytes(index_path(prefix, exts[f]));
        if (sz[f] < 0) {
            swm_set_error("index file %s is missing", index_path(prefix, exts[f]).c_str());
            return SWM_ERR_IO;
        }
    }
    const uint64_t nb = 1ull << (2 * k);
    const uint64_t S = (uint64_t)sz[1] / 4;
    if ((uint64_t)sz[0] != nb * 4 || sz[1] % 4 || (uint64_t)sz[2] != S * 2 || sz[3] % 8 || sz[3] != 2 * sz[4] ||
        S >= 0xffffffffull) {
        swm_set_error("index files under %s have inconsistent sizes for k=%u (hash_count %lld, positions %lld, "
                      "pos_lseeds %lld, base_2bits %lld, base_3bits %lld bytes)",
                      prefix, k, (long long)sz[0], (long long)sz[1], (long long)sz[2], (long long)sz[3],
                      (long long)sz[4]);
        return SWM_ERR_IO;
    }
    SWM_CUDA(cudaSetDevice(device));
    swm_index *ix = (swm_index *)calloc(1, sizeof(swm_index));
    if (!ix) return SWM_ERR_OOM;
    ix->device = device;
    ix->k = k;
    ix->n_seeds = S;
    ix->n_words2 = (uint64_t)sz[3] / 4;
    ix->n_words3 = (uint64_t)sz[4] / 4;
    ix->ref_length = (uint64_t)sz[3] * 16; // mapper_mpe.c:288
    ix->n = 32 * ix->n_words3;
    void *info = nullptr;
    size_t ninfo = 0;
    if (swmf_read(prefix, ".ref_info", &info, &ninfo) == 0) {
        const uint64_t t = swmf_ref_info_total((const char *)info, ninfo);
        if (t) ix->n = t;
        free(info);
    }
    uint32_t *d_tmp = nullptr;
    int rc = SWM_OK;
    if (dalloc(&ix->d_count, nb) || dalloc(&ix->d_off, nb + 1) || dalloc(&ix->d_pos, S + 8) ||
        dalloc(&ix->d_ls, S + 8) || dalloc(&ix->d_b2, ix->n_words2 + SWM_PAD_WORDS) ||
        dalloc(&ix->d_b3, ix->n_words3 + SWM_PAD_WORDS) || dalloc(&d_tmp, swm_scan_tmp_words(nb))) {
        rc = SWM_ERR_OOM;
    }
    if (rc == SWM_OK) {
        FileLoad loads[5];
        void *dst[5] = {ix->d_count, ix->d_pos, ix->d_ls, ix->d_b2, ix->d_b3};
        for (int f = 0; f < 5; f++) {
            loads[f].path = index_path(prefix, exts[f]);
            loads[f].bytes = (uint64_t)sz[f];
            loads[f].d_dst = dst[f];
            loads[f].sum_words = f == 0;
            loads[f].err[0] = 0;
        }
        std::vector<std::thread> th;
        for (int f = 1; f < 5; f++) th.emplace_back(load_file, &loads[f], device);
        load_file(&loads[0], device);
        for (auto &t : th) t.join();
        for (int f = 0; f < 5 && rc == SWM_OK; f++)
            if (loads[f].rc != SWM_OK) {
                swm_set_error("%s", loads[f].err);
                rc = loads[f].rc;
            }
        if (rc == SWM_OK && loads[0].sum != S) {
            swm_set_error("index files under %s are inconsistent: hash_count adds up to %llu, positions hold %llu",
                          prefix, (unsigned long long)loads[0].sum, (unsigned long long)S);
            rc = SWM_ERR_IO;
        }
    }
    if (rc == SWM_OK) {
        if (cudaMemset(ix->d_pos + S, 0, 32) != cudaSuccess || cudaMemset(ix->d_ls + S, 0, 16) != cudaSuccess ||
            cudaMemset(ix->d_b2 + ix->n_words2, 0, SWM_PAD_WORDS * 4) != cudaSuccess ||
            cudaMemset(ix->d_b3 + ix->n_words3, 0, SWM_PAD_WORDS * 4) != cudaSuccess) {
            swm_set_error("clearing the index padding under %s failed", prefix);
            rc = SWM_ERR_CUDA;
        }
    }
    if (rc == SWM_OK) {
        // hash_offset rebuilt from the counts (mapper_mpe.c:250-255)
        rc = swm_exclusive_scan(ix->d_count, ix->d_off, nullptr, nb, nb, d_tmp, nullptr, 0);
        if (rc == SWM_OK && cudaDeviceSynchronize() != cudaSuccess) {
            swm_set_error("rebuilding hash_offset under %s failed", prefix);
            rc = SWM_ERR_CUDA;
        }
    }
    cudaFree(d_tmp);
    if (rc != SWM_OK) {
        index_release(ix);
        return rc;
    }
    *out = ix;
    return SWM_OK;
}

extern "C" void swm_index_free(swm_index *ix) {
    if (!ix) return;
    cudaSetDevice(ix->device);
    index_release(ix);
}

static std::mutex g_ctab_mu;

// Device bytes of the candidate table of ix.
static uint64_t ctab_bytes(const swm_index *ix) { return (SWM_CTAB_KEYS + 1) * 4 + (4 * ix->n_seeds + 8) * 4; }

// Build the candidate table when it is missing, k is 12, the caller has not
// dropped it, and the device holds it with a margin (8 GiB) to spare. Not
// building it is not an error: the mapper then filters the buckets entry by
// entry. Returns SWM_OK in both cases; a CUDA error while building is returned.
int swm_ctab_build(swm_index *ix, int forced) {
    std::lock_guard<std::mutex> lk(g_ctab_mu);
    if (ix->d_ctab_off || ix->ctab_off || ix->k != 12 || 4 * ix->n_seeds + 8 >= 0xffffffffull) return SWM_OK;
    // Built on its own only for genomes whose buckets average SWM_CTAB_MIN_MEAN
    // entries or more: its lookup is a random read of a 17 GiB array per
    // selected seed, which costs more than filtering a bucket of a few entries
    // (a 100 Mbp genome averages 1.5 per bucket, a 3.1 Gbp one 44).
    if (!forced && ix->n_seeds < (uint64_t)SWM_CTAB_MIN_MEAN << (2 * ix->k)) return SWM_OK;
    SWM_CUDA(cudaSetDevice(ix->device));
    size_t fr = 0, total = 0;
    if (cudaMemGetInfo(&fr, &total) != cudaSuccess || fr < ctab_bytes(ix) + (8ull << 30)) {
        cudaGetLastError();
        return SWM_OK;
    }
    uint32_t *d_o = nullptr, *d_p = nullptr;
    if (cudaMalloc(&d_o, (SWM_CTAB_KEYS + 1) * 4) != cudaSuccess ||
        cudaMalloc(&d_p, (4 * ix->n_seeds + 8) * 4) != cudaSuccess) {
        cudaFree(d_o);
        cudaGetLastError();
        return SWM_OK;
    }
    const uint64_t nb = 1ull << (2 * ix->k);
    const uint32_t last = (uint32_t)(4 * ix->n_seeds);
    cudaError_t e = cudaMemcpy(d_o + SWM_CTAB_KEYS, &last, 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_p + 4 * ix->n_seeds, 0, 32);
    if (e == cudaSuccess) {
        kb_ctab<<<grid_for(nb * 32, CTAB_WARPS * 32, ix->device, 8), CTAB_WARPS * 32>>>(ix->d_off, nb, ix->d_pos,
                                                                                       ix->d_ls, d_o, d_p);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        cudaFree(d_o);
        cudaFree(d_p);
        swm_set_error("building the candidate table: %s", cudaGetErrorString(e));
        return SWM_ERR_CUDA;
    }
    ix->d_ctab_off = d_o;
    ix->d_ctab_pos = d_p;
    ix->ctab_gen++;
    return SWM_OK;
}

extern "C" int swm_index_candidate_table(swm_index *ix, int enable, uint64_t *bytes) {
    if (!ix) return SWM_ERR_ARG;
    if (enable < 0) { // query only
        std::lock_guard<std::mutex> lk(g_ctab_mu);
        if (bytes) *bytes = ix->d_ctab_off ? ctab_bytes(ix) : 0;
        return SWM_OK;
    }
    if (enable) {
        {
            std::lock_guard<std::mutex> lk(g_ctab_mu);
            ix->ctab_off = 0;
        }
        const int rc = swm_ctab_build(ix, 1);
        if (rc) return rc;
    } else {
        std::lock_guard<std::mutex> lk(g_ctab_mu);
        ix->ctab_off = 1;
        if (ix->d_ctab_off) {
            SWM_CUDA(cudaSetDevice(ix->device));
            cudaDeviceSynchronize(); // no block may still read the table
            cudaFree(ix->d_ctab_off);
            cudaFree(ix->d_ctab_pos);
            ix->d_ctab_off = ix->d_ctab_pos = nullptr;
            ix->ctab_gen++;
        }
    }
    if (bytes) *bytes = ix->d_ctab_off ? ctab_bytes(ix) : 0;
    return SWM_OK;
}

// ------------------------------------------------ allocation-free offsets

// Scratch of swm_hash_offset_noalloc: the scan's block partial sums, one word
// per 2048 counts, so 32768 words cover 4^13 buckets (k <= 13). Every device
// that loads this library holds these 128 KB until the process exits.
#define NOALLOC_PARTIALS 32768
static __device__ __align__(256) uint32_t g_noalloc_partials[NOALLOC_PARTIALS + 64];

#define NOALLOC_MAX_DEVICES 64
static std::mutex g_noalloc_mu;
static uint32_t *g_noalloc_addr[NOALLOC_MAX_DEVICES]; // device address of the array, per device

// For callers that must not allocate device memory: the caller owns both
// arrays, and the scan's partial sums go to the static array above instead of
// a cudaMalloc'ed buffer. Its first call on a device looks up the array's
// device address (cudaGetSymbolAddress) with that device current; make that
// first call before any stream capture. The address is cached for the life of
// the process: a cudaDeviceReset of the primary context would leave it stale,
// so resetting a device the library uses is not supported.
extern "C" int swm_hash_offset_noalloc(const uint32_t *d_hash_count, uint32_t *d_hash_offset, uint32_t k,
                                       void *stream) {
    if (!d_hash_count || !d_hash_offset || k < 1 || k > 16) {
        swm_set_error("swm_hash_offset_noalloc: null array or k out of range (k=%u)", k);
        return SWM_ERR_ARG;
    }
    const uint64_t n = 1ull << (2 * k);
    const uint64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb > NOALLOC_PARTIALS) {
        swm_set_error("swm_hash_offset_noalloc: k=%u needs %llu partial sums, the static scratch holds %d (k <= 13)",
                      k, (unsigned long long)nb, NOALLOC_PARTIALS);
        return SWM_ERR_ARG;
    }
    int dev = 0;
    SWM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        swm_set_error("swm_hash_offset_noalloc: device %d beyond the %d supported", dev, NOALLOC_MAX_DEVICES);
        return SWM_ERR_ARG;
    }
    uint32_t *scratch;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            void *addr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_partials);
            if (e != cudaSuccess || !addr) {
                swm_set_error("swm_hash_offset_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
                return SWM_ERR_CUDA;
            }
            g_noalloc_addr[dev] = (uint32_t *)addr;
        }
        scratch = g_noalloc_addr[dev];
    }
    // every partial the scan reads is written earlier in the same call, so
    // nothing in the scratch has to be cleared between calls
    return swm_exclusive_scan(d_hash_count, d_hash_offset, nullptr, n, n, scratch, nullptr, (cudaStream_t)stream);
}

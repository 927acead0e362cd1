// swm_common.cuh -- shared definitions of the GB300 mapper library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "swmapper.h"

#define SWM_SEED_STEP 4          // fm_define.h:13
#define SWM_PAD_WORDS 64         // zero words after base_2bits (genome end reads base A)
#define SWM_BATCH_POSITIONS 2048 // positions_size, mapper_cpe.c:2129
#define SWM_PER_FETCH 32         // seeds_per_block, mapper_cpe.c:2178
#define SWM_MAX_RUNS_BLOCK 256   // block_size bound, mapper_cpe.c:2265
#define SWM_MAX_SEL 64           // (SWM_MAX_ERRORS + 1) * SWM_SEED_STEP
#define SWM_MAXERROR 10000       // MAXERROR, mapper_cpe.c:17
#define SWM_WIN_WORDS 12         // aligned window words per plane (L + 2e + 32 < 384)
#define SWM_CIGAR_SLOT 128       // CIGAR text bytes kept per verified candidate

// error helpers (implemented in swm_index.cu)
void swm_set_error(const char *fmt, ...);

#define SWM_CUDA(call)                                                                          \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            swm_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));   \
            return SWM_ERR_CUDA;                                                                \
        }                                                                                       \
    } while (0)

// Device-resident index (mapper layout).
struct swm_index {
    int device;
    uint32_t k;
    uint64_t n, n_seeds, n_words2, n_words3, ref_length;
    uint32_t *d_count;     // 4^k
    uint32_t *d_off;       // 4^k + 1 start offsets (mapper_mpe.c:250-255)
    uint32_t *d_pos;       // n_seeds (+8): positions, bucket order (.positions)
    uint16_t *d_ls;        // n_seeds (+8): their 12-bit flank codes (.pos_lseeds)
    uint32_t *d_b2;        // n_words2 + SWM_PAD_WORDS
    uint32_t *d_b3;        // n_words3 + SWM_PAD_WORDS
    // Candidate table (k = 12 only; device-only, derived from the arrays
    // above): the entries of every bucket grouped, for each seed shift t, by
    // the 6 flank bits the filter of shift t compares, so that the entries a
    // read's seed keeps form one contiguous, position-ordered range.
    uint32_t *d_ctab_off;  // SWM_CTAB_KEYS + 1 start offsets into d_ctab_pos
    uint32_t *d_ctab_pos;  // 4 * n_seeds (+8) positions
    uint32_t ctab_gen;     // bumped whenever the table is built or dropped
    int ctab_off;          // the caller dropped the table: no automatic build
    // swm_index_serialize_mappers: when chain is set, every mapper of this
    // index queues its block's kernels behind chain_ev (the completion of the
    // block queued before it, by any mapper) and records chain_ev after them
    int chain;
    cudaEvent_t chain_ev;
};

// Key of the candidate table: seed code << 8 | shift << 6 | flank, where
// flank = rl | rh << 3 are the lo / hi bits of the 3 long-seed bases outside
// the 12-mer (the bits long_seeds_filter compares, mapper_cpe.c:2107-2112).
#define SWM_CTAB_KEYS (1ull << 32)
__host__ __device__ __forceinline__ uint32_t swm_ctab_key(uint32_t seed, uint32_t shift, uint32_t flank) {
    return (seed << 8) | (shift << 6) | flank;
}
// The flank value an index entry with flank code ls offers to shift t.
__host__ __device__ __forceinline__ uint32_t swm_ctab_flank(uint32_t ls, uint32_t t) {
    const uint32_t sh = SWM_SEED_STEP - 1 - t;
    return ((ls >> sh) & 7u) | (((ls >> (6 + sh)) & 7u) << 3);
}
// Build the table (swm_index.cu) when it is missing and the device has room:
// forced = 1 for an explicit request, 0 when a mapper is made (then only for
// indexes averaging SWM_CTAB_MIN_MEAN or more entries per bucket).
#define SWM_CTAB_MIN_MEAN 8
int swm_ctab_build(swm_index *ix, int forced);

// Exclusive scan of n u32 values (n read from *d_n when d_n is not NULL,
// else n_host; clamped to n_cap); out gets n + 1 entries, out[n] = total,
// and *d_total = total when d_total is not NULL. A total of 2^32 - 1 or more
// is written as SWM_SCAN_SATURATED (the offsets are then meaningless). tmp
// needs swm_scan_tmp_words(n_cap) words. Implemented in swm_index.cu.
#define SWM_SCAN_SATURATED 0xffffffffu
uint64_t swm_scan_tmp_words(uint64_t n_cap);
int swm_exclusive_scan(const uint32_t *d_in, uint32_t *d_out, const uint32_t *d_n, uint64_t n_host, uint64_t n_cap,
                       uint32_t *d_tmp, uint32_t *d_total, cudaStream_t st);

__device__ __forceinline__ uint32_t swm_fsr(uint32_t lo, uint32_t hi, uint32_t s) {
    // (hi:lo) >> s for s in [0, 31]; s == 0 gives lo (defined form of the
    // reference's x >> s | y << (32 - s))
    return __funnelshift_r(lo, hi, s);
}

/*
 * swm_oracle.h -- CPU oracle for the SWMapper hot path.
 *
 * TEST INFRASTRUCTURE. This library is the parity checker for the CUDA
 * implementation in swmapper_gb300/. Only tests/, __graft_entry__.smoke() and
 * the cpu_baseline / reference legs of bench.py may load it. The product path
 * never links or calls it.
 *
 * It restates, in plain C, the reference's index build (serial_index.c) and
 * its per-read mapping kernel (mapper_cpe.c), with every undefined behaviour
 * of the reference given one defined meaning (listed in swm_oracle.c). Parity
 * of this restatement is pinned against the reference's own source compiled
 * here (oracle/build_ref.sh -> oracle/_ref/).
 */
#ifndef SWM_ORACLE_H
#define SWM_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Record layout of the reference's output buffers (fm_define.h:17-19,
 * mapper_cpe.c:1468,1481): one record = [cur_read, n | primary<<31, loc * n]
 * at a stride of MAX_CIGAR + 2 words, and its CIGAR bytes at a stride of
 * MAX_CIGAR * CIGAR_LEN bytes. */
#define SWO_MAX_CIGAR 256
#define SWO_RECORD_WORDS (SWO_MAX_CIGAR + 2)
#define SWO_CIGAR_STRIDE (SWO_MAX_CIGAR * 16)

/* Zero words appended after base_2bits / base_3bits so that any window read
 * past the end of the genome reads base A (defined replacement for the
 * reference's read past the end of its buffer, mapper_mpe.c:290). */
#define SWO_PAD_WORDS 64

typedef struct {
    uint32_t k;
    uint64_t n;            /* bases in the concatenated reference            */
    uint64_t n_seeds;      /* S: valid sampled 12-mers                       */
    uint32_t *hash_count;  /* 4^k                                            */
    uint32_t *hash_offset; /* 4^k + 1, END offsets as serial_index writes    */
    uint32_t *positions;   /* S                                              */
    uint16_t *pos_lseeds;  /* S                                              */
    uint32_t *base_2bits;  /* 2*ceil(n/32) (+ pad zeros)                     */
    uint32_t *base_3bits;  /* ceil(n/32) (+ pad zeros)                       */
} swo_index;

/* Build the k-mer index of the concatenated reference sequence `seq`
 * (serial_index.c:157-445 with defined shifts and a guarded final flush).
 * Returns 0 on success. */
int swo_index_build(const uint8_t *seq, uint64_t n, uint32_t k, swo_index *out);
/* The same index built with nthreads host threads (identical output). */
int swo_index_build_mt(const uint8_t *seq, uint64_t n, uint32_t k, uint32_t nthreads, swo_index *out);
void swo_index_free(swo_index *ix);

/* Read-only view used by the mapper (mapper_mpe.c:198-314). */
typedef struct {
    uint32_t k;
    const uint32_t *hash_offset;  /* 4^k + 1 START offsets (rebuilt from counts) */
    const uint32_t *positions;
    const uint16_t *pos_lseeds;
    const uint32_t *base_2bits;   /* must carry SWO_PAD_WORDS zero words at the end */
    uint64_t n_words2;            /* words in base_2bits without the pad          */
    uint64_t ref_length;          /* bytes(base_2bits) * 16 (mapper_mpe.c:288)    */
} swo_mapidx;

typedef struct {
    uint32_t *ref_pos;   /* cap_records * SWO_RECORD_WORDS */
    uint8_t *cigar;      /* cap_records * SWO_CIGAR_STRIDE */
    uint32_t *unmapped;  /* cap_unmapped                   */
    uint64_t cap_records, cap_unmapped;
    uint64_t n_records, n_unmapped;
    int overflow;        /* set when a capacity was too small */
} swo_out;

typedef struct {
    uint64_t items;        /* (read, strand) pairs processed                  */
    uint64_t batches;      /* candidate batches (alignment_rmdup flushes)     */
    uint64_t fetched;      /* positions fetched from buckets                  */
    uint64_t candidates;   /* candidates verified by banded Myers             */
    uint64_t cells;        /* sum over candidates of L * (2e + 1)             */
    uint64_t passed;       /* candidates with error <= e                      */
    uint64_t hamming;      /* passed candidates resolved by the Hamming check */
    uint64_t traceback;    /* passed candidates resolved by traceback         */
    uint64_t emitted;      /* locations written                               */
    uint64_t mapped_reads; /* reads with >= 1 location on either strand       */
    /* how often each defined meaning of a reference UB was used */
    uint64_t ub_shift_out;      /* traceback bit lookup outside bits 0..31     */
    uint64_t ub_walk_stop;      /* traceback stopped below window position 0  */
    uint64_t ub_empty_merge;    /* batch with no candidate left after filter  */
    uint64_t ub_short_seeds;    /* strands with fewer long seeds than e + 1    */
    uint64_t ub_err0_traceback; /* traceback entered with error 0              */
} swo_stats;

/* Map `nreads` reads stored at a fixed stride (mapper_mpe.c:935-960) with
 * error threshold e. Records come out in (read, strand, record) order.
 * nthreads > 1 runs reads on a pthread pool pulling from an atomic counter
 * (the reference's faaw queue, mapper_cpe.c:2620,2644). Returns 0 on success,
 * -1 on bad arguments, -2 on output overflow. */
int swo_map_reads(const swo_mapidx *ix, const char *reads, uint64_t stride,
                  const uint32_t *lens, uint64_t nreads, uint32_t e,
                  uint32_t nthreads, swo_out *out, swo_stats *stats);

/* --- stage-level views, used to test the GPU stages one at a time --- */

/* Read encodings after choose_seed (mapper_cpe.c:1246-1364): w[0..15] the
 * 2-bit packed read, w[16..31] the lo/hi bit planes. */
void swo_encode_read(const char *seq, uint32_t L, uint32_t k, uint32_t w[32]);

/* Banded Myers (mapper_cpe.c:519-660) on an aligned window: wlo/whi hold the
 * window bit planes (bit b of word j = window base 32j+b), rl the window
 * length. Returns the error (10000 when > e) and sets *loc (-1 when none). */
int swo_banded_myers(const uint32_t w2[16], uint32_t L, uint32_t e,
                     const uint32_t *wlo, const uint32_t *whi, uint32_t rl,
                     int *loc);

/* Per-item trace: every candidate verified for one (read, strand), in
 * verification order. Arrays are allocated by the callee (free with
 * swo_trace_free). */
typedef struct {
    uint32_t n;          /* candidates */
    uint32_t *batch;     /* batch index within the item                */
    uint32_t *pos;       /* candidate position (after adjust + dedup)  */
    int32_t *err;        /* Myers error (10000 when above e)           */
    int32_t *loc;        /* Myers location (-1 when none)              */
    uint32_t nbatches;
    uint32_t nsel;       /* selected seeds                              */
    uint32_t sel_start[64], sel_count[64], sel_base[64];
    uint8_t sel_shift[64], sel_rl[64], sel_rh[64];
    uint32_t w[32];
} swo_trace;

int swo_trace_item(const swo_mapidx *ix, const char *seq, uint32_t L,
                   uint32_t e, swo_trace *tr);
void swo_trace_free(swo_trace *tr);

/* FASTA records -> concatenated sequence, following kseq.h:198-237 for FASTA
 * input (name = first word of the header, sequence = line contents without
 * '\n' and one trailing '\r'). Writes `.ref_info` text to ref_info (may be
 * NULL). Caller frees *seq and *info. */
int swo_read_fasta(const char *path, uint8_t **seq, uint64_t *n,
                   char **ref_info, size_t *ref_info_len);

/* Write the seven index files under `prefix` (serial_index.c:73-138). */
int swo_index_write(const swo_index *ix, const char *prefix,
                    const char *ref_info, size_t ref_info_len);

#ifdef __cplusplus
}
#endif
#endif

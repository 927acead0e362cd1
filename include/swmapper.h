/*
 * swmapper.h -- C ABI of the GB300 short-read mapper hot path
 * (libswmapper_gb300.so).
 *
 * Drop-in boundary for SWMapper's index build and mapping kernel:
 *   index build   serial_index.c main (818-865) and construct_hash_index
 *                 (359-445): the same seven files under the same prefix.
 *   index load    mapper_mpe.c load_ref_info (198-314).
 *   mapping       athread_spawn(find_positions, &ref_info_h) / athread_join
 *                 (mapper_mpe.c:972,1056; mapper_cpe.c:2592-2663) with the
 *                 in/out fields of ref_info_t (fm_define.h:22-55).
 * Plain pointers and sizes only; every call returns an int status (0 = OK,
 * < 0 = one of the SWM_ERR_* codes) where the reference returns void.
 */
#ifndef SWMAPPER_H
#define SWMAPPER_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Output layout of the reference (fm_define.h:17-19; mapper_cpe.c:1468,1481). */
#define SWM_MAX_CIGAR 256
#define SWM_RECORD_WORDS (SWM_MAX_CIGAR + 2) /* [cur_read, n | primary<<31, loc * n] */
#define SWM_CIGAR_STRIDE (SWM_MAX_CIGAR * 16) /* [NM, len, text] per location     */
/* Envelope: read length and error threshold (mapper_cpe.c:15,686,2515). */
#define SWM_MAX_READ_LEN 254
#define SWM_MAX_ERRORS 15

enum {
    SWM_OK = 0,
    SWM_ERR_ARG = -1,      /* bad argument or outside the envelope          */
    SWM_ERR_IO = -2,       /* file missing, short or unwritable             */
    SWM_ERR_OOM = -3,      /* device or host allocation failed              */
    SWM_ERR_CUDA = -4,     /* a CUDA call failed (see swm_last_error)       */
    SWM_ERR_OVERFLOW = -5, /* a caller buffer is too small for the results  */
    SWM_ERR_TIMEOUT = -6,  /* a bounded wait gave up                        */
    SWM_ERR_STATE = -7     /* call out of order (e.g. wait without submit)  */
};

/* Text of the last error on this thread (never NULL). */
const char *swm_last_error(void);

/* ------------------------------------------------------------------ index */

typedef struct swm_index swm_index;

typedef struct {
    uint32_t k;          /* seed length (-s)                                */
    uint64_t n;          /* bases in the concatenated reference             */
    uint64_t n_seeds;    /* entries in .positions / .pos_lseeds             */
    uint64_t n_words2;   /* words in .base_2bits                            */
    uint64_t n_words3;   /* words in .base_3bits                            */
    uint64_t ref_length; /* bytes(.base_2bits) * 16, as mapper_mpe.c:288    */
    int device;
} swm_index_info;

/* Replaces serial_index.c main + construct_hash_index (serial_index.c:818-852,
 * 359-445): read the FASTA at fasta_path, build the k-mer index on the GPU and
 * write <prefix>.{ref_info,hash_count,hash_offset,positions,pos_lseeds,
 * base_2bits,base_3bits}. */
int swm_index_build_fasta(const char *fasta_path, const char *prefix, uint32_t k, int device);

/* Build a device-resident index from n bases already concatenated in host
 * memory (the body of construct_hash_index, serial_index.c:396-438). */
int swm_index_build(const uint8_t *seq, uint64_t n, uint32_t k, int device, swm_index **out);

/* As swm_index_build, with the bases already in device memory. */
int swm_index_build_device(const uint8_t *d_seq, uint64_t n, uint32_t k, int device, swm_index **out);

/* Replaces load_ref_info (mapper_mpe.c:198-314): load the index files of
 * `prefix` into device memory (hash_offset rebuilt from .hash_count). */
int swm_index_open(const char *prefix, uint32_t k, int device, swm_index **out);

/* Write the index files of a device-resident index (serial_index.c:73-138);
 * ref_info is the text of <prefix>.ref_info (may be NULL for an empty file). */
int swm_index_save(const swm_index *ix, const char *prefix, const char *ref_info, size_t ref_info_len);

int swm_index_get_info(const swm_index *ix, swm_index_info *info);

/* No counterpart in the reference. The mapper's hash_offset (4^k + 1 start
 * offsets, rebuilt from .hash_count as mapper_mpe.c:250-255 does) computed
 * into device memory the caller already owns, for callers that cannot
 * allocate device memory -- code running where allocation is forbidden or
 * would stall, such as a serving loop inside another framework's memory pool,
 * a stream being captured into a CUDA graph, or a host callback. The call
 * allocates nothing: its scratch is a 128 KB static device array, so k <= 13
 * (larger k returns SWM_ERR_ARG). The first call on a device looks up that
 * array's address and should come before any stream capture; the address is
 * kept for the life of the process, so the device's primary context must not
 * be reset (cudaDeviceReset) while the library is in use. All calls on a
 * device share the array: calls that overlap on the GPU (other streams,
 * other threads) race; serialise them. stream is a cudaStream_t (NULL =
 * default stream); the call is asynchronous on it. */
int swm_hash_offset_noalloc(const uint32_t *d_hash_count, uint32_t *d_hash_offset, uint32_t k, void *stream);

/* No counterpart in the reference (a device-only structure derived from the
 * index arrays; the files are unchanged). For k = 12 the first mapper made on
 * an index whose buckets average 8 or more entries (a genome of about 540 Mbp
 * or more) builds a candidate table when the device has room for it: the
 * entries of every bucket grouped, for each seed shift, by the 6 flank bits
 * long_seeds_filter compares (mapper_cpe.c:2090-2123), behind a directly
 * indexed table of 2^32 + 1 offsets (about 17 GiB, plus 16 bytes per index
 * entry). The candidate stage then reads only the entries the filter keeps
 * instead of every entry of the fetched buckets; results are identical
 * either way. enable = 0 drops the table and keeps it from being built again
 * (mappers fall back to filtering every entry; call it with no block in
 * flight), enable = 1 builds it now if it is missing and fits, whatever the
 * bucket sizes, enable < 0
 * only reports. *bytes (may be NULL) gets the table's device bytes, 0 when
 * there is none. */
int swm_index_candidate_table(swm_index *ix, int enable, uint64_t *bytes);

/* No counterpart in the reference, whose host loop keeps one block running on
 * the CPEs while it reads the next block and writes the previous one
 * (mapper_mpe.c:972-1106). on = 1: the mappers of this index run their
 * blocks' kernels one block at a time, in the order the blocks were queued,
 * while each mapper's input and result copies overlap the kernels of the
 * others -- that double buffering with two mappers. on = 0 (the default):
 * the kernels of different mappers' blocks share the GPU. Results are the
 * same either way. Call it with no block in flight. */
int swm_index_serialize_mappers(swm_index *ix, int on);

/* Copy the index arrays to host memory in file layout (any pointer may be
 * NULL). hash_offset_end gets the END offsets serial_index writes. */
int swm_index_download(const swm_index *ix, uint32_t *hash_count, uint32_t *hash_offset_end, uint32_t *positions,
                       uint16_t *pos_lseeds, uint32_t *base_2bits, uint32_t *base_3bits);

void swm_index_free(swm_index *ix);

/* ---------------------------------------------------------------- mapping */

typedef struct swm_mapper swm_mapper;

/* Inputs of one block of reads: ref_info_t.reads[cur_block],
 * reads_seq_len[cur_block], reads_seq_length, reads_num, errors
 * (fm_define.h:30-40; filled at mapper_mpe.c:886-904,966-967). */
typedef struct {
    const char *reads;             /* reads_num reads at a fixed stride           */
    const uint32_t *reads_len;     /* length of each read (<= SWM_MAX_READ_LEN)    */
    uint64_t stride;               /* reads_seq_length (-l)                        */
    uint64_t reads_num;            /* reads in this block                          */
    uint32_t errors;               /* -e                                           */
    const uint8_t *errors_per_read;/* optional per-read threshold (NULL = errors). */
} swm_batch;

/* Outputs: ref_info_t.ref_pos_buffer / cigar_buffer / cigar_num and the
 * counters *cigar_ind / *unmap_ind (fm_define.h:42-49). Records are written in
 * (read, strand, record) order; cur_read = 2 * read + strand as in
 * mapper_cpe.c:2628. */
typedef struct {
    uint32_t *ref_pos_buffer;   /* records_cap * SWM_RECORD_WORDS words          */
    uint8_t *cigar_buffer;      /* records_cap * SWM_CIGAR_STRIDE bytes (may be NULL) */
    uint32_t *unmapped;         /* unmapped_cap cur_read ids (2 * read + 1)      */
    uint64_t records_cap, unmapped_cap;
    uint64_t n_records;         /* *cigar_ind                                    */
    uint64_t n_unmapped;        /* *unmap_ind                                    */
} swm_result;

/* Work counters of the last completed block. */
typedef struct {
    uint64_t reads, items;      /* reads and (read, strand) items               */
    uint64_t chunks;            /* bucket fetches of <= 32 positions            */
    uint64_t batches;           /* candidate batches (alignment_rmdup flushes)  */
    uint64_t fetched;           /* positions fetched                            */
    uint64_t candidates;        /* windows verified by banded Myers              */
    uint64_t cells;             /* sum over candidates of L * (2e + 1)           */
    uint64_t passed;            /* candidates with error <= e                    */
    uint64_t records;           /* output records                                */
    uint64_t locations;         /* output locations                              */
    uint64_t mapped_reads;      /* reads with >= 1 location on either strand     */
    uint64_t retries;           /* block re-runs after growing a work buffer     */
    uint64_t h2d_bytes;         /* host -> device bytes of the block (0 when resident) */
    uint64_t d2h_bytes;         /* device -> host bytes of the block's results   */
    uint64_t myers_steps;       /* read bases run through the Myers recurrence,
                                   summed over candidates and both passes       */
    uint64_t kept;              /* positions the flank filter kept, before each
                                   batch's merge and dedup                       */
} swm_map_stats;

/* Create a mapping context on the index's device with its own CUDA stream and
 * work buffers for blocks of up to max_reads reads (mapper_mpe.c:727 uses
 * 10,000). */
int swm_mapper_create(swm_index *ix, uint64_t max_reads, swm_mapper **out);

/* find_positions over one block, synchronously: copy the reads in, map both
 * strands of every read, copy the records out. */
int swm_map_batch(swm_mapper *m, const swm_batch *b, swm_result *r);

/* Asynchronous pair, the analog of athread_spawn / athread_join
 * (mapper_mpe.c:972,1036): submit copies the inputs to pinned staging and
 * queues all the work on the mapper's stream; wait blocks until it is done
 * and fills r. One block may be in flight per mapper. */
int swm_map_submit(swm_mapper *m, const swm_batch *b);
int swm_map_wait(swm_mapper *m, swm_result *r);

/* Device-resident variant (no host copies): d_reads / d_lens / d_errors are
 * device pointers. Results stay on the device until swm_map_fetch. */
int swm_map_device(swm_mapper *m, const char *d_reads, const uint32_t *d_lens, uint64_t stride,
                   uint64_t reads_num, uint32_t errors, const uint8_t *d_errors);
int swm_map_fetch(swm_mapper *m, swm_result *r);

/* Asynchronous form of swm_map_device (no reference counterpart: the
 * reference's reads are always host buffers): submit queues the block on the
 * mapper's stream and returns; wait blocks until it is mapped (results stay
 * on the device until swm_map_fetch). The device inputs must stay valid until
 * wait returns. Two mappers used in turn keep the GPU busy while the host
 * handles the other's results. */
int swm_map_device_submit(swm_mapper *m, const char *d_reads, const uint32_t *d_lens, uint64_t stride,
                          uint64_t reads_num, uint32_t errors, const uint8_t *d_errors);
int swm_map_device_wait(swm_mapper *m);

/* Packed results: the same records without the reference's fixed strides
 * (record q's words follow record q - 1's; its CIGAR bytes likewise), for
 * callers that do not need the ref_info_t layout. */
typedef struct {
    uint32_t *words;            /* [cur_read, n | primary<<31, loc * n] per record */
    uint8_t *cigar;             /* [NM, len, text] per location, records back to back */
    uint32_t *record_cigar_len; /* CIGAR bytes of each record                      */
    uint32_t *unmapped;         /* cur_read ids (2 * read + 1) of unmapped reads   */
    uint64_t words_cap, cigar_cap, records_cap, unmapped_cap;
    uint64_t n_words, n_cigar, n_records, n_unmapped;
} swm_packed_result;

int swm_map_fetch_packed(swm_mapper *m, swm_packed_result *r);

/* swm_map_wait with packed results. */
int swm_map_wait_packed(swm_mapper *m, swm_packed_result *r);

int swm_mapper_stats(const swm_mapper *m, swm_map_stats *s);

/* Per-stage device time of the last block in milliseconds (CUDA events on the
 * mapper's stream); names are "seed", "plan", "candidates", "compact",
 * "verify", "traceback", "records", "total". Returns SWM_ERR_ARG for an
 * unknown name. */
int swm_mapper_stage_ms(const swm_mapper *m, const char *stage, float *ms);

/* Settings of a mapper that change its speed, never its results (no
 * reference counterpart; the autotuner sets them per read-length bucket). */
typedef struct {
    uint32_t verify_head_bases; /* two-pass verification: bases of every candidate
                                   the first pass runs before its exact stop test,
                                   32 or 64                                       */
    uint32_t verify_chunk;      /* 0: two-pass verification; 8 or 16 (default 16):
                                   streaming verification, each lane running its
                                   own candidate and testing the stop bound every
                                   8 / 16 bases, refilled from the queue as
                                   candidates stop (verify_head_bases is then
                                   ignored)                                       */
    uint32_t verify_pairs;      /* 1 (with verify_chunk 16): two candidates per lane
                                   in 15-bit halves of each word, for blocks whose
                                   thresholds are all <= 7 (others run with one per
                                   lane); 0: one per lane                         */
} swm_tuning;

/* Apply *set (may be NULL) and report the current settings in *get (may be
 * NULL); SWM_ERR_ARG for a value outside the lists above, SWM_ERR_STATE while a
 * block is in flight. */
int swm_mapper_tuning(swm_mapper *m, const swm_tuning *set, swm_tuning *get);

/* Kernel launches queued for the last block. */
uint64_t swm_mapper_launches(const swm_mapper *m);

/* The CUDA stream of the mapper (a cudaStream_t), for callers that order
 * their own work around it. */
void *swm_mapper_stream(const swm_mapper *m);

/* Verified candidates of the last block in verification order: item
 * (= 2 * read + strand), window-start candidate position, Myers error and
 * location. For tests; n gets the total even when cap is smaller. */
int swm_mapper_debug_candidates(const swm_mapper *m, uint32_t *item, uint32_t *pos, int32_t *err, int32_t *loc,
                                uint64_t cap, uint64_t *n);

/* Read encodings of the last block, 32 words per item: [0..15] the bit
 * planes of the 2-bit packed read that banded Myers scans (lo, hi per 32
 * bases), [16..31] the planes the Hamming check uses (reads_2bits[16..31] of
 * get_seed_from_reads, mapper_cpe.c:1246-1364). For tests. */
int swm_mapper_debug_read_words(const swm_mapper *m, uint32_t *words, uint64_t cap_items);

void swm_mapper_free(swm_mapper *m);

/* ---------------------------------------------------------------- serving */

/* Request loop over a resident index. Replaces the reference's block loop
 * with spawn / join double buffering (mapper_mpe.c:945-1106), which maps one
 * fixed block at a time: a server takes requests of any size as they arrive
 * and an engine thread coalesces the waiting ones into the next block (up to
 * block_reads reads) whenever a block slot is free, so requests that arrive
 * while other blocks are on the GPU are admitted as slots free up and their
 * blocks overlap on the device. A block slot is one mapper (its own CUDA
 * stream and work buffers); slots are made on demand, each only when the
 * device reports the memory for it free at that moment and the caller's limit
 * allows it. Results are the same as mapping each request alone. */
typedef struct swm_server swm_server;

typedef struct {
    uint64_t block_reads;       /* reads per block slot (the coalescing limit)   */
    uint32_t max_slots;         /* block slots at most (blocks in flight)        */
    uint64_t stride;            /* read stride inside the server (>= the longest
                                   read; reads are copied to it at submission)  */
    uint64_t max_queued_reads;  /* reads waiting for a slot at most (>= block_reads);
                                   a request beyond it is refused               */
    uint64_t device_mem_limit;  /* device bytes the slots may hold (0 = no limit
                                   beyond the device's free memory)             */
    uint64_t device_mem_reserve;/* device bytes to leave free when making a slot */
} swm_serve_config;

typedef struct {
    uint64_t slots;                /* block slots made                            */
    uint64_t slot_bytes;           /* device memory of one slot (measured)        */
    uint64_t blocks;               /* blocks launched                             */
    uint64_t max_blocks_in_flight; /* most blocks on the GPU at once              */
    uint64_t requests_admitted, requests_done, reads_done;
    uint64_t refused_memory;       /* submissions refused: no slot fits (SWM_ERR_OOM) */
    uint64_t refused_queue;        /* submissions refused: queue full (SWM_ERR_STATE) */
    uint64_t queued_reads;         /* reads waiting for a slot now                */
} swm_serve_counters;

typedef struct {
    uint64_t id;
    uint64_t reads;        /* reads of the request                          */
    uint64_t block_reads;  /* reads of the block it was mapped in           */
    double latency_ms;     /* submission to results ready (host clock)      */
} swm_request_info;

/* Start a server on a resident index. Makes the first block slot (which
 * measures a slot's device memory); SWM_ERR_OOM when the device cannot hold
 * one. The index must outlive the server. */
int swm_serve_open(swm_index *ix, const swm_serve_config *cfg, swm_server **out);

/* Admit one request of 1..block_reads reads (host memory; copied before the
 * call returns) and return its id. Refused with SWM_ERR_OOM when no block slot
 * can ever be made within the memory allowed, with SWM_ERR_STATE when the
 * reads already waiting plus these would exceed max_queued_reads (or the
 * server is closing), with SWM_ERR_ARG for reads outside the envelope. */
int swm_serve_submit(swm_server *s, const swm_batch *b, uint64_t *id);

/* The next finished request, waiting up to timeout_ms (< 0: no limit; 0: do
 * not wait): its id, its packed records with read ids relative to the request
 * (cur_read = 2 * read + strand), and optionally info. SWM_ERR_TIMEOUT when
 * none finished in time; SWM_ERR_OVERFLOW when r's buffers are too small (the
 * n_* fields hold the sizes needed and the result stays first in line); a
 * request whose block failed returns that block's status once. r may be NULL
 * to drop the records. */
int swm_serve_poll(swm_server *s, int timeout_ms, uint64_t *id, swm_packed_result *r, swm_request_info *info);

int swm_serve_stats(swm_server *s, swm_serve_counters *out);

/* Stop admitting, finish the requests already admitted, free the slots and
 * any results not polled. */
int swm_serve_close(swm_server *s);

/* Rate at which the device serves independent random 32-byte reads from a
 * buffer of the given size (>= 1 MiB; larger than L2 for DRAM, smaller for
 * L2), in sectors per second: the ceiling of the gather kernels (seed
 * lookups, candidate gathers), which read scattered sectors rather than
 * streams. No reference counterpart: measurement of this device, used for
 * the roofline the benchmark reports. Allocates and frees the buffer. */
int swm_probe_random_reads(int device, uint64_t bytes, double *sectors_per_s);

#ifdef __cplusplus
}
#endif
#endif

/* mapper_driver.c -- drives the reference's own get_positions()
 * (mapper_cpe.c:2500-2590, compiled on the host by oracle/build_ref.sh) over a
 * batch of reads, the way find_positions (mapper_cpe.c:2592-2663) does on the
 * CPEs: a shared counter hands out one read at a time to each worker, and the
 * output slots come from fetch-and-add counters. TEST INFRASTRUCTURE: used by
 * the pinning tests and by the reference leg of bench.py. */
#include <pthread.h>
#include <stdlib.h>
#include "mapper_prelude.h"

void get_positions(ref_info_t *ref_info_s, char *reads_s, sindex_t *reads_l, sindex_t reads_per_core);

typedef struct {
    ref_info_t proto;
    const char *reads;
    uint64_t stride, nreads;
    const uint32_t *lens;
    uint64_t next;
} swref_job;

static void *swref_worker(void *arg) {
    swref_job *jb = arg;
    ref_info_t ri = jb->proto; /* private copy per worker, like the CPE's LDM copy (2602-2604) */
    char buf[READ_LEN + 16];
    sindex_t len;
    for (;;) {
        uint64_t r = __atomic_fetch_add(&jb->next, 1, __ATOMIC_RELAXED);
        if (r >= jb->nreads) break;
        len = jb->lens[r];
        memcpy(buf, jb->reads + r * jb->stride, len);
        ri.cur_read = 2 * r;
        get_positions(&ri, buf, &len, 1);
    }
    return NULL;
}

/* Returns 0 on success, -1 on bad arguments. Output layout is the reference's
 * (records at stride MAX_CIGAR + 2 words, CIGAR bytes at 4096 bytes). */
int swref_map(const uint32_t *hash_offset, const uint32_t *positions, const uint16_t *lseeds,
              const uint32_t *base_2bits, uint64_t ref_length, uint32_t k, uint32_t e,
              const char *reads, uint64_t stride, const uint32_t *lens, uint64_t nreads,
              int nthreads, uint32_t *ref_pos, uint8_t *cigar, uint32_t *unmapped,
              uint64_t *n_records, uint64_t *n_unmapped) {
    if (stride > READ_LEN || nthreads < 1) return -1;
    for (uint64_t r = 0; r < nreads; r++)
        if (lens[r] > 254) return -1;
    index_t cind = 0, uind = 0;
    swref_job jb;
    memset(&jb, 0, sizeof jb);
    jb.proto.hash_offset = (sindex_t *)hash_offset;
    jb.proto.hash_positions = (sindex_t *)positions;
    jb.proto.pos_lseeds = (half_word_t *)lseeds;
    jb.proto.base_2bits = (sindex_t *)base_2bits;
    jb.proto.reads_seq_length = stride;
    jb.proto.seed_length = k;
    jb.proto.errors = e;
    jb.proto.ref_length = ref_length;
    jb.proto.cigars_per_read = 1024;
    jb.proto.cigar_avg_len = 16;
    jb.proto.reads_num = nreads;
    jb.proto.cigar_buffer[0] = (char *)cigar;
    jb.proto.cigar_num[0] = unmapped;
    jb.proto.ref_pos_buffer[0] = ref_pos;
    jb.proto.cigar_ind = &cind;
    jb.proto.unmap_ind = &uind;
    jb.proto.cur_block = 0;
    jb.reads = reads;
    jb.stride = stride;
    jb.nreads = nreads;
    jb.lens = lens;
    if (nthreads == 1) {
        swref_worker(&jb);
    } else {
        pthread_t *th = malloc(sizeof(pthread_t) * (size_t)nthreads);
        for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, swref_worker, &jb);
        for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
        free(th);
    }
    *n_records = cind;
    *n_unmapped = uind;
    return 0;
}

/*
 * swm_mapper -- drop-in for SWMapper's mapper (mapper_mpe.c:697-1125):
 *
 *     swm_mapper -l<max read length> -e <errors> -p <index prefix> [-s<k>]
 *                (-i<reads.fa|fq> | -f<list of read files>) -o<output prefix> [-h]
 *
 * maps every read on the GPU (both strands, k-mer index of swm_index) and
 * writes SAM to <output prefix>.sam.gz (<output prefix>_0000.sam.gz with -f,
 * the first file of the list, as rank 0 of the reference does); without
 * zlib at build time the output is uncompressed <prefix>.sam. Reads are taken
 * in blocks; two mappers alternate so one block maps while the previous
 * one's SAM is written (the reference's cur_block / pre_block double
 * buffering). Exit status 0 on success, 1 on an error.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "swm_sam.h"
#include "swmapper.h"

#ifdef HAVE_ZLIB
#include <zlib.h>
typedef gzFile out_file;
static out_file out_open(const char *p) { return gzopen(p, "w1"); }
static int out_write(out_file f, const char *s, size_t n) { return n == 0 || gzwrite(f, s, (unsigned)n) == (int)n; }
static void out_close(out_file f) { gzclose(f); }
#define OUT_EXT ".sam.gz"
#else
typedef FILE *out_file;
static out_file out_open(const char *p) { return fopen(p, "w"); }
static int out_write(out_file f, const char *s, size_t n) { return fwrite(s, 1, n, f) == n; }
static void out_close(out_file f) { fclose(f); }
#define OUT_EXT ".sam"
#endif

#define NAME_STRIDE 128

static void help(void) {
    printf("-l\tmax length (less than 200)\n");
    printf("-o\toutput file prefix\n");
    printf("-e\terror size\n");
    printf("-p\tindex prefix\n");
    printf("-s\t[opt, default:12] seed length\n");
    printf("-i\t[opt, default:12] single data input\n");
    exit(0);
}

static int die(const char *what) {
    fprintf(stderr, "swm_mapper: %s: %s\n", what, swm_last_error());
    return 1;
}

typedef struct {
    swm_read_block b;
    swm_packed_result r;
} slot_t;

static int slot_init(slot_t *s, uint64_t cap, uint64_t stride) {
    memset(s, 0, sizeof *s);
    s->b.name_stride = NAME_STRIDE;
    s->b.seq_stride = stride;
    s->b.n_cap = cap;
    s->b.names = (char *)malloc(cap * NAME_STRIDE);
    s->b.name_len = (uint32_t *)malloc(cap * 4);
    s->b.seqs = (char *)malloc(cap * stride);
    s->b.quals = (char *)malloc(cap * stride);
    s->b.seq_len = (uint32_t *)malloc(cap * 4);
    s->r.words_cap = cap * 16;
    s->r.cigar_cap = cap * 64;
    s->r.records_cap = cap * 4;
    s->r.unmapped_cap = cap;
    s->r.words = (uint32_t *)malloc(s->r.words_cap * 4);
    s->r.cigar = (uint8_t *)malloc(s->r.cigar_cap);
    s->r.record_cigar_len = NULL;
    s->r.unmapped = (uint32_t *)malloc(cap * 4);
    return (s->b.names && s->b.name_len && s->b.seqs && s->b.quals && s->b.seq_len && s->r.words && s->r.cigar &&
            s->r.unmapped) ? 0 : -1;
}

static void slot_free(slot_t *s) {
    free(s->b.names); free(s->b.name_len); free(s->b.seqs); free(s->b.quals); free(s->b.seq_len);
    free(s->r.words); free(s->r.cigar); free(s->r.unmapped);
}

/* wait for the slot's block and fetch its packed results, growing the
 * buffers when they are too small */
static int collect(swm_mapper *m, slot_t *s) {
    int rc = swm_map_wait_packed(m, &s->r);
    while (rc == SWM_ERR_OVERFLOW) {
        if (s->r.n_words > s->r.words_cap) {
            s->r.words_cap = s->r.n_words;
            free(s->r.words);
            s->r.words = (uint32_t *)malloc(s->r.words_cap * 4);
        }
        if (s->r.n_cigar > s->r.cigar_cap) {
            s->r.cigar_cap = s->r.n_cigar;
            free(s->r.cigar);
            s->r.cigar = (uint8_t *)malloc(s->r.cigar_cap);
        }
        if (s->r.n_records > s->r.records_cap) s->r.records_cap = s->r.n_records;
        if (!s->r.words || !s->r.cigar) return SWM_ERR_OOM;
        rc = swm_map_fetch_packed(m, &s->r);
    }
    return rc;
}

static int write_sam(out_file out, const swm_refs *refs, slot_t *s, char **buf, size_t *cap) {
    size_t n = 0;
    int rc = swm_sam_block(refs, &s->b, &s->r, *buf, *cap, &n);
    if (rc == SWM_ERR_OVERFLOW) {
        free(*buf);
        *cap = n + n / 4;
        *buf = (char *)malloc(*cap);
        if (!*buf) return SWM_ERR_OOM;
        rc = swm_sam_block(refs, &s->b, &s->r, *buf, *cap, &n);
    }
    if (rc) return rc;
    return out_write(out, *buf, n) ? SWM_OK : SWM_ERR_IO;
}

int main(int argc, char *argv[]) {
    const char *prefix = NULL, *reads_path = NULL, *list = NULL, *out_prefix = NULL;
    unsigned k = 12, errors = 4;
    uint64_t stride = 120; /* reads_seq_length default, mapper_mpe.c:725 */
    int opt;
    while ((opt = getopt(argc, argv, "h::l::s::p:i::o::e:f::")) != -1) {
        switch (opt) {
        case 'l': if (optarg) stride = (uint64_t)atoi(optarg); break;
        case 'p': prefix = optarg; break;
        case 's': if (optarg) k = (unsigned)atoi(optarg); break;
        case 'h': help(); break;
        case 'o': out_prefix = optarg; break;
        case 'e': errors = (unsigned)atoi(optarg); break;
        case 'i': reads_path = optarg; break;
        case 'f': list = optarg; break;
        default: return 1;
        }
    }
    if (!prefix || !out_prefix || (!reads_path && !list)) {
        fprintf(stderr, "swm_mapper: -p <prefix>, -o<prefix> and -i<reads> or -f<list> are required\n");
        return 1;
    }
    char path[4096], result[4096];
    if (list) { /* the first file of the list: rank 0 of the reference (mapper_mpe.c:852-859) */
        FILE *lf = fopen(list, "r");
        if (!lf || fscanf(lf, "%4095s", path) != 1) {
            fprintf(stderr, "swm_mapper: cannot read the list %s\n", list);
            return 1;
        }
        fclose(lf);
        reads_path = path;
        snprintf(result, sizeof result, "%s_%04d" OUT_EXT, out_prefix, 0);
    } else {
        snprintf(result, sizeof result, "%s" OUT_EXT, out_prefix);
    }
    const char *dev = getenv("SWM_DEVICE");
    const char *blk = getenv("SWM_BLOCK_READS");
    const uint64_t cap = blk ? (uint64_t)atoll(blk) : 262144;
    swm_index *ix = NULL;
    if (swm_index_open(prefix, k, dev ? atoi(dev) : 0, &ix)) return die("index");
    swm_refs refs;
    if (swm_refs_load(prefix, &refs)) {
        fprintf(stderr, "swm_mapper: cannot read %s.ref_info\n", prefix);
        return 1;
    }
    swm_fastx *fx = NULL;
    if (swm_fastx_open(reads_path, &fx)) {
        fprintf(stderr, "swm_mapper: cannot open %s\n", reads_path);
        return 1;
    }
    out_file out = out_open(result);
    if (!out) {
        fprintf(stderr, "swm_mapper: cannot write %s\n", result);
        return 1;
    }
    swm_mapper *mp[2] = {NULL, NULL};
    slot_t sl[2];
    if (swm_mapper_create(ix, cap, &mp[0]) || swm_mapper_create(ix, cap, &mp[1])) return die("mapper");
    if (slot_init(&sl[0], cap, stride) || slot_init(&sl[1], cap, stride)) {
        fprintf(stderr, "swm_mapper: out of host memory\n");
        return 1;
    }
    size_t bcap = 1 << 20, n = 0;
    char *buf = (char *)malloc(bcap);
    int rc = buf ? swm_sam_header(&refs, buf, bcap, &n) : SWM_ERR_OOM;
    if (!rc && !out_write(out, buf, n)) rc = SWM_ERR_IO;
    int pending[2] = {0, 0};
    uint64_t total = 0, mapped = 0;
    for (int cur = 0; !rc;) {
        /* read and submit the next block into slot cur */
        rc = swm_fastx_read_block(fx, &sl[cur].b);
        if (rc) {
            fprintf(stderr, "swm_mapper: %s: %s\n", reads_path, rc == SWM_ERR_ARG ? "a read is longer than -l" :
                                                               "malformed record");
            break;
        }
        if (sl[cur].b.n) {
            swm_batch bt = {sl[cur].b.seqs, sl[cur].b.seq_len, stride, sl[cur].b.n, errors, NULL};
            if ((rc = swm_map_submit(mp[cur], &bt))) { die("map"); break; }
            pending[cur] = 1;
        }
        /* finish the other slot's block while this one maps */
        const int oth = cur ^ 1;
        if (pending[oth]) {
            if ((rc = collect(mp[oth], &sl[oth]))) { die("map"); break; }
            pending[oth] = 0;
            total += sl[oth].b.n;
            mapped += sl[oth].b.n - sl[oth].r.n_unmapped;
            if ((rc = write_sam(out, &refs, &sl[oth], &buf, &bcap))) break;
        }
        if (!sl[cur].b.n) break;
        cur = oth;
    }
    for (int s = 0; s < 2 && !rc; s++) /* a block still mapping when the input ended */
        if (pending[s]) {
            if ((rc = collect(mp[s], &sl[s]))) { die("map"); break; }
            total += sl[s].b.n;
            mapped += sl[s].b.n - sl[s].r.n_unmapped;
            rc = write_sam(out, &refs, &sl[s], &buf, &bcap);
        }
    out_close(out);
    fprintf(stderr, "swm_mapper: %llu reads, %llu mapped -> %s\n", (unsigned long long)total,
            (unsigned long long)mapped, result);
    free(buf);
    slot_free(&sl[0]);
    slot_free(&sl[1]);
    swm_mapper_free(mp[0]);
    swm_mapper_free(mp[1]);
    swm_fastx_close(fx);
    swm_refs_free(&refs);
    swm_index_free(ix);
    return rc ? 1 : 0;
}

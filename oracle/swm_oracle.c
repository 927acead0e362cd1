/*
 * swm_oracle.c -- CPU oracle for the SWMapper hot path (TEST INFRASTRUCTURE).
 *
 * Restates the reference's k-mer index build (serial_index.c:157-445) and its
 * per-read mapping kernel (mapper_cpe.c:229-2590) step for step, in plain C.
 * The GPU implementation in swmapper_gb300/csrc must agree with this file bit
 * for bit. Parity of this file is pinned against the reference source itself,
 * compiled here by oracle/build_ref.sh (tests/test_oracle_golden.py).
 *
 * Defined meanings for the reference's undefined behaviour (each one is also
 * applied to the reference build used for pinning, see build_ref.sh):
 *  D1  x >> s | y << (32 - s) at s == 0 is taken as x (funnel shift), at
 *      serial_index.c:286,298-299,307-308,321 and mapper_cpe.c:262-263,
 *      1565-1566,2474,2477.
 *  D2  The final partial-word flush (serial_index.c:423-426) only runs when
 *      n is not a multiple of 32 (16 for the 2-bit seed words).
 *  D3  Seed slots beyond floor(L/15) long seeds read bucket count 0
 *      (mapper_cpe.c:2195-2196 reads stale hash_count there).
 *  D4  A batch whose filter leaves nothing yields no candidates
 *      (block_heap_sort reads an unset pos_heap[1], mapper_cpe.c:2074).
 *  D5  Genome words past the end of base_2bits read as zero (base A).
 *  D6  Traceback bit lookups outside bits 0..31 read 0, and the walk stops
 *      once it would compare a window position below 0
 *      (mapper_cpe.c:380-466 shift by negative / >= 32 and index below the
 *      window there).
 *  D7  Buffers are large enough for every read length up to 254 and every
 *      e up to 15 (the reference overflows its 16-word window slot for
 *      L + 2e > 224, mapper_cpe.c:1600,1613).
 */
#include "swm_oracle.h"

#include <ctype.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define SEED_STEP 4
#define MAXERROR 10000
#define BATCH_POSITIONS 2048   /* positions_size, mapper_cpe.c:2129 */
#define PER_FETCH 32           /* seeds_per_block, mapper_cpe.c:2178 */
#define MAX_RUNS_BLOCK 256     /* block_size limit, mapper_cpe.c:2265 */
#define MAX_READ_LEN 254
#define MAX_E 15

/* D1: funnel shift right of the pair (lo, hi) by s in [0, 31]. */
static inline uint32_t fsr(uint32_t lo, uint32_t hi, uint32_t s) {
    return s ? (lo >> s) | (hi << (32 - s)) : lo;
}

/* ======================================================================
 * Index build: serial_index.c:157-445
 * ====================================================================== */

static inline int base_code(uint8_t ch) {
    switch (toupper(ch)) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    default: return -1; /* N and every other byte: serial_index.c:203-214 */
    }
}

int swo_index_build(const uint8_t *seq, uint64_t n, uint32_t k, swo_index *ix) {
    memset(ix, 0, sizeof(*ix));
    if (k < 1 || k > 14 || n >= 0xffffffffull) return -1;
    const uint64_t nb = 1ull << (2 * k);
    const uint64_t W = (n + 31) / 32;
    ix->k = k;
    ix->n = n;
    ix->hash_count = calloc(nb, 4);
    ix->hash_offset = calloc(nb + 1, 4);
    ix->base_2bits = calloc(2 * W + SWO_PAD_WORDS, 4);
    ix->base_3bits = calloc(W + SWO_PAD_WORDS, 4);
    uint32_t *seeds2 = calloc((n + 15) / 16 + SWO_PAD_WORDS, 4);
    if (!ix->hash_count || !ix->hash_offset || !ix->base_2bits || !ix->base_3bits || !seeds2) {
        free(seeds2);
        swo_index_free(ix);
        return -3;
    }
    /* get_seed (serial_index.c:157-245): bit planes, N mask, 2-bit seed words
     * and the rolling k-mer; a k-mer is counted when its start is a multiple
     * of SEED_STEP (chromo_hash_index, serial_index.c:253-269). State carries
     * across FASTA records, so the concatenation is indexed as one stream. */
    const uint64_t kmask = (k == 32) ? ~0ull : ((1ull << (2 * k)) - 1);
    uint64_t seed = 0, run = 0, S = 0;
    for (uint64_t p = 0; p < n; p++) {
        int c = base_code(seq[p]);
        const uint64_t w = p / 32, b = p % 32;
        if (c < 0) {
            ix->base_3bits[w] |= 1u << b;
            run = 0;
            seed = 0;
            continue;
        }
        ix->base_2bits[2 * w] |= (uint32_t)(c & 1) << b;
        ix->base_2bits[2 * w + 1] |= (uint32_t)(c >> 1) << b;
        seeds2[p / 16] |= (uint32_t)c << (2 * (p % 16));
        seed = ((seed >> 2) | ((uint64_t)c << (2 * (k - 1)))) & kmask;
        if (run < k) run++;
        if (run == k && ((p + 1 - k) % SEED_STEP) == 0) {
            ix->hash_count[seed]++;
            S++;
        }
    }
    ix->n_seeds = S;
    ix->positions = malloc((S + 8) * 4);
    ix->pos_lseeds = malloc((S + 8) * 2);
    if (!ix->positions || !ix->pos_lseeds) {
        free(seeds2);
        swo_index_free(ix);
        return -3;
    }
    /* store_positions (serial_index.c:332-356): start offsets, then a stable
     * scatter of every valid sampled position in ascending order. */
    uint32_t *cursor = ix->hash_offset;
    cursor[0] = 0;
    for (uint64_t i = 0; i < nb; i++) cursor[i + 1] = cursor[i] + ix->hash_count[i];
    const uint32_t smask = (uint32_t)kmask;
    const uint32_t nmask = (k >= 32) ? ~0u : ((1u << k) - 1);
    const uint32_t res = SEED_STEP - 1, rmask = (1u << res) - 1;
    for (uint64_t i = 0; n >= k && i < n - k + 1; i += SEED_STEP) {
        /* get_seed_from_enc_bits, serial_index.c:280-331 */
        uint32_t sd = fsr(seeds2[i / 16], seeds2[i / 16 + 1], (uint32_t)(i % 16) * 2) & smask;
        uint32_t nf = fsr(ix->base_3bits[i / 32], ix->base_3bits[i / 32 + 1], (uint32_t)(i % 32)) & nmask;
        if (nf) continue;
        uint64_t sp = (i >= res) ? i - res : 0;
        uint32_t fl = fsr(ix->base_2bits[(sp / 32) * 2], ix->base_2bits[(sp / 32 + 1) * 2], sp % 32) & rmask;
        uint32_t fh = fsr(ix->base_2bits[(sp / 32) * 2 + 1], ix->base_2bits[(sp / 32 + 1) * 2 + 1], sp % 32) & rmask;
        sp = i + k;
        uint32_t bl = fsr(ix->base_2bits[(sp / 32) * 2], ix->base_2bits[(sp / 32 + 1) * 2], sp % 32) & rmask;
        uint32_t bh = fsr(ix->base_2bits[(sp / 32) * 2 + 1], ix->base_2bits[(sp / 32 + 1) * 2 + 1], sp % 32) & rmask;
        fl |= bl << res;
        fh |= bh << res;
        uint16_t lseed = (uint16_t)(fl | (fh << (res * 2)));
        uint32_t slot = cursor[sd]++;
        ix->positions[slot] = (uint32_t)i;
        ix->pos_lseeds[slot] = lseed;
    }
    /* cursor (== hash_offset) now holds END offsets, the way the reference
     * writes its .hash_offset file (serial_index.c:105-110). */
    free(seeds2);
    return 0;
}

/* The same index with nthreads host threads, identical output (the serial
 * build above is the restatement; this one only splits its loops). Phase 1:
 * thread t encodes the 32-base words of its slice of the genome and counts
 * the k-mers starting there in its own histogram (a sampled start i is
 * counted when bases i .. i + k - 1 are all A/C/G/T, which is the serial
 * loop's run == k test). Phase 2: start offsets, and each thread's first slot
 * in every bucket = the bucket's start + the counts of the slices before it.
 * Phase 3: each thread scatters its slice's positions in ascending order, so
 * every bucket holds its positions in ascending order, as the serial scatter
 * leaves them (serial_index.c:343-352). */
typedef struct {
    const uint8_t *seq;
    uint64_t n, w0, w1;
    uint32_t k, phase;
    uint32_t *hist;
    uint32_t *seeds2;
    swo_index *ix;
} ibuild_t;

static void *ibuild_worker(void *arg) {
    ibuild_t *a = (ibuild_t *)arg;
    swo_index *ix = a->ix;
    const uint32_t k = a->k;
    const uint64_t n = a->n;
    const uint32_t smask = (k >= 16) ? ~0u : ((1u << (2 * k)) - 1);
    const uint64_t i0 = a->w0 * 32, i1 = a->w1 * 32 < n ? a->w1 * 32 : n;
    if (a->phase == 1) {
        for (uint64_t p = i0; p < i1; p++) {
            const int c = base_code(a->seq[p]);
            const uint64_t w = p / 32, b = p % 32;
            if (c < 0) {
                ix->base_3bits[w] |= 1u << b;
                continue;
            }
            ix->base_2bits[2 * w] |= (uint32_t)(c & 1) << b;
            ix->base_2bits[2 * w + 1] |= (uint32_t)(c >> 1) << b;
            a->seeds2[p / 16] |= (uint32_t)c << (2 * (p % 16));
        }
        for (uint64_t i = i0; n >= k && i < i1 && i < n - k + 1; i += SEED_STEP) {
            uint32_t sd = 0, ok = 1;
            for (uint32_t j = 0; j < k && ok; j++) {
                const int c = base_code(a->seq[i + j]);
                if (c < 0) ok = 0;
                else sd |= (uint32_t)c << (2 * j);
            }
            if (ok) a->hist[sd & smask]++;
        }
        return NULL;
    }
    const uint32_t nmask = (k >= 32) ? ~0u : ((1u << k) - 1);
    const uint32_t res = SEED_STEP - 1, rmask = (1u << res) - 1;
    const uint32_t *b2 = ix->base_2bits, *s2 = a->seeds2;
    uint32_t *cursor = a->hist; /* this slice's next slot in every bucket */
    for (uint64_t i = i0; n >= k && i < i1 && i < n - k + 1; i += SEED_STEP) {
        uint32_t sd = fsr(s2[i / 16], s2[i / 16 + 1], (uint32_t)(i % 16) * 2) & smask;
        uint32_t nf = fsr(ix->base_3bits[i / 32], ix->base_3bits[i / 32 + 1], (uint32_t)(i % 32)) & nmask;
        if (nf) continue;
        uint64_t sp = (i >= res) ? i - res : 0;
        uint32_t fl = fsr(b2[(sp / 32) * 2], b2[(sp / 32 + 1) * 2], sp % 32) & rmask;
        uint32_t fh = fsr(b2[(sp / 32) * 2 + 1], b2[(sp / 32 + 1) * 2 + 1], sp % 32) & rmask;
        sp = i + k;
        uint32_t bl = fsr(b2[(sp / 32) * 2], b2[(sp / 32 + 1) * 2], sp % 32) & rmask;
        uint32_t bh = fsr(b2[(sp / 32) * 2 + 1], b2[(sp / 32 + 1) * 2 + 1], sp % 32) & rmask;
        fl |= bl << res;
        fh |= bh << res;
        const uint32_t slot = cursor[sd]++;
        ix->positions[slot] = (uint32_t)i;
        ix->pos_lseeds[slot] = (uint16_t)(fl | (fh << (res * 2)));
    }
    return NULL;
}

int swo_index_build_mt(const uint8_t *seq, uint64_t n, uint32_t k, uint32_t nthreads, swo_index *ix) {
    if (nthreads <= 1 || n < (1u << 20)) return swo_index_build(seq, n, k, ix);
    memset(ix, 0, sizeof(*ix));
    if (k < 1 || k > 14 || n >= 0xffffffffull) return -1;
    if (nthreads > 64) nthreads = 64;
    const uint64_t nb = 1ull << (2 * k);
    const uint64_t W = (n + 31) / 32;
    ix->k = k;
    ix->n = n;
    ix->hash_count = calloc(nb, 4);
    ix->hash_offset = calloc(nb + 1, 4);
    ix->base_2bits = calloc(2 * W + SWO_PAD_WORDS, 4);
    ix->base_3bits = calloc(W + SWO_PAD_WORDS, 4);
    uint32_t *seeds2 = calloc((n + 15) / 16 + SWO_PAD_WORDS, 4);
    uint32_t *hist = calloc((size_t)nthreads * nb, 4);
    ibuild_t args[64];
    pthread_t th[64];
    if (!ix->hash_count || !ix->hash_offset || !ix->base_2bits || !ix->base_3bits || !seeds2 || !hist) {
        free(seeds2);
        free(hist);
        swo_index_free(ix);
        return -3;
    }
    const uint64_t per = (W + nthreads - 1) / nthreads;
    for (uint32_t t = 0; t < nthreads; t++) {
        const uint64_t w0 = t * per < W ? t * per : W, w1 = (t + 1) * per < W ? (t + 1) * per : W;
        args[t] = (ibuild_t){seq, n, w0, w1, k, 1, hist + (size_t)t * nb, seeds2, ix};
    }
    for (uint32_t t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, ibuild_worker, &args[t]);
    for (uint32_t t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    /* counts, start offsets, and each slice's first slot per bucket */
    uint64_t S = 0;
    for (uint64_t b = 0; b < nb; b++) {
        uint32_t c = 0;
        for (uint32_t t = 0; t < nthreads; t++) {
            const uint32_t h = hist[(size_t)t * nb + b];
            hist[(size_t)t * nb + b] = (uint32_t)(S + c);
            c += h;
        }
        ix->hash_count[b] = c;
        S += c;
        ix->hash_offset[b] = (uint32_t)S; /* END offsets, as the serial build leaves them */
    }
    ix->hash_offset[nb] = (uint32_t)S;
    ix->n_seeds = S;
    ix->positions = malloc((S + 8) * 4);
    ix->pos_lseeds = malloc((S + 8) * 2);
    if (!ix->positions || !ix->pos_lseeds) {
        free(seeds2);
        free(hist);
        swo_index_free(ix);
        return -3;
    }
    for (uint32_t t = 0; t < nthreads; t++) args[t].phase = 3;
    for (uint32_t t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, ibuild_worker, &args[t]);
    for (uint32_t t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(seeds2);
    free(hist);
    return 0;
}

void swo_index_free(swo_index *ix) {
    free(ix->hash_count);
    free(ix->hash_offset);
    free(ix->positions);
    free(ix->pos_lseeds);
    free(ix->base_2bits);
    free(ix->base_3bits);
    memset(ix, 0, sizeof(*ix));
}

/* ======================================================================
 * FASTA input and index files
 * ====================================================================== */

typedef struct {
    char *p;
    size_t n, cap;
} sbuf;

static int sb_put(sbuf *b, const void *src, size_t len) {
    if (b->n + len + 1 > b->cap) {
        size_t nc = b->cap ? b->cap : 1024;
        while (nc < b->n + len + 1) nc *= 2;
        char *q = realloc(b->p, nc);
        if (!q) return -1;
        b->p = q;
        b->cap = nc;
    }
    memcpy(b->p + b->n, src, len);
    b->n += len;
    b->p[b->n] = 0;
    return 0;
}

int swo_read_fasta(const char *path, uint8_t **seq, uint64_t *n, char **ref_info, size_t *ref_info_len) {
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    sbuf s = {0}, info = {0}, name = {0};
    int c = fgetc(f);
    /* skip to the first header (kseq.h:202-205) */
    while (c != EOF && c != '>' && c != '@') c = fgetc(f);
    while (c != EOF) {
        name.n = 0;
        if (name.p) name.p[0] = 0;
        /* name: up to the first whitespace (kseq.h:208); rest of line ignored */
        c = fgetc(f);
        while (c != EOF && !isspace(c)) {
            char ch = (char)c;
            sb_put(&name, &ch, 1);
            c = fgetc(f);
        }
        while (c != EOF && c != '\n') c = fgetc(f);
        uint64_t len0 = s.n;
        /* sequence lines until the next '>' / '@' / '+' at a line start */
        for (;;) {
            c = fgetc(f);
            if (c == EOF || c == '>' || c == '+' || c == '@') break;
            if (c == '\n') continue;
            size_t line0 = s.n;
            while (c != EOF && c != '\n') {
                char ch = (char)c;
                sb_put(&s, &ch, 1);
                c = fgetc(f);
            }
            /* kseq strips one trailing '\r' when the accumulated sequence of
             * this record is longer than 1 (kseq.h:151) */
            if (s.n - len0 > 1 && s.n > line0 && s.p[s.n - 1] == '\r') s.n--;
            if (c == EOF) break;
        }
        char line[64];
        int ln = snprintf(line, sizeof line, "%lu\n%lu\n", (unsigned long)(s.n - len0), (unsigned long)name.n);
        sb_put(&info, line, (size_t)ln);
        sb_put(&info, name.p ? name.p : "", name.n);
        sb_put(&info, "\n", 1);
        while (c != EOF && c != '>' && c != '@') c = fgetc(f);
    }
    fclose(f);
    free(name.p);
    *seq = (uint8_t *)(s.p ? s.p : calloc(1, 1));
    *n = s.n;
    if (ref_info) {
        *ref_info = info.p ? info.p : calloc(1, 1);
        *ref_info_len = info.n;
    } else {
        free(info.p);
    }
    return 0;
}

static int write_file(const char *prefix, const char *ext, const void *data, size_t bytes) {
    char path[4096];
    snprintf(path, sizeof path, "%s%s", prefix, ext);
    FILE *f = fopen(path, "wb");
    if (!f) return -1;
    size_t w = bytes ? fwrite(data, 1, bytes, f) : 0;
    fclose(f);
    return w == bytes ? 0 : -1;
}

int swo_index_write(const swo_index *ix, const char *prefix, const char *ref_info, size_t ref_info_len) {
    const uint64_t nb = 1ull << (2 * ix->k);
    const uint64_t W = (ix->n + 31) / 32;
    int rc = 0;
    rc |= write_file(prefix, ".ref_info", ref_info ? ref_info : "", ref_info ? ref_info_len : 0);
    rc |= write_file(prefix, ".hash_count", ix->hash_count, nb * 4);
    rc |= write_file(prefix, ".hash_offset", ix->hash_offset, (nb + 1) * 4);
    rc |= write_file(prefix, ".positions", ix->positions, ix->n_seeds * 4);
    rc |= write_file(prefix, ".pos_lseeds", ix->pos_lseeds, ix->n_seeds * 2);
    rc |= write_file(prefix, ".base_2bits", ix->base_2bits, 2 * W * 4);
    rc |= write_file(prefix, ".base_3bits", ix->base_3bits, W * 4);
    return rc;
}

/* ======================================================================
 * Mapping: mapper_cpe.c
 * ====================================================================== */

/* Encode one read base the way get_seed_from_reads does (mapper_cpe.c:
 * 1260-1305): into the 2-bit accumulator and the lo/hi planes; anything but
 * A/C/G/T is encoded as C. */
static inline void enc_base(uint32_t w[32], uint32_t *acc, uint64_t rp, char ch) {
    uint32_t code;
    switch (ch) {
    case 'A': code = 0; break;
    case 'C': code = 1; break;
    case 'G': code = 2; break;
    case 'T': code = 3; break;
    default: code = 1; break;
    }
    *acc |= code << ((rp % 16) * 2);
    w[16 + (rp >> 5) * 2] |= (code & 1u) << (rp & 31);
    w[16 + (rp >> 5) * 2 + 1] |= (code >> 1) << (rp & 31);
    if (rp % 16 == 15) {
        w[rp / 16] = *acc;
        *acc = 0;
    }
}

/* get_seed_from_reads, mapper_cpe.c:1246-1364, including its tail encoder
 * (1312-1362) that re-runs after every seed whose last base lies within k of
 * the read end. Returns the rolling seed for slot j. */
static uint32_t read_seed(const char *s, uint32_t w[32], uint32_t *acc, uint32_t pre,
                          uint32_t k, uint32_t j, uint32_t L) {
    uint64_t i = (j % SEED_STEP == 0) ? 0 : k - 1;
    const uint64_t base = (uint64_t)(j / SEED_STEP) * (k + SEED_STEP - 1) + j % SEED_STEP;
    uint32_t seed = pre;
    uint64_t rp = base + i;
    for (; i < k; i++) {
        rp = base + i;
        char ch = s[rp];
        uint32_t sc;
        switch (ch) {
        case 'A': sc = 0; break;
        case 'C': sc = 1; break;
        case 'G': sc = 2; break;
        case 'T': sc = 3; break;
        default: sc = (uint32_t)(i % 4); break; /* mapper_cpe.c:1294 */
        }
        seed = (uint32_t)((seed >> 2) | ((uint64_t)sc << ((k - 1) * 2)));
        enc_base(w, acc, rp, ch);
    }
    if ((uint64_t)L - rp < k) {
        for (; rp < L; rp++) enc_base(w, acc, rp, s[rp]);
        w[(rp - 1) / 16] = *acc;
    }
    return seed;
}

void swo_encode_read(const char *seq, uint32_t L, uint32_t k, uint32_t w[32]) {
    memset(w, 0, 32 * 4);
    uint32_t acc = 0, seed = 0;
    const uint32_t ns = (L / (k + SEED_STEP - 1)) * SEED_STEP;
    for (uint32_t j = 0; j < ns; j++) seed = read_seed(seq, w, &acc, seed, k, j, L);
}

typedef struct {
    uint32_t count, index;
} slot_t; /* hash_count_t, mapper_cpe.c:78-81 */

/* Window of one candidate: aligned bit planes, bit b of word j = window base
 * 32j + b (shift_ref_pos_v, mapper_cpe.c:1509-1586). */
#define WIN_WORDS 12
typedef struct {
    uint32_t lo[WIN_WORDS], hi[WIN_WORDS];
    uint32_t ws, rl;
} window_t;

static inline uint32_t ref_word(const swo_mapidx *ix, uint64_t w) {
    /* D5: zero beyond the end of the genome (plus pad) */
    return (w < ix->n_words2 + SWO_PAD_WORDS) ? ix->base_2bits[w] : 0u;
}

/* adjust_ref_len + pos_start, mapper_cpe.c:1403-1435, with the reference's
 * integer types. Returns the window start or 0xffffffff when rejected. */
static uint32_t window_start(const swo_mapidx *ix, uint32_t base_pos, uint32_t L, uint32_t e, uint32_t *rl_out) {
    const uint64_t dist_error = e;
    uint64_t shift_tmp = e;
    uint64_t ref_len = (uint64_t)L + 2 * shift_tmp;
    if (base_pos <= shift_tmp) {
        shift_tmp = base_pos;
        ref_len -= (dist_error - base_pos);
    }
    int64_t front = (int64_t)ix->ref_length - (int64_t)((uint64_t)base_pos - dist_error);
    int64_t back = (int64_t)((uint64_t)(uint32_t)(base_pos + L) + dist_error) - (int64_t)ix->ref_length;
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

static void load_window(const swo_mapidx *ix, uint32_t ws, uint32_t rl, window_t *win) {
    const uint64_t w0 = (uint64_t)(ws / 32) * 2;
    const uint32_t s = ws & 31;
    win->ws = ws;
    win->rl = rl;
    for (uint32_t j = 0; j < WIN_WORDS; j++) {
        win->lo[j] = fsr(ref_word(ix, w0 + 2 * j), ref_word(ix, w0 + 2 * j + 2), s);
        win->hi[j] = fsr(ref_word(ix, w0 + 2 * j + 1), ref_word(ix, w0 + 2 * j + 3), s);
    }
}

static inline uint32_t win_base(const uint32_t *lo, const uint32_t *hi, uint32_t p) {
    return ((lo[p >> 5] >> (p & 31)) & 1u) | (((hi[p >> 5] >> (p & 31)) & 1u) << 1);
}

/* Banded Myers / Hyyro recurrence, banded_myers_simd (mapper_cpe.c:519-660).
 * When d0h/hph are given the per-step D0/HP words are kept for traceback
 * (align_reads, mapper_cpe.c:288-362). */
static int myers(const uint32_t w2[16], uint32_t L, uint32_t e, const uint32_t *lo, const uint32_t *hi,
                 uint32_t rl, int *loc_out, uint32_t *d0h, uint32_t *hph) {
    const int dist_error = (int)e;
    const uint32_t band = 2 * e + 1, down = 2 * e;
    uint32_t peq[4] = {0, 0, 0, 0};
    uint32_t t = 1;
    for (uint32_t j = 0; j < band; j++) {
        peq[win_base(lo, hi, j)] |= t;
        t <<= 1;
    }
    const int last_high = (int)band - (int)L + (int)rl - (int)down - 1;
    uint32_t vp = 0, vn = 0, x, d0, hn, hp;
    int err = 0;
    uint32_t ibd = down;
    const uint32_t top = 1u << (band - 1);
    for (uint32_t i = 0; i < L; i++) {
        uint32_t c = (w2[i / 16] >> ((i % 16) * 2)) & 3u;
        x = peq[c] | vn;
        d0 = ((vp + (x & vp)) ^ vp) | x;
        hn = vp & d0;
        hp = vn | ~(vp | d0);
        x = d0 >> 1;
        vn = x & hp;
        vp = hn | ~(x | hp);
        if (d0h) {
            d0h[i] = d0;
            hph[i] = hp;
        }
        if (!(d0 & 1u)) err++;
        peq[0] >>= 1;
        peq[1] >>= 1;
        peq[2] >>= 1;
        peq[3] >>= 1;
        ++ibd;
        peq[win_base(lo, hi, ibd)] |= top;
    }
    const int site = (int)rl - last_high - 1;
    int location = -1, error = MAXERROR;
    if (err <= dist_error && err < error) {
        error = err;
        location = site;
    }
    for (int i = 0; i < last_high; i++) {
        err += (int)((vp >> i) & 1u);
        err -= (int)((vn >> i) & 1u);
        if (err <= dist_error && err < error) {
            error = err;
            location = site + i + 1;
        }
    }
    *loc_out = location;
    return error;
}

int swo_banded_myers(const uint32_t w2[16], uint32_t L, uint32_t e, const uint32_t *wlo, const uint32_t *whi,
                     uint32_t rl, int *loc) {
    if (L == 0 || L > MAX_READ_LEN || e > MAX_E) return -1;
    uint32_t lo[WIN_WORDS] = {0}, hi[WIN_WORDS] = {0};
    uint32_t nw = (L + 2 * e + 1) / 32 + 1;
    for (uint32_t j = 0; j < nw && j < WIN_WORDS; j++) {
        lo[j] = wlo[j];
        hi[j] = whi[j];
    }
    return myers(w2, L, e, lo, hi, rl, loc, NULL, NULL);
}

/* Per-strand output accumulator: the reference's cigar_t (mapper_cpe.c:
 * 98-108, 2160-2169) plus the records it has put so far. */
typedef struct {
    uint32_t loc[2 * SWO_MAX_CIGAR + 8];
    uint8_t cig[8 * SWO_CIGAR_STRIDE]; /* room for a group of pathological CIGARs */
    uint32_t num, len;
    int main_flag;
} acc_t;

typedef struct {
    uint32_t *w;   /* packed records: [cur_read, numflag, loc...] */
    size_t nw, capw;
    uint8_t *c;    /* packed cigar bytes per record */
    size_t nc, capc;
    uint32_t *clen; /* cigar byte count per record */
    uint32_t nrec, caprec;
    int unmapped;
    int overflow;
    uint64_t cigar_size; /* ref_info_s->cigar_size, reset per read (2528) */
} oread_t;

static int grow(void **p, size_t *cap, size_t need, size_t elt) {
    if (need <= *cap) return 0;
    size_t nc = *cap ? *cap : 64;
    while (nc < need) nc *= 2;
    void *q = realloc(*p, nc * elt);
    if (!q) return -1;
    *p = q;
    *cap = nc;
    return 0;
}

/* put_cigar, mapper_cpe.c:1437-1507 */
static void put_cigar(acc_t *a, oread_t *o, uint32_t cur_read, int last) {
    o->cigar_size += a->num;
    if (last && o->cigar_size == 0) o->unmapped = 1;
    if (a->num > 0) {
        uint32_t numflag = a->num;
        if (a->main_flag) {
            numflag |= 1u << 31;
            a->main_flag = 0;
        }
        if (a->len > SWO_CIGAR_STRIDE) o->overflow = 1;
        size_t cr = o->caprec;
        if (grow((void **)&o->w, &o->capw, o->nw + 2 + a->num, 4) ||
            grow((void **)&o->c, &o->capc, o->nc + a->len, 1) ||
            grow((void **)&o->clen, &cr, o->nrec + 1, 4)) {
            o->overflow = 1;
        } else {
            o->caprec = (uint32_t)cr;
            o->w[o->nw++] = cur_read;
            o->w[o->nw++] = numflag;
            memcpy(o->w + o->nw, a->loc, a->num * 4);
            o->nw += a->num;
            memcpy(o->c + o->nc, a->cig, a->len);
            o->nc += a->len;
            o->clen[o->nrec++] = a->len;
        }
    }
    a->num = 0;
    a->len = 0;
}

/* sprint_length, mapper_cpe.c:214-228. Its digit is '0' + (char)rlen % 10:
 * the cast binds first, so with the signed char of the reference's targets a
 * value whose low byte is >= 128 yields a non-digit ('0' + (-118 % 10) = '('
 * for 138). Reproduced with explicit signed-byte arithmetic so the result does
 * not depend on the host's char signedness. */
static int put_len(uint8_t *p, uint32_t v) {
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

typedef struct {
    uint64_t ss_out, ms_stop, empty_merge, short_seeds, err0_tb;
} ubstat_t;

/* align_reads for one passing candidate (mapper_cpe.c:243-509): Hamming
 * shortcut, else traceback with run-length route and CIGAR text. */
static void align_one(const uint32_t w[32], uint32_t L, uint32_t e, const window_t *win, int error, int location,
                      acc_t *a, swo_stats *st, ubstat_t *ub) {
    (void)e;
    int start = location - (int)L + 1;
    int ham = 0;
    for (uint32_t ii = 0; ii * 32 < L; ii++) {
        uint32_t mask = 0xffffffffu;
        if ((ii + 1) * 32 > L) mask >>= (32 - (L - ii * 32));
        uint32_t lref = fsr(win->lo[ii], win->lo[ii + 1], (uint32_t)start);
        uint32_t href = fsr(win->hi[ii], win->hi[ii + 1], (uint32_t)start);
        uint32_t x = ((w[16 + 2 * ii + 1] ^ href) | (w[16 + 2 * ii] ^ lref)) & mask;
        ham += __builtin_popcount(x);
    }
    if (ham == error) {
        uint8_t *cs = a->cig + a->len;
        uint32_t n = 0;
        cs[n++] = (uint8_t)ham;
        n++;
        n += (uint32_t)put_len(cs + n, L);
        cs[n++] = 'M';
        cs[1] = (uint8_t)(n - 2);
        a->len += n;
        a->loc[a->num++] = win->ws + (uint32_t)start + 1;
        if (st) {
            st->hamming++;
            st->emitted++;
        }
        return;
    }
    /* traceback: re-run Myers keeping D0/HP per read base */
    uint32_t d0h[MAX_READ_LEN + 2], hph[MAX_READ_LEN + 2];
    int loc2;
    myers(w, L, e, win->lo, win->hi, win->rl, &loc2, d0h, hph);
    if (st) st->traceback++;
    if (error == 0 && ub) ub->err0_tb++;
    int match_site = location;
    int search_site = match_site - ((int)L - 1);
    int i = (int)L - 1, sum_err = 0, j = 1;
    int pre_size = 1;
    char pre_char = 'N';
    int rsz[3 * MAX_READ_LEN + 64];
    char rch[3 * MAX_READ_LEN + 64];
#define TB_BIT(arr, ii, s) (((s) >= 0 && (s) < 32) ? (((arr)[ii] >> (s)) & 1u) : (ub ? ub->ss_out++ : 0, 0u))
#define TB_REF(m) win_base(win->lo, win->hi, (uint32_t)(m))
#define TB_READ(r) ((w[(r) / 16] >> (2 * ((r) % 16))) & 3u)
    /* first step, mapper_cpe.c:380-410 */
    if (TB_BIT(d0h, i, search_site) && TB_REF(match_site) == TB_READ(i)) {
        i--; pre_size = 1; pre_char = 'M'; match_site--;
    } else if (!TB_BIT(d0h, i, search_site) && TB_REF(match_site) != TB_READ(i)) {
        i--; pre_size = 1; pre_char = 'S'; match_site--; sum_err++;
    } else if (TB_BIT(hph, i, search_site)) {
        i--; search_site++; pre_size = 1; pre_char = 'S'; sum_err++; start++;
    } else {
        search_site--; pre_size = 1; pre_char = 'D'; match_site--; sum_err++; start--;
    }
    /* mapper_cpe.c:412-466 */
    while (i >= 0) {
        if (sum_err == error) break;
        if (match_site < 0) { /* D6 */
            if (ub) ub->ms_stop++;
            break;
        }
        if (TB_BIT(d0h, i, search_site) && TB_REF(match_site) == TB_READ(i)) {
            i--; match_site--;
            if (pre_char != 'M') { rsz[j] = pre_size; rch[j++] = pre_char; pre_size = 1; pre_char = 'M'; }
            else pre_size++;
        } else if (!TB_BIT(d0h, i, search_site) && TB_REF(match_site) != TB_READ(i)) {
            i--; match_site--; sum_err++;
            if (pre_char != 'S') { rsz[j] = pre_size; rch[j++] = pre_char; pre_size = 1; pre_char = 'S'; }
            else pre_size++;
        } else if (TB_BIT(hph, i, search_site)) {
            i--; search_site++; sum_err++;
            if (pre_char != 'I') { rsz[j] = pre_size; rch[j++] = pre_char; pre_size = 1; pre_char = 'I'; }
            else pre_size++;
            start++;
        } else {
            search_site--; match_site--; sum_err++;
            if (pre_char != 'D') { rsz[j] = pre_size; rch[j++] = pre_char; pre_size = 1; pre_char = 'D'; }
            else pre_size++;
            start--;
        }
    }
#undef TB_BIT
#undef TB_REF
#undef TB_READ
    rsz[j] = pre_size;
    rch[j++] = pre_char;
    if (i >= 0) {
        rsz[j] = i + 1;
        rch[j++] = 'M';
    }
    const uint32_t out_loc = win->ws + (uint32_t)start + 1;
    if (a->num > 0 && a->loc[a->num - 1] == out_loc) return; /* mapper_cpe.c:475-477 */
    uint8_t *cs = a->cig + a->len;
    uint32_t n = 0;
    cs[n++] = (uint8_t)error;
    n++;
    a->loc[a->num++] = out_loc;
    for (j = j - 1; j > 0; j--) {
        if (rch[j] == 'M' || rch[j] == 'S') {
            int sm = 0;
            while (j > 0 && (rch[j] == 'M' || rch[j] == 'S')) {
                sm += rsz[j];
                j--;
            }
            j++;
            n += (uint32_t)put_len(cs + n, (uint32_t)sm);
            cs[n++] = 'M';
        } else {
            n += (uint32_t)put_len(cs + n, (uint32_t)rsz[j]);
            cs[n++] = (uint8_t)rch[j];
        }
    }
    cs[1] = (uint8_t)(n - 2);
    a->len += n;
    if (st) st->emitted++;
}

/* Candidate sink: verification (banded_myers, mapper_cpe.c:1590-1864) in
 * groups of 8 with the record flush test after every group (1790, 1858). */
typedef struct {
    const swo_mapidx *ix;
    const uint32_t *w;
    uint32_t L, e;
    acc_t *a;
    oread_t *o;
    uint32_t cur_read;
    swo_stats *st;
    ubstat_t *ub;
    swo_trace *tr;
    uint32_t batch;
} verify_ctx;

static int trace_push(swo_trace *tr, uint32_t batch, uint32_t pos, int err, int loc) {
    static const size_t chunk = 1024;
    if (tr->n % chunk == 0) {
        size_t nc = tr->n + chunk;
        uint32_t *b = realloc(tr->batch, nc * 4), *p;
        if (!b) return -1;
        tr->batch = b;
        p = realloc(tr->pos, nc * 4);
        if (!p) return -1;
        tr->pos = p;
        int32_t *er = realloc(tr->err, nc * 4);
        if (!er) return -1;
        tr->err = er;
        int32_t *lc = realloc(tr->loc, nc * 4);
        if (!lc) return -1;
        tr->loc = lc;
    }
    tr->batch[tr->n] = batch;
    tr->pos[tr->n] = pos;
    tr->err[tr->n] = err;
    tr->loc[tr->n] = loc;
    tr->n++;
    return 0;
}

/* record flush test after each group of 8 (mapper_cpe.c:1790, 1858) */
static void flush_check(verify_ctx *v) {
    if (v->a && (v->a->num + 8 > SWO_MAX_CIGAR || v->a->len + 16 * 16 > SWO_MAX_CIGAR * 16))
        put_cigar(v->a, v->o, v->cur_read, 0);
}

static void verify_batch(verify_ctx *v, const uint32_t *cand, uint32_t nc) {
    uint32_t in_group = 0;
    for (uint32_t c = 0; c < nc; c++) {
        uint32_t rl;
        uint32_t ws = window_start(v->ix, cand[c], v->L, v->e, &rl);
        if (ws == 0xffffffffu) continue;
        window_t win;
        load_window(v->ix, ws, rl, &win);
        int loc;
        int err = myers(v->w, v->L, v->e, win.lo, win.hi, rl, &loc, NULL, NULL);
        if (v->st) {
            v->st->candidates++;
            v->st->cells += (uint64_t)v->L * (2 * v->e + 1);
        }
        if (v->tr) trace_push(v->tr, v->batch, cand[c], err, loc);
        if (err <= (int)v->e) {
            if (v->st) v->st->passed++;
            if (v->a) align_one(v->w, v->L, v->e, &win, err, loc, v->a, v->st, v->ub);
        }
        if (++in_group == 8) {
            in_group = 0;
            flush_check(v);
        }
    }
    if (in_group > 0) flush_check(v);
}

/* One fetched chunk of a bucket, with the fields the filter needs. */
typedef struct {
    uint32_t pos;   /* adjusted position */
    uint16_t lseed;
    uint8_t sel;    /* selected seed slot i */
} elem_t;

/* block_heap_sort, mapper_cpe.c:1999-2089: k-way merge of the (sorted)
 * filtered runs with duplicate removal. pi holds [start, end) per run. */
static uint32_t merge_runs(uint32_t *P, uint32_t *pi, uint32_t nruns, uint32_t *out, ubstat_t *ub) {
    uint32_t hpos[MAX_RUNS_BLOCK + 8], hind[MAX_RUNS_BLOCK + 8];
    uint32_t hs = 0;
    for (uint32_t r = 0; r < nruns; r++) {
        if (pi[2 * r] < pi[2 * r + 1]) {
            hs++;
            hpos[hs] = P[pi[2 * r]];
            hind[hs] = 2 * r;
            pi[2 * r]++;
            uint32_t ci = hs, p = ci / 2;
            while (ci > 1) {
                if (hpos[p] > hpos[ci]) {
                    uint32_t t = hpos[ci]; hpos[ci] = hpos[p]; hpos[p] = t;
                    t = hind[ci]; hind[ci] = hind[p]; hind[p] = t;
                } else break;
                ci /= 2;
                p = ci / 2;
            }
        }
    }
    if (hs == 0) { /* D4 */
        if (ub) ub->empty_merge++;
        return 0;
    }
    uint32_t pre = 0xffffffffu, n = 0;
    while (hs > 1) {
        uint32_t id = hind[1];
        if (pre != hpos[1]) {
            out[n++] = hpos[1];
            pre = hpos[1];
        }
        if (pi[id] < pi[id + 1]) {
            hpos[1] = P[pi[id]];
            pi[id]++;
        } else {
            hpos[1] = hpos[hs];
            hind[1] = hind[hs];
            hs--;
            if (hs == 1) break;
        }
        uint32_t h = 1;
        while (h * 2 <= hs) {
            uint32_t l = h * 2, r = l + 1, s = l;
            if (r <= hs && hpos[l] > hpos[r]) s = r;
            if (hpos[h] > hpos[s]) {
                uint32_t t = hpos[h]; hpos[h] = hpos[s]; hpos[s] = t;
                t = hind[h]; hind[h] = hind[s]; hind[s] = t;
            } else break;
            h = s;
        }
    }
    uint32_t id = hind[1];
    for (uint32_t i = pi[id] - 1; i < pi[id + 1]; i++) {
        if (P[i] != pre) {
            out[n++] = P[i];
            pre = P[i];
        }
    }
    return n;
}

typedef struct {
    uint32_t start, count, base, rl, rh, shift, pc;
} sel_t;

/* Filter (long_seeds_filter, mapper_cpe.c:2090-2123: element 0 of every
 * batch is dropped by its `pos_size != j` test), merge and verify one batch. */
static void process_batch(verify_ctx *v, const elem_t *el, uint32_t nel, const uint32_t *run_end, uint32_t nruns,
                          const sel_t *sel) {
    uint32_t P[BATCH_POSITIONS + 64], pi[2 * MAX_RUNS_BLOCK + 8], out[BATCH_POSITIONS + 64];
    uint32_t keep = 0, j = 0;
    for (uint32_t r = 0; r < nruns; r++) {
        const uint32_t s0 = keep;
        for (; j < run_end[r]; j++) {
            const sel_t *sd = &sel[el[j].sel];
            uint32_t sl = (uint32_t)el[j].lseed >> sd->shift;
            uint32_t sh = (uint32_t)el[j].lseed >> (6 + sd->shift);
            uint32_t res = ((sl ^ sd->rl) | (sh ^ sd->rh)) & 7u;
            if (res == 0 && keep != j) P[keep++] = el[j].pos;
        }
        pi[2 * r] = s0;
        pi[2 * r + 1] = keep;
    }
    (void)nel;
    uint32_t nc = (keep > 0) ? merge_runs(P, pi, nruns, out, v->ub) : 0;
    if (nc > 0) verify_batch(v, out, nc);
    if (v->st) v->st->batches++;
}

/* seeds_heap_insert / seeds_heap_pop_and_insert, mapper_cpe.c:1919-1962.
 * The pop keeps the reference's `i * 2 < size` loop bound. */
typedef struct {
    uint32_t loc[72];
    uint32_t idx[72];
    uint32_t size;
} sheap_t;

static void sheap_insert(sheap_t *h, uint32_t loc, uint32_t idx) {
    h->size++;
    h->loc[h->size] = loc;
    h->idx[h->size] = idx;
    uint32_t i = h->size;
    while (i > 1) {
        uint32_t t = i / 2;
        if (h->loc[t] > h->loc[i]) {
            uint32_t a = h->loc[t]; h->loc[t] = h->loc[i]; h->loc[i] = a;
            a = h->idx[t]; h->idx[t] = h->idx[i]; h->idx[i] = a;
        } else break;
        i = t;
    }
}

static void sheap_pop_insert(sheap_t *h, uint32_t loc, int del) {
    if (del) {
        h->loc[1] = h->loc[h->size];
        h->idx[1] = h->idx[h->size];
        h->size--;
    } else {
        h->loc[1] = loc;
    }
    uint32_t i = 1, ti;
    while (i * 2 < h->size) {
        ti = i * 2;
        if (i * 2 + 1 <= h->size && h->loc[i * 2] > h->loc[i * 2 + 1]) ti = i * 2 + 1;
        if (h->loc[ti] < h->loc[i]) {
            uint32_t a = h->loc[ti]; h->loc[ti] = h->loc[i]; h->loc[i] = a;
            a = h->idx[ti]; h->idx[ti] = h->idx[i]; h->idx[i] = a;
        } else break;
        i = ti;
    }
}

/* Seed selection for one strand: choose_seed (mapper_cpe.c:1365-1401),
 * set_read_long_seeds (2451-2499) and the slot table alignment_rmdup reads
 * (2194-2196). Returns the number of selected seed slots. */
static uint32_t select_seeds(const swo_mapidx *ix, const char *s, uint32_t L, uint32_t e, uint32_t w[32],
                             sel_t *sel, ubstat_t *ub) {
    const uint32_t k = ix->k, klong = k + SEED_STEP - 1;
    const uint32_t nl = L / klong, ns_all = nl * SEED_STEP;
    uint32_t cnt[64], start[64];
    memset(w, 0, 32 * 4);
    uint32_t acc = 0, seed = 0;
    for (uint32_t j = 0; j < ns_all; j++) {
        seed = read_seed(s, w, &acc, seed, k, j, L);
        start[j] = ix->hash_offset[seed];
        cnt[j] = ix->hash_offset[seed + 1] - ix->hash_offset[seed];
    }
    slot_t info[16];
    for (uint32_t j = 0; j < 16; j++) {
        info[j].count = 0;
        info[j].index = j;
    }
    for (uint32_t j = 0; j < ns_all; j++) info[j / SEED_STEP].count += cnt[j];
    for (uint32_t j = 0; j < nl; j++)
        for (uint32_t m = j + 1; m < nl; m++)
            if (info[j].count > info[m].count) {
                slot_t t = info[j]; info[j] = info[m]; info[m] = t;
            }
    /* read flank codes (set_read_long_seeds) */
    uint8_t res[128];
    const uint32_t lmask = (klong >= 32) ? ~0u : ((1u << klong) - 1), rmask = (1u << (SEED_STEP - 1)) - 1;
    for (uint32_t i = 0; i < nl; i++) {
        uint32_t off = i * klong, wj = off >> 5, sh = off & 31;
        uint32_t nxt = 16 + (wj + 1) * 2;
        uint32_t l = fsr(w[16 + wj * 2], nxt < 32 ? w[nxt] : 0u, sh) & lmask;
        uint32_t h = fsr(w[16 + wj * 2 + 1], nxt + 1 < 32 ? w[nxt + 1] : 0u, sh) & lmask;
        for (uint32_t j = 0; j < SEED_STEP; j++) {
            uint32_t sft = k + j, m = (1u << j) - 1;
            res[2 * (SEED_STEP * i + j)] = (uint8_t)(((l & m) | ((l >> sft) << j)) & rmask);
            res[2 * (SEED_STEP * i + j) + 1] = (uint8_t)(((h & m) | ((h >> sft) << j)) & rmask);
        }
    }
    const uint32_t nsl = (e + 1 < nl) ? e + 1 : nl; /* D3 */
    if (e + 1 > nl && ub) ub->short_seeds++;
    for (uint32_t i = 0; i < nsl * SEED_STEP; i++) {
        uint32_t sidx = info[i / SEED_STEP].index * SEED_STEP + i % SEED_STEP;
        sel[i].start = start[sidx];
        sel[i].count = cnt[sidx];
        sel[i].base = info[i / SEED_STEP].index * klong + i % SEED_STEP;
        sel[i].shift = SEED_STEP - 1 - sidx % SEED_STEP;
        sel[i].rl = res[2 * sidx];
        sel[i].rh = res[2 * sidx + 1];
        sel[i].pc = 0;
    }
    return nsl * SEED_STEP;
}

/* alignment_rmdup (mapper_cpe.c:2124-2426) for one strand. */
static void map_strand(const swo_mapidx *ix, const char *s, uint32_t L, uint32_t e, uint32_t cur_read,
                       oread_t *o, swo_stats *st, ubstat_t *ub, swo_trace *tr) {
    uint32_t w[32];
    sel_t sel[64];
    const uint32_t ns = select_seeds(ix, s, L, e, w, sel, ub);
    if (tr) {
        tr->nsel = ns;
        memcpy(tr->w, w, sizeof w);
        for (uint32_t i = 0; i < ns; i++) {
            tr->sel_start[i] = sel[i].start;
            tr->sel_count[i] = sel[i].count;
            tr->sel_base[i] = sel[i].base;
            tr->sel_shift[i] = (uint8_t)sel[i].shift;
            tr->sel_rl[i] = (uint8_t)sel[i].rl;
            tr->sel_rh[i] = (uint8_t)sel[i].rh;
        }
    }
    acc_t *a = NULL;
    if (o) {
        a = malloc(sizeof(acc_t));
        a->num = 0;
        a->len = 0;
        a->main_flag = 1;
    }
    verify_ctx v = {ix, w, L, e, a, o, cur_read, st, ub, tr, 0};
    elem_t el[BATCH_POSITIONS + 64];
    uint32_t run_end[MAX_RUNS_BLOCK + 8];
    uint32_t nel = 0, nruns = 0;
    sheap_t h;
    h.size = 0;
#define FETCH(i, get)                                                                 \
    do {                                                                              \
        sel_t *sd_ = &sel[i];                                                         \
        for (uint32_t q_ = 0; q_ < (get); q_++) {                                     \
            uint32_t g_ = sd_->start + sd_->pc + q_;                                   \
            uint32_t raw_ = ix->positions[g_];                                        \
            el[nel].pos = raw_ > sd_->base ? raw_ - sd_->base : 0;                    \
            el[nel].lseed = ix->pos_lseeds[g_];                                       \
            el[nel].sel = (uint8_t)(i);                                               \
            nel++;                                                                    \
        }                                                                             \
        sd_->pc += (get);                                                             \
        run_end[nruns++] = nel;                                                       \
        if (st) st->fetched += (get);                                                 \
    } while (0)
    /* initial fetch of up to 32 positions per seed (2194-2236) */
    for (uint32_t i = 0; i < ns; i++) {
        uint32_t get = sel[i].count > PER_FETCH ? PER_FETCH : sel[i].count;
        if (get > 0) FETCH(i, get);
    }
    for (uint32_t i = 0; i < ns; i++)
        if (sel[i].pc != sel[i].count) sheap_insert(&h, ix->positions[sel[i].start + sel[i].pc - 1], i);
    /* refill / flush loop (2261-2419) */
    for (;;) {
        if (h.size > 0 && nel + PER_FETCH <= BATCH_POSITIONS && 1 + 2 * nruns < MAX_RUNS_BLOCK) {
            uint32_t i = h.idx[1];
            uint32_t left = sel[i].count - sel[i].pc;
            uint32_t get = left > PER_FETCH ? PER_FETCH : left;
            FETCH(i, get);
            int del = sel[i].pc == sel[i].count;
            sheap_pop_insert(&h, ix->positions[sel[i].start + sel[i].pc - 1], del);
        }
        if (nel + PER_FETCH > BATCH_POSITIONS || h.size == 0 || 1 + 2 * nruns >= MAX_RUNS_BLOCK) {
            if (nel > 0) process_batch(&v, el, nel, run_end, nruns, sel);
            v.batch++;
            nel = 0;
            nruns = 0;
            if (h.size == 0) break;
        }
    }
#undef FETCH
    if (tr) tr->nbatches = v.batch;
    if (a) {
        put_cigar(a, o, cur_read, (int)(cur_read & 1));
        free(a);
    }
}

/* reverse_read, mapper_cpe.c:2429-2450 */
static void revcomp(char *dst, const char *src, uint32_t L) {
    for (uint32_t i = 0; i < L; i++) {
        char c = src[i], r;
        switch (c) {
        case 'A': r = 'T'; break;
        case 'C': r = 'G'; break;
        case 'G': r = 'C'; break;
        case 'T': r = 'A'; break;
        default: r = c; break;
        }
        dst[L - 1 - i] = r;
    }
}

int swo_trace_item(const swo_mapidx *ix, const char *seq, uint32_t L, uint32_t e, swo_trace *tr) {
    memset(tr, 0, sizeof(*tr));
    if (L > MAX_READ_LEN || e > MAX_E) return -1;
    map_strand(ix, seq, L, e, 0, NULL, NULL, NULL, tr);
    return 0;
}

void swo_trace_free(swo_trace *tr) {
    free(tr->batch);
    free(tr->pos);
    free(tr->err);
    free(tr->loc);
    memset(tr, 0, sizeof(*tr));
}

/* ---------------- threaded driver (find_positions + get_positions) ------ */

typedef struct {
    const swo_mapidx *ix;
    const char *reads;
    uint64_t stride;
    const uint32_t *lens;
    uint64_t nreads;
    uint32_t e;
    oread_t *per;
    uint64_t next;
    int bad;
    pthread_mutex_t mu;
    swo_stats st;
} job_t;

static void map_read(job_t *jb, uint64_t r, swo_stats *st, ubstat_t *ub) {
    const uint32_t L = jb->lens[r];
    oread_t *o = &jb->per[r];
    memset(o, 0, sizeof(*o));
    if (L > MAX_READ_LEN) {
        jb->bad = 1;
        return;
    }
    const char *s = jb->reads + r * jb->stride;
    char rc[MAX_READ_LEN + 1];
    /* get_positions, mapper_cpe.c:2522-2588: forward then reverse complement */
    map_strand(jb->ix, s, L, jb->e, (uint32_t)(2 * r), o, st, ub, NULL);
    revcomp(rc, s, L);
    map_strand(jb->ix, rc, L, jb->e, (uint32_t)(2 * r + 1), o, st, ub, NULL);
    st->items += 2;
    if (o->cigar_size > 0) st->mapped_reads++;
}

static void *worker(void *arg) {
    job_t *jb = arg;
    swo_stats st;
    ubstat_t ub;
    memset(&st, 0, sizeof st);
    memset(&ub, 0, sizeof ub);
    for (;;) {
        uint64_t r = __atomic_fetch_add(&jb->next, 1, __ATOMIC_RELAXED);
        if (r >= jb->nreads) break;
        map_read(jb, r, &st, &ub);
    }
    st.ub_shift_out = ub.ss_out;
    st.ub_walk_stop = ub.ms_stop;
    st.ub_empty_merge = ub.empty_merge;
    st.ub_short_seeds = ub.short_seeds;
    st.ub_err0_traceback = ub.err0_tb;
    pthread_mutex_lock(&jb->mu);
    uint64_t *d = (uint64_t *)&jb->st, *sv = (uint64_t *)&st;
    for (size_t i = 0; i < sizeof(swo_stats) / 8; i++) d[i] += sv[i];
    pthread_mutex_unlock(&jb->mu);
    return NULL;
}

int swo_map_reads(const swo_mapidx *ix, const char *reads, uint64_t stride, const uint32_t *lens, uint64_t nreads,
                  uint32_t e, uint32_t nthreads, swo_out *out, swo_stats *stats) {
    if (e > MAX_E || ix->k < 1 || ix->k > 14) return -1;
    job_t jb;
    memset(&jb, 0, sizeof jb);
    jb.ix = ix;
    jb.reads = reads;
    jb.stride = stride;
    jb.lens = lens;
    jb.nreads = nreads;
    jb.e = e;
    jb.per = calloc(nreads ? nreads : 1, sizeof(oread_t));
    if (!jb.per) return -3;
    pthread_mutex_init(&jb.mu, NULL);
    if (nthreads <= 1) {
        worker(&jb);
    } else {
        pthread_t *th = malloc(sizeof(pthread_t) * nthreads);
        for (uint32_t t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, worker, &jb);
        for (uint32_t t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
        free(th);
    }
    pthread_mutex_destroy(&jb.mu);
    int rc = jb.bad ? -1 : 0;
    if (out) {
        out->n_records = 0;
        out->n_unmapped = 0;
        out->overflow = 0;
        for (uint64_t r = 0; r < nreads; r++) {
            oread_t *o = &jb.per[r];
            if (o->overflow) out->overflow = 1;
            size_t wp = 0, cp = 0;
            for (uint32_t q = 0; q < o->nrec; q++) {
                uint32_t nloc = o->w[wp + 1] & 0x7fffffffu;
                if (out->n_records < out->cap_records) {
                    uint32_t *dst = out->ref_pos + out->n_records * SWO_RECORD_WORDS;
                    memset(dst, 0, SWO_RECORD_WORDS * 4);
                    memcpy(dst, o->w + wp, (2 + (nloc < SWO_MAX_CIGAR ? nloc : SWO_MAX_CIGAR)) * 4);
                    uint8_t *cd = out->cigar + out->n_records * SWO_CIGAR_STRIDE;
                    memset(cd, 0, SWO_CIGAR_STRIDE);
                    uint32_t cl = o->clen[q] < SWO_CIGAR_STRIDE ? o->clen[q] : SWO_CIGAR_STRIDE;
                    memcpy(cd, o->c + cp, cl);
                } else {
                    out->overflow = 1;
                }
                out->n_records++;
                wp += 2 + nloc;
                cp += o->clen[q];
            }
            if (o->unmapped) {
                if (out->n_unmapped < out->cap_unmapped) out->unmapped[out->n_unmapped] = (uint32_t)(2 * r + 1);
                else out->overflow = 1;
                out->n_unmapped++;
            }
        }
        if (out->overflow && rc == 0) rc = -2;
    }
    for (uint64_t r = 0; r < nreads; r++) {
        free(jb.per[r].w);
        free(jb.per[r].c);
        free(jb.per[r].clen);
    }
    free(jb.per);
    if (stats) *stats = jb.st;
    return rc;
}

/*
 * swm_sam.c -- SAM text of mapping results (sam_header / sam_format_2,
 * mapper_mpe.c:315-687) and FASTA/FASTQ read blocks (the kseq reading of
 * mapper_mpe.c:935-960). Host code of libswmapper_gb300.so.
 */
#define _GNU_SOURCE
#include "swm_sam.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------ references */

int swm_refs_load(const char *prefix, swm_refs *r) {
    if (!prefix || !r) return SWM_ERR_ARG;
    memset(r, 0, sizeof *r);
    char path[4096];
    if (snprintf(path, sizeof path, "%s.ref_info", prefix) >= (int)sizeof path) return SWM_ERR_ARG;
    FILE *f = fopen(path, "r");
    if (!f) return SWM_ERR_IO;
    uint32_t cap = 16;
    r->name = (char **)calloc(cap, sizeof(char *));
    r->name_len = (uint32_t *)calloc(cap, sizeof(uint32_t));
    r->start = (uint32_t *)calloc(cap + 3, sizeof(uint32_t));
    int rc = (r->name && r->name_len && r->start) ? SWM_OK : SWM_ERR_OOM;
    char *line = NULL;
    size_t lcap = 0;
    ssize_t ln;
    uint64_t acc = 0;
    while (rc == SWM_OK && (ln = getline(&line, &lcap, f)) != -1) { /* length, name length, name */
        const uint64_t len = strtoull(line, NULL, 10);
        if (getline(&line, &lcap, f) == -1) { rc = SWM_ERR_IO; break; }
        if ((ln = getline(&line, &lcap, f)) == -1) { rc = SWM_ERR_IO; break; }
        if (ln > 0 && line[ln - 1] == '\n') line[--ln] = 0;
        if (r->n == cap) {
            cap *= 2;
            char **nn = (char **)realloc(r->name, cap * sizeof(char *));
            uint32_t *nl = (uint32_t *)realloc(r->name_len, cap * sizeof(uint32_t));
            uint32_t *ns = (uint32_t *)realloc(r->start, (cap + 3) * sizeof(uint32_t));
            if (nn) r->name = nn;
            if (nl) r->name_len = nl;
            if (ns) r->start = ns;
            if (!nn || !nl || !ns) { rc = SWM_ERR_OOM; break; }
        }
        r->name[r->n] = strdup(line);
        if (!r->name[r->n]) { rc = SWM_ERR_OOM; break; }
        r->name_len[r->n] = (uint32_t)ln;
        r->start[r->n] = (uint32_t)acc;
        acc += len;
        r->n++;
    }
    free(line);
    fclose(f);
    if (rc == SWM_OK) {
        /* starts n .. n + 2: the end, then zeros (get_ref_name looks two ahead) */
        r->start[r->n] = (uint32_t)acc;
        r->start[r->n + 1] = 0;
        r->start[r->n + 2] = 0;
    } else {
        swm_refs_free(r);
    }
    return rc;
}

void swm_refs_free(swm_refs *r) {
    if (!r) return;
    for (uint32_t i = 0; i < r->n; i++) free(r->name[i]);
    free(r->name);
    free(r->name_len);
    free(r->start);
    memset(r, 0, sizeof *r);
}

/* Chromosome of 1-based global position loc (get_ref_name, mapper_mpe.c:374-404):
 * the previous chromosome or the next one first, else its binary search. */
static uint32_t ref_of(const swm_refs *rf, uint32_t loc, uint32_t pre) {
    const uint32_t *s = rf->start;
    if (loc >= s[pre] && loc < s[pre + 1]) return pre;
    if (loc >= s[pre + 1] && loc < s[pre + 2]) return pre + 1;
    uint32_t left = 0, right = rf->n, mid = rf->n / 2;
    while (right > left) {
        if (loc < s[mid]) right = mid - 1;
        else if (loc > s[mid]) left = mid + 1;
        else return mid;
        mid = (left + right) / 2;
    }
    return loc < s[mid] ? mid - 1 : mid;
}

/* ------------------------------------------------------------ writer */

typedef struct {
    char *p;
    size_t n, cap;
} out_t;

static inline void put(out_t *o, const void *s, size_t len) {
    if (o->n + len <= o->cap) memcpy(o->p + o->n, s, len);
    o->n += len;
}
static inline void putc_(out_t *o, char c) {
    if (o->n < o->cap) o->p[o->n] = c;
    o->n++;
}
static inline void putu(out_t *o, uint32_t v) {
    char t[12];
    int i = 12;
    do {
        t[--i] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    put(o, t + i, (size_t)(12 - i));
}
#define PUTS(o, lit) put(o, lit, sizeof(lit) - 1)

int swm_sam_header(const swm_refs *rf, char *out, size_t cap, size_t *n) {
    if (!rf || !n || (!out && cap)) return SWM_ERR_ARG;
    out_t o = {out, 0, cap};
    PUTS(&o, "@HD\tVN:1.4\tSO:unsorted\n");
    for (uint32_t i = 0; i < rf->n; i++) {
        PUTS(&o, "@SQ\tSN:");
        put(&o, rf->name[i], rf->name_len[i]);
        PUTS(&o, "\tLN:");
        putu(&o, rf->start[i + 1] - rf->start[i]);
        putc_(&o, '\n');
    }
    PUTS(&o, "@PG\tID:XXX\tVN:1.0\tPN:XXX\tCL:\"CMDLINE\"\n");
    *n = o.n;
    return o.n <= cap ? SWM_OK : SWM_ERR_OVERFLOW;
}

static void put_seq_qual(out_t *o, const swm_read_block *b, uint64_t rd, int reverse) {
    const char *sq = b->seqs + rd * b->seq_stride;
    const uint32_t L = b->seq_len[rd];
    if (!reverse) {
        put(o, sq, L);
    } else { /* reverse_read, 350-373: A<->T, C<->G, anything else kept */
        for (uint32_t i = 0; i < L; i++) {
            const char c = sq[L - 1 - i];
            putc_(o, c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : c == 'T' ? 'A' : c);
        }
    }
    putc_(o, '\t');
    if (!b->have_qual) {
        putc_(o, '*');
    } else {
        const char *qu = b->quals + rd * b->seq_stride;
        if (!reverse) put(o, qu, L);
        else
            for (uint32_t i = 0; i < L; i++) putc_(o, qu[L - 1 - i]);
    }
}

int swm_sam_block(const swm_refs *rf, const swm_read_block *b, const swm_packed_result *r, char *out, size_t cap,
                  size_t *n) {
    if (!rf || !b || !r || !n || (!out && cap)) return SWM_ERR_ARG;
    out_t o = {out, 0, cap};
    for (uint64_t u = 0; u < r->n_unmapped; u++) { /* 436-461 */
        const uint64_t rd = r->unmapped[u] / 2;
        if (rd >= b->n) return SWM_ERR_ARG;
        put(&o, b->names + rd * b->name_stride, b->name_len[rd]);
        PUTS(&o, "\t4\t*\t0\t0\t*\t*\t0\t0\t");
        put_seq_qual(&o, b, rd, 0);
        putc_(&o, '\n');
    }
    const uint32_t *w = r->words;
    const uint8_t *cg = r->cigar;
    uint64_t wq = 0, cq = 0;
    for (uint64_t q = 0; q < r->n_records; q++) { /* 462-686 */
        if (wq + 2 > r->n_words) return SWM_ERR_ARG;
        const uint32_t cur = w[wq], word1 = w[wq + 1];
        const uint64_t rd = cur / 2;
        const int reverse = (int)(cur & 1u), primary = (int)(word1 >> 31);
        const uint32_t nloc = word1 & 0xfffffffu; /* the reference's 28-bit mask */
        if (rd >= b->n || wq + 2 + nloc > r->n_words) return SWM_ERR_ARG;
        uint32_t ri = 0;
        for (uint32_t j = 0; j < nloc; j++) {
            const uint32_t loc = w[wq + 2 + j];
            if (cq + 2 > r->n_cigar) return SWM_ERR_ARG;
            const uint32_t nm = cg[cq], cl = cg[cq + 1];
            if (cq + 2 + cl > r->n_cigar) return SWM_ERR_ARG;
            ri = ref_of(rf, loc, ri);
            if (ri >= rf->n) ri = rf->n - 1; /* past the last chromosome (padding): the last one */
            put(&o, b->names + rd * b->name_stride, b->name_len[rd]);
            putc_(&o, '\t');
            if (primary && j == 0) {
                if (reverse) PUTS(&o, "16");
                else putc_(&o, '0');
            } else {
                if (reverse) PUTS(&o, "272");
                else PUTS(&o, "256");
            }
            putc_(&o, '\t');
            put(&o, rf->name[ri], rf->name_len[ri]);
            putc_(&o, '\t');
            putu(&o, loc - rf->start[ri]);
            PUTS(&o, "\t255\t");
            put(&o, cg + cq + 2, cl);
            PUTS(&o, "\t*\t0\t0\t");
            if (primary && j == 0) {
                put_seq_qual(&o, b, rd, reverse);
                putc_(&o, '\t');
            } else {
                PUTS(&o, "*\t*\t");
            }
            PUTS(&o, "NM:i:");
            putc_(&o, (char)('0' + nm));
            PUTS(&o, "\tXM:i:");
            putc_(&o, (char)('0' + nm));
            putc_(&o, '\n');
            cq += 2 + cl;
        }
        wq += 2 + nloc;
    }
    *n = o.n;
    return o.n <= cap ? SWM_OK : SWM_ERR_OVERFLOW;
}

/* ------------------------------------------------------------ FASTA / FASTQ */

struct swm_fastx {
    FILE *f;
    char *line;
    size_t lcap;
    ssize_t llen;   /* the line read ahead (a header), or -1 */
};

int swm_fastx_open(const char *path, swm_fastx **out) {
    if (!path || !out) return SWM_ERR_ARG;
    swm_fastx *x = (swm_fastx *)calloc(1, sizeof *x);
    if (!x) return SWM_ERR_OOM;
    x->f = fopen(path, "r");
    if (!x->f) {
        free(x);
        return SWM_ERR_IO;
    }
    x->llen = -1;
    *out = x;
    return SWM_OK;
}

void swm_fastx_close(swm_fastx *x) {
    if (!x) return;
    if (x->f) fclose(x->f);
    free(x->line);
    free(x);
}

static ssize_t next_line(swm_fastx *x) {
    ssize_t n = getline(&x->line, &x->lcap, x->f);
    while (n > 0 && (x->line[n - 1] == '\n' || x->line[n - 1] == '\r')) x->line[--n] = 0;
    return n;
}

int swm_fastx_read_block(swm_fastx *x, swm_read_block *b) {
    if (!x || !b || !b->names || !b->name_len || !b->seqs || !b->seq_len) return SWM_ERR_ARG;
    b->n = 0;
    b->have_qual = 1;
    while (b->n < b->n_cap) {
        ssize_t n = x->llen >= 0 ? x->llen : next_line(x);
        x->llen = -1;
        while (n == 0) n = next_line(x); /* blank lines */
        if (n < 0) break;
        const char kind = x->line[0];
        if (kind != '>' && kind != '@') return SWM_ERR_IO;
        /* name: up to the first blank (kseq) */
        size_t nl = 1;
        while ((ssize_t)nl < n && x->line[nl] != ' ' && x->line[nl] != '\t') nl++;
        nl -= 1;
        if (nl > b->name_stride) nl = b->name_stride;
        const uint64_t rd = b->n;
        memcpy(b->names + rd * b->name_stride, x->line + 1, nl);
        b->name_len[rd] = (uint32_t)nl;
        char *sq = b->seqs + rd * b->seq_stride;
        uint64_t L = 0;
        for (;;) { /* sequence lines up to the next header / '+' */
            n = next_line(x);
            if (n < 0) break;
            if (n > 0 && (x->line[0] == '>' || x->line[0] == '@' || x->line[0] == '+')) break;
            if (L + (uint64_t)n > b->seq_stride) return SWM_ERR_ARG;
            memcpy(sq + L, x->line, (size_t)n);
            L += (uint64_t)n;
        }
        b->seq_len[rd] = (uint32_t)L;
        if (kind == '@') {
            if (n < 0 || x->line[0] != '+') return SWM_ERR_IO;
            uint64_t Q = 0; /* quality: exactly L characters, possibly over lines */
            while (Q < L) {
                n = next_line(x);
                if (n < 0) return SWM_ERR_IO;
                if (Q + (uint64_t)n > L) return SWM_ERR_IO;
                if (b->quals) memcpy(b->quals + rd * b->seq_stride + Q, x->line, (size_t)n);
                Q += (uint64_t)n;
            }
        } else {
            b->have_qual = 0;
            if (n >= 0) x->llen = n; /* the next header */
        }
        b->n++;
    }
    if (!b->quals || b->n == 0) b->have_qual = 0;
    return SWM_OK;
}

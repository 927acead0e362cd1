/*
 * swm_files.c -- index files and FASTA input on the host.
 *
 * FASTA handling follows what serial_index.c gets from kseq.h (kseq.h:198-237):
 * the record name is the first whitespace-delimited word of the header line,
 * the sequence is the concatenation of the following lines without '\n' and
 * with one trailing '\r' per line removed, up to the next line that starts
 * with '>', '@' or '+'. serial_index.c writes one `len\nnamelen\nname\n`
 * triple per record to .ref_info (serial_index.c:406-408) and indexes the
 * concatenation of all records as one stream.
 */
#include "swm_files.h"

#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    char *p;
    size_t n, cap;
} buf_t;

static int buf_reserve(buf_t *b, size_t extra) {
    if (b->n + extra + 1 <= b->cap) return 0;
    size_t nc = b->cap ? b->cap : 1 << 16;
    while (nc < b->n + extra + 1) nc *= 2;
    char *q = realloc(b->p, nc);
    if (!q) return -1;
    b->p = q;
    b->cap = nc;
    return 0;
}

static int buf_add(buf_t *b, const char *s, size_t len) {
    if (buf_reserve(b, len)) return -1;
    memcpy(b->p + b->n, s, len);
    b->n += len;
    b->p[b->n] = 0;
    return 0;
}

int swmf_read_fasta(const char *path, uint8_t **seq, uint64_t *n, char **info, size_t *info_len) {
    FILE *f = fopen(path, "rb");
    if (!f) return -2;
    buf_t s = {0}, ri = {0}, name = {0};
    char *line = NULL;
    size_t cap = 0;
    ssize_t got;
    int in_rec = 0, rc = 0;
    uint64_t rec0 = 0;
#define CLOSE_RECORD()                                                                              \
    do {                                                                                            \
        char hdr[64];                                                                               \
        int hn = snprintf(hdr, sizeof hdr, "%lu\n%lu\n", (unsigned long)(s.n - rec0),               \
                          (unsigned long)name.n);                                                   \
        if (buf_add(&ri, hdr, (size_t)hn) || buf_add(&ri, name.p ? name.p : "", name.n) ||          \
            buf_add(&ri, "\n", 1))                                                                  \
            rc = -3;                                                                                \
    } while (0)
    while (rc == 0 && (got = getline(&line, &cap, f)) != -1) {
        size_t len = (size_t)got;
        if (len > 0 && line[len - 1] == '\n') len--;
        if (len > 0 && (line[0] == '>' || line[0] == '@')) {
            if (in_rec) CLOSE_RECORD();
            in_rec = 1;
            rec0 = s.n;
            name.n = 0;
            size_t j = 1;
            while (j < len && !isspace((unsigned char)line[j])) j++;
            if (buf_add(&name, line + 1, j - 1)) rc = -3;
            continue;
        }
        if (!in_rec) continue; /* text before the first header is skipped */
        if (len > 0 && line[0] == '+') {
            /* '+' ends a FASTA record's sequence in kseq; such a file is not
             * FASTA, stop the record's sequence here */
            continue;
        }
        if (len == 0) continue;
        if (buf_add(&s, line, len)) {
            rc = -3;
            break;
        }
        if (s.n - rec0 > 1 && s.p[s.n - 1] == '\r') s.n--;
    }
    if (rc == 0 && in_rec) CLOSE_RECORD();
#undef CLOSE_RECORD
    free(line);
    free(name.p);
    fclose(f);
    if (rc) {
        free(s.p);
        free(ri.p);
        return rc;
    }
    *seq = (uint8_t *)(s.p ? s.p : calloc(1, 1));
    *n = s.n;
    *info = ri.p ? ri.p : calloc(1, 1);
    *info_len = ri.n;
    return 0;
}

int swmf_read(const char *prefix, const char *ext, void **data, size_t *bytes) {
    char path[4096];
    snprintf(path, sizeof path, "%s%s", prefix, ext);
    FILE *f = fopen(path, "rb");
    if (!f) return -2;
    if (fseek(f, 0, SEEK_END) != 0) {
        fclose(f);
        return -2;
    }
    long sz = ftell(f);
    if (sz < 0 || fseek(f, 0, SEEK_SET) != 0) {
        fclose(f);
        return -2;
    }
    void *p = malloc((size_t)sz + 16);
    if (!p) {
        fclose(f);
        return -3;
    }
    size_t r = sz ? fread(p, 1, (size_t)sz, f) : 0;
    fclose(f);
    if (r != (size_t)sz) {
        free(p);
        return -2;
    }
    *data = p;
    *bytes = (size_t)sz;
    return 0;
}

int swmf_write(const char *prefix, const char *ext, const void *data, size_t bytes) {
    char path[4096];
    snprintf(path, sizeof path, "%s%s", prefix, ext);
    FILE *f = fopen(path, "wb");
    if (!f) return -2;
    size_t w = bytes ? fwrite(data, 1, bytes, f) : 0;
    int ok = (w == bytes);
    if (fclose(f) != 0) ok = 0;
    return ok ? 0 : -2;
}

uint64_t swmf_ref_info_total(const char *info, size_t len) {
    uint64_t total = 0;
    size_t p = 0;
    int field = 0;
    while (p < len) {
        size_t q = p;
        while (q < len && info[q] != '\n') q++;
        if (field == 0) total += strtoull(info + p, NULL, 10);
        field = (field + 1) % 3;
        p = q + 1;
    }
    return total;
}

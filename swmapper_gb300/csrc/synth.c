/*
 * synth.c -- seeded synthetic genomes and reads with the shapes of the
 * benchmark workloads (uniform or GC-biased sequence, diverged repeat copies,
 * N runs; reads of fixed or uniform length with substitution / 1-bp indel
 * errors on both strands). Deterministic across machines: the generator is a
 * counter-based splitmix64 keyed by (seed, block), so x86 and Arm hosts make
 * the same bytes.
 */
#include "../../include/swm_synth.h"

#include <stdlib.h>
#include <string.h>

static inline uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

typedef struct {
    uint64_t s;
} rng_t;

static inline uint64_t rnext(rng_t *r) {
    r->s += 0x9e3779b97f4a7c15ull;
    uint64_t z = r->s;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
/* uniform in [0, 1) with 53 bits */
static inline double runif(rng_t *r) { return (double)(rnext(r) >> 11) * (1.0 / 9007199254740992.0); }
static inline uint64_t rrange(rng_t *r, uint64_t lo, uint64_t hi) { /* [lo, hi] */
    return lo + rnext(r) % (hi - lo + 1);
}

static const char ACGT[4] = {'A', 'C', 'G', 'T'};

static inline char rbase(rng_t *r, double gc) {
    double u = runif(r);
    if (u < gc) return (u < gc * 0.5) ? 'C' : 'G';
    return (u < gc + (1.0 - gc) * 0.5) ? 'A' : 'T';
}

static inline char other_base(rng_t *r, char b) {
    char c;
    do c = ACGT[rnext(r) & 3]; while (c == b);
    return c;
}

int swm_synth_reference(uint8_t *out, uint64_t n, const swm_synth_ref_cfg *cfg) {
    if (!out || !cfg) return -1;
    const uint64_t BLK = 1ull << 20;
    /* background, generated per 1 Mbp block so the result does not depend on
     * how the work is split */
    for (uint64_t b0 = 0; b0 < n; b0 += BLK) {
        rng_t r = {mix64(cfg->seed ^ mix64(b0 / BLK + 1))};
        uint64_t b1 = b0 + BLK < n ? b0 + BLK : n;
        for (uint64_t p = b0; p < b1; p++) out[p] = (uint8_t)rbase(&r, cfg->gc);
    }
    rng_t r = {mix64(cfg->seed ^ 0x5eed5eedull)};
    /* repeat families: each family is a consensus copied with substitutions
     * at a per-copy divergence drawn from [div_min, div_max] */
    uint64_t target = (uint64_t)(cfg->repeat_frac * (double)n);
    if (target > 0 && cfg->rep_len_max >= cfg->rep_len_min && cfg->rep_len_min > 0 &&
        cfg->rep_len_max < n) {
        const uint64_t avg = (cfg->rep_len_min + cfg->rep_len_max) / 2;
        uint64_t copies = cfg->copies_per_family ? cfg->copies_per_family : 8;
        uint64_t nfam = target / (avg * copies);
        if (nfam == 0) nfam = 1;
        uint64_t covered = 0, fam = 0;
        char *cons = malloc(cfg->rep_len_max);
        if (!cons) return -3;
        while (covered < target) {
            uint64_t flen = rrange(&r, cfg->rep_len_min, cfg->rep_len_max);
            for (uint64_t i = 0; i < flen; i++) cons[i] = rbase(&r, cfg->gc);
            for (uint64_t c = 0; c < copies && covered < target; c++) {
                uint64_t len = flen;
                if (len > n) len = n;
                uint64_t at = rrange(&r, 0, n - len);
                double div = cfg->div_min + (cfg->div_max - cfg->div_min) * runif(&r);
                for (uint64_t i = 0; i < len; i++) {
                    char b = cons[i];
                    if (runif(&r) < div) b = other_base(&r, b);
                    out[at + i] = (uint8_t)b;
                }
                covered += len;
            }
            fam++;
        }
        (void)nfam;
        (void)fam;
        free(cons);
    }
    /* N runs */
    uint64_t ntarget = (uint64_t)(cfg->n_frac * (double)n);
    if (ntarget > 0 && cfg->nrun_max >= cfg->nrun_min && cfg->nrun_min > 0) {
        uint64_t covered = 0;
        while (covered < ntarget) {
            uint64_t len = rrange(&r, cfg->nrun_min, cfg->nrun_max);
            if (len > ntarget - covered) len = ntarget - covered;
            if (len > n) len = n;
            uint64_t at = rrange(&r, 0, n - len);
            memset(out + at, 'N', len);
            covered += len;
        }
    }
    return 0;
}

int swm_synth_reads(const uint8_t *ref, uint64_t n, const swm_synth_read_cfg *cfg, char *reads, uint64_t stride,
                    uint32_t *lens, uint32_t *truth_pos, uint8_t *truth_strand) {
    if (!ref || !cfg || !reads || !lens || cfg->len_min == 0 || cfg->len_max < cfg->len_min ||
        cfg->len_max > stride || n < (uint64_t)cfg->len_max * 2 + 64)
        return -1;
    char fwd[1024];
    for (uint64_t q = 0; q < cfg->nreads; q++) {
        rng_t r = {mix64(cfg->seed ^ mix64(q + 0x1234567ull))};
        uint32_t L = (uint32_t)rrange(&r, cfg->len_min, cfg->len_max);
        uint64_t start = 0;
        int tries = 0;
        for (;;) {
            start = rrange(&r, 0, n - (uint64_t)L * 2 - 16);
            /* avoid reads that are mostly N */
            uint32_t nn = 0;
            for (uint32_t i = 0; i < L; i++) nn += ref[start + i] == 'N';
            if (nn * 10 <= L || ++tries > 64) break;
        }
        /* walk the reference applying errors: 70% substitution, 15% 1-bp
         * insertion, 15% 1-bp deletion */
        uint64_t p = start;
        uint32_t o = 0;
        while (o < L && p < n) {
            double u = runif(&r);
            if (u < cfg->err_rate) {
                double t = runif(&r);
                if (t < 0.70) {
                    fwd[o++] = other_base(&r, (char)ref[p]);
                    p++;
                } else if (t < 0.85) {
                    fwd[o++] = ACGT[rnext(&r) & 3];
                } else {
                    p++;
                }
            } else {
                fwd[o++] = (char)ref[p++];
            }
        }
        while (o < L) fwd[o++] = 'A';
        int rev = (rnext(&r) & 1) != 0;
        char *dst = reads + q * stride;
        if (rev) {
            for (uint32_t i = 0; i < L; i++) {
                char c = fwd[i], rc;
                switch (c) {
                case 'A': rc = 'T'; break;
                case 'C': rc = 'G'; break;
                case 'G': rc = 'C'; break;
                case 'T': rc = 'A'; break;
                default: rc = c; break;
                }
                dst[L - 1 - i] = rc;
            }
        } else {
            memcpy(dst, fwd, L);
        }
        if (stride > L) memset(dst + L, 0, stride - L);
        lens[q] = L;
        if (truth_pos) truth_pos[q] = (uint32_t)start;
        if (truth_strand) truth_strand[q] = (uint8_t)rev;
    }
    return 0;
}

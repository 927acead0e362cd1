/*
 * swm_synth.h -- seeded synthetic workloads (libswm_synth.so).
 *
 * Not part of the reference interface: the reference ships no data, so the
 * benchmark and the tests generate genomes and reads with the shapes the
 * workloads name (sizes, GC content, repeat copies, N runs, read lengths and
 * error mix). The bytes depend only on the configuration and the seed.
 */
#ifndef SWM_SYNTH_H
#define SWM_SYNTH_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    uint64_t seed;
    double gc;                  /* G+C fraction of the background            */
    double repeat_frac;         /* fraction of the genome made of copies     */
    uint64_t rep_len_min, rep_len_max; /* family consensus length range      */
    uint64_t copies_per_family; /* copies written per family                 */
    double div_min, div_max;    /* per-copy substitution divergence range    */
    double n_frac;              /* fraction of the genome in N runs          */
    uint64_t nrun_min, nrun_max;/* N run length range                        */
} swm_synth_ref_cfg;

typedef struct {
    uint64_t seed;
    uint64_t nreads;
    uint32_t len_min, len_max;  /* read length, uniform in [min, max]        */
    double err_rate;            /* per-base error probability                */
} swm_synth_read_cfg;

/* Fill out[0..n) with A/C/G/T/N bytes. Returns 0 on success. */
int swm_synth_reference(uint8_t *out, uint64_t n, const swm_synth_ref_cfg *cfg);

/* Sample cfg->nreads reads from ref into a fixed-stride buffer (zero padded
 * to the stride), their lengths into lens, and optionally the true start and
 * strand (1 = reverse complement). Returns 0 on success. */
int swm_synth_reads(const uint8_t *ref, uint64_t n, const swm_synth_read_cfg *cfg, char *reads,
                    uint64_t stride, uint32_t *lens, uint32_t *truth_pos, uint8_t *truth_strand);

#ifdef __cplusplus
}
#endif
#endif

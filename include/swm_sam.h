/*
 * swm_sam.h -- SAM text of mapping results and FASTA/FASTQ read blocks
 * (host side of libswmapper_gb300.so).
 *
 * The SAM writer restates sam_header / sam_format_2 (mapper_mpe.c:315-687)
 * for the packed results of swm_map_wait_packed: the same header lines, one
 * line per reported location with the reference's flags (0 / 256 forward,
 * 16 / 272 reverse), POS within the record's chromosome (get_ref_name,
 * mapper_mpe.c:374-404), MAPQ 255, the CIGAR text, SEQ / QUAL on the primary
 * line only (reverse complemented for the reverse strand, reverse_read
 * 350-373), NM:i / XM:i as the single character '0' + NM, and one line per
 * unmapped read (flag 4). Lines come unmapped reads first, then records, in
 * read order (the reference's order follows its CPE queue).
 *
 * The block reader fills the fixed-stride buffers the mapper takes from
 * FASTA or FASTQ text (the kseq parsing of mapper_mpe.c:935-960): name up to
 * the first blank, sequence lines joined, quality for FASTQ ('*'-free: a
 * FASTA record gets no quality).
 */
#ifndef SWM_SAM_H
#define SWM_SAM_H
#include <stddef.h>
#include <stdint.h>

#include "swmapper.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Chromosomes of an index: the .ref_info text (serial_index.c:406-408). */
typedef struct {
    uint32_t n;            /* chromosomes                                    */
    char **name;           /* n names (NUL terminated)                        */
    uint32_t *name_len;
    uint32_t *start;       /* n + 1 cumulative starts: ref_len of mapper_mpe.c */
} swm_refs;

/* Parse <prefix>.ref_info into r (free with swm_refs_free). */
int swm_refs_load(const char *prefix, swm_refs *r);
void swm_refs_free(swm_refs *r);

/* A block of reads in the mapper's fixed-stride layout (mapper_mpe.c:779-789). */
typedef struct {
    char *names;           /* n_cap * name_stride                            */
    uint32_t *name_len;
    char *seqs;            /* n_cap * seq_stride (the mapper's reads)        */
    char *quals;           /* n_cap * seq_stride (FASTQ only; else '*' lines) */
    uint32_t *seq_len;     /* the mapper's reads_len                          */
    uint64_t name_stride, seq_stride, n_cap, n;
    int have_qual;         /* 1 when every read of the block had a quality    */
} swm_read_block;

typedef struct swm_fastx swm_fastx;

/* Open a FASTA / FASTQ file for block reading. */
int swm_fastx_open(const char *path, swm_fastx **out);
/* Fill b with up to b->n_cap reads (b->n gets the count; 0 at the end).
 * Returns SWM_ERR_ARG for a read longer than seq_stride, SWM_ERR_IO for a
 * truncated record. */
int swm_fastx_read_block(swm_fastx *f, swm_read_block *b);
void swm_fastx_close(swm_fastx *f);

/* SAM header text (sam_header, mapper_mpe.c:315-337) into out; *n gets its
 * length. SWM_ERR_OVERFLOW (and the needed size in *n) when cap is short. */
int swm_sam_header(const swm_refs *refs, char *out, size_t cap, size_t *n);

/* SAM lines of one mapped block (packed results of swm_map_wait_packed /
 * swm_map_fetch_packed for the reads of b) into out; *n gets the length.
 * SWM_ERR_OVERFLOW (and the needed size in *n) when cap is short. */
int swm_sam_block(const swm_refs *refs, const swm_read_block *b, const swm_packed_result *r, char *out, size_t cap,
                  size_t *n);

#ifdef __cplusplus
}
#endif
#endif

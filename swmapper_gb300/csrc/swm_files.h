/* swm_files.h -- host-side file handling of the index (C). */
#ifndef SWM_FILES_H
#define SWM_FILES_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* FASTA -> concatenated bases and the .ref_info text (serial_index.c:396-420
 * with kseq.h:198-237 FASTA semantics). Caller frees *seq and *info. */
int swmf_read_fasta(const char *path, uint8_t **seq, uint64_t *n, char **info, size_t *info_len);

/* Whole-file read / write of <prefix><ext>. */
int swmf_read(const char *prefix, const char *ext, void **data, size_t *bytes);
int swmf_write(const char *prefix, const char *ext, const void *data, size_t bytes);

/* Total bases listed in a .ref_info text (len / namelen / name triples). */
uint64_t swmf_ref_info_total(const char *info, size_t len);

#ifdef __cplusplus
}
#endif
#endif

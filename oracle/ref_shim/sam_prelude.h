/* sam_prelude.h -- host stand-ins for the SAM writer of the reference's
 * mapper_mpe.c (sam_header .. sam_format_2, 315-687), compiled on the host by
 * oracle/build_ref.sh (TEST INFRASTRUCTURE). zlib's gzwrite / gzprintf become
 * appends to a memory buffer (swref_sam_out), so the text can be compared
 * with the library's SAM writer; the globals the functions read are the ones
 * mapper_mpe.c declares at 142-180. */
#ifndef SWM_SAM_PRELUDE_H
#define SWM_SAM_PRELUDE_H
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "fm_define.h"

typedef void *gzFile;
int swref_gzwrite(void *f, const void *buf, unsigned len);
int swref_gzprintf(void *f, const char *fmt, ...);
#define gzwrite swref_gzwrite
#define gzprintf swref_gzprintf

extern gzFile *sam_ptr;
extern index_t max_match_size;
extern sindex_t ref_len[500];
extern sindex_t ref_name_len[500];
extern char ref_name[500][25];
extern sindex_t ref_num;
extern index_t cigar_block_size_pre;
extern index_t cigar_unmap_size_pre;
#endif

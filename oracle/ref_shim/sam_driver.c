/* sam_driver.c -- runs the reference's own sam_header and sam_format_2
 * (mapper_mpe.c:315-687, compiled on the host by oracle/build_ref.sh) on one
 * block of results in the reference's strided layout and returns the SAM
 * text. TEST INFRASTRUCTURE: the pinning test of the library's SAM writer. */
#include "sam_prelude.h"

gzFile *sam_ptr;
index_t max_match_size;
sindex_t ref_len[500];
sindex_t ref_name_len[500];
char ref_name[500][25];
sindex_t ref_num;
index_t cigar_block_size_pre;
index_t cigar_unmap_size_pre;

void sam_header(void);
void sam_format_2(char *reads_name, char *reads_seq, char *reads_qual, char *cigar_buffer, sindex_t *ref_pos,
                  sindex_t *reads_name_len, sindex_t *reads_seq_len, sindex_t *cigar_num2, index_t reads_size,
                  sindex_t read_name_max_len, sindex_t read_seq_max_len);

static char *g_out;
static size_t g_cap, g_n;

int swref_gzwrite(void *f, const void *buf, unsigned len) {
    (void)f;
    if (g_n + len <= g_cap) memcpy(g_out + g_n, buf, len);
    g_n += len;
    return (int)len;
}

int swref_gzprintf(void *f, const char *fmt, ...) {
    char tmp[4096];
    va_list ap;
    va_start(ap, fmt);
    int n = vsnprintf(tmp, sizeof tmp, fmt, ap);
    va_end(ap);
    if (n > 0) swref_gzwrite(f, tmp, (unsigned)n);
    return n;
}

/* Chromosomes (lengths, names), then the block; returns the text length
 * (more than cap when cap is short). */
size_t swref_sam(uint32_t nref, const uint32_t *lens, const char *names, uint32_t name_stride,
                 const uint32_t *name_lens, char *reads_name, char *reads_seq, char *reads_qual,
                 char *cigar_buffer, uint32_t *ref_pos, uint32_t *rname_len, uint32_t *rseq_len,
                 uint32_t *unmapped, uint64_t n_unmapped, uint64_t n_records, uint64_t reads_size,
                 uint32_t read_name_max_len, uint32_t read_seq_max_len, char *out, size_t cap) {
    g_out = out;
    g_cap = cap;
    g_n = 0;
    ref_num = nref;
    ref_len[0] = 0;
    for (uint32_t i = 0; i < nref; i++) { /* load_ref_info, mapper_mpe.c:198-240 */
        ref_len[i + 1] = ref_len[i] + lens[i];
        ref_name_len[i] = name_lens[i];
        memcpy(ref_name[i], names + (size_t)i * name_stride, name_lens[i]);
        ref_name[i][name_lens[i]] = 0;
    }
    cigar_unmap_size_pre = n_unmapped;
    cigar_block_size_pre = n_records;
    sam_header();
    sam_format_2(reads_name, reads_seq, reads_qual, cigar_buffer, ref_pos, rname_len, rseq_len, unmapped,
                 reads_size, read_name_max_len, read_seq_max_len);
    return g_n;
}

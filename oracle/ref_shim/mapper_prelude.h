/* mapper_prelude.h -- host stand-ins for the Sunway CPE environment of the
 * reference's mapper_cpe.c (TEST INFRASTRUCTURE). oracle/build_ref.sh cuts
 * the scalar functions of mapper_cpe.c out of the reference tree and compiles
 * them with this prelude: DMA becomes memcpy, the scalar banded Myers is
 * selected (SIMD_BM / SIMD_BM_ASM left undefined), every other compile-time
 * switch keeps its value from mapper_cpe.c:24-32. */
#ifndef SWM_MAPPER_PRELUDE_H
#define SWM_MAPPER_PRELUDE_H
#include <assert.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include "fm_define.h"
#include "ub_defined.h"

#define READ_LEN 256
#define SIMD_WIDTH 8
#define MAXERROR 10000
#define word_t uint32_t
#define WORD_BITS 32
#define READ_INT_LEN (256 / 16)
#define BALANCE
#define DMA_ASYN
#define LSEED_FILTER
#define SORT_POS
#define OUT_CIGAR

#define dma_declare()
#define dma_syn() ((void)0)
#define pe_get(mem, ldm, size) memcpy((void *)(ldm), (const void *)(mem), (size_t)(size))
#define pe_put(mem, ldm, size) memcpy((void *)(mem), (const void *)(ldm), (size_t)(size))
typedef long dma_desc;
/* 256-bit Sunway vector, used by banded_myers only as storage */
typedef struct {
    uint32_t v[8];
} __attribute__((aligned(32))) uintv8;
#define DMA_GET 0
#define dma_set_op(d, op) ((void)0)
#define dma_set_reply(d, r) ((void)0)
#define dma_set_size(d, s) (*(d) = (long)(s))
#define dma_rpl(desc, mem, ldm, reply)                                   \
    do {                                                                 \
        memcpy((void *)(ldm), (const void *)(mem), (size_t)(desc));      \
        (reply)++;                                                       \
    } while (0)
#endif

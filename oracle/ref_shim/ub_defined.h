/* ub_defined.h -- gives the reference's `y << (32 - s)` idiom a defined
 * result of 0 at s == 0 (it is undefined in C; x86 computes y << 0). Used by
 * oracle/build_ref.sh when it builds the reference source for the pinning
 * tests (TEST INFRASTRUCTURE). */
#ifndef SWM_UB_DEFINED_H
#define SWM_UB_DEFINED_H
#include <stdint.h>
#define ZMASK(n) (((uint64_t)(n) >= 32u) ? 0u : 0xffffffffu)
/* traceback bit lookup with an out-of-range shift reading 0 */
#define TBBIT(x, s) ((((long)(s)) >= 0 && ((long)(s)) < 32) ? (((x) >> (s)) & 1u) : 0u)
#endif

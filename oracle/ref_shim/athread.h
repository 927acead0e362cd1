/* athread.h -- host stand-in for the Sunway athread runtime, so that the
 * reference's serial_index.c compiles on a CPU for the pinning tests
 * (TEST INFRASTRUCTURE). serial_index.c only spawns CPE work on its
 * non-default path (construct_hash_index_cpe); these no-ops drop it. */
#ifndef SWM_ATHREAD_SHIM_H
#define SWM_ATHREAD_SHIM_H
#include <ctype.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
void *__real_malloc(size_t size);
static inline void athread_init(void) {}
#define athread_spawn(fn, arg) ((void)(arg))
#define athread_join() ((void)0)
#endif

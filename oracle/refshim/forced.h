/* Force-included into every in-place compile of the reference sources:
 * prototypes the reference uses without declaring (it was built with the
 * Intel compiler, which provides them implicitly).  Without these, C would
 * assume int returns and truncate pointers. */
#ifndef REFSHIM_FORCED_H
#define REFSHIM_FORCED_H
#include <stddef.h>
#include <stdlib.h>
#include <alloca.h>
void *_mm_malloc(size_t size, size_t align);
void _mm_free(void *p);
/* Intel offload placement attribute (local_barrier.c/.h): no meaning here */
#define __declspec(x)
#endif

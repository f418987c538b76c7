/* Host stand-ins for the two CUDA runtime calls the reference's USE_CPU_ONLY
 * programs still make (examples/advection_2d/main.cpp:117-132): managed
 * allocations become plain heap allocations, so no GPU is needed. */
#include <stdlib.h>
int cudaMallocManaged(void** p, size_t n, unsigned int flags) {
  (void)flags;
  *p = calloc(n, 1);
  return *p ? 0 : 2;
}
int cudaFree(void* p) {
  free(p);
  return 0;
}

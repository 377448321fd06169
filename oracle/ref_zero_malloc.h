/* Test infrastructure only (oracle build).  Force-included (-include) into
 * the reference's CPU sources: their malloc calls become zero-filled
 * allocations, which makes reads of never-written slots deterministic (see
 * Makefile).  The C/C++ standard headers are included first so that their
 * own declarations are not renamed. */
#include <stdlib.h>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <omp.h>
extern "C" void* ref_zero_malloc(size_t n);
#define malloc ref_zero_malloc

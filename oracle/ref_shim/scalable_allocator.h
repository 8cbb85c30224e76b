/* Stand-in for TBB's scalable allocator header, which the reference includes
 * (BRMerge-SpGEMM/inc/utils.h:3) but which is not installed here: the two
 * functions the reference calls map onto the C heap. */
#ifndef BRM_REF_SHIM_SCALABLE_ALLOCATOR_H
#define BRM_REF_SHIM_SCALABLE_ALLOCATOR_H
#include <cstdlib>
inline void *scalable_malloc(size_t bytes) { return std::malloc(bytes); }
inline void scalable_free(void *p) { std::free(p); }
#endif

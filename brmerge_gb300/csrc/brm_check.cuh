// brm_check.cuh -- bounds checks of the checked device build (-DBRM_CHECKED).
//
// In a checked build BRM_IN(cnt, index, bound) tests 0 <= index < bound;
// when it fails it ORs kErrChecked into the device error word, records the
// first failure (source line, index, bound) in the counters and yields
// false, and the caller skips the access, so the kernel finishes and the call
// returns BRM_ERR_INTERNAL (brm_last_check_failure names the line).  It
// never traps.  In the normal build it is `true` and costs nothing.  The
// guards sit on the accesses whose index comes from data: writes into C, the
// scratch arrays, the segment descriptors and split table, shared-memory
// slots indexed by computed ranks, and gathers from B.
#pragma once

#include "brm_plan.h"

namespace brm {

#ifdef BRM_CHECKED
constexpr bool kCheckedBuild = true;

__device__ __noinline__ inline void check_failed(Counters *c, int line, long long idx,
                                                 long long bound)
{
    atomicOr(&c->err, kErrChecked);
    if (atomicCAS(&c->chk_line, 0, line) == 0) {
        c->chk_idx = idx;
        c->chk_bound = bound;
    }
}

#define BRM_IN(cnt, idx, bound)                                                           \
    ((unsigned long long)(long long)(idx) < (unsigned long long)(long long)(bound)        \
         ? true                                                                           \
         : (::brm::check_failed((cnt), __LINE__, (long long)(idx), (long long)(bound)), \
            false))
#else
constexpr bool kCheckedBuild = false;
#define BRM_IN(cnt, idx, bound) true
#endif

}  // namespace brm

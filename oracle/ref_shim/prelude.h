/* Forced-include prelude for building the reference's BRMerge path unmodified.
 * It stands in for BRMerge-SpGEMM/inc/common.h, whose timer reads the x86 TSC
 * with inline assembly and cpuid (common.h:17-47): that neither builds on an
 * Arm host nor gives a usable frequency on a VM.  Defining the header guard
 * _Z_COMMON_ first makes the reference's own #include "common.h" a no-op; this
 * file provides the same includes and a wall-clock fast_clock_time(). */
#ifndef BRM_REF_PRELUDE_H
#define BRM_REF_PRELUDE_H
#define _Z_COMMON_
#include "define.h"
#include <stdio.h>
#include <stdlib.h>
#include <omp.h>
#include <algorithm>
#include <numeric>
#include <cmath>
#include <cassert>
#include <cstring>
#include <stdexcept>
#include <string>
#include "Timings.h"
#include "utils.h"
inline double fast_clock_time() { return omp_get_wtime(); }
#endif

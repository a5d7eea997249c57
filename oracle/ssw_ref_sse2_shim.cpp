// ssw_ref_sse2_shim.cpp -- compiles the reference's SSW core through oracle/sse2_shim/.
//
// TEST INFRASTRUCTURE ONLY (the timed CPU baseline and its parity check).  The
// reference's src/ssw/ssw_core.cpp takes its SSE2 branch only where __x86_64__ is
// defined.  This unit includes every system header that source uses first, then
// defines __x86_64__ (when the host does not) and includes the source unmodified, so
// its intrinsics resolve to oracle/sse2_shim/emmintrin.h (NEON on aarch64).  The
// include path (-I) names the directory holding the reference sources; oracle/Makefile
// builds this into oracle/_ref/ (git-ignored) together with ssw.cpp and ssw_ref_shim.cpp.
#include <assert.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <string>
#include <vector>

#include "emmintrin.h"  // oracle/sse2_shim (first on the include path)

#ifndef __x86_64__
#define __x86_64__ 1
#define MHSW_DEFINED_X86_64
#endif
#include "ssw_core.cpp"
#ifdef MHSW_DEFINED_X86_64
#undef __x86_64__
#endif

/* Pre-included into every reference translation unit of the oracle build.
 * It supplies the few MSVC-only names the reference's sources use, and the
 * CUDA runtime declarations its SoA containers name (never called on the CPU
 * path), and gives unqualified abs() the meaning it has on the reference's
 * own Windows build.  Oracle build only. */
#pragma once
#include <cstdlib>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <ctime>
#include <cuda_runtime.h>
using std::isnan;
/* MSVC declares the floating-point overloads of abs() in the global
 * namespace, so the reference's unqualified abs(double) calls (e.g.
 * FVMR/src/time/CalculateDt.cpp:48, space/convection/Roe.cpp:480-482) take
 * |x| there.  With glibc alone only C's int abs(int) would be found and the
 * argument truncated; this brings the same overloads into scope. */
using std::abs;
#ifndef _countof
#define _countof(a) (sizeof(a) / sizeof((a)[0]))
#endif
#define sprintf_s snprintf
static inline int localtime_s(struct tm* out, const time_t* t) { return localtime_r(t, out) ? 0 : 1; }

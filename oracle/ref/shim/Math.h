/* On the reference's Windows build, `#include "Math.h"` from FVMR/src/legacy
 * (FVM_2D.h:5, Edge_2D.cpp:3) falls through to the C library's <math.h>
 * because the file system ignores case.  This header reproduces that lookup
 * on Linux.  Oracle build only. */
#pragma once
#include <cmath>

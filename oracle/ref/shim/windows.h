/* Linux stand-in for <windows.h> as named by FVMR/src/output/ConsolePrinter.h:4.
 * That header only needs COORD, which FVMR/src/legacy/head.h:31-36 already
 * declares for Linux, so this file includes it instead of declaring a second
 * one.  Oracle build only. */
#pragma once
#include "legacy/head.h"
typedef void* HANDLE;

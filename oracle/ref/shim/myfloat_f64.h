/* Pre-included ahead of the reference sources to build its CPU path with
 * `myfloat` = double.  It claims the include guard of
 * FVMR/src/gpu/datatype/DefineType.h (lines 1-2) and restates that header's
 * four declarations (lines 12-17) with double, so no reference file is
 * edited.  Oracle build only. */
#pragma once
#define DEFINE_TYPE_H
using myfloat = double;
using integer = int;
using myint = integer;
typedef void (*func_bin_myfloat)(myfloat&, const myfloat&);

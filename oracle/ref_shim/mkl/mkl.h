/* Stand-in for <mkl.h> in Code/OutputNu/stdafx.h.  The receiver-evaluation
 * sources built against it (T_Brick.cpp, OutputArbitrary.cpp, For_Solvers.cpp,
 * in_out.cpp) call no MKL routine.  The smoothing sources (OutputResultant3d,
 * Subdomain, FormatConverter) name MKL's 64-bit integer type; their PARDISO
 * calls go to oracle/ref_shim/pardiso_shim.cpp instead of MKL. */
#pragma once
#include <cstdio>
/* glibc's own 64-bit type, spelled without `long` (llp64.h maps that
 * keyword to int once the system headers are in) */
typedef __int64_t MKL_INT64;

/* Stand-in for <mkl.h> in Code/OutputNu/stdafx.h.  The receiver-evaluation
 * sources built against it (T_Brick.cpp, OutputArbitrary.cpp, For_Solvers.cpp,
 * in_out.cpp) call no MKL routine; the PARDISO smoothing path that does is not
 * built. */
#pragma once

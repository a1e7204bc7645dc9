/* Shim: Accelerate umbrella header -> the LAPACK/BLAS shims. Test only. */
#pragma once
#include <vecLib/blas_new.h>
#include <vecLib/lapack.h>

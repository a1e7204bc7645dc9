/* Shim for building the reference's CPU path on Linux: Accelerate's LAPACK
 * integer types mapped onto the LP64 OpenBLAS bundled with scipy.
 * Test infrastructure only (oracle/_ref); never linked into the product. */
#pragma once
typedef int __LAPACK_int;
typedef int __LAPACK_bool;

/*
 * Test infrastructure only (never linked into the product library).
 *
 * Macro shim that lets the reference's OpenCL C step kernels
 * (D3Q19_opencl/kernel.cl, D3Q27_opencl/kernel.cl) compile as plain C11 so
 * the reference arithmetic can be executed on the host as the parity oracle
 * and as the timed CPU baseline.  Each OpenCL work-item becomes one call of
 * the kernel function with a thread-local global id.
 *
 * REF_REAL selects the arithmetic type of the build: float (the reference's
 * FP32 path) or double (the FP64 oracle build; the build script passes
 * -Dfloat=double, so min/max must map to the double functions).
 */
#ifndef LBFFS_REF_SHIM_H
#define LBFFS_REF_SHIM_H

#include <math.h>
#include <stdbool.h>
#include <stdint.h>

#define __kernel
#define __global
#define __local
#define __constant const
#define inline static inline

typedef unsigned int uint;

extern __thread int lbffs_ref_gid;
#define get_global_id(dim) (lbffs_ref_gid)

#ifdef REF_DOUBLE
#define min(a, b) fmin((a), (b))
#define max(a, b) fmax((a), (b))
#else
#define min(a, b) fminf((a), (b))
#define max(a, b) fmaxf((a), (b))
#endif

/* 32-bit compare-and-swap; only used by the reference's float atomic add. */
#define atom_cmpxchg(p, cmp, val) __sync_val_compare_and_swap((p), (cmp), (val))

#endif

// One instantiation unit of the fused step kernels.  The build compiles this file once per
// (lattice LBFFS_Q, storage LBFFS_S, collision LBFFS_C, part LBFFS_PART) so every heavy template
// instantiation compiles in parallel; step_dispatch.cu selects among them at run time.
//   LBFFS_PART 0: k_bulk, Smagorinsky with LES off;  1: k_bulk, Smagorinsky with LES on;
//              2: k_bulk, WALE;                      3: k_special
#include "launch.h"
#include "step_kernels.cuh"

#if !defined(LBFFS_Q) || !defined(LBFFS_S) || !defined(LBFFS_C) || !defined(LBFFS_PART)
#error "LBFFS_Q, LBFFS_S, LBFFS_C and LBFFS_PART must be defined by the build"
#endif

#define LBFFS_NAME2(q, s, c, p) launch_step_q##q##_s##s##_c##c##_p##p
#define LBFFS_NAME(q, s, c, p) LBFFS_NAME2(q, s, c, p)

namespace lbffs {

cudaError_t LBFFS_NAME(LBFFS_Q, LBFFS_S, LBFFS_C, LBFFS_PART)(const StepArgs& a, cudaStream_t st)
{
#if LBFFS_PART == 3
    if (a.n_special <= 0) return cudaSuccess;
#if LBFFS_Q == 19
    if (a.special_kind == 1) {
        constexpr int per = SPECIAL_BS / LBFFS_SPECIAL_LANES;
        const dim3 grid((unsigned)((a.n_special + per - 1) / per));
        k_special_warp<LBFFS_Q, LBFFS_S, LBFFS_C><<<grid, SPECIAL_BS, 0, st>>>(a);
        return cudaGetLastError();
    }
#endif
    const dim3 grid((unsigned)((a.n_special + SPECIAL_BS - 1) / SPECIAL_BS));
    k_special<LBFFS_Q, LBFFS_S, LBFFS_C><<<grid, SPECIAL_BS, 0, st>>>(a);
#else
    constexpr int V = bulk_v<LBFFS_Q, LBFFS_C, LBFFS_PART == 2 ? SGS_WALE : SGS_SMAG>();
    const dim3 grid((a.nx + BULK_BX * V - 1) / (BULK_BX * V), a.ny, a.nz);
    constexpr int SGS = LBFFS_PART == 2 ? SGS_WALE : SGS_SMAG;
    constexpr bool LES = LBFFS_PART == 1;
    if (a.border_pulls == 3) {  // x-face cells write their ghost slots
        k_bulk<LBFFS_Q, LBFFS_S, LBFFS_C, SGS, LES, 2><<<grid, BULK_BX, 0, st>>>(a);
        return cudaGetLastError();
    }
    // the x-face pull kernels where they are built (xface_pulls_built: D3Q19, FP32 D3Q27)
#if LBFFS_Q == 19 || LBFFS_S == 0
    static_assert(xface_pulls_built(LBFFS_Q, LBFFS_S), "x-face pull kernel list");
    if (a.border_pulls == 2) {
        k_bulk<LBFFS_Q, LBFFS_S, LBFFS_C, SGS, LES, 1><<<grid, BULK_BX, 0, st>>>(a);
        return cudaGetLastError();
    }
#else
    static_assert(!xface_pulls_built(LBFFS_Q, LBFFS_S), "x-face pull kernel list");
    if (a.border_pulls == 2) return cudaErrorInvalidValue;  // the context never selects a mode without its kernel
#endif
    k_bulk<LBFFS_Q, LBFFS_S, LBFFS_C, SGS, LES, 0><<<grid, BULK_BX, 0, st>>>(a);
#endif
    return cudaGetLastError();
}

}  // namespace lbffs

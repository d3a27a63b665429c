// One instantiation unit of the fused step kernels.  The build compiles this file once
// per (lattice LBFFS_Q, storage LBFFS_S, part LBFFS_PART) so the heavy template
// instantiations compile in parallel; step_dispatch.cu selects among them at run time.
#include "launch.h"
#include "step_kernels.cuh"

#ifndef LBFFS_Q
#error "LBFFS_Q, LBFFS_S and LBFFS_PART must be defined by the build"
#endif

#define LBFFS_CAT2(a, b, c, d) launch_##a##_q##b##_s##c##_##d
#define LBFFS_CAT(a, b, c, d) LBFFS_CAT2(a, b, c, d)

namespace lbffs {

#if LBFFS_PART == 0
template <int COLL>
static void bulk_c(const StepArgs& a, const StepConfig& c, cudaStream_t st)
{
    const dim3 grid((a.nx + BULK_BX - 1) / BULK_BX, a.ny, a.nz);
    if (c.sgs == SGS_WALE) k_bulk<LBFFS_Q, LBFFS_S, COLL, SGS_WALE, false><<<grid, BULK_BX, 0, st>>>(a);
    else if (c.les) k_bulk<LBFFS_Q, LBFFS_S, COLL, SGS_SMAG, true><<<grid, BULK_BX, 0, st>>>(a);
    else k_bulk<LBFFS_Q, LBFFS_S, COLL, SGS_SMAG, false><<<grid, BULK_BX, 0, st>>>(a);
}

cudaError_t LBFFS_CAT(bulk, LBFFS_Q, LBFFS_S, inst)(const StepArgs& a, const StepConfig& c, cudaStream_t st)
{
#if LBFFS_Q == 27
    if (c.collision == COLL_CUMULANT) bulk_c<COLL_CUMULANT>(a, c, st);
    else
#endif
        bulk_c<COLL_RR>(a, c, st);
    return cudaGetLastError();
}
#else
cudaError_t LBFFS_CAT(special, LBFFS_Q, LBFFS_S, inst)(const StepArgs& a, const StepConfig& c, cudaStream_t st)
{
    if (a.n_special <= 0) return cudaSuccess;
    const dim3 grid((unsigned)((a.n_special + SPECIAL_BS - 1) / SPECIAL_BS));
#if LBFFS_Q == 27
    if (c.collision == COLL_CUMULANT) k_special<LBFFS_Q, LBFFS_S, COLL_CUMULANT><<<grid, SPECIAL_BS, 0, st>>>(a);
    else
#endif
        k_special<LBFFS_Q, LBFFS_S, COLL_RR><<<grid, SPECIAL_BS, 0, st>>>(a);
    return cudaGetLastError();
}
#endif

}  // namespace lbffs

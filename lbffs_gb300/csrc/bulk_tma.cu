// Launchers of the warp-specialised D3Q19 bulk kernel (bulk_tma.cuh), compiled once per
// storage format (LBFFS_S).  The grid is persistent: as many CTAs as fit on the device at once,
// each walking the row tiles with a stride of the grid size.
#include "bulk_tma.cuh"
#include "launch.h"

#ifndef LBFFS_S
#error "compile with -DLBFFS_S=<storage>"
#endif

#define LBFFS_CAT2(a, b) a##b
#define LBFFS_CAT(a, b) LBFFS_CAT2(a, b)

namespace lbffs {
namespace {

template <int SGS, bool LES>
cudaError_t run(const StepArgs& a, cudaStream_t st)
{
    constexpr int S = LBFFS_S;
    using L = RingLayout<S>;
    auto kern = k_bulk_tma<S, SGS, LES>;
    // per process: the kernel's shared-memory opt-in and its resident CTAs per SM
    static int per_sm = 0;
    if (per_sm == 0) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L::SMEM);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, RING_THREADS, L::SMEM);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int tiles_x = (a.nx + RING_TW - 1) / RING_TW;
    const long long ntiles = (long long)tiles_x * a.ny * a.nz;  // < 2^31: fewer tiles than cells
    long long grid = (long long)nsm * per_sm;
    if (grid > ntiles) grid = ntiles;
    kern<<<(unsigned)grid, RING_THREADS, L::SMEM, st>>>(a, (int)ntiles, tiles_x);
    return cudaGetLastError();
}

}  // namespace

cudaError_t LBFFS_CAT(launch_bulk_tma_s, LBFFS_S)(const StepArgs& a, int sgs, bool les, cudaStream_t st)
{
    if (sgs == SGS_WALE) return run<SGS_WALE, false>(a, st);
    return les ? run<SGS_SMAG, true>(a, st) : run<SGS_SMAG, false>(a, st);
}

}  // namespace lbffs

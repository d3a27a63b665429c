// Batched D3Q19 step kernels for one storage format (compiled once per LBFFS_S).  They run the
// same per-tile and per-cell code as k_bulk / k_special (bulk_block, special_cell), so a case
// computes the same numbers alone, in a batch, or through lbffs_step.
#include <type_traits>

#include "batch.h"
#include "step_kernels.cuh"

#ifndef LBFFS_S
#error "compile with -DLBFFS_S=<storage>"
#endif

namespace lbffs {
namespace {

constexpr int S = LBFFS_S;

// last index c in [0, n) with start[c] <= key (start ascending, start[0] = 0)
template <class T>
__device__ __forceinline__ int find_case(const T* __restrict__ start, int n, T key)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(start + mid) <= key) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// resident CTAs per SM the batched bulk kernel is compiled for (0: the compiler's choice); a
// build-time tuning value.  The compiler's choice measured 8-10 % slower on the served sample.
#ifndef LBFFS_BATCH_MINB
#define LBFFS_BATCH_MINB 8
#endif
#if LBFFS_BATCH_MINB > 0
#define LBFFS_BATCH_BOUNDS __launch_bounds__(BULK_BX, LBFFS_BATCH_MINB)
#else
#define LBFFS_BATCH_BOUNDS __launch_bounds__(BULK_BX)
#endif

// kernel arguments of the batched bulk kernel: 1 = a copy in shared memory per CTA, 0 = read
// in place from the case table (cached); a build-time choice
#ifndef LBFFS_BATCH_ARGS_SMEM
#define LBFFS_BATCH_ARGS_SMEM 0
#endif

// ROWS: the cases in k_bulk's row tiles (BatchCase::rowtile), else those in the segment mapping; the
// two mappings are separate kernels so that each keeps its own register allocation
template <bool LES, bool ROWS>
__global__ void LBFFS_BATCH_BOUNDS k_bulk_batch(const BatchCase* __restrict__ cases,
                                                        const int2* __restrict__ cta_run,
                                                        const long long* __restrict__ done)
{
    // the CTA's case and run of tiles, one read (no search over the case table)
    const int2 cr = __ldg(cta_run + blockIdx.x);
    const int c = cr.x, run = cr.y;
#if LBFFS_BATCH_ARGS_SMEM
    __shared__ StepArgs sa;
    __shared__ int s_parity, s_last;
    if (threadIdx.x == 0) {
        const long long d = done[cases[c].slot];
        s_parity = d < cases[c].nsteps ? (int)(d & 1) : -1;
        s_last = d + 1 == cases[c].nsteps;
    }
    __syncthreads();
    if (s_parity < 0) return;  // the case has finished; it leaves the batch at the next rebuild
    const int* src = reinterpret_cast<const int*>(&cases[c].args[s_parity]);
    int* dst = reinterpret_cast<int*>(&sa);
    for (int w = threadIdx.x; w < (int)(sizeof(StepArgs) / sizeof(int)); w += blockDim.x) dst[w] = src[w];
    __syncthreads();
    if (threadIdx.x == 0 && s_last) sa.store_all = 1;  // full macroscopic fields on the final step
    __syncthreads();
#else
    const long long d = done[cases[c].slot];
    if (d >= cases[c].nsteps) return;  // the case has finished; it leaves the batch at the next rebuild
    const StepArgs& sa = d + 1 == cases[c].nsteps ? cases[c].last : cases[c].args[d & 1];
#endif
    const int tiles = cases[c].tiles;
    const int t1 = min(tiles, (run + 1) * BATCH_TILES_PER_CTA);
    if constexpr (ROWS) {
        // wide rows: k_bulk's own row tiles (the same pair paths, without its launch-order prefetch)
        const int nxb = cases[c].nxb;
        for (int tile = run * BATCH_TILES_PER_CTA; tile < t1; tile++) {
            const int r = tile / nxb;
            const int k = (int)fdiv(r, cases[c].dny);
            bulk_block<19, S, COLL_RR, SGS_SMAG, LES, false>(sa, tile - r * nxb, r - k * sa.ny, k);
        }
    } else {
        const int spr = cases[c].seg_per_row;
        const int nseg = spr * sa.ny * sa.nz;
        for (int tile = run * BATCH_TILES_PER_CTA; tile < t1; tile++)
            bulk_segments<19, S, COLL_RR, SGS_SMAG, LES>(sa, tile * BATCH_SEG_PER_TILE, spr, nseg, cases[c].dspr,
                                                         cases[c].dny);
    }
}

__global__ void __launch_bounds__(SPECIAL_BS) k_special_batch(const BatchCase* __restrict__ cases,
                                                              const long long* __restrict__ sp_start, int ncases,
                                                              const long long* __restrict__ done)
{
    const long long t = (long long)blockIdx.x * SPECIAL_BS + threadIdx.x;
    if (t >= sp_start[ncases]) return;
    const int c = find_case<long long>(sp_start, ncases, t);
    const long long d = done[cases[c].slot];
    if (d >= cases[c].nsteps) return;
    special_cell<19, S, COLL_RR>(cases[c].args[d & 1], t - sp_start[c]);
}

// a group of LBFFS_SPECIAL_LANES lanes per listed cell (special_cell with G lanes), for short lists
__global__ void __launch_bounds__(SPECIAL_BS) k_special_batch_warp(const BatchCase* __restrict__ cases,
                                                                   const long long* __restrict__ sp_start,
                                                                   int ncases, const long long* __restrict__ done)
{
    constexpr int G = LBFFS_SPECIAL_LANES;
    const long long t = (long long)blockIdx.x * (SPECIAL_BS / G) + (threadIdx.x / G);
    if (t >= sp_start[ncases]) return;
    const int c = find_case<long long>(sp_start, ncases, t);
    const long long d = done[cases[c].slot];
    if (d >= cases[c].nsteps) return;
    special_cell<19, S, COLL_RR, LBFFS_SPECIAL_LANES>(cases[c].args[d & 1], t - sp_start[c]);
}

using W = typename std::conditional<S == ST_FP32, uint32_t, uint16_t>::type;

// CTA b runs ghost-fill block b - h_start[c] of case c (h_start: prefix sums of halo blocks)
// CTA b fills ghost block y of case x, (x, y) = cta_block[b]
__global__ void __launch_bounds__(HALO_BS) k_halo_batch(const BatchCase* __restrict__ cases,
                                                        const int2* __restrict__ cta_block,
                                                        const long long* __restrict__ done)
{
    const int2 cb = __ldg(cta_block + blockIdx.x);
    const int c = cb.x;
    const long long d = done[cases[c].slot];
    if (d >= cases[c].nsteps) return;
    const StepArgs& a = cases[c].args[d & 1];
    const PadGeom g{a.nx, a.ny, a.nz, a.px, a.pxy, a.porg, a.pE};
    // the ghosts of this step's source copy (k_bulk / k_special read it only after this launch)
    halo_block<19, W>(static_cast<W*>(const_cast<void*>(a.f_in)), a.flags, a.bc, g, cb.y, threadIdx.x);
}

}  // namespace

#define LBFFS_CAT2(a, b) a##b
#define LBFFS_CAT(a, b) LBFFS_CAT2(a, b)

cudaError_t LBFFS_CAT(batch_bulk_s, LBFFS_S)(bool les, bool rows, const BatchCase* cases, const int2* cta_run,
                                             int nctas, const long long* done, cudaStream_t st)
{
    if (nctas <= 0) return cudaSuccess;
    if (rows) {
        if (les) k_bulk_batch<true, true><<<nctas, BULK_BX, 0, st>>>(cases, cta_run, done);
        else k_bulk_batch<false, true><<<nctas, BULK_BX, 0, st>>>(cases, cta_run, done);
    } else {
        if (les) k_bulk_batch<true, false><<<nctas, BULK_BX, 0, st>>>(cases, cta_run, done);
        else k_bulk_batch<false, false><<<nctas, BULK_BX, 0, st>>>(cases, cta_run, done);
    }
    return cudaGetLastError();
}

cudaError_t LBFFS_CAT(batch_special_s, LBFFS_S)(bool warp, const BatchCase* cases, const long long* sp_start,
                                                int ncases, long long nspecial, const long long* done,
                                                cudaStream_t st)
{
    if (nspecial <= 0) return cudaSuccess;
    if (warp) {
        constexpr int per = SPECIAL_BS / LBFFS_SPECIAL_LANES;
        k_special_batch_warp<<<(unsigned)((nspecial + per - 1) / per), SPECIAL_BS, 0, st>>>(cases, sp_start, ncases,
                                                                                            done);
        return cudaGetLastError();
    }
    const unsigned nb = (unsigned)((nspecial + SPECIAL_BS - 1) / SPECIAL_BS);
    k_special_batch<<<nb, SPECIAL_BS, 0, st>>>(cases, sp_start, ncases, done);
    return cudaGetLastError();
}

cudaError_t LBFFS_CAT(batch_halo_s, LBFFS_S)(const BatchCase* cases, const int2* cta_block,
                                             long long nblocks, const long long* done, cudaStream_t st)
{
    if (nblocks <= 0) return cudaSuccess;
    k_halo_batch<<<(unsigned)nblocks, HALO_BS, 0, st>>>(cases, cta_block, done);
    return cudaGetLastError();
}

}  // namespace lbffs

// Batched step kernels of the server: one launch advances every resident case of a group
// (same storage format and LES switch).  A case is described by the kernel arguments of its two
// ping-pong parities; its device step counter picks the parity and stops it at exactly nsteps.
#pragma once
#include <cuda_runtime.h>

#include "launch.h"

namespace lbffs {

struct BatchCase {
    StepArgs args[2];  // args[p]: source populations and macroscopics are copy p
    StepArgs last;     // the final step's arguments (args[(nsteps - 1) & 1], full macroscopic fields)
    long long nsteps;  // steps the case runs in total
    int slot;          // index of the case's step counter
    int seg_per_row;   // 32-cell x segments per row: ceil(nx / 32)
    int rowtile;       // 1: the case's bulk tiles are k_bulk's row tiles (bulk_block), 0: segments
    int nxb;           // row tiles per row: ceil(nx / (BULK_BX * BULK_V))
    int tiles;         // bulk tiles of the case: nxb * ny * nz row tiles, or
                       // ceil(seg_per_row * ny * nz / BATCH_SEG_PER_TILE) segment tiles
    FastDiv dspr, dny;  // division by seg_per_row and by ny
};

// x segments one bulk tile covers (BULK_V per warp of a BULK_BX-thread CTA; bulk_segments)
constexpr int BATCH_SEG_PER_TILE = (BULK_BX / 32) * BULK_V;
// bulk tiles one CTA of the batched kernel runs (consecutive tiles of one case); a build-time
// tuning value.  On the 48-request served sample 2 measured best (GPU busy time 1.680 s; 4: 1.688 s,
// 8: 1.717 s; with the shared-memory argument copy 1: 1.859 s).
#ifndef LBFFS_BATCH_TILES
#define LBFFS_BATCH_TILES 2
#endif
constexpr int BATCH_TILES_PER_CTA = LBFFS_BATCH_TILES;
// cases whose rows fill at least 70 % of k_bulk's row tiles run in them (1), or every case in the
// segment mapping (0); a build-time choice
#ifndef LBFFS_BATCH_ROWTILE
#define LBFFS_BATCH_ROWTILE 1
#endif

// Bulk step of every case in cases[0..ncases), in k_bulk's row tiles (bulk_block) for wide rows and
// in the segment mapping of bulk_segments (narrow rows keep the lanes busy) for the others: CTA b
// runs tiles [BATCH_TILES_PER_CTA y, BATCH_TILES_PER_CTA (y + 1)) of case x, (x, y) = cta_run[b],
// nctas CTAs.  rows: the launch over the row-tile cases, else over the segment cases.
cudaError_t batch_bulk(int storage, bool les, bool rows, const BatchCase* cases, const int2* cta_run, int nctas,
                       const long long* done, cudaStream_t st);
// Boundary step: thread (warp: warp) t runs entry t - sp_start[c] of case c's special list.
cudaError_t batch_special(int storage, bool warp, const BatchCase* cases, const long long* sp_start, int ncases,
                          long long nspecial, const long long* done, cudaStream_t st);
// Ghost layers: CTA b fills ghost block y of case x's source populations, (x, y) = cta_block[b].
cudaError_t batch_halo(int storage, const BatchCase* cases, const int2* cta_block, long long nblocks,
                       const long long* done, cudaStream_t st);
// Advance the step counters of the listed slots that have not reached their nsteps.
cudaError_t batch_tick(const int* slots, const long long* nsteps, int n, long long* done, cudaStream_t st);

// per storage format (batch_inst.cu compiled once per format)
cudaError_t batch_bulk_s0(bool, bool, const BatchCase*, const int2*, int, const long long*, cudaStream_t);
cudaError_t batch_bulk_s1(bool, bool, const BatchCase*, const int2*, int, const long long*, cudaStream_t);
cudaError_t batch_bulk_s2(bool, bool, const BatchCase*, const int2*, int, const long long*, cudaStream_t);
cudaError_t batch_special_s0(bool, const BatchCase*, const long long*, int, long long, const long long*, cudaStream_t);
cudaError_t batch_halo_s0(const BatchCase*, const int2*, long long, const long long*, cudaStream_t);
cudaError_t batch_halo_s1(const BatchCase*, const int2*, long long, const long long*, cudaStream_t);
cudaError_t batch_halo_s2(const BatchCase*, const int2*, long long, const long long*, cudaStream_t);
cudaError_t batch_special_s1(bool, const BatchCase*, const long long*, int, long long, const long long*, cudaStream_t);
cudaError_t batch_special_s2(bool, const BatchCase*, const long long*, int, long long, const long long*, cudaStream_t);

}  // namespace lbffs

// Warp-specialised D3Q19 bulk kernel: a producer warp streams the pulled rows of each tile into
// a ring of shared-memory stages with bulk async copies (cp.async.bulk, completion counted on an
// mbarrier), four consumer warps collide the tile's cells from shared memory and store the
// results (from registers, or for clean 64-cell segments through bulk async stores from a
// per-warp output buffer: LBFFS_RING_STORE).
//
// A tile is RING_TW consecutive cells of one row (j, k).  Population q of cell x is pulled from
// x - c_q, so the tile needs, per direction, the row (j - cy, k - cz) over x0 - 1 .. x0 + n: one
// bulk copy per direction of that row widened to 16-byte boundaries (the padded planes put every
// row start on a 32-byte sector, so the widened copy is aligned), plus one copy of the tile's
// flag bytes.  The producer runs up to NST tiles ahead; a stage is handed back (the "empty"
// barrier) as soon as every consumer warp has read its inputs, before the collision.
//
// What this buys over the per-thread kernel: the bytes in flight no longer cost registers and
// the consumers address shared memory with fixed offsets (no per-direction pointer arithmetic
// for the loads).  For 2-byte storage a lane owns two adjacent cells, so the two results of a
// direction are packed into one 32-bit store by one conversion.
//
// Only active cells are written: a lane stores its own active cells, and with bulk stores a
// segment goes through the output buffer only when all its cells are plain bulk cells and its
// length is a multiple of 16 bytes (others fall back to the lane stores), so cells owned by
// another kernel or by nobody are never written.
//
// Every mbarrier wait is bounded and its outcome is taken by the whole warp; when a wait runs
// out the warp sets bit 2 of the error word and leaves its loop (the other warps' waits then run
// out in turn), and before the CTA exits the producer waits (bounded) for the copies it still has
// in flight.  No CTA-wide barrier sits inside the loops.
#pragma once
#include <stdint.h>

#include "step_kernels.cuh"

namespace lbffs {

constexpr int RING_TW = 256;                      // cells per tile
constexpr int RING_CW = 4;                        // consumer warps
constexpr int RING_SEG = RING_TW / RING_CW;       // cells per consumer warp (2 per lane)
constexpr int RING_THREADS = 32 * (RING_CW + 1);  // consumers + one producer warp
constexpr unsigned TMA_WAIT_LIMIT = 1u << 20;
// results: 0 = each lane stores its own cells from registers, 1 = clean 64-cell segments through
// a per-warp shared-memory buffer and bulk stores (build-time choices, as is the stage count)
#ifndef LBFFS_RING_STORE
#define LBFFS_RING_STORE 0
#endif
#ifndef LBFFS_RING_NST
#define LBFFS_RING_NST 0
#endif
// resident CTAs per SM the kernel is compiled for (0: the compiler's register choice)
#ifndef LBFFS_RING_MINB
#define LBFFS_RING_MINB 6
#endif
#if LBFFS_RING_MINB > 0
#define LBFFS_RING_BOUNDS __launch_bounds__(RING_THREADS, LBFFS_RING_MINB)
#else
#define LBFFS_RING_BOUNDS __launch_bounds__(RING_THREADS)
#endif

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// bounded wait for the phase with the given parity
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity)
{
    for (unsigned n = 0; n < TMA_WAIT_LIMIT; n++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void bulk_load(void* sdst, const void* gsrc, unsigned bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(sdst)),
                 "l"(gsrc), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void bulk_store(void* gdst, const void* ssrc, unsigned bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(smem_addr(ssrc)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// the source of every committed group but the newest `N` has been read
template <int N>
__device__ __forceinline__ void bulk_wait_read()
{
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// held value <-> stored element (the bulk kernel's held form: f for FP32, 2^15 (f - w) for
// FP16S, f - w for BF16S)
__device__ __forceinline__ float held_of(float x) { return x; }
__device__ __forceinline__ float held_of(__half x) { return __half2float(x); }
__device__ __forceinline__ float held_of(__nv_bfloat16 x) { return __bfloat162float(x); }
template <class T>
__device__ __forceinline__ T held_to(float v);
template <>
__device__ __forceinline__ float held_to<float>(float v)
{
    return v;
}
template <>
__device__ __forceinline__ __half held_to<__half>(float v)
{
    return __float2half_rn(v);
}
template <>
__device__ __forceinline__ __nv_bfloat16 held_to<__nv_bfloat16>(float v)
{
    return __float2bfloat16_rn(v);
}
// x components of the D3Q19 directions as bit masks (c_x = +1, c_x = -1)
__host__ __device__ constexpr unsigned cx_mask19(int s)
{
    unsigned m = 0;
    for (int q = 0; q < 19; q++)
        if (lat_c(19, q, 0) == s) m |= 1u << q;
    return m;
}

template <int S>
struct RingLayout {
    using T = typename Codec<S>::T;
    static constexpr int SZ = (int)sizeof(T);
    static constexpr bool ADJ = SZ == 2;                // a lane owns cells 2l, 2l + 1 (else l, l + 32)
    static constexpr int E16 = 16 / SZ;                 // elements per 16 bytes
    static constexpr int ROW = RING_TW + 2 * E16;       // staged elements per direction
    static constexpr int NST = LBFFS_RING_NST > 0 ? LBFFS_RING_NST : (SZ == 2 ? 3 : 2);  // input stages
    static constexpr int IN_BYTES = 19 * ROW * SZ;      // one input stage
    static constexpr int FL_BYTES = RING_TW + 32;       // a tile's flag bytes, widened to 16 bytes
    static constexpr int OUT_BYTES = LBFFS_RING_STORE ? 19 * RING_SEG * SZ : 0;  // one consumer warp's output rows
    static constexpr int OFF_FL = NST * IN_BYTES;
    static constexpr int OFF_OUT = OFF_FL + NST * FL_BYTES;
    static constexpr int OFF_HDR = OFF_OUT + RING_CW * OUT_BYTES;
    static constexpr int OFF_BAR = OFF_HDR + NST * 32;
    static constexpr int SMEM = OFF_BAR + 2 * NST * 8;
    static_assert(IN_BYTES % 16 == 0 && OUT_BYTES % 16 == 0 && FL_BYTES % 16 == 0, "16-byte stages");
};

// tile header written by the producer: first cell, cells, row, offset of the first cell's flag
// byte in the staged flag bytes
struct RingHdr {
    int x0, n, j, k, foff, pad0, pad1, pad2;
};

template <int S, int SGS, bool LES>
__global__ void LBFFS_RING_BOUNDS k_bulk_tma(const StepArgs a, int ntiles, int tiles_x)
{
    using T = typename Codec<S>::T;
    using L = RingLayout<S>;
    constexpr int NST = L::NST, ROW = L::ROW, E16 = L::E16, SZ = L::SZ;
    constexpr unsigned CXP = cx_mask19(1), CXM = cx_mask19(-1);
    extern __shared__ __align__(128) unsigned char smem[];
    T* in = reinterpret_cast<T*>(smem);                                  // [NST][19][ROW]
    uint8_t* flb = smem + L::OFF_FL;                                     // [NST][FL_BYTES]
    T* outb = reinterpret_cast<T*>(smem + L::OFF_OUT);                   // [RING_CW][19][RING_SEG]
    RingHdr* hdr = reinterpret_cast<RingHdr*>(smem + L::OFF_HDR);        // [NST]
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L::OFF_BAR);     // [NST]
    uint64_t* empty = full + NST;                                        // [NST]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], RING_CW);
        }
        fence_mbar_init();
    }
    __syncthreads();

    int issued = 0;  // producer: tiles whose copies were issued
    if (warp == RING_CW) {
        // ---- producer ----
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, issued++) {
            const int st = issued % NST, u = issued / NST;
            // the stage's previous tile has been read by every consumer warp
            if (u > 0 && !__all_sync(0xffffffffu, mbar_wait(&empty[st], (unsigned)((u - 1) & 1)))) {
                if (lane == 0 && a.err) atomicOr(a.err, 2);
                break;
            }
            const int row = t / tiles_x;
            const int x0 = (t - row * tiles_x) * RING_TW;
            const int j = row % a.ny, k = row / a.ny;
            const int n = min(RING_TW, a.nx - x0);
            const int count = (n + 2 * E16) / E16 * E16;  // x0 - E16 .. x0 + n, whole 16-byte units
            const int fo = row * a.nx + x0;
            const int fstart = fo & ~15;
            const int fbytes = ((fo + n + 15) & ~15) - fstart;
            if (lane == 0) {
                hdr[st] = RingHdr{x0, n, j, k, fo - fstart, 0, 0, 0};
                mbar_expect_tx(&full[st], 19u * (unsigned)(count * SZ) + (unsigned)fbytes);
            }
            __syncwarp();
            if (lane < 19) {
                // row (j - cy, k - cz) from x0 - E16: the pulled plane base moved back by c_x
                const int cx = (int)((CXP >> lane) & 1u) - (int)((CXM >> lane) & 1u);
                const T* src = static_cast<const T*>(a.fin_s[lane]) + (pidx(a, x0 - E16, j, k) + cx);
                bulk_load(in + (st * 19 + lane) * ROW, src, (unsigned)(count * SZ), &full[st]);
            } else if (lane == 19) {
                bulk_load(flb + st * L::FL_BYTES, a.flags + fstart, (unsigned)fbytes, &full[st]);
            }
        }
    } else {
        // ---- consumers: lane l of warp w owns cells xi[0], xi[1] of the tile ----
        const int xi[2] = {L::ADJ ? RING_SEG * warp + 2 * lane : RING_SEG * warp + lane,
                           L::ADJ ? RING_SEG * warp + 2 * lane + 1 : RING_SEG * warp + lane + 32};
        T* ob = outb + warp * 19 * RING_SEG;
        int it = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
            const int st = it % NST, u = it / NST;
            if (!__all_sync(0xffffffffu, mbar_wait(&full[st], (unsigned)(u & 1)))) {
                if (lane == 0 && a.err) atomicOr(a.err, 2);
                break;
            }
            const RingHdr h = hdr[st];
            const uint8_t* fls = flb + st * L::FL_BYTES + h.foff;
            uint8_t fl[2];
            bool act[2], valid[2];
#pragma unroll
            for (int v = 0; v < 2; v++) {
                valid[v] = xi[v] < h.n;
                fl[v] = valid[v] ? fls[xi[v]] : FL_SOLID;
                act[v] = !(fl[v] & (FL_SOLID | FL_SPECIAL));
            }
            const T* r = in + st * 19 * ROW + E16;
            F2 ft[19];
#pragma unroll
            for (int q = 0; q < 19; q++) {
                const int cx = lat_c(19, q, 0);
                const T* p = r + q * ROW - cx;
                if constexpr (L::ADJ) {
                    if (cx == 0) {
                        // the two cells' elements are one aligned 32-bit word
                        ft[q] = held_unpack(T{}, *reinterpret_cast<const uint32_t*>(p + xi[0]));
                    } else {
                        ft[q] = pk(held_of(p[xi[0]]), held_of(p[xi[1]]));
                    }
                } else {
                    ft[q] = pk(held_of(p[xi[0]]), held_of(p[xi[1]]));
                }
            }
            // inputs read: hand the stage back to the producer
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
            if (!__any_sync(0xffffffffu, act[0] || act[1])) continue;
            const int row = h.k * a.ny + h.j;
            const int ci[2] = {h.x0 + xi[0], h.x0 + xi[1]}, cj[2] = {h.j, h.j}, ck[2] = {h.k, h.k};
            const int ic[2] = {row * a.nx + ci[0], row * a.nx + ci[1]};
            if constexpr (SGS != SGS_WALE) {
                const bool plain = __all_sync(0xffffffffu, plain_pair(a, fl, act));
                bulk_collide2<S, LES>(a, ft, fl, act, ci, cj, ck, ic, plain);
            } else {
                // WALE: the scalar path, one cell at a time
#pragma unroll
                for (int v = 0; v < 2; v++) {
                    float fs[19];
#pragma unroll
                    for (int q = 0; q < 19; q++) fs[q] = v == 0 ? lane0(ft[q]) : lane1(ft[q]);
                    if (act[v]) bulk_collide<19, S, COLL_RR, SGS, LES>(a, fs, fl[v], ci[v], h.j, h.k, ic[v]);
#pragma unroll
                    for (int q = 0; q < 19; q++) ft[q] = v == 0 ? pk(fs[q], lane1(ft[q])) : pk(lane0(ft[q]), fs[q]);
                }
            }
            const int m = min(max(h.n - RING_SEG * warp, 0), RING_SEG);
            const bool ok = (!valid[0] || act[0]) && (!valid[1] || act[1]);
            const bool clean = LBFFS_RING_STORE && __all_sync(0xffffffffu, ok) && (m * SZ) % 16 == 0;
            if (clean) {
                // this warp's previous bulk stores have read the output buffer
                if (lane < 19) bulk_wait_read<0>();
                __syncwarp();
#pragma unroll
                for (int q = 0; q < 19; q++) {
                    if constexpr (L::ADJ)
                        reinterpret_cast<uint32_t*>(ob + q * RING_SEG)[lane] = held_pack(T{}, lane0(ft[q]), lane1(ft[q]));
                    else {
                        ob[q * RING_SEG + lane] = held_to<T>(lane0(ft[q]));
                        ob[q * RING_SEG + lane + 32] = held_to<T>(lane1(ft[q]));
                    }
                }
                fence_async_smem();
                __syncwarp();
                if (lane < 19) {
                    T* dst = static_cast<T*>(a.fout_q[lane]) + pidx(a, h.x0 + RING_SEG * warp, h.j, h.k);
                    bulk_store(dst, ob + lane * RING_SEG, (unsigned)(m * SZ));
                    bulk_commit();
                }
            } else {
                const int ip[2] = {pidx(a, ci[0], h.j, h.k), pidx(a, ci[1], h.j, h.k)};
                // adjacent 2-byte cells, both active: one 32-bit store (ip[0] is even: every row
                // starts on a 32-byte sector and the pair on an even cell)
                const bool both = L::ADJ && act[0] && act[1];
#pragma unroll
                for (int q = 0; q < 19; q++) {
                    T* p = static_cast<T*>(a.fout_q[q]);
                    if constexpr (L::ADJ) {
                        if (both) {
                            *reinterpret_cast<uint32_t*>(p + ip[0]) = held_pack(T{}, lane0(ft[q]), lane1(ft[q]));
                            continue;
                        }
                    }
                    if (act[0]) Codec<S>::store_held(p + ip[0], lane0(ft[q]));
                    if (act[1]) Codec<S>::store_held(p + ip[1], lane1(ft[q]));
                }
            }
        }
        if (LBFFS_RING_STORE && lane < 19) bulk_wait_all();
    }
    __syncthreads();
    // copies still in flight into this CTA's shared memory (only after a wait ran out): the last
    // tile issued into each stage has landed
    if (warp == RING_CW && lane == 0) {
        for (int s = 0; s < NST && s < issued; s++) {
            const int u_last = (issued - 1 - s) / NST;
            if (!mbar_wait(&full[s], (unsigned)(u_last & 1)) && a.err) atomicOr(a.err, 2);
        }
    }
}

}  // namespace lbffs

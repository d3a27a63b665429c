// Row-staged D3Q19 bulk kernel: the pulled rows of a tile reach shared memory by bulk async
// copies (cp.async.bulk, completion on an mbarrier), the compute threads read them back with
// fixed shared-memory offsets, and clean tiles leave through bulk async stores.
//
// A tile is TMA_TW consecutive cells of one row (j, k).  Population q of cell x is pulled from
// x - c_q, so the tile needs, per direction, the row (j - cy, k - cz) over x0 - 1 .. x0 + n: one
// bulk copy per direction of that row widened to 16-byte boundaries (the padded planes put every
// row start on a 32-byte sector, so the widened copy is aligned).  Two stages alternate: while
// the tile of one stage is computed, thread 0 has the next tile's 19 rows in flight.
//
// A tile whose cells are all plain bulk cells and whose length is a multiple of 16 bytes is
// written back by 19 bulk stores from a shared-memory output row; any other tile (solid,
// special, or row-tail cells) has each active thread store its own cell, so cells owned by
// another kernel or by nobody are never written.
//
// Every mbarrier wait is bounded; when a wait runs out, the CTA (deciding together) sets bit 2 of
// the error word, waits (bounded) for the copies still in flight and leaves the kernel.
#pragma once
#include <stdint.h>

#include "step_kernels.cuh"

namespace lbffs {

constexpr int TMA_TW = 128;  // cells per tile = threads per CTA
constexpr unsigned TMA_WAIT_LIMIT = 1u << 20;

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

template <int S>
struct TmaLayout {
    using T = typename Codec<S>::T;
    static constexpr int E16 = 16 / (int)sizeof(T);           // elements per 16 bytes
    static constexpr int ROW = TMA_TW + 2 * E16;              // staged elements per direction
    static constexpr int IN_BYTES = 19 * ROW * (int)sizeof(T);  // one input stage
    static constexpr int OUT_BYTES = 19 * TMA_TW * (int)sizeof(T);
    static constexpr int SMEM = 2 * (IN_BYTES + OUT_BYTES) + 64;
};

template <int S, int SGS, bool LES>
__global__ void __launch_bounds__(TMA_TW) k_bulk_tma(const StepArgs a, long long ntiles, int tiles_x)
{
    using T = typename Codec<S>::T;
    using L = TmaLayout<S>;
    extern __shared__ __align__(128) unsigned char smem[];
    T* in = reinterpret_cast<T*>(smem);                            // [2][19][ROW]
    T* out = reinterpret_cast<T*>(smem + 2 * L::IN_BYTES);         // [2][19][TW]
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + 2 * (L::IN_BYTES + L::OUT_BYTES));
    const int tid = threadIdx.x;

    // tile -> first cell x0, cells n, row (j, k)
    auto decode = [&](long long t, int& x0, int& n, int& j, int& k) {
        const int xb = (int)(t % tiles_x);
        const long long row = t / tiles_x;
        j = (int)(row % a.ny);
        k = (int)(row / a.ny);
        x0 = xb * TMA_TW;
        n = min(TMA_TW, a.nx - x0);
    };
    // thread 0: the 19 pulled rows of tile t into stage st
    auto issue = [&](long long t, int st) {
        int x0, n, j, k;
        decode(t, x0, n, j, k);
        const int count = ((n + 1 + L::E16) + L::E16 - 1) / L::E16 * L::E16;  // covers x0 - E16 .. x0 + n
        const unsigned bytes = (unsigned)count * (unsigned)sizeof(T);
        mbar_expect_tx(&bar[st], 19u * bytes);
#pragma unroll
        for (int q = 0; q < 19; q++) {
            const T* src = static_cast<const T*>(a.fin_q[q]) +
                           pidx(a, x0 - L::E16, j - lat_c(19, q, 1), k - lat_c(19, q, 2));
            bulk_load(in + (st * 19 + q) * L::ROW, src, bytes, &bar[st]);
        }
    };

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    long long tile = blockIdx.x;
    if (tid == 0 && tile < ntiles) issue(tile, 0);
    int it = 0;
    bool failed = false;
    for (; tile < ntiles; tile += gridDim.x, it++) {
        const int st = it & 1;
        const long long next = tile + gridDim.x;
        // stage st ^ 1 was last read in the previous iteration, which ended with a barrier
        if (tid == 0 && next < ntiles) issue(next, st ^ 1);
        // every thread observes the phase itself (acquiring the copied rows); the give-up decision
        // is taken by the whole CTA together so that no thread is left at a barrier
        const bool got = mbar_wait(&bar[st], (unsigned)((it >> 1) & 1));
        if (!__syncthreads_and(got)) {
            failed = true;
            break;
        }
        int x0, n, j, k;
        decode(tile, x0, n, j, k);
        const bool valid = tid < n;
        const int i = x0 + tid;
        const int ic = (k * a.ny + j) * a.nx + i;
        const uint8_t fl = valid ? __ldg(a.flags + ic) : FL_SOLID;
        const bool act = !(fl & (FL_SOLID | FL_SPECIAL));
        const bool clean = __syncthreads_and(!valid || act) && (n % L::E16) == 0;
        if (act) {
            const T* row = in + st * 19 * L::ROW + L::E16 + tid;
            float ft[19];
            if constexpr (SGS != SGS_WALE) {
                // the two-lane collision of the per-thread kernel with the second lane idle, so
                // both variants round every cell the same way
                F2 fp[19];
#pragma unroll
                for (int q = 0; q < 19; q++) fp[q] = pk(held_of(row[q * L::ROW - lat_c(19, q, 0)]), 0.f);
                const uint8_t fl2[2] = {fl, FL_SOLID};
                const bool act2[2] = {true, false};
                const int ci[2] = {i, i}, cj[2] = {j, j}, ck[2] = {k, k}, ic2[2] = {ic, ic};
                bulk_collide2<S, LES>(a, fp, fl2, act2, ci, cj, ck, ic2);
#pragma unroll
                for (int q = 0; q < 19; q++) ft[q] = lane0(fp[q]);
            } else {
#pragma unroll
                for (int q = 0; q < 19; q++) ft[q] = held_of(row[q * L::ROW - lat_c(19, q, 0)]);
                bulk_collide<19, S, COLL_RR, SGS, LES>(a, ft, fl, i, j, k, ic);
            }
            if (clean) {
                T* o = out + st * 19 * TMA_TW + tid;
#pragma unroll
                for (int q = 0; q < 19; q++) o[q * TMA_TW] = held_to<T>(ft[q]);
            } else {
                const int ip = pidx(a, i, j, k);
#pragma unroll
                for (int q = 0; q < 19; q++) Codec<S>::store_held(static_cast<T*>(a.fout_q[q]) + ip, ft[q]);
            }
        }
        // each writer orders its shared-memory stores before the bulk stores that read them
        if (clean) fence_async_smem();
        __syncthreads();  // output rows of stage st written; input stage st fully read
        if (tid == 0) {
            if (clean) {
                const int ip0 = pidx(a, x0, j, k);
                const unsigned bytes = (unsigned)n * (unsigned)sizeof(T);
#pragma unroll
                for (int q = 0; q < 19; q++)
                    bulk_store(static_cast<T*>(a.fout_q[q]) + ip0, out + (st * 19 + q) * TMA_TW, bytes);
            }
            bulk_commit();
            bulk_wait_read<1>();  // the previous iteration's output stage may be rewritten
        }
        __syncthreads();
    }
    if (failed) {
        if (tid == 0) {
            if (a.err) atomicOr(a.err, 2);
            // the next tile's rows may still be in flight into this CTA's shared memory
            const long long next = tile + gridDim.x;
            if (next < ntiles) mbar_wait(&bar[(it & 1) ^ 1], (unsigned)(((it + 1) >> 1) & 1));
        }
    }
    if (tid == 0) bulk_wait_all();
}

}  // namespace lbffs

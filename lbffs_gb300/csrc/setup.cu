// Geometry commit, population format conversion and FP64 reductions.
//
// The reference hands the device one int32 array per boundary code and u8 solid /
// neiSolid arrays (D3Q19_opencl/ns.cpp:405-436).  Here they are condensed once per
// geometry change into a u16 boundary word and a u8 flag per cell plus a compact list
// of the cells that need the general boundary path; the time step never touches the
// int32 arrays again.
#include <algorithm>
#include <climits>

#include "launch.h"
#include "step_kernels.cuh"

namespace lbffs {

__global__ void k_pack_bc(const int* boundary, const int* b1, const int* b2, const int* b3, uint16_t* bc, int nx,
                          int ny, int nz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx) return;
    const long long ic = ((long long)blockIdx.z * ny + blockIdx.y) * nx + i;
    bc[ic] = (uint16_t)((b1[ic] & 7) | ((b2[ic] & 7) << 3) | ((b3[ic] & 7) << 6) | ((boundary[ic] == 1) << 9));
}

cudaError_t setup_pack_bc(const int* boundary, const int* b1, const int* b2, const int* b3, uint16_t* bc, int nx,
                          int ny, int nz, cudaStream_t st)
{
    k_pack_bc<<<dim3((nx + 127) / 128, ny, nz), 128, 0, st>>>(boundary, b1, b2, b3, bc, nx, ny, nz);
    return cudaGetLastError();
}

// pass 1: solid / face / link / special bits
template <int Q>
__global__ void k_classify1(const uint16_t* bc, const uint8_t* solid, const uint8_t* nei, uint8_t* flags, int nx,
                            int ny, int nz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx) return;
    const int j = blockIdx.y, k = blockIdx.z;
    const long long ic = ((long long)k * ny + j) * nx + i;
    if (solid[ic]) {
        flags[ic] = FL_SOLID;
        return;
    }
    const uint16_t bw = bc[ic];
    const int b[3] = {bw & 7, (bw >> 3) & 7, (bw >> 6) & 7};
    const bool face = (bw >> 9) & 1;
    const bool border = i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || (nz > 1 && (k == 0 || k == nz - 1));
    bool link = false;
    if (nei[ic] == 1) {
        const int x[3] = {i, j, k}, N[3] = {nx, ny, nz};
#pragma unroll
        for (int q = 1; q < Q; q++) {
            const long long up = upwind<Q>(q, x, N, b, face);
            link |= (up >= 0 && solid[up] == 1);
        }
    }
    // faces with an Outlet, FixedVelocity, FixedDensity or WallFunction code need the boundary operators of the
    // general kernel; wall / periodic / symmetry faces only change where populations come from
    // and stay in the bulk kernel
    bool complex_bc = false;
#pragma unroll
    for (int d = 0; d < 3; d++)
        complex_bc |= (b[d] == BC_OUTLET || b[d] == BC_FIXVEL || b[d] == BC_FIXDEN || b[d] == BC_WALLFN);
    complex_bc &= (face || border);
    uint8_t fl = 0;
    if (face || border) fl |= FL_FACE;
    if (link) fl |= FL_LINK;
    if (link || complex_bc) fl |= FL_SPECIAL;
    flags[ic] = fl;
}

// pass 2: cells next to a special cell store their macroscopics; damping / omega read bits.  A cell
// reads its wall distance when the damping can change its eddy viscosity: the reference's factor
// min(1, 0.41 y / Cs)^2 only below y = Cs / 0.41, the Van Driest factor wherever a distance is set.
__global__ void k_classify2(const uint8_t* pass1, uint8_t* flags, const float* sdf, const float* omega, float omega0,
                            float cs, int damping, int nx, int ny, int nz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx) return;
    const int j = blockIdx.y, k = blockIdx.z;
    const long long ic = ((long long)k * ny + j) * nx + i;
    uint8_t fl = pass1[ic];
    if (fl & FL_SOLID) {
        flags[ic] = fl;
        return;
    }
    bool near = false;
    for (int dk = -1; dk <= 1; dk++)
        for (int dj = -1; dj <= 1; dj++)
            for (int di = -1; di <= 1; di++) {
                int ii = i + di, jj = j + dj, kk = k + dk;
                if (ii < 0) ii += nx;
                if (ii >= nx) ii -= nx;
                if (jj < 0) jj += ny;
                if (jj >= ny) jj -= ny;
                if (kk < 0) kk += nz;
                if (kk >= nz) kk -= nz;
                near |= (pass1[((long long)kk * ny + jj) * nx + ii] & FL_SPECIAL) != 0;
            }
    fl &= (FL_SPECIAL | FL_LINK | FL_FACE);
    if (near) fl |= FL_STORE;
    const float s = sdf[ic];
    if (s != 10000.f && s > 0.f &&
        ((damping == LBFFS_DAMP_WALL && 0.41f * s / cs < 1.f) || damping == LBFFS_DAMP_VAN_DRIEST))
        fl |= FL_SDF;
    if (__float_as_uint(omega[ic]) != __float_as_uint(omega0)) fl |= FL_OMEGA;
    flags[ic] = fl;
}

cudaError_t setup_classify(int Q, const uint16_t* bc, const uint8_t* solid, const uint8_t* nei, const float* sdf,
                           const float* omega, float omega0, float cs, int damping, uint8_t* flags, uint8_t* scratch,
                           int nx, int ny, int nz, cudaStream_t st)
{
    const dim3 grid((nx + 127) / 128, ny, nz);
    if (Q == 19) k_classify1<19><<<grid, 128, 0, st>>>(bc, solid, nei, scratch, nx, ny, nz);
    else k_classify1<27><<<grid, 128, 0, st>>>(bc, solid, nei, scratch, nx, ny, nz);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_classify2<<<grid, 128, 0, st>>>(scratch, flags, sdf, omega, omega0, cs, damping, nx, ny, nz);
    return cudaGetLastError();
}

__global__ void k_count_special(const uint8_t* flags, long long E, uint8_t mask, unsigned* counts)
{
    const long long ic = (long long)blockIdx.x * SETUP_CHUNK + threadIdx.x;
    const bool sp = ic < E && (flags[ic] & mask) && !(flags[ic] & FL_SOLID);
    const int n = __syncthreads_count(sp);
    if (threadIdx.x == 0) counts[blockIdx.x] = (unsigned)n;
}

cudaError_t setup_count_special(const uint8_t* flags, long long E, uint8_t mask, unsigned* counts, cudaStream_t st)
{
    const unsigned nb = (unsigned)((E + SETUP_CHUNK - 1) / SETUP_CHUNK);
    k_count_special<<<nb, SETUP_CHUNK, 0, st>>>(flags, E, mask, counts);
    return cudaGetLastError();
}

__global__ void k_scatter_special(const uint8_t* flags, long long E, uint8_t mask, const unsigned long long* offsets,
                                  uint32_t* out)
{
    __shared__ unsigned warp_base[SETUP_CHUNK / 32];
    const long long ic = (long long)blockIdx.x * SETUP_CHUNK + threadIdx.x;
    const bool sp = ic < E && (flags[ic] & mask) && !(flags[ic] & FL_SOLID);
    const unsigned m = __ballot_sync(0xffffffffu, sp);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_base[warp] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned s = 0;
        for (int w = 0; w < SETUP_CHUNK / 32; w++) {
            const unsigned c = warp_base[w];
            warp_base[w] = s;
            s += c;
        }
    }
    __syncthreads();
    if (sp) {
        const unsigned pos = warp_base[warp] + __popc(m & ((1u << lane) - 1u));
        out[offsets[blockIdx.x] + pos] = (uint32_t)ic;
    }
}

cudaError_t setup_scatter_special(const uint8_t* flags, long long E, uint8_t mask, const unsigned long long* offsets,
                                  uint32_t* out, cudaStream_t st)
{
    const unsigned nb = (unsigned)((E + SETUP_CHUNK - 1) / SETUP_CHUNK);
    k_scatter_special<<<nb, SETUP_CHUNK, 0, st>>>(flags, E, mask, offsets, out);
    return cudaGetLastError();
}

// bit q set: (cell, q) is an STL link, i.e. neiSolid[cell] && solid[upwind(cell, q)] (kernel.cl:1940-1943)
template <int Q>
__global__ void k_link_masks(const uint32_t* special, long long n, const uint16_t* bc, const uint8_t* solid,
                             const uint8_t* nei, int nx, int ny, int nz, uint32_t* masks)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const long long ic = special[t];
    const int x[3] = {(int)(ic % nx), (int)((ic / nx) % ny), (int)(ic / ((long long)nx * ny))}, N[3] = {nx, ny, nz};
    const uint16_t bw = bc[ic];
    const int b[3] = {bw & 7, (bw >> 3) & 7, (bw >> 6) & 7};
    const bool face = (bw >> 9) & 1;
    uint32_t m = 0;
    if (nei[ic] == 1 && !solid[ic]) {
#pragma unroll
        for (int q = 1; q < Q; q++) {
            const long long up = upwind<Q>(q, x, N, b, face);
            if (up >= 0 && solid[up] == 1) m |= 1u << q;
        }
    }
    masks[t] = m;
}

cudaError_t setup_link_masks(int Q, const uint32_t* special, long long n, const uint16_t* bc, const uint8_t* solid,
                             const uint8_t* nei, int nx, int ny, int nz, uint32_t* masks, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const unsigned nb = (unsigned)((n + 127) / 128);
    if (Q == 19) k_link_masks<19><<<nb, 128, 0, st>>>(special, n, bc, solid, nei, nx, ny, nz, masks);
    else k_link_masks<27><<<nb, 128, 0, st>>>(special, n, bc, solid, nei, nx, ny, nz, masks);
    return cudaGetLastError();
}

// ---- population format conversion (host float32 layout <-> storage) ----
// Populations between the reference's packed layout (Q*ny*nz rows of nx values) and the padded
// device planes, one block per row: rows [row0, row0 + nrows) of the packed array live in src /
// dst, the device planes in the padded layout of g.
template <int Q>
__device__ __forceinline__ float weight_of(int q)
{
    float w = 0.f;
#pragma unroll
    for (int p = 0; p < Q; p++)
        if (p == q) w = lat_w(Q, p);
    return w;
}

__device__ __forceinline__ long long padded_row(const PadGeom& g, long long r, int& q)
{
    const long long plane_rows = (long long)g.ny * g.nz;
    q = (int)(r / plane_rows);
    const long long jk = r - (long long)q * plane_rows;
    const int j = (int)(jk % g.ny), k = (int)(jk / g.ny);
    return (long long)q * g.pE + g.porg + (long long)k * g.pxy + (long long)j * g.px;
}

// src may be host memory the device can address (pinned); dst2, when set, receives the same values
template <int S, int Q>
__global__ void k_encode(const float* src, typename Codec<S>::T* dst, typename Codec<S>::T* dst2, long long row0,
                         PadGeom g)
{
    int q;
    const long long base = padded_row(g, row0 + blockIdx.x, q);
    const float w = weight_of<Q>(q);
    const float* s = src + (long long)blockIdx.x * g.nx;
    for (int i = threadIdx.x; i < g.nx; i += blockDim.x) {
        const float v = s[i];
        Codec<S>::store(dst + base + i, v, w);
        if (dst2) Codec<S>::store(dst2 + base + i, v, w);
    }
}

template <int S, int Q>
__global__ void k_decode(const typename Codec<S>::T* src, float* dst, long long row0, PadGeom g)
{
    int q;
    const long long base = padded_row(g, row0 + blockIdx.x, q);
    const float w = weight_of<Q>(q);
    float* d = dst + (long long)blockIdx.x * g.nx;
    for (int i = threadIdx.x; i < g.nx; i += blockDim.x) d[i] = Codec<S>::load(src + base + i, w);
}

template <int S>
static cudaError_t enc_q(int Q, const float* src, void* dst, void* dst2, long long row0, long long nrows,
                         const PadGeom& g, cudaStream_t st)
{
    using T = typename Codec<S>::T;
    if (Q == 19)
        k_encode<S, 19><<<(unsigned)nrows, 256, 0, st>>>(src, static_cast<T*>(dst), static_cast<T*>(dst2), row0, g);
    else
        k_encode<S, 27><<<(unsigned)nrows, 256, 0, st>>>(src, static_cast<T*>(dst), static_cast<T*>(dst2), row0, g);
    return cudaGetLastError();
}

template <int S>
static cudaError_t dec_q(int Q, const void* src, float* dst, long long row0, long long nrows, const PadGeom& g,
                         cudaStream_t st)
{
    using T = typename Codec<S>::T;
    if (Q == 19) k_decode<S, 19><<<(unsigned)nrows, 256, 0, st>>>(static_cast<const T*>(src), dst, row0, g);
    else k_decode<S, 27><<<(unsigned)nrows, 256, 0, st>>>(static_cast<const T*>(src), dst, row0, g);
    return cudaGetLastError();
}

cudaError_t encode_f(int storage, int Q, const float* src, void* dst, void* dst2, long long row0, long long nrows,
                     const PadGeom& g, cudaStream_t st)
{
    if (nrows <= 0) return cudaSuccess;
    switch (storage) {
        case ST_FP32: return enc_q<ST_FP32>(Q, src, dst, dst2, row0, nrows, g, st);
        case ST_FP16S: return enc_q<ST_FP16S>(Q, src, dst, dst2, row0, nrows, g, st);
        case ST_BF16S: return enc_q<ST_BF16S>(Q, src, dst, dst2, row0, nrows, g, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t decode_f(int storage, int Q, const void* src, float* dst, long long row0, long long nrows,
                     const PadGeom& g, cudaStream_t st)
{
    if (nrows <= 0) return cudaSuccess;
    switch (storage) {
        case ST_FP32: return dec_q<ST_FP32>(Q, src, dst, row0, nrows, g, st);
        case ST_FP16S: return dec_q<ST_FP16S>(Q, src, dst, row0, nrows, g, st);
        case ST_BF16S: return dec_q<ST_BF16S>(Q, src, dst, row0, nrows, g, st);
    }
    return cudaErrorInvalidValue;
}

// ---- ghost layer (halo_block in step_kernels.cuh) ----
template <int Q, typename W, bool SPEC>
__global__ void __launch_bounds__(HALO_BS) k_halo(W* f, const uint8_t* __restrict__ flags,
                                                  const uint16_t* __restrict__ bc, PadGeom g)
{
    halo_block<Q, W, SPEC>(f, flags, bc, g, blockIdx.x, threadIdx.x);
}

template <int Q, typename W>
static void launch_halo(bool spec, long long nb, void* f, const uint8_t* flags, const uint16_t* bc, const PadGeom& g,
                        cudaStream_t st)
{
    if (spec) k_halo<Q, W, true><<<(unsigned)nb, HALO_BS, 0, st>>>(static_cast<W*>(f), flags, bc, g);
    else k_halo<Q, W, false><<<(unsigned)nb, HALO_BS, 0, st>>>(static_cast<W*>(f), flags, bc, g);
}

cudaError_t halo_fill(int Q, int tsize, void* f, const uint8_t* flags, const uint16_t* bc, const PadGeom& g,
                      cudaStream_t st)
{
    const long long n0 = halo_blocks(g, Q, 0), n1 = halo_blocks(g, Q, 1), n2 = halo_blocks(g, Q, 2);
    const long long nb = n0 + n1 + n2;
    // D3Q19: the per-face code paths when one axis holds at least two thirds of the face cells
    // (the run-time path is measured on D3Q19 only; D3Q27 keeps the per-face paths)
    const bool spec = Q != 19 || 3 * std::max(n0, std::max(n1, n2)) >= 2 * nb;
    if (Q == 19) {
        if (tsize == 4) launch_halo<19, uint32_t>(spec, nb, f, flags, bc, g, st);
        else launch_halo<19, uint16_t>(spec, nb, f, flags, bc, g, st);
    } else {
        if (tsize == 4) launch_halo<27, uint32_t>(spec, nb, f, flags, bc, g, st);
        else launch_halo<27, uint16_t>(spec, nb, f, flags, bc, g, st);
    }
    return cudaGetLastError();
}

// Boundary-code check over the three per-axis code arrays: out[0] bit 0 = a WallFunction code
// (7) is present, bit 1 = a value outside {0, 1, 3, 4, 5, 6, 7} is present, out[1] = the largest
// such value.
__global__ void k_check_codes(const int* __restrict__ b1, const int* __restrict__ b2, const int* __restrict__ b3,
                              long long E, int* out)
{
    int bits = 0, bad = INT_MIN;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < E; i += (long long)gridDim.x * blockDim.x) {
        const int v[3] = {b1[i], b2[i], b3[i]};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            if (v[d] == BC_WALLFN) bits |= 1;
            else if (!(v[d] == 0 || v[d] == 1 || v[d] == 3 || v[d] == 4 || v[d] == 5 || v[d] == 6)) {
                bits |= 2;
                bad = max(bad, v[d]);
            }
        }
    }
    bits = __reduce_or_sync(0xffffffffu, bits);
    bad = __reduce_max_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && bits) {
        atomicOr(out, bits);
        atomicMax(out + 1, bad);
    }
}

cudaError_t setup_check_codes(const int* b1, const int* b2, const int* b3, long long E, int* out, cudaStream_t st)
{
    k_check_codes<<<512, 256, 0, st>>>(b1, b2, b3, E, out);
    return cudaGetLastError();
}

__global__ void k_check_faces(const int* __restrict__ boundary, const int* __restrict__ b1,
                              const int* __restrict__ b2, const int* __restrict__ b3, int codes, int nx, int ny,
                              int nz, int* bad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx) return;
    const int j = blockIdx.y, k = blockIdx.z;
    const long long ic = ((long long)k * ny + j) * nx + i;
    const int x[3] = {i, j, k}, N[3] = {nx, ny, nz};
    const int* b[3] = {b1, b2, b3};
    const bool border = i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || (nz > 1 && (k == 0 || k == nz - 1));
    bool ok = boundary[ic] == (border ? 1 : 0);
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int e = x[d] == 0 ? (codes >> (6 * d)) & 7 : x[d] == N[d] - 1 ? (codes >> (6 * d + 3)) & 7 : 0;
        ok &= b[d][ic] == e;
    }
    if (!ok) atomicOr(bad, 1);
}

cudaError_t setup_check_faces(const int* boundary, const int* b1, const int* b2, const int* b3, int codes, int nx,
                              int ny, int nz, int* bad, cudaStream_t st)
{
    const dim3 grid((nx + 127) / 128, ny, nz);
    k_check_faces<<<grid, 128, 0, st>>>(boundary, b1, b2, b3, codes, nx, ny, nz, bad);
    return cudaGetLastError();
}

// Cells per class: counts[0] fluid, [1] special, [2] STL-link, [3] storing macroscopics.
__global__ void k_count_flags(const uint8_t* __restrict__ flags, long long E, unsigned long long* counts)
{
    unsigned c[4] = {0, 0, 0, 0};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < E; i += (long long)gridDim.x * blockDim.x) {
        const uint8_t v = flags[i];
        if (v & FL_SOLID) continue;
        c[0]++;
        c[1] += (v & FL_SPECIAL) != 0;
        c[2] += (v & FL_LINK) != 0;
        c[3] += (v & FL_STORE) != 0;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const unsigned t = __reduce_add_sync(0xffffffffu, c[k]);
        if ((threadIdx.x & 31) == 0 && t) atomicAdd(counts + k, (unsigned long long)t);
    }
}

cudaError_t setup_count_flags(const uint8_t* flags, long long E, unsigned long long* counts, cudaStream_t st)
{
    k_count_flags<<<512, 256, 0, st>>>(flags, E, counts);
    return cudaGetLastError();
}

__global__ void k_fill(float* p, float v, long long n)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) p[t] = v;
}

cudaError_t fill_f32(float* p, float v, long long n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_fill<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p, v, n);
    return cudaGetLastError();
}

// ---- FP64 reductions (per-block partials, summed in a fixed order on the host) ----
__device__ __forceinline__ double block_sum(double v, double* sh)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sh[w];
    __syncthreads();
    return s;
}

__global__ void k_reduce_force(const uint32_t* cells, long long n, const float* fx, const float* fy, const float* fz,
                               double* partial)
{
    __shared__ double sh[REDUCE_BS / 32];
    double a = 0.0, b = 0.0, c = 0.0;
    for (long long t = (long long)blockIdx.x * REDUCE_BS + threadIdx.x; t < n; t += (long long)gridDim.x * REDUCE_BS) {
        const long long ic = cells[t];
        a += (double)fx[ic];
        b += (double)fy[ic];
        c += (double)fz[ic];
    }
    a = block_sum(a, sh);
    b = block_sum(b, sh);
    c = block_sum(c, sh);
    if (threadIdx.x == 0) {
        partial[3 * blockIdx.x + 0] = a;
        partial[3 * blockIdx.x + 1] = b;
        partial[3 * blockIdx.x + 2] = c;
    }
}

cudaError_t reduce_force(const uint32_t* cells, long long n, const float* fx, const float* fy, const float* fz,
                         double* partial, int nblocks, cudaStream_t st)
{
    k_reduce_force<<<nblocks, REDUCE_BS, 0, st>>>(cells, n, fx, fy, fz, partial);
    return cudaGetLastError();
}

template <int S, int Q>
__global__ void k_reduce_mass(const typename Codec<S>::T* f, const uint8_t* flags, long long E, PadGeom g,
                              double* partial)
{
    __shared__ double sh[REDUCE_BS / 32];
    double acc = 0.0;
    for (long long ic = (long long)blockIdx.x * REDUCE_BS + threadIdx.x; ic < E; ic += (long long)gridDim.x * REDUCE_BS) {
        if (flags[ic] & FL_SOLID) continue;
        const long long row = ic / g.nx;
        const long long ip = g.porg + (row / g.ny) * g.pxy + (row % g.ny) * g.px + (ic - row * g.nx);
        float r = 0.f;
#pragma unroll
        for (int q = 0; q < Q; q++) r += Codec<S>::load(f + (long long)q * g.pE + ip, lat_w(Q, q));
        acc += (double)r;
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

cudaError_t reduce_mass(int storage, int Q, const void* f, const uint8_t* flags, long long E, const PadGeom& g,
                        double* partial, int nblocks, cudaStream_t st)
{
#define LBFFS_MASS(S)                                                                                                  \
    (Q == 19 ? (k_reduce_mass<S, 19><<<nblocks, REDUCE_BS, 0, st>>>(static_cast<const Codec<S>::T*>(f), flags, E, g, partial), 0) \
             : (k_reduce_mass<S, 27><<<nblocks, REDUCE_BS, 0, st>>>(static_cast<const Codec<S>::T*>(f), flags, E, g, partial), 0))
    switch (storage) {
        case ST_FP32: LBFFS_MASS(ST_FP32); break;
        case ST_FP16S: LBFFS_MASS(ST_FP16S); break;
        case ST_BF16S: LBFFS_MASS(ST_BF16S); break;
        default: return cudaErrorInvalidValue;
    }
#undef LBFFS_MASS
    return cudaGetLastError();
}

}  // namespace lbffs

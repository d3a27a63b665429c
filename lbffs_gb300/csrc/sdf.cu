// Wall-distance field of an STL surface on the device: setSDF (src/walls.hpp:218-268) followed by
// setSDFnearBwalls (walls.hpp:372-467), the LES set-up sequence of D3Q19_opencl/ns.cpp:200-225.
//
// setSDF marks every cell within a Chebyshev box of half-width int(dr) around a neiSolid cell
// ("near" cells) and gives each of them the inverse-distance-weighted signed distance
//     sdf = sum_t sd_t r_t^-p / sum_t r_t^-p   over the triangles t with r_t < dr,
// r_t the distance from the cell to the triangle's centroid, sd_t the projection of that offset on
// the triangle's normal (sdfIni when no triangle is that close).  ns.cpp calls it once per STL
// patch, and every call rewrites every near cell, so the sequence ends with the last patch's
// values: that pass is the one run here.
//
// Device form: the near mask is a separable box dilation of neiSolid (three axis passes).  The
// triangles are binned on the host into bricks of 8 x 4 x 4 cells (every brick whose box lies
// within dr + 1 of the centroid), each brick's list in ascending triangle order; one CTA per
// brick stages its list through shared memory and every near cell accumulates its triangles in
// that order.  Arithmetic follows the reference's expression types as its host compiler
// evaluates them: the offsets and sd in float, the squared distance and its square root in double
// (r rounded to float), and the weight r^-p, the products sd * r^-p and both running sums in double,
// each sum rounded back to float after every term.  The weight is formed in double by repeated
// squaring for an integral p (by pow otherwise); it is not bit-identical to the host library's pow
// in every case, so the result agrees with the reference to a few float ulps of the sums.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "ctx.h"

namespace lbffs {
namespace {

constexpr int SDF_BX = 8, SDF_BY = 4, SDF_BZ = 4;
constexpr int SDF_BS = SDF_BX * SDF_BY * SDF_BZ;

struct SdfTri {
    float c[3];  // centroid ((v0 + v1) + v2) / 3 (stl.hpp:177-186)
    float n[3];  // facet normal as read from the STL
};

// out = OR of in over [x - r, x + r] along one axis, clipped to the domain (the nearSTL box of
// walls.hpp:223-252, one axis at a time)
__global__ void k_dilate(const uint8_t* __restrict__ in, uint8_t* __restrict__ out, int nx, int ny, int nz, int axis,
                         int r)
{
    const long long ic = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long E = (long long)nx * ny * nz;
    if (ic >= E) return;
    const int i = (int)(ic % nx), j = (int)((ic / nx) % ny), k = (int)(ic / ((long long)nx * ny));
    const int pos = axis == 0 ? i : (axis == 1 ? j : k);
    const int n = axis == 0 ? nx : (axis == 1 ? ny : nz);
    const long long stride = axis == 0 ? 1 : (axis == 1 ? (long long)nx : (long long)nx * ny);
    const int lo = max(0, pos - r), hi = min(n - 1, pos + r);
    uint8_t v = 0;
    for (int p = lo; p <= hi && !v; p++) v = in[ic + (long long)(p - pos) * stride] != 0;
    out[ic] = v;
}

// r^-p in double: an integral p by repeated squaring, any other by pow
__device__ __forceinline__ double inv_pow(double r, float p)
{
    if (p >= 1.f && p <= 64.f && p == floorf(p)) {
        int n = (int)p;
        double x = 1.0, b = r;
        while (n) {
            if (n & 1) x *= b;
            b *= b;
            n >>= 1;
        }
        return 1.0 / x;
    }
    return pow(r, -(double)p);
}

// One CTA per brick; thread t owns cell (x0 + t % 8, y0 + (t / 8) % 4, z0 + t / 32).
__global__ void __launch_bounds__(SDF_BS) k_sdf_bricks(const SdfTri* __restrict__ tris,
                                                       const long long* __restrict__ off, const int* __restrict__ ent,
                                                       const uint8_t* __restrict__ near, int nx, int ny, int nz,
                                                       int nbx, int nby, float dr, float p, float sdf_ini,
                                                       float* __restrict__ sdf)
{
    __shared__ SdfTri st[SDF_BS];
    const int b = blockIdx.x;
    const int bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
    const int t = threadIdx.x;
    const int i = bx * SDF_BX + (t % SDF_BX), j = by * SDF_BY + (t / SDF_BX) % SDF_BY;
    const int k = bz * SDF_BZ + t / (SDF_BX * SDF_BY);
    const bool in = i < nx && j < ny && k < nz;
    const long long ic = ((long long)k * ny + j) * nx + i;
    const bool mine = in && near[ic] != 0;
    if (!__syncthreads_or(mine)) return;
    const float fi = (float)i, fj = (float)j, fk = (float)k;
    float acc = 0.f, sum = 0.f;
    const long long e0 = off[b], e1 = off[b + 1];
    for (long long base = e0; base < e1; base += SDF_BS) {
        __syncthreads();
        if (base + t < e1) st[t] = tris[ent[base + t]];
        __syncthreads();
        const int n = (int)min((long long)SDF_BS, e1 - base);
        if (mine) {
            for (int m = 0; m < n; m++) {
                const float dx = __fsub_rn(fi, st[m].c[0]);
                const float dy = __fsub_rn(fj, st[m].c[1]);
                const float dz = __fsub_rn(fk, st[m].c[2]);
                const double ddx = dx, ddy = dy, ddz = dz;
                const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)), __dmul_rn(ddz, ddz));
                const float r = __double2float_rn(__dsqrt_rn(r2));
                if (r < dr) {
                    const float sd = __fadd_rn(__fadd_rn(__fmul_rn(dx, st[m].n[0]), __fmul_rn(dy, st[m].n[1])),
                                               __fmul_rn(dz, st[m].n[2]));
                    const double w = inv_pow((double)r, p);
                    sum = __double2float_rn(__dadd_rn((double)sum, w));
                    acc = __double2float_rn(__dadd_rn((double)acc, __dmul_rn((double)sd, w)));
                }
            }
        }
    }
    if (mine) sdf[ic] = sum != 0.f ? __fdiv_rn(acc, sum) : sdf_ini;
}

__global__ void k_sdf_fill(float* __restrict__ sdf, long long E, float v)
{
    const long long ic = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (ic < E) sdf[ic] = v;
}

// setSDFnearBwalls: the x-face loops run first, then y, then z, and in each the far face's loop
// after the near one, so the last write a cell receives is the first match in the order
// z far, z near, y far, y near, x far, x near.  n = int(dr): cells up to n from a face whose
// boundary code is 1 (half-way bounce-back) get 0.5 + their distance from it.
__global__ void k_sdf_bwalls(float* __restrict__ sdf, const int* __restrict__ b1, const int* __restrict__ b2,
                             const int* __restrict__ b3, int nx, int ny, int nz, int n)
{
    const long long ic = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long E = (long long)nx * ny * nz;
    if (ic >= E) return;
    const int i = (int)(ic % nx), j = (int)((ic / nx) % ny), k = (int)(ic / ((long long)nx * ny));
    const long long nxy = (long long)nx * ny;
    const long long row = ic - i;                   // (0, j, k)
    const long long col = ic - (long long)j * nx;   // (i, 0, k)
    const long long pil = ic - (long long)k * nxy;  // (i, j, 0)
    int d = -1;
    if (b3[pil + (long long)(nz - 1) * nxy] == 1 && nz - 1 - k <= n && k > 0) d = nz - 1 - k;
    else if (b3[pil] == 1 && k <= n && k < nz - 1) d = k;
    else if (b2[col + (long long)(ny - 1) * nx] == 1 && ny - 1 - j <= n && j > 0) d = ny - 1 - j;
    else if (b2[col] == 1 && j <= n && j < ny - 1) d = j;
    else if (b1[row + nx - 1] == 1 && nx - 1 - i <= n && i > 0) d = nx - 1 - i;
    else if (b1[row] == 1 && i <= n && i < nx - 1) d = i;
    if (d >= 0) sdf[ic] = 0.5f + (float)d;
}

}  // namespace
}  // namespace lbffs

using namespace lbffs;

extern "C" int lbffs_build_sdf(lbffs_ctx* c, const float* verts, const float* normals, const long long* patch_ntri,
                               int npatch, float dr, float p, float sdf_ini, float dr_walls)
{
    if (!c || npatch < 0 || (npatch > 0 && !patch_ntri)) return ctx_fail(c, LBFFS_E_ARG, "lbffs_build_sdf: bad argument");
    long long ntri = 0, last = 0;
    for (int s = 0; s < npatch; s++) {
        if (patch_ntri[s] < 0) return ctx_fail(c, LBFFS_E_ARG, "lbffs_build_sdf: negative patch size");
        last = ntri;
        ntri += patch_ntri[s];
        if (ntri > (1LL << 30)) return ctx_fail(c, LBFFS_E_ARG, "lbffs_build_sdf: too many triangles");
    }
    if ((ntri > 0 && (!verts || !normals)) || !(dr >= 0.f) || !(dr < 1024.f) || !std::isfinite(dr_walls) ||
        dr_walls > 1e6f)
        return ctx_fail(c, LBFFS_E_ARG, "lbffs_build_sdf: bad argument");
    {
        const int rc = ctx_io_wait(c);  // an asynchronous file write may still read the geometry fields
        if (rc != LBFFS_OK) return rc;
    }
    cudaError_t e = cudaSetDevice(c->d.device);
    if (e != cudaSuccess) return ctx_fail(c, LBFFS_E_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    const int nx = c->d.nx, ny = c->d.ny, nz = c->d.nz;
    const long long E = c->E;
    const unsigned nb = (unsigned)((E + 255) / 256);

    // the last patch's triangles, binned into bricks in ascending order
    const long long t0 = last, nt = ntri - t0;
    const int nbx = (nx + SDF_BX - 1) / SDF_BX, nby = (ny + SDF_BY - 1) / SDF_BY, nbz = (nz + SDF_BZ - 1) / SDF_BZ;
    const long long nbricks = (long long)nbx * nby * nbz;
    std::vector<SdfTri> tri((size_t)nt);
    std::vector<long long> off((size_t)nbricks + 1, 0);
    const double reach = (double)dr + 1.0;
    const int bsz[3] = {SDF_BX, SDF_BY, SDF_BZ}, nbv[3] = {nbx, nby, nbz};
    auto brick_span = [&](const SdfTri& T, int lo[3], int hi[3]) {
        for (int d = 0; d < 3; d++) {
            if (!std::isfinite(T.c[d])) return false;
            lo[d] = (int)std::max(0.0, std::floor(((double)T.c[d] - reach) / bsz[d]));
            hi[d] = (int)std::min((double)nbv[d] - 1, std::floor(((double)T.c[d] + reach) / bsz[d]));
            if (lo[d] > hi[d]) return false;
        }
        return true;
    };
    auto touches = [&](const SdfTri& T, int bx, int by, int bz) {  // brick box within dr + 1 of the centroid
        const int b0[3] = {bx * SDF_BX, by * SDF_BY, bz * SDF_BZ};
        double d2 = 0.0;
        for (int d = 0; d < 3; d++) {
            const double x = T.c[d], a = b0[d], b = b0[d] + bsz[d] - 1;
            const double g = x < a ? a - x : (x > b ? x - b : 0.0);
            d2 += g * g;
        }
        return d2 <= reach * reach;
    };
    for (long long t = 0; t < nt; t++) {
        const float* v = verts + 9 * (t0 + t);
        const float* nr = normals + 3 * (t0 + t);
        SdfTri& T = tri[(size_t)t];
        for (int d = 0; d < 3; d++) {
            T.c[d] = ((v[d] + v[3 + d]) + v[6 + d]) / 3.f;  // float arithmetic, each step rounded
            T.n[d] = nr[d];
        }
        int lo[3], hi[3];
        if (!brick_span(T, lo, hi)) continue;
        for (int bz = lo[2]; bz <= hi[2]; bz++)
            for (int by = lo[1]; by <= hi[1]; by++)
                for (int bx = lo[0]; bx <= hi[0]; bx++)
                    if (touches(T, bx, by, bz)) off[(size_t)(((long long)bz * nby + by) * nbx + bx) + 1]++;
    }
    for (size_t b = 0; b < (size_t)nbricks; b++) off[b + 1] += off[b];
    const size_t nent = (size_t)off[(size_t)nbricks];
    std::vector<int> ent(nent > 0 ? nent : 1);
    {
        std::vector<long long> fill(off.begin(), off.end() - 1);
        for (long long t = 0; t < nt; t++) {
            const SdfTri& T = tri[(size_t)t];
            int lo[3], hi[3];
            if (!brick_span(T, lo, hi)) continue;
            for (int bz = lo[2]; bz <= hi[2]; bz++)
                for (int by = lo[1]; by <= hi[1]; by++)
                    for (int bx = lo[0]; bx <= hi[0]; bx++)
                        if (touches(T, bx, by, bz))
                            ent[(size_t)fill[(size_t)(((long long)bz * nby + by) * nbx + bx)]++] = (int)t;
        }
    }

    SdfTri* d_tri = nullptr;
    long long* d_off = nullptr;
    int* d_ent = nullptr;
    uint8_t *m0 = nullptr, *m1 = nullptr;
    e = ctx_alloc_bytes(c, (void**)&d_tri, sizeof(SdfTri) * (size_t)(nt > 0 ? nt : 1));
    if (e == cudaSuccess) e = ctx_alloc_bytes(c, (void**)&d_off, sizeof(long long) * off.size());
    if (e == cudaSuccess) e = ctx_alloc_bytes(c, (void**)&d_ent, sizeof(int) * ent.size());
    if (e == cudaSuccess) e = ctx_alloc_bytes(c, (void**)&m0, (size_t)E);
    if (e == cudaSuccess) e = ctx_alloc_bytes(c, (void**)&m1, (size_t)E);
    if (e == cudaSuccess && nt > 0)
        e = cudaMemcpyAsync(d_tri, tri.data(), sizeof(SdfTri) * (size_t)nt, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_off, off.data(), sizeof(long long) * off.size(), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_ent, ent.data(), sizeof(int) * ent.size(), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        k_sdf_fill<<<nb, 256, 0, c->stream>>>(c->sdf, E, sdf_ini);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && npatch > 0) {
        const int r = (int)dr;
        k_dilate<<<nb, 256, 0, c->stream>>>(c->nei, m0, nx, ny, nz, 0, r);
        k_dilate<<<nb, 256, 0, c->stream>>>(m0, m1, nx, ny, nz, 1, r);
        k_dilate<<<nb, 256, 0, c->stream>>>(m1, m0, nx, ny, nz, 2, r);
        e = cudaGetLastError();
        if (e == cudaSuccess && nbricks > 0) {
            k_sdf_bricks<<<(unsigned)nbricks, SDF_BS, 0, c->stream>>>(d_tri, d_off, d_ent, m0, nx, ny, nz, nbx, nby, dr,
                                                                      p, sdf_ini, c->sdf);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) {
        const int n = (int)dr_walls;  // int(dr) of the loops `i < int(dr) + 1`
        if (n >= 0) {
            k_sdf_bwalls<<<nb, 256, 0, c->stream>>>(c->sdf, c->iarr[1], c->iarr[2], c->iarr[3], nx, ny, nz, n);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    ctx_free(c, d_tri);
    ctx_free(c, d_off);
    ctx_free(c, d_ent);
    ctx_free(c, m0);
    ctx_free(c, m1);
    if (e != cudaSuccess) return ctx_fail(c, LBFFS_E_CUDA, std::string("lbffs_build_sdf: ") + cudaGetErrorString(e));
    c->dirty = true;
    return LBFFS_OK;
}

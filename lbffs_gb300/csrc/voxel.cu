// Solid / neiSolid voxelisation of an STL surface on the device (src/walls.hpp:24-216), bit for bit
// the reference's host result.
//
// isInner (walls.hpp:73-157) counts, for a cell (i, j, k) inside the STL's bounding box, the
// triangles whose y/z box contains (j, k) and that the ray from the cell along +x crosses
// (isCross, walls.hpp:24-71: Cramer's rule on the triangle edges with the ray direction
// (-1, 0, 0) as third column); an odd count makes the cell solid.  Here the triangles are binned
// once per (j, k) column on the host with the same inclusive float comparisons, and one CTA per
// column tests every cell of the column against its candidates.  Every float operation is the
// reference's, in its order and without contraction (__fmul_rn / __fadd_rn / __fsub_rn /
// __fdiv_rn), and the comparisons are IEEE, so NaN results behave as in the reference.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "ctx.h"

namespace lbffs {
namespace {

struct VoxTri {
    float v0[3], a[3], b[3];  // first vertex, v1 - v0, v2 - v0
};

// det(a, b, c) of walls.hpp:18-22, left to right
__device__ __forceinline__ float det3(const float (&a)[3], const float (&b)[3], const float (&c)[3])
{
    float t = __fmul_rn(__fmul_rn(a[0], b[1]), c[2]);
    t = __fadd_rn(t, __fmul_rn(__fmul_rn(a[1], b[2]), c[0]));
    t = __fadd_rn(t, __fmul_rn(__fmul_rn(a[2], b[0]), c[1]));
    t = __fsub_rn(t, __fmul_rn(__fmul_rn(a[0], b[2]), c[1]));
    t = __fsub_rn(t, __fmul_rn(__fmul_rn(a[1], b[0]), c[2]));
    t = __fsub_rn(t, __fmul_rn(__fmul_rn(a[2], b[1]), c[0]));
    return t;
}

// isCross (walls.hpp:24-71)
__device__ __forceinline__ bool is_cross(const VoxTri& t, int i, int j, int k)
{
    const float a[3] = {t.a[0], t.a[1], t.a[2]};
    const float b[3] = {t.b[0], t.b[1], t.b[2]};
    const float c[3] = {-1.f, 0.f, 0.f};
    const float d[3] = {__fsub_rn((float)i, t.v0[0]), __fsub_rn((float)j, t.v0[1]), __fsub_rn((float)k, t.v0[2])};
    const float x = __fdiv_rn(det3(d, b, c), det3(a, b, c));
    const float y = __fdiv_rn(det3(a, d, c), det3(a, b, c));
    const float z = __fdiv_rn(det3(a, b, d), det3(a, b, c));
    if (x < 0.f || x > 1.f) return false;
    if (y < 0.f || y > 1.f) return false;
    const float xy = __fadd_rn(x, y);
    if (xy < 0.f || xy > 1.f) return false;
    if (z < 0.f) return false;
    return true;
}

constexpr int VOX_BS = 128;

// One CTA per (j, k) column: solid[ic] = 1 for the cells of the column inside the STL box with an
// odd crossing count (setSolid, walls.hpp:159-184), then the optional inversion.
__global__ void __launch_bounds__(VOX_BS) k_voxel_columns(const VoxTri* __restrict__ tris, const int* __restrict__ col_off,
                                                          const int* __restrict__ col_tri, int nx, int ny, int nz,
                                                          float xmin, float xmax, float ymin, float ymax, float zmin,
                                                          float zmax, int invert, uint8_t* __restrict__ solid)
{
    __shared__ VoxTri st[VOX_BS];
    const int col = blockIdx.x;
    const int j = col % ny, k = col / ny;
    const bool in_yz = !((float)j < ymin || (float)j > ymax || (float)k < zmin || (float)k > zmax);
    const int t0 = col_off[col], t1 = col_off[col + 1];
    for (int i0 = 0; i0 < nx; i0 += VOX_BS) {
        const int i = i0 + threadIdx.x;
        int cross = 0;
        if (in_yz) {
            for (int base = t0; base < t1; base += VOX_BS) {
                __syncthreads();
                if (base + threadIdx.x < t1) st[threadIdx.x] = tris[col_tri[base + threadIdx.x]];
                __syncthreads();
                const int n = min(VOX_BS, t1 - base);
                if (i < nx)
                    for (int m = 0; m < n; m++) cross += is_cross(st[m], i, j, k) ? 1 : 0;
            }
        }
        if (i < nx) {
            const bool in_x = !((float)i < xmin || (float)i > xmax);
            const bool inner = in_yz && in_x && (cross % 2) != 0;
            const uint8_t s = inner ? 1 : 0;
            solid[((long long)k * ny + j) * nx + i] = invert ? (uint8_t)(1 - s) : s;
        }
    }
}

// setNeiSolid (walls.hpp:187-216): fluid cells off the domain faces (an axis of one cell excepted)
// with a solid upwind neighbour under periodic wrap
template <int Q>
__global__ void k_nei_solid(const uint8_t* __restrict__ solid, int nx, int ny, int nz, uint8_t* __restrict__ nei)
{
    const long long ic = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long E = (long long)nx * ny * nz;
    if (ic >= E) return;
    const int i = (int)(ic % nx), j = (int)((ic / nx) % ny), k = (int)(ic / ((long long)nx * ny));
    const bool inner = (nx == 1 && j != 0 && j != ny - 1 && k != 0 && k != nz - 1) ||
                       (ny == 1 && i != 0 && i != nx - 1 && k != 0 && k != nz - 1) ||
                       (nz == 1 && i != 0 && i != nx - 1 && j != 0 && j != ny - 1) ||
                       (i != 0 && i != nx - 1 && j != 0 && j != ny - 1 && k != 0 && k != nz - 1);
    uint8_t out = 0;
    if (inner && solid[ic] == 0) {
#pragma unroll
        for (int q = 0; q < Q; q++) {
            int ii = i - lat_c(Q, q, 0), jj = j - lat_c(Q, q, 1), kk = k - lat_c(Q, q, 2);
            ii = ii < 0 ? ii + nx : (ii >= nx ? ii - nx : ii);
            jj = jj < 0 ? jj + ny : (jj >= ny ? jj - ny : jj);
            kk = kk < 0 ? kk + nz : (kk >= nz ? kk - nz : kk);
            if (solid[((long long)kk * ny + jj) * nx + ii] == 1) out = 1;
        }
    }
    nei[ic] = out;
}

}  // namespace
}  // namespace lbffs

using namespace lbffs;

extern "C" int lbffs_voxelize(lbffs_ctx* c, const float* verts, long long ntri, int invert)
{
    if (!c || (ntri > 0 && !verts) || ntri < 0 || ntri > (1LL << 30))
        return ctx_fail(c, LBFFS_E_ARG, "lbffs_voxelize: bad argument");
    {
        const int rc = ctx_io_wait(c);  // an asynchronous file write may still read the geometry fields
        if (rc != LBFFS_OK) return rc;
    }
    cudaError_t e = cudaSetDevice(c->d.device);
    if (e != cudaSuccess) return ctx_fail(c, LBFFS_E_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    const int nx = c->d.nx, ny = c->d.ny, nz = c->d.nz;
    // triangle data and boxes exactly as stl.hpp:188-266 and the STL constructor (stl.hpp:538-553,
    // which starts the overall box at 0) compute them
    std::vector<VoxTri> tri((size_t)ntri);
    float xmin = 0.f, xmax = 0.f, ymin = 0.f, ymax = 0.f, zmin = 0.f, zmax = 0.f;
    std::vector<int> cnt((size_t)ny * nz + 1, 0);
    std::vector<int> jlo((size_t)ntri), jhi((size_t)ntri), klo((size_t)ntri), khi((size_t)ntri);
    for (long long t = 0; t < ntri; t++) {
        const float* v = verts + 9 * t;
        VoxTri& T = tri[(size_t)t];
        for (int d = 0; d < 3; d++) {
            T.v0[d] = v[d];
            T.a[d] = v[3 + d] - v[d];
            T.b[d] = v[6 + d] - v[d];
        }
        const float eymin = fminf(v[1], fminf(v[4], v[7])), eymax = fmaxf(v[1], fmaxf(v[4], v[7]));
        const float ezmin = fminf(v[2], fminf(v[5], v[8])), ezmax = fmaxf(v[2], fmaxf(v[5], v[8]));
        xmin = fminf(xmin, fminf(v[0], fminf(v[3], v[6])));
        xmax = fmaxf(xmax, fmaxf(v[0], fmaxf(v[3], v[6])));
        ymin = fminf(ymin, eymin);
        ymax = fmaxf(ymax, eymax);
        zmin = fminf(zmin, ezmin);
        zmax = fmaxf(zmax, ezmax);
        // columns (j, k) with float(j) >= eymin && float(j) <= eymax && the same for k (walls.hpp:118-124)
        auto lo = [](float m) { return std::isnan(m) ? 1 : (int)std::max(-1.0, std::ceil((double)m)); };
        auto hi = [](float m, int n) { return std::isnan(m) ? 0 : (int)std::min((double)n - 1, std::floor((double)m)); };
        jlo[(size_t)t] = std::max(0, lo(eymin));
        jhi[(size_t)t] = hi(eymax, ny);
        klo[(size_t)t] = std::max(0, lo(ezmin));
        khi[(size_t)t] = hi(ezmax, nz);
        for (int k = klo[(size_t)t]; k <= khi[(size_t)t]; k++)
            for (int j = jlo[(size_t)t]; j <= jhi[(size_t)t]; j++) cnt[(size_t)k * ny + j + 1]++;
    }
    for (size_t col = 0; col < (size_t)ny * nz; col++) cnt[col + 1] += cnt[col];
    const size_t nent = (size_t)cnt[(size_t)ny * nz];
    std::vector<int> ent(nent > 0 ? nent : 1), fill(cnt.begin(), cnt.end() - 1);
    for (long long t = 0; t < ntri; t++)  // ascending triangle order inside every column
        for (int k = klo[(size_t)t]; k <= khi[(size_t)t]; k++)
            for (int j = jlo[(size_t)t]; j <= jhi[(size_t)t]; j++) ent[(size_t)fill[(size_t)k * ny + j]++] = (int)t;

    VoxTri* d_tri = nullptr;
    int *d_off = nullptr, *d_ent = nullptr;
    e = ctx_alloc_bytes(c, (void**)&d_tri, sizeof(VoxTri) * (size_t)(ntri > 0 ? ntri : 1));
    if (e == cudaSuccess) e = ctx_alloc_bytes(c, (void**)&d_off, sizeof(int) * cnt.size());
    if (e == cudaSuccess) e = ctx_alloc_bytes(c, (void**)&d_ent, sizeof(int) * ent.size());
    if (e == cudaSuccess && ntri > 0)
        e = cudaMemcpyAsync(d_tri, tri.data(), sizeof(VoxTri) * (size_t)ntri, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_off, cnt.data(), sizeof(int) * cnt.size(), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_ent, ent.data(), sizeof(int) * ent.size(), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        k_voxel_columns<<<(unsigned)((long long)ny * nz), VOX_BS, 0, c->stream>>>(
            d_tri, d_off, d_ent, nx, ny, nz, xmin, xmax, ymin, ymax, zmin, zmax, invert, c->solid);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        const unsigned nb = (unsigned)((c->E + 255) / 256);
        if (c->Q == 19) k_nei_solid<19><<<nb, 256, 0, c->stream>>>(c->solid, nx, ny, nz, c->nei);
        else k_nei_solid<27><<<nb, 256, 0, c->stream>>>(c->solid, nx, ny, nz, c->nei);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    ctx_free(c, d_tri);
    ctx_free(c, d_off);
    ctx_free(c, d_ent);
    if (e != cudaSuccess) return ctx_fail(c, LBFFS_E_CUDA, std::string("lbffs_voxelize: ") + cudaGetErrorString(e));
    c->dirty = true;  // flags, boundary words and lists are rebuilt at the next step
    return LBFFS_OK;
}

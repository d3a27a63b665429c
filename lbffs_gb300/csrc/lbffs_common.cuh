// Shared device definitions of the GB300 LBFFS step: lattice tables, population
// storage codecs, per-cell flag bits and the kernel argument block.
//
// Data layout in HBM (one context = one lattice):
//   populations   two copies (pull ping-pong) of Q planes; each plane is the grid with a
//                 one-cell ghost layer on every side, rows padded so that every row of
//                 interior cells starts on a 32-byte sector: cell (i,j,k) lives at
//                 ip = porg + k*pxy + j*px + i of plane q (plane stride pE).  Elements are
//                 float (FP32), or a shifted/scaled half / bfloat16.  The ghost layer holds,
//                 for each population that crosses the domain border, the value the
//                 reference's face streaming would pull (wrap, bounce-back or mirror), so
//                 every cell pulls population q from ip - (c_x + c_y*px + c_z*pxy).
//   cell arrays   everything else is indexed by ic = (k*ny + j)*nx + i (the reference's
//                 own layout, src/base.hpp:20)
//   flags         u8 per cell (FL_* bits below), built on the device from the
//                 reference's boundary/solid/neiSolid/sdf/omega arrays
//   bc            u16 per cell: boundary1 | boundary2<<3 | boundary3<<6 | face<<9
//   macroscopics  rho,u,v,w,tauSGS, two copies (previous step / this step); only
//                 cells whose values are read later are written each step
//   special list  u32 indices of domain-face and STL-link cells, which take the
//                 general boundary path; every other fluid cell takes the lean
//                 bulk path (19 or 27 loads, collision, 19 or 27 stores)
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lbffs_cuda.h"

namespace lbffs {

// Boundary codes: src/input.hpp:221-256
enum BcCode { BC_CYCLIC = 0, BC_BB = 1, BC_OUTLET = 3, BC_SYM = 4, BC_FIXVEL = 5, BC_FIXDEN = 6, BC_WALLFN = 7 };
enum Storage { ST_FP32 = 0, ST_FP16S = 1, ST_BF16S = 2 };
enum Collision { COLL_RR = 0, COLL_CUMULANT = 1 };
enum Sgs { SGS_SMAG = 0, SGS_WALE = 1 };
enum Wall { WALL_BB = 0, WALL_IBB = 1 };

// Cell flags
constexpr uint8_t FL_SOLID = 1;    // solid cell: skipped (kernel.cl:3549)
constexpr uint8_t FL_SPECIAL = 2;  // domain-face or STL-link cell: general path
constexpr uint8_t FL_STORE = 4;    // macroscopics are read by a neighbour next step: store them
constexpr uint8_t FL_SDF = 8;      // near-wall damping factor < 1: read sdf
constexpr uint8_t FL_OMEGA = 16;   // omega differs from the uniform omega0: read omega[]
constexpr uint8_t FL_LINK = 32;    // has at least one STL link
constexpr uint8_t FL_FACE = 64;    // on the domain border (face codes apply)

// bulk kernel tiling: BULK_BX threads per block, BULK_V cells per thread (32 apart)
constexpr int BULK_BX = 128;
constexpr int BULK_V = 2;
// cells per thread of the D3Q27 cumulant and WALE bulk kernels (a build-time tuning value).  One:
// 27 populations per thread leave room for twice the resident warps of two cells (80 against 116
// registers), which measured 11-15 % faster on the 768x192x192 LES step and 1.5 % on the 256^3 cavity.
#ifndef LBFFS_BULK_V27
#define LBFFS_BULK_V27 1
#endif
// D3Q27 recursive regularised bulk cells with Smagorinsky (or no) SGS: two cells per thread with the
// moment-form collision on packed FP32x2 pairs (1), or the generic one-cell path (0); build-time
#ifndef LBFFS_BULK_PAIR27
#define LBFFS_BULK_PAIR27 1
#endif
// the step kernels can pull across the grid's border themselves (StepArgs::border_pulls); 0 compiles
// that choice out, and the library then fills the ghost layer before every step (a build-time choice)
#ifndef LBFFS_BORDER_PULLS
#define LBFFS_BORDER_PULLS 1
#endif
// the bulk kernels with pulls across the x faces (border_pulls 2) are built for D3Q19 and for FP32
// D3Q27; with 2-byte D3Q27 storage they measured slower than the ghost fill they replace (the
// 256^3 cavity: 0.430 against 0.419 ms per step), and those lattices keep the ghost layer
__host__ __device__ constexpr bool xface_pulls_built(int Q, int S) { return Q == 19 || S == ST_FP32; }

template <int Q, int COLL = 0, int SGS = 0>
__host__ __device__ constexpr int bulk_v()
{
    return Q == 19 ? BULK_V : (LBFFS_BULK_PAIR27 && COLL == 0 && SGS == 0) ? 2 : LBFFS_BULK_V27;
}

constexpr float FP16S_SCALE = 32768.0f;  // (f - w) * 2^15 keeps |f - w| < 2 in range, 1.9e-9 above subnormals
constexpr float FP16S_INV = 1.0f / 32768.0f;

// ---- lattice tables (reference order: D3Q19 kernel.cl:3555-3560, D3Q27 kernel.cl:2742-2747) ----
__host__ __device__ constexpr int lat_c(int Q, int q, int a)
{
    constexpr int c19[19][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},   {0, 0, -1},
                                {1, 1, 0},  {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 0, 1},  {-1, 0, -1}, {1, 0, -1},
                                {-1, 0, 1}, {0, 1, 1},   {0, -1, -1}, {0, 1, -1}, {0, -1, 1}};
    constexpr int c27[27][3] = {{0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},   {0, -1, 0}, {0, 0, 1},  {0, 0, -1},
                                {1, 1, 0},   {-1, -1, 0}, {1, -1, 0},  {-1, 1, 0},  {1, 0, 1},  {-1, 0, -1}, {1, 0, -1},
                                {-1, 0, 1},  {0, 1, 1},   {0, -1, -1}, {0, 1, -1},  {0, -1, 1}, {1, 1, 1},  {-1, -1, -1},
                                {-1, 1, 1},  {1, -1, -1}, {1, -1, 1},  {-1, 1, -1}, {1, 1, -1}, {-1, -1, 1}};
    return Q == 19 ? c19[q][a] : c27[q][a];
}

__host__ __device__ constexpr int lat_n2(int Q, int q)
{
    return lat_c(Q, q, 0) * lat_c(Q, q, 0) + lat_c(Q, q, 1) * lat_c(Q, q, 1) + lat_c(Q, q, 2) * lat_c(Q, q, 2);
}

__host__ __device__ constexpr float lat_w(int Q, int q)
{
    return Q == 19 ? (lat_n2(Q, q) == 0 ? 1.0f / 3.0f : lat_n2(Q, q) == 1 ? 1.0f / 18.0f : 1.0f / 36.0f)
                   : (lat_n2(Q, q) == 0   ? float(8.0 / 27.0)
                      : lat_n2(Q, q) == 1 ? float(2.0 / 27.0)
                      : lat_n2(Q, q) == 2 ? float(1.0 / 54.0)
                                          : float(1.0 / 216.0));
}

__host__ __device__ constexpr int lat_find(int Q, int x, int y, int z)
{
    for (int q = 0; q < Q; q++)
        if (lat_c(Q, q, 0) == x && lat_c(Q, q, 1) == y && lat_c(Q, q, 2) == z) return q;
    return -1;
}

__host__ __device__ constexpr int lat_opp(int Q, int q)
{
    return lat_find(Q, -lat_c(Q, q, 0), -lat_c(Q, q, 1), -lat_c(Q, q, 2));
}

// the wall codes: a population crossing a face with one of them is missing (bounce-back / mirror)
__host__ __device__ __forceinline__ bool is_wall_code(int b) { return b == 1 || b == 4 || b == 5 || b == 6 || b == 7; }

// bounce-back / mirror direction for a missing link on a domain face (reflectOrMirrorQ, D3Q19
// kernel.cl:114-326; D3Q27 kernel.cl:1133-1146 with mirrorQx/y/z)
template <int Q>
__host__ __device__ __forceinline__ int missing_dir(int q, const int (&b)[3])
{
    const int c0 = lat_c(Q, q, 0), c1 = lat_c(Q, q, 1), c2 = lat_c(Q, q, 2);
    const int r = lat_opp(Q, q);
    if (Q == 19) {
        if ((c0 != 0) + (c1 != 0) + (c2 != 0) < 2) return r;
        if (c0 != 0 && b[0] == BC_SYM) return lat_find(Q, -c0, c1, c2);
        if (c1 != 0 && b[1] == BC_SYM) return lat_find(Q, c0, -c1, c2);
        if (c2 != 0 && b[2] == BC_SYM) return lat_find(Q, c0, c1, -c2);
        return r;
    }
    int out = r;
    if (b[0] == BC_SYM) out = c0 ? lat_find(Q, -c0, c1, c2) : r;
    if (b[1] == BC_SYM) out = c1 ? lat_find(Q, c0, -c1, c2) : r;
    if (b[2] == BC_SYM) out = c2 ? lat_find(Q, c0, c1, -c2) : r;
    return out;
}

// ---- population storage codecs ----
template <int S>
struct Codec;

template <>
struct Codec<ST_FP32> {
    using T = float;
    static __device__ __forceinline__ float load(const T* p, float) { return __ldg(p); }
    static __device__ __forceinline__ void store(T* p, float v, float) { __stcs(p, v); }
    // held value in the bulk kernel: f itself (DEV = false), unscaled (HS = 1)
    static constexpr bool DEV = false;
    static constexpr int HS = 1;
    static __device__ __forceinline__ float load_held(const T* p) { return __ldg(p); }
    static __device__ __forceinline__ void store_held(T* p, float v) { __stcs(p, v); }
};

// FP16S: IEEE half of (f - w_q) * 2^15; arithmetic stays FP32.
template <>
struct Codec<ST_FP16S> {
    using T = __half;
    static __device__ __forceinline__ float load(const T* p, float w)
    {
        return fmaf(__half2float(__ldg(p)), FP16S_INV, w);
    }
    static __device__ __forceinline__ void store(T* p, float v, float w)
    {
        *p = __float2half_rn((v - w) * FP16S_SCALE);
    }
    // held value in the bulk kernel: the stored number itself, 2^15 (f - w) (DEV = true,
    // HS = 2^15); the collision folds the power-of-two scale into its constants, which
    // leaves every rounding unchanged
    static constexpr bool DEV = true;
    static constexpr int HS = 32768;
    static __device__ __forceinline__ float load_held(const T* p) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ void store_held(T* p, float gs) { *p = __float2half_rn(gs); }
};

// BF16S: bfloat16 of (f - w_q); arithmetic stays FP32.
template <>
struct Codec<ST_BF16S> {
    using T = __nv_bfloat16;
    static __device__ __forceinline__ float load(const T* p, float w) { return __bfloat162float(__ldg(p)) + w; }
    static __device__ __forceinline__ void store(T* p, float v, float w) { *p = __float2bfloat16_rn(v - w); }
    static constexpr bool DEV = true;
    static constexpr int HS = 1;
    static __device__ __forceinline__ float load_held(const T* p) { return __bfloat162float(__ldg(p)); }
    static __device__ __forceinline__ void store_held(T* p, float g) { *p = __float2bfloat16_rn(g); }
};

// x / d for 0 <= x < 2^31 by a multiply-high and a shift (round-up method of Granlund and
// Montgomery, 1994): l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, x / d = (mulhi(x, m) + x)
// >> l, the sum staying below 2^32 for x < 2^31
struct FastDiv {
    uint32_t m;
    int l;
};
inline FastDiv fast_div(uint32_t d)
{
    int l = 0;
    while ((1ull << l) < d) l++;
    const uint64_t m = ((1ull << 32) * ((1ull << l) - d)) / d + 1;
    return FastDiv{(uint32_t)m, l};
}
__device__ __forceinline__ int fdiv(int x, FastDiv f)
{
    const uint32_t t = __umulhi((uint32_t)x, f.m);
    return (int)((t + (uint32_t)x) >> f.l);
}

// Padded population planes: cell (i,j,k) at porg + k*pxy + j*px + i of a plane of pE elements.
struct PadGeom {
    int nx, ny, nz, px, pxy, porg;
    long long pE;
};


// ---- kernel argument block ----
struct StepArgs {
    const void* f_in;
    void* f_out;
    const uint8_t* flags;
    const uint16_t* bc;
    const uint8_t* solid;
    const uint8_t* nei_solid;
    const float *u0, *v0, *w0, *omega, *sdf;
    const float *rho_p, *u_p, *v_p, *w_p, *tau_p;  // previous step
    float *rho_n, *u_n, *v_n, *w_n, *tau_n;        // this step
    float *fwx, *fwy, *fwz;
    float *gx, *gy, *gz;
    const uint32_t* special;
    long long n_special;
    long long E;
    int nx, ny, nz;
    float omega0, dpdx, les, omega_b, spz, clim, cs;
    int damping;      // near-wall damping of the Smagorinsky eddy viscosity (enum lbffs_damping)
    // pulls across the grid's border: 0, from the ghost layer filled before each step (k_halo); 1 and
    // 2, straight from where the face streaming takes them (every face carries one boundary code per
    // axis: face_codes holds code (axis d, low / high face s) in bits 3 (2 d + s) .. 3 (2 d + s) + 2).
    // 1: both x faces carry boundary-kernel codes, so bulk cells cross only y / z faces; 2 and 3: bulk
    // cells lie on the x faces too (nz > 1), those of rows crossing no y / z face pulling their
    // x-crossing directions from fin_xlo / fin_xhi (2) or from the ghost slots at x = -1 / nx, which
    // they write for the next step after their collision (3: no Cyclic x face)
    int border_pulls;
    int face_codes;
    int sponge_mask;  // bit s set: face centre s (x-,x+,y-,y+,z-,z+) is Outlet/FixedDensity
    int store_all;    // store rho/u/v/w/tau for every fluid cell this step
    int bulk_kind;    // D3Q19 bulk kernel: 0 per-thread loads, 1 row-staged bulk copies (launch choice)
    int special_kind;  // boundary kernel: 0 one thread per listed cell, 1 a lane group per cell (launch choice)
    int l2_policy;    // L2 policy of the 2-byte bulk pairs' accesses: 0 none, 1 evict-first (2 evict-normal)
    int sgs, wall;    // Sgs / Wall selections (runtime in the boundary kernel)
    const int* ibm_box;  // device int[6] lo/hi of the marker box (cells inside store macroscopics), or null
    int* err;            // device error word (non-finite density seen), may be null
    // padded population planes: cell (i,j,k) at ip = porg + k*pxy + j*px + i (< 2^31)
    int px, pxy, porg;
    long long pE;
    // per-direction plane bases: fin_q[q][ip] is the cell's own value of population q,
    // fin_s[q][ip] the value it pulls (the plane base moved by the pull offset), and
    // fout_q[q][ip] where it writes
    const void* fin_q[27];
    const void* fin_s[27];
    void* fout_q[27];
    // border_pulls 2: the plane base from which a cell on the low (xlo, directions c_x > 0) / high
    // (xhi, c_x < 0) x face of a row crossing no other face pulls: the base of the missing direction's
    // own plane (fin_q) when the face carries a wall code, else the pull base shifted to the periodic
    // image (fin_s -+ nx elements); the other directions' entries are fin_s
    const void* fin_xlo[27];
    const void* fin_xhi[27];
};

__host__ __device__ __forceinline__ int pidx(const StepArgs& a, int i, int j, int k)
{
    return a.porg + k * a.pxy + j * a.px + i;
}

__device__ __forceinline__ bool in_box(const StepArgs& a, int i, int j, int k)
{
    if (!a.ibm_box) return false;
    const int* b = a.ibm_box;
    return i >= b[0] && i <= b[3] && j >= b[1] && j <= b[4] && k >= b[2] && k <= b[5];
}

// tauSpongeZone (D3Q19 kernel.cl:2444-2503); the blend is fused explicitly so that its rounding
// does not depend on the code around it
__device__ __forceinline__ float sponge_tau(const StepArgs& a, float tau, float tsgs, int i, int j, int k)
{
    if (a.sponge_mask == 0) return tau;
    const int x[3] = {i, j, k};
    const int N[3] = {a.nx, a.ny, a.nz};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const float n = (float)N[d];
        if ((a.sponge_mask >> (2 * d)) & 1) {
            if ((float)x[d] < n * a.spz) {
                const float fx = (float)x[d] / (n * a.spz);
                tau = fmaf(fx, tau, (1.f - fx) * (1.f - tsgs));
            }
        }
        if ((a.sponge_mask >> (2 * d + 1)) & 1) {
            if ((float)x[d] > n * (1.f - a.spz)) {
                const float fx = (float)(N[d] - x[d]) / (n * a.spz);
                tau = fmaf(fx, tau, (1.f - fx) * (1.f - tsgs));
            }
        }
    }
    return tau;
}

}  // namespace lbffs

// Fused pull-streaming + collision kernels (one LBM time step = k_bulk + k_special).
//
// k_bulk     one thread per cell of an x-row, grid (ceil(nx/BX), ny, nz).  Handles every
//            fluid cell that is neither on the domain border nor next to an STL wall:
//            Q coalesced loads (the x-shifted ones are served by L1/L2 sectors), local
//            macroscopics, Smagorinsky / WALE eddy viscosity, sponge ramp, collision,
//            Q streaming stores.  Macroscopics are written only for cells flagged
//            FL_STORE (someone reads them next step), in the IBM box, or on request.
// k_special  one thread per listed domain-face / STL-link cell: the reference's face
//            streaming with wall / mirror bounce-back, corner rule, FixedVelocity,
//            FixedDensity and Geier outlet, then STL bounce-back or Filippova-Hanel /
//            Mei-Luo-Shyy interpolated bounce-back with the momentum-exchange force.
//            Ordering of the boundary operators follows k_streamingCollision
//            (D3Q19_opencl/kernel.cl:3525-3646).
//
// Both kernels read only the previous-step populations and previous-step macroscopic
// buffers and write disjoint cells, so they need no ordering between them.
#pragma once
#include <type_traits>

#include "collide.cuh"
#include "lbffs_common.cuh"

namespace lbffs {

constexpr int SPECIAL_BS = 128;

// CTAs ahead whose pulled rows a 2-byte D3Q19 bulk CTA prefetches into L2 (0: none); a build-time
// tuning value.  608 (half a wave of 8-CTA-per-SM residency) measured 4 % faster on the 256^3
// FP16S / BF16S cavity than none or 304, the same as 1216.
// 2-byte D3Q19 bulk cells of k_bulk: the pulls are issued together with the flag loads (1) or
// after them (0); a build-time choice
#ifndef LBFFS_BULK_EAGER
#define LBFFS_BULK_EAGER 1
#endif
// the same for the D3Q19 pairs 32 apart (FP32 storage)
#ifndef LBFFS_BULK_EAGER32
#define LBFFS_BULK_EAGER32 1
#endif
// 2-byte D3Q19 bulk cells: a lane owns two adjacent cells (1) or two cells 32 apart (0); a
// build-time choice
#ifndef LBFFS_BULK_ADJ
#define LBFFS_BULK_ADJ 1
#endif
// L2 eviction priority of the 2-byte bulk pair path's pulls and stores: with LBFFS_BULK_EVICT 1
// they carry the L2 policy StepArgs::l2_policy chooses: evict-first when both population copies
// fit in L2 (the boundary kernel's scattered accesses then stay cached; 1024x256x4 FP16S cylinder
// channel +22 % MLUPS), none otherwise (256^3: evict-first measured 11 % slower, adjacent warps'
// shared sectors being evicted before their second read; evict-normal the same as none) and for
// the server's batches (an evict-last policy on the ghost fill's accesses measured no better).
// A build-time choice.
#ifndef LBFFS_BULK_EVICT
#define LBFFS_BULK_EVICT 1
#endif
#ifndef LBFFS_BULK_PREFETCH
#define LBFFS_BULK_PREFETCH 608
#endif

template <int Q>
__device__ __forceinline__ void macroscopics(const float (&ft)[Q], float dpdx, float& rho, float& u, float& v, float& w)
{
    float r = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
#pragma unroll
    for (int q = 0; q < Q; q++) {
        r += ft[q];
        if (lat_c(Q, q, 0)) mx += (float)lat_c(Q, q, 0) * ft[q];
        if (lat_c(Q, q, 1)) my += (float)lat_c(Q, q, 1) * ft[q];
        if (lat_c(Q, q, 2)) mz += (float)lat_c(Q, q, 2) * ft[q];
    }
    rho = r;
    u = mx / r;
    v = my / r;
    w = mz / r;
    u += 0.5f * dpdx / r;  // updateRhoUVW (kernel.cl:3509-3523)
}

// smagorinskyTauSGS (D3Q19 kernel.cl:2133-2201) without the damping factor
template <int Q>
__device__ __forceinline__ float smagorinsky(const float (&ft)[Q], float rho, float u, float v, float w, float omega,
                                             float les, float cs)
{
    const float tau = 1.f / omega;
    const float usq = u * u + v * v + w * w;
    float P[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // xx yy zz xy xz yz
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int cx = lat_c(Q, q, 0), cy = lat_c(Q, q, 1), cz = lat_c(Q, q, 2);
        const float cu = u * (float)cx + v * (float)cy + w * (float)cz;
        const float feq = (rho + 3.f * cu + 4.5f * cu * cu - 1.5f * usq) * lat_w(Q, q);
        const float d = ft[q] - feq;
        if (cx) P[0] += d;
        if (cy) P[1] += d;
        if (cz) P[2] += d;
        if (cx * cy) P[3] += (float)(cx * cy) * d;
        if (cx * cz) P[4] += (float)(cx * cz) * d;
        if (cy * cz) P[5] += (float)(cy * cz) * d;
    }
    const float pp = P[0] * P[0] + P[1] * P[1] + P[2] * P[2] + 2.f * (P[3] * P[3] + P[4] * P[4] + P[5] * P[5]);
    return les * 0.5f * (-tau + sqrtf(tau * tau + 18.f * 1.41421356237f * cs * cs * sqrtf(pp) / rho));
}

// Van Driest mixing length over Cs, (kappa / Cs) (1 - exp(-y+ / A+)) y, of the block the reference
// keeps commented out in smagorinskyTauSGS (D3Q19 kernel.cl:2178-2197, D3Q27 kernel.cl:2072-2091):
// y+ from the log law u+ = ln(E y+) / kappa at wall distance y with the cell's own speed, by the
// fixed-point iteration y+ <- (kappa |u| y / nu + y+) / (1 + ln(E y+)) from y+ = 1 (at most 10 times,
// until y+ moves by at most 0.001); kappa 0.41, A+ 26, E 9.8, nu = (tau - 1/2) / 3.  1 + 1e-10 is 1 in
// FP32, as in the reference's float expression.  The iteration runs on the hardware logarithm and
// an approximate division (a few ulp per step of a contraction whose result is used to 1e-3); the
// loop-invariant kappa |u| y / nu is formed once.
static __device__ __forceinline__ float van_driest_ratio(float y, float umag, float nu, float cs)
{
    const float kappa = 0.41f, Aplus = 26.f, Ek = 9.8f;
    const float a = kappa * umag * y / nu;
    float yp = 1.f, ypn;
    int it = 0;
    do {
        ypn = yp;
        yp = __fdividef(a + yp, 1.f + __logf(Ek * yp));
        it++;
    } while (fabsf(yp - ypn) > 0.001f && it < 10);
    return (kappa / cs) * (1.f - expf(-yp / Aplus)) * y;
}

// near-wall damping of the eddy relaxation time t (smagorinskyTauSGS, kernel.cl:2166-2199) for a
// cell at wall distance sdf with velocity (u, v, w) and relaxation rate omega
__device__ __forceinline__ float damping(const StepArgs& a, float t, float sdf, float u, float v, float w,
                                         float omega)
{
    if (sdf != 10000.f && sdf > 0.f && a.damping != LBFFS_DAMP_NONE) {
        float d;
        if (a.damping == LBFFS_DAMP_VAN_DRIEST)
            d = van_driest_ratio(sdf, sqrtf(u * u + v * v + w * w), (1.f / omega - 0.5f) / 3.f, a.cs);
        else
            d = 0.41f * sdf / a.cs;
        d = fminf(1.f, d);
        t *= d * d;
    }
    return t;
}

// waleTauSGS (D3Q19 kernel.cl:2267-2365) from a velocity-gradient tensor g[c][d] = du_c/dx_d
__device__ __forceinline__ float wale_from_grad(const float (&g)[3][3])
{
    float SS = 0.f;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const float s = 0.5f * (g[a][b] + g[b][a]);
            SS += s * s;
        }
    float gg[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) gg[a][b] = g[0][a] * g[b][0] + g[1][a] * g[b][1] + g[2][a] * g[b][2];
    const float tr = gg[0][0] + gg[1][1] + gg[2][2];
    float SdSd = 0.f;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const float sd = 0.5f * (gg[a][b] + gg[b][a]) - (a == b ? tr * (1.f / 3.f) : 0.f);
            SdSd += sd * sd;
        }
    const float cw = 0.325f;
    if (SS > 1e-24f && SdSd > 1e-24f)
        return 3.f * (cw * cw * powf(SdSd, 1.5f) / (powf(SS, 2.5f) + powf(SdSd, 1.25f))) * 3.f;
    return 0.f;
}

// previous-step neighbour velocity, own cell from the current step (reference read order)
__device__ __forceinline__ float vel_at(const StepArgs& a, int c, long long idx, long long self, const float (&own)[3])
{
    if (idx == self) return own[c];
    const float* p = c == 0 ? a.u_p : c == 1 ? a.v_p : a.w_p;
    return __ldg(p + idx);
}

static __device__ float wale_general(const StepArgs& a, int i, int j, int k, long long ic, const float (&own)[3])
{
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    // indices are clamped into the grid so axes shorter than 2 cells never read outside it
    auto id = [&](int ii, int jj, int kk) {
        ii = min(max(ii, 0), nx - 1);
        jj = min(max(jj, 0), ny - 1);
        kk = min(max(kk, 0), nz - 1);
        return ((long long)kk * ny + jj) * nx + ii;
    };
    float g[3][3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        g[c][0] = (i > 0 && i < nx - 1) ? 0.5f * (vel_at(a, c, id(i + 1, j, k), ic, own) - vel_at(a, c, id(i - 1, j, k), ic, own))
                  : (i == 0)            ? vel_at(a, c, id(1, j, k), ic, own) - vel_at(a, c, id(0, j, k), ic, own)
                                        : vel_at(a, c, id(nx - 1, j, k), ic, own) - vel_at(a, c, id(nx - 2, j, k), ic, own);
        g[c][1] = (j > 0 && j < ny - 1) ? 0.5f * (vel_at(a, c, id(i, j + 1, k), ic, own) - vel_at(a, c, id(i, j - 1, k), ic, own))
                  : (j == 0)            ? vel_at(a, c, id(i, 1, k), ic, own) - vel_at(a, c, id(i, 0, k), ic, own)
                                        : vel_at(a, c, id(i, ny - 1, k), ic, own) - vel_at(a, c, id(i, ny - 2, k), ic, own);
        g[c][2] = (k > 0 && k < nz - 1) ? 0.5f * (vel_at(a, c, id(i, j, k + 1), ic, own) - vel_at(a, c, id(i, j, k - 1), ic, own))
                  : (nz - 1 == 0 || k == 0) ? 0.f
                                            : vel_at(a, c, id(i, j, nz - 1), ic, own) - vel_at(a, c, id(i, j, nz - 2), ic, own);
    }
    return wale_from_grad(g);
}

template <int Q, int COLL>
__device__ __forceinline__ void collide(float (&ft)[Q], float rho, float u, float v, float w, float we, const StepArgs& a)
{
    if constexpr (Q == 19) {
        const float U[3] = {u - 0.5f * a.dpdx / rho, v, w};
        collide_rr19(ft, rho, U, we, a.omega_b, a.dpdx);
    } else if constexpr (COLL == COLL_CUMULANT) {
        collide_cumulant(ft, rho, u, v, w, we, a.omega_b, a.clim);
    } else {
        const float U[3] = {u - 0.5f * a.dpdx / rho, v, w};
        collide_rr27(ft, rho, U, we, a.omega_b, a.dpdx);
    }
}

// calcTauw (D3Q19 kernel.cl:1621-1655, D3Q27 1487-1522): wall shear stress from the tangential
// speed magUp 1.5 cells from the wall by Newton iterations on Spalding's law (kappa 0.42, E 9.1).
// As in the reference, the convergence test compares each new y+ with the first one (the
// loop's yPlus update declares a new variable), for at most 100 iterations.
__device__ __forceinline__ float calc_tauw(float rhow, float magUp, float nu)
{
    const float y = 1.5f, kappa = 0.42f, E = 9.1f;
    float ut = sqrtf(nu * magUp);
    const float yPlus = y * ut / nu;
    int iter = 0;
    float err;
    do {
        const float kUu = fminf(kappa * magUp / ut, 50.f);
        const float fkUu = expf(kUu) - 1.f - kUu * (1.f + 0.5f * kUu);
        const float func = -ut * y / nu + magUp / ut + (fkUu - kUu * kUu * kUu / 6.f) / E;
        const float dfunc = y / nu + magUp / (ut * ut) + (kUu * fkUu / ut) / E;
        ut = ut + func / dfunc;
        err = fabsf(yPlus - y * ut / nu);
    } while (err > 0.005f && ++iter < 100);
    ut = fmaxf(ut, 0.f);
    return rhow * ut * ut;
}

// ------------------------------------------------------------------------------------------

// upwindID_B with per-axis wall codes (face cells) or plain periodic wrap (other cells); -1 = missing
template <int Q>
__device__ __forceinline__ long long upwind(int q, const int (&x)[3], const int (&N)[3], const int (&b)[3], bool face)
{
    int n[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        n[d] = x[d] - lat_c(Q, q, d);
        if (n[d] < 0) {
            if (face && is_wall_code(b[d])) return -1;
            n[d] += N[d];
        } else if (n[d] >= N[d]) {
            if (face && is_wall_code(b[d])) return -1;
            n[d] -= N[d];
        }
    }
    return ((long long)n[2] * N[1] + n[1]) * N[0] + n[0];
}

// ---- border pulls (StepArgs::border_pulls 1-3): the face streaming without a ghost fill ----
// A cell on the grid's border pulls population q from outside the grid when P - c_q lies there.  The
// reference's face streaming (upwindID_B + reflectOrMirrorQ, D3Q19 kernel.cl:114-575, D3Q27
// kernel.cl:1133-1146) then takes P's own previous value of missing_dir(q) when a crossed face of P
// carries a wall code, else the previous value of q of the periodically wrapped upwind cell.  In this
// mode the cell reads that value where it lies instead of from a ghost layer filled before the step.
// A cell's face codes come from face_codes (one code per face and axis, checked when the geometry is
// committed); the face flag is set on every border cell (on the z faces only when nz > 1).
__device__ __forceinline__ int face_code(const StepArgs& a, int d, int s) { return (a.face_codes >> (3 * (2 * d + s))) & 7; }

// the code of axis d of a cell at coordinate xd: its face's code when the cell is on a face of that
// axis (the low face when the axis is one cell long), else 0
__device__ __forceinline__ int cell_code(const StepArgs& a, int xd, int Nd, int d)
{
    return xd == 0 ? face_code(a, d, 0) : xd == Nd - 1 ? face_code(a, d, 1) : 0;
}

// Where a border cell's pulls come from: its border flags, face flag and codes, and per axis the
// padded-index shift to the periodic image (grid extent times the axis stride).
struct BorderCell {
    bool lo[3], hi[3];
    bool face;
    int b[3];
    int wrap[3];
};

__device__ __forceinline__ BorderCell border_cell(const StepArgs& a, int i, int j, int k)
{
    BorderCell g;
    const int x[3] = {i, j, k}, N[3] = {a.nx, a.ny, a.nz}, st[3] = {1, a.px, a.pxy};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        g.lo[d] = x[d] == 0;
        g.hi[d] = x[d] == N[d] - 1;
        g.b[d] = cell_code(a, x[d], N[d], d);
        g.wrap[d] = N[d] * st[d];
    }
    g.face = i == 0 || i == a.nx - 1 || j == 0 || j == a.ny - 1 || (a.nz > 1 && (k == 0 || k == a.nz - 1));
    return g;
}

// The border of a bulk row (j, k) in a border-pull context: the y / z faces it crosses (row_crosses:
// the row lies on one of them).  row_border leaves the row's x flags and x code clear, so every
// cell of the row off the x faces shares its mapping; the cells of such a row take border_cell.
__device__ __forceinline__ bool row_crosses(const StepArgs& a, int j, int k)
{
    return a.border_pulls && (j == 0 || j == a.ny - 1 || k == 0 || k == a.nz - 1);
}

// Bulk cells on the x faces (border_pulls 2 and 3; the bulk kernels' XM 1 and 2 instantiations):
// xface_cell, cell i of a row lies on an x face.  In a row that crosses a y / z face such a cell takes
// its own border (border_cell) for the directions with c_x != 0.  In a row that crosses no other face
// it pulls its x-crossing directions (c_x > 0 on the low face, c_x < 0 on the high face) from the
// plane bases fin_xlo / fin_xhi (XM 1, any x-face codes), or from the ghost slots at x = -1 / nx
// like every other cell, which it wrote itself at the end of the previous step (XM 2, x faces
// without a Cyclic code: xface_push).
__device__ __forceinline__ bool xface_cell(const StepArgs& a, int i) { return i == 0 || i == a.nx - 1; }

// the x-face bits of a pair of cells i0 < i1 of rows crossing no y / z face (-1: no cell): bit 0, i0
// on the low face; bit 1, i0 on the high face; bit 2, i1 on the high face
__device__ __forceinline__ int xface_bits(const StepArgs& a, int i0, int i1)
{
    return (i0 == 0 ? 1 : 0) | (i0 == a.nx - 1 ? 2 : 0) | (i1 == a.nx - 1 ? 4 : 0);
}

// the plane base direction q of a cell at the low (lo) / high (hi) x face of a row crossing no other
// face pulls from
template <int Q>
__device__ __forceinline__ const void* xface_base(const StepArgs& a, int q, bool lo, bool hi)
{
    if (lat_c(Q, q, 0) > 0 && lo) return a.fin_xlo[q];
    if (lat_c(Q, q, 0) < 0 && hi) return a.fin_xhi[q];
    return a.fin_s[q];
}

__device__ __forceinline__ BorderCell row_border(const StepArgs& a, int j, int k)
{
    BorderCell g;
    g.lo[0] = g.hi[0] = false;
    g.b[0] = 0;
    g.wrap[0] = a.nx;
    g.lo[1] = j == 0;
    g.hi[1] = j == a.ny - 1;
    g.lo[2] = k == 0;
    g.hi[2] = k == a.nz - 1;
    g.b[1] = cell_code(a, j, a.ny, 1);
    g.b[2] = cell_code(a, k, a.nz, 2);
    g.wrap[1] = a.ny * a.px;
    g.wrap[2] = a.nz * a.pxy;
    g.face = j == 0 || j == a.ny - 1 || (a.nz > 1 && (k == 0 || k == a.nz - 1));
    return g;
}

// the element index (in the population array a.f_in, planes pE apart) that population q of border
// cell g at padded index ip pulls: the ghost position ip - c_q of plane q moved to the periodic image,
// or the cell's own element of the missing direction.  Plane and offset are formed arithmetically.
template <int Q>
__device__ __forceinline__ long long border_pull(const StepArgs& a, const BorderCell& g, int q, int ip)
{
    const int c[3] = {lat_c(Q, q, 0), lat_c(Q, q, 1), lat_c(Q, q, 2)};
    int shift = 0;
    bool out = false, wall = false;
#pragma unroll
    for (int e = 0; e < 3; e++) {
        if (c[e] > 0 && g.lo[e]) {  // P - c_q below the low face
            out = true;
            shift += g.wrap[e];
            wall |= is_wall_code(g.b[e]);
        } else if (c[e] < 0 && g.hi[e]) {  // above the high face
            out = true;
            shift -= g.wrap[e];
            wall |= is_wall_code(g.b[e]);
        }
    }
    const long long pull = (long long)q * a.pE + (ip - (c[0] + c[1] * a.px + c[2] * a.pxy));
    if (!out) return pull;
    if (!(g.face && wall)) return pull + shift;
    return (long long)missing_dir<Q>(q, g.b) * a.pE + ip;
}

// The collision of one bulk cell whose Q pulled populations are in ft (held form for D3Q19):
// macroscopics, eddy viscosity, sponge, stores of the macroscopic fields that are read later, and
// the collision in place.
template <int Q, int S, int COLL, int SGS, bool LES>
__device__ __forceinline__ void bulk_collide(const StepArgs& a, float (&ft)[Q], uint8_t fl, int i, int j, int k,
                                             int ic)
{
    const float omega = (fl & FL_OMEGA) ? __ldg(a.omega + ic) : a.omega0;
    float rho, u, v, w, tsgs = 0.f;
    if constexpr (Q == 19) {
        constexpr int HS = Codec<S>::HS;
        const Mom19 m = moments19<Codec<S>::DEV, HS>(ft);
        rho = m.rho;
        const float ir = 1.f / rho;
        const float irs = ir * (1.f / HS);
        const float hd = ir * (0.5f * a.dpdx);
        u = fmaf(m.j[0], irs, hd);  // updateRhoUVW (kernel.cl:3509-3523)
        v = m.j[1] * irs;
        w = m.j[2] * irs;
        if constexpr (SGS == SGS_WALE) {
            const float own[3] = {u, v, w};
            tsgs = wale_general(a, i, j, k, ic, own);
        } else if constexpr (LES) {
            tsgs = smagorinsky19<HS>(m, u, v, w, omega, a.les, a.cs);
            if (fl & FL_SDF) tsgs = damping(a, tsgs, __ldg(a.sdf + ic), u, v, w, omega);
        }
        if (a.err && !(rho == rho)) atomicOr(a.err, 1);
        const float tau = sponge_tau(a, 1.f / omega, tsgs, i, j, k);
        const float we = 1.f / (tau + tsgs);
        if (a.store_all || (fl & FL_STORE) || SGS == SGS_WALE || in_box(a, i, j, k)) {
            a.rho_n[ic] = rho;
            a.u_n[ic] = u;
            a.v_n[ic] = v;
            a.w_n[ic] = w;
            a.tau_n[ic] = tsgs;
        }
        const float U[3] = {u - hd, v, w};
        collide_rr19m<HS>(ft, m, U, we, ir, a.omega_b, a.dpdx);
    } else if constexpr (SGS != SGS_WALE) {
        // D3Q27: one pass over the 13 opposite pairs gives rho, j and the second moments that both
        // the Smagorinsky stress and the recursive regularised collision need
        const Mom27 m = moments27(ft);
        rho = m.rho;
        const float ir = 1.f / rho;
        u = m.j[0] * ir + 0.5f * a.dpdx * ir;  // updateRhoUVW (kernel.cl:3509-3523)
        v = m.j[1] * ir;
        w = m.j[2] * ir;
        if constexpr (LES) {
            tsgs = smag_tau(smag_pp_raw(m.s, rho, u, v, w), rho, omega, a.les, a.cs);
            if (fl & FL_SDF) tsgs = damping(a, tsgs, __ldg(a.sdf + ic), u, v, w, omega);
        }
        if (a.err && !(rho == rho)) atomicOr(a.err, 1);
        const float tau = sponge_tau(a, 1.f / omega, tsgs, i, j, k);
        const float we = 1.f / (tau + tsgs);
        if (a.store_all || (fl & FL_STORE) || in_box(a, i, j, k)) {
            a.rho_n[ic] = rho;
            a.u_n[ic] = u;
            a.v_n[ic] = v;
            a.w_n[ic] = w;
            a.tau_n[ic] = tsgs;
        }
        if constexpr (COLL == COLL_CUMULANT) {
            collide_cumulant(ft, rho, u, v, w, we, a.omega_b, a.clim);
        } else {
            const float U[3] = {u - 0.5f * a.dpdx * ir, v, w};
            collide_rr27m(ft, m, U, we, a.omega_b, a.dpdx);
        }
    } else {
        macroscopics<Q>(ft, a.dpdx, rho, u, v, w);
        const float own[3] = {u, v, w};
        tsgs = wale_general(a, i, j, k, ic, own);
        if (a.err && !(rho == rho)) atomicOr(a.err, 1);
        const float tau = sponge_tau(a, 1.f / omega, tsgs, i, j, k);
        const float we = 1.f / (tau + tsgs);
        a.rho_n[ic] = rho;
        a.u_n[ic] = u;
        a.v_n[ic] = v;
        a.w_n[ic] = w;
        a.tau_n[ic] = tsgs;
        collide<Q, COLL>(ft, rho, u, v, w, we, a);
    }
}

// The bulk step of one fluid cell: bulk_collide, then the Q streaming stores at ip.
template <int Q, int S, int COLL, int SGS, bool LES>
__device__ __forceinline__ void bulk_cell(const StepArgs& a, float (&ft)[Q], uint8_t fl, int i, int j, int k, int ic,
                                          int ip)
{
    using T = typename Codec<S>::T;
    constexpr bool HELD = (Q == 19);
    bulk_collide<Q, S, COLL, SGS, LES>(a, ft, fl, i, j, k, ic);
#pragma unroll
    for (int q = 0; q < Q; q++) {
        T* p = static_cast<T*>(a.fout_q[q]) + ip;
        if constexpr (HELD) Codec<S>::store_held(p, ft[q]);
        else Codec<S>::store(p, ft[q], lat_w(Q, q));
    }
}

// the per-lane test of bulk_collide2's plain path (the caller takes it over the whole warp)
__device__ __forceinline__ bool plain_pair(const StepArgs& a, const uint8_t (&fl)[2], const bool (&act)[2])
{
    return act[0] && act[1] && !((fl[0] | fl[1]) & (FL_OMEGA | FL_SDF | FL_STORE)) && !a.store_all && !a.ibm_box &&
           a.sponge_mask == 0;
}

// cell (i, j, k) lies in a sponge zone: the conditions of sponge_tau, which leaves tau unchanged
// everywhere else
__device__ __forceinline__ bool in_sponge(const StepArgs& a, int i, int j, int k)
{
    if (a.sponge_mask == 0) return false;
    const int x[3] = {i, j, k};
    const int N[3] = {a.nx, a.ny, a.nz};
    bool s = false;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const float n = (float)N[d];
        if ((a.sponge_mask >> (2 * d)) & 1) s |= (float)x[d] < n * a.spz;
        if ((a.sponge_mask >> (2 * d + 1)) & 1) s |= (float)x[d] > n * (1.f - a.spz);
    }
    return s;
}

// plain_pair for the cells (i0, j, k) and (i1, j, k): a sponge zone elsewhere in the lattice does not
// take them off the plain path
__device__ __forceinline__ bool plain_pair(const StepArgs& a, const uint8_t (&fl)[2], const bool (&act)[2], int i0,
                                           int i1, int j, int k)
{
    return act[0] && act[1] && !((fl[0] | fl[1]) & (FL_OMEGA | FL_SDF | FL_STORE)) && !a.store_all && !a.ibm_box &&
           !in_sponge(a, i0, j, k) && !in_sponge(a, i1, j, k);
}

// bulk_collide for the two cells of a thread at once (D3Q19, Smagorinsky or no SGS): the moments,
// the velocity and the recursive regularised collision run on packed FP32x2 lanes (lane v = cell
// v); the per-cell parts (relaxation rates, eddy viscosity square roots, sponge, field stores)
// run per lane.  act[v]: cell v is a bulk cell (the other lane's values are computed and dropped).
// plain (the same for the whole warp, see plain_pair): both cells active, uniform omega, no wall
// damping, no field stores and outside the sponge zones, so the per-lane part reduces to the
// relaxation rates;
// it computes the same numbers as the general path.
// Q = 27: the same with the D3Q27 moments and recursive regularised collision (collide_rr27p).
// The per-cell side data of a pair that bulk_collide2 reads (its relaxation rate where it differs
// from the uniform one, its wall distance where the damping needs it), loaded as soon as the flags
// are known so that the reads overlap the pulls instead of following the moments.
struct PairSide {
    float om[2];
    float sdf[2];
};
template <bool LES>
__device__ __forceinline__ PairSide pair_side(const StepArgs& a, const uint8_t (&fl)[2], const int (&ic)[2])
{
    PairSide p;
#pragma unroll
    for (int v = 0; v < 2; v++) {
        p.om[v] = (fl[v] & FL_OMEGA) ? __ldg(a.omega + ic[v]) : a.omega0;
        p.sdf[v] = (LES && (fl[v] & FL_SDF)) ? __ldg(a.sdf + ic[v]) : 0.f;
    }
    return p;
}

template <int S, bool LES, int Q = 19>
__device__ __forceinline__ void bulk_collide2(const StepArgs& a, F2 (&ft)[Q], const uint8_t (&fl)[2],
                                              const bool (&act)[2], const int (&ci)[2], const int (&cj)[2],
                                              const int (&ck)[2], const int (&ic)[2], bool plain = false,
                                              const PairSide* side = nullptr)
{
    constexpr int HS = Codec<S>::HS;
    Mom19T<F2> m;
    if constexpr (Q == 19) m = moments19<Codec<S>::DEV, HS>(ft);
    else m = moments27p<Codec<S>::DEV, HS>(ft);
    float irl[2], oml[2];
#pragma unroll
    for (int v = 0; v < 2; v++) {
        if (side) oml[v] = plain ? a.omega0 : side->om[v];
        else oml[v] = (!plain && (fl[v] & FL_OMEGA)) ? __ldg(a.omega + ic[v]) : a.omega0;
        irl[v] = 1.f / lane(m.rho, v);
    }
    const F2 ir = pk(irl[0], irl[1]);
    F2 irs;
    if constexpr (HS == 1) irs = ir;
    else irs = ir * (1.f / HS);
    const F2 hd = ir * (0.5f * a.dpdx);
    const F2 u = mad(m.j[0], irs, hd);  // updateRhoUVW (kernel.cl:3509-3523)
    const F2 v = m.j[1] * irs;
    const F2 w = m.j[2] * irs;
    float tsl[2] = {0.f, 0.f}, wel[2];
    F2 pp;
    if constexpr (LES) pp = smag_pp19<HS>(m, u, v, w);
    if (plain) {
        const float tau0 = 1.f / a.omega0;
#pragma unroll
        for (int c = 0; c < 2; c++) {
            if constexpr (LES) tsl[c] = smag_tau(lane(pp, c), lane(m.rho, c), a.omega0, a.les, a.cs);
            wel[c] = 1.f / (tau0 + tsl[c]);
        }
        if (a.err && !(lane0(m.rho) == lane0(m.rho) && lane1(m.rho) == lane1(m.rho))) atomicOr(a.err, 1);
    } else
#pragma unroll
    for (int c = 0; c < 2; c++) {
        const float rho = lane(m.rho, c);
        if constexpr (LES) {
            tsl[c] = smag_tau(lane(pp, c), rho, oml[c], a.les, a.cs);
            if (fl[c] & FL_SDF)
                tsl[c] = damping(a, tsl[c], side ? side->sdf[c] : __ldg(a.sdf + ic[c]), lane(u, c), lane(v, c),
                                 lane(w, c), oml[c]);
        }
        if (act[c]) {
            if (a.err && !(rho == rho)) atomicOr(a.err, 1);
            if (a.store_all || (fl[c] & FL_STORE) || in_box(a, ci[c], cj[c], ck[c])) {
                a.rho_n[ic[c]] = rho;
                a.u_n[ic[c]] = lane(u, c);
                a.v_n[ic[c]] = lane(v, c);
                a.w_n[ic[c]] = lane(w, c);
                a.tau_n[ic[c]] = tsl[c];
            }
        }
        const float tau = sponge_tau(a, 1.f / oml[c], tsl[c], ci[c], cj[c], ck[c]);
        wel[c] = 1.f / (tau + tsl[c]);
    }
    const F2 U[3] = {u - hd, v, w};
    if constexpr (Q == 19) collide_rr19m<HS>(ft, m, U, pk(wel[0], wel[1]), ir, a.omega_b, a.dpdx);
    else collide_rr27p<HS, !Codec<S>::DEV>(ft, m, U, pk(wel[0], wel[1]), ir, a.omega_b, a.dpdx);
}

// Two cells of one thread through bulk_collide2, then the stores of the active ones.
template <int S, bool LES, int XM = 0>
__device__ __forceinline__ void bulk_pair(const StepArgs& a, const uint8_t (&fl)[2], const bool (&act)[2],
                                          const int (&ci)[2], const int (&cj)[2], const int (&ck)[2],
                                          const int (&ic)[2], const int (&ip)[2], bool plain = false)
{
    using T = typename Codec<S>::T;
    F2 ft[19];
    if (row_crosses(a, cj[0], ck[0]) || row_crosses(a, cj[1], ck[1]) ||
        (XM != 0 && (xface_cell(a, ci[0]) || xface_cell(a, ci[1])))) {
        const BorderCell rb[2] = {XM ? border_cell(a, ci[0], cj[0], ck[0]) : row_border(a, cj[0], ck[0]),
                                  XM ? border_cell(a, ci[1], cj[1], ck[1]) : row_border(a, cj[1], ck[1])};
        const T* f = static_cast<const T*>(a.f_in);
#pragma unroll
        for (int q = 0; q < 19; q++) {
            const float x0 = act[0] ? Codec<S>::load_held(f + border_pull<19>(a, rb[0], q, ip[0])) : 0.f;
            const float x1 = act[1] ? Codec<S>::load_held(f + border_pull<19>(a, rb[1], q, ip[1])) : 0.f;
            ft[q] = pk(x0, x1);
        }
    } else {
#pragma unroll
        for (int q = 0; q < 19; q++) {
            const T* p = static_cast<const T*>(a.fin_s[q]);
            const float x0 = act[0] ? Codec<S>::load_held(p + ip[0]) : 0.f;
            const float x1 = act[1] ? Codec<S>::load_held(p + ip[1]) : 0.f;
            ft[q] = pk(x0, x1);
        }
    }
    bulk_collide2<S, LES>(a, ft, fl, act, ci, cj, ck, ic, plain);
#pragma unroll
    for (int q = 0; q < 19; q++) {
        T* p = static_cast<T*>(a.fout_q[q]);
        if (act[0]) Codec<S>::store_held(p + ip[0], lane0(ft[q]));
        if (act[1]) Codec<S>::store_held(p + ip[1], lane1(ft[q]));
    }
}

// two held values as one 32-bit word of 2-byte elements, x in the low half (each element
// rounded exactly as held_to rounds it)
__device__ __forceinline__ uint32_t held_pack(__half, float x, float y)
{
    const __half2 h = __floats2half2_rn(x, y);
    return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ uint32_t held_pack(__nv_bfloat16, float x, float y)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(x, y);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// a 32-bit word of two 2-byte elements as held values (low half in lane 0)
__device__ __forceinline__ F2 held_unpack(__half, uint32_t wd)
{
    __half2 h;
    memcpy(&h, &wd, 4);
    return pk(__low2float(h), __high2float(h));
}
__device__ __forceinline__ F2 held_unpack(__nv_bfloat16, uint32_t wd)
{
    __nv_bfloat162 h;
    memcpy(&h, &wd, 4);
    return pk(__low2float(h), __high2float(h));
}

// global accesses with an L2 cache policy (createpolicy): loads through the non-coherent path
__device__ __forceinline__ uint64_t l2_policy_evict_first()
{
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t l2_policy_evict_normal()
{
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint32_t ld_hint_b32(const void* p, uint64_t pol)
{
    uint32_t v;
    asm("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ uint16_t ld_hint_b16(const void* p, uint64_t pol)
{
    unsigned short v;
    asm("ld.global.nc.L2::cache_hint.b16 %0, [%1], %2;" : "=h"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ void st_hint_b32(void* p, uint32_t v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}
// a stored 2-byte element (its bits) as the held value
__device__ __forceinline__ float held_bits(__half, uint16_t b) { return __half2float(__ushort_as_half(b)); }
__device__ __forceinline__ float held_bits(__nv_bfloat16, uint16_t b) { return __bfloat162float(__ushort_as_bfloat16(b)); }

// XM 2: the ghost slots of an active bulk cell on the low (hi false) / high x face of a row crossing
// no y / z face, lane L of the pair ft, at padded index ip, after its collision, written by its own
// thread (the D3Q19 kernels; see xface_push_warp for what is written where).
template <int Q, int S, int L>
__device__ __forceinline__ void xface_push(const StepArgs& a, const F2 (&ft)[Q], bool hi, int ip)
{
    using T = typename Codec<S>::T;
    constexpr int A = 32 / (int)sizeof(T);
    const int code = hi ? (a.face_codes >> 3) & 7 : a.face_codes & 7;
    const bool sym = code == BC_SYM;
    const bool whole = !hi || a.nx % A == 0;
#pragma unroll
    for (int q = 1; q < Q; q++) {
        const int cx = lat_c(Q, q, 0), cy = lat_c(Q, q, 1), cz = lat_c(Q, q, 2);
        if (cx == 0 || (cx < 0) != hi) continue;
        const int r = lat_opp(Q, q), m = lat_find(Q, -cx, cy, cz);
        const F2 src = sym ? ft[m] : ft[r];
        const float v = L == 0 ? lane0(src) : lane1(src);
        T* p = static_cast<T*>(a.fout_q[q]) + (ip - (cx + cy * a.px + cz * a.pxy));
        if (whole) {
            uint32_t w32;
            if constexpr (sizeof(T) == 4) w32 = __float_as_uint(v);
            else w32 = held_pack(T{}, v, v);
            const uint4 quad = make_uint4(w32, w32, w32, w32);
            uint4* sec = reinterpret_cast<uint4*>(hi ? p : p - (A - 1));
            sec[0] = quad;
            sec[1] = quad;
        } else {
            Codec<S>::store_held(p, v);
        }
    }
}

// XM 2, a pair's x-face cells (xf: xface_bits, act: its active cells), by the lane's own thread
template <int Q, int S>
__device__ __forceinline__ void xface_push_lane(const StepArgs& a, const F2 (&ft)[Q], int xf, const bool (&act)[2],
                                                int ip0, int ip1)
{
    if ((xf & 1) && act[0]) xface_push<Q, S, 0>(a, ft, false, ip0);
    if ((xf & 2) && act[0]) xface_push<Q, S, 0>(a, ft, true, ip0);
    if ((xf & 4) && act[1]) xface_push<Q, S, 1>(a, ft, true, ip1);
}

// XM 2: the ghost slots of a warp's x-face cell, written by the warp's lanes together (every lane
// of the warp calls, with the same arguments).  The cell is on the low (HI false) / high x face of a
// row crossing no y / z face, cell `second` of lane src's pair ft, at padded index ip, after its
// collision.  For each direction q crossing its face inward (c_x > 0 on the low face, c_x < 0 on the
// high one; 5 for D3Q19, 9 for D3Q27) its next step pulls from the ghost position ip - c_q of plane
// q a value the face streaming takes from the cell itself: its new value of the missing direction
// (missing_dir with the face's code: the x mirror on a Symmetry face, else the opposite
// direction), stored as the row stores it.  The values reach the lanes by shuffles, lane 2 n + h
// writing half h of direction n's slot: the slot at x = -1, and at x = nx when the row fills whole
// 32-byte sectors, is alone in its sector, which is written whole (the value replicated) so that
// L2 need not merge a partial sector; otherwise lane 2 n writes the element.  The D3Q27 kernels
// write their 9 slots per face this way; the D3Q19 ones, whose 5 slots one thread writes in turn
// (xface_push), measured faster with the serial form (the cavity's FP16S step 0.264 against 0.269 ms;
// D3Q27 FP16S 0.390 against 0.403 ms the other way round).
template <int Q, int S, bool HI>
__device__ __forceinline__ void xface_push_warp(const StepArgs& a, const F2 (&ft)[Q], int src, bool second, int ip)
{
    using T = typename Codec<S>::T;
    constexpr int A = 32 / (int)sizeof(T);
    const int lane = threadIdx.x & 31, slot = lane >> 1, half = lane & 1;
    const int code = HI ? (a.face_codes >> 3) & 7 : a.face_codes & 7;
    const bool sym = code == BC_SYM;
    float mine = 0.f;
    T* p = nullptr;
    int n = 0;
#pragma unroll
    for (int q = 1; q < Q; q++) {
        const int cx = lat_c(Q, q, 0), cy = lat_c(Q, q, 1), cz = lat_c(Q, q, 2);
        if (cx == 0 || (cx < 0) != HI) continue;
        const int r = lat_opp(Q, q), m = lat_find(Q, -cx, cy, cz);
        const F2 s2 = sym ? ft[m] : ft[r];
        const float v = __shfl_sync(0xffffffffu, second ? lane1(s2) : lane0(s2), src);
        if (slot == n) {
            mine = v;
            p = static_cast<T*>(a.fout_q[q]) + (ip - (cx + cy * a.px + cz * a.pxy));
        }
        n++;
    }
    if (slot >= n) return;
    if (!HI || a.nx % A == 0) {
        uint32_t w32;
        if constexpr (sizeof(T) == 4) w32 = __float_as_uint(mine);
        else w32 = held_pack(T{}, mine, mine);
        uint4* sec = reinterpret_cast<uint4*>(HI ? p : p - (A - 1));
        sec[half] = make_uint4(w32, w32, w32, w32);
    } else if (half == 0) {
        Codec<S>::store_held(p, mine);
    }
}

// XM 2: the ghost slots of the x-face cells among a warp's pairs (xf: xface_bits of the lane's pair,
// act: its active cells), by every lane of the warp; the row's cells start at padded index prow
template <int Q, int S>
__device__ __forceinline__ void xface_push_pairs(const StepArgs& a, const F2 (&ft)[Q], int xf, const bool (&act)[2],
                                                 int prow)
{
    const unsigned lo = __ballot_sync(0xffffffffu, (xf & 1) && act[0]);
    const unsigned hi = __ballot_sync(0xffffffffu, ((xf & 2) && act[0]) || ((xf & 4) && act[1]));
    const unsigned hi2 = __ballot_sync(0xffffffffu, (xf & 4) && act[1]);
    if (lo) xface_push_warp<Q, S, false>(a, ft, __ffs(lo) - 1, false, prow);
    if (hi) xface_push_warp<Q, S, true>(a, ft, __ffs(hi) - 1, hi2 != 0, prow + a.nx - 1);
}

// the Q pulls of two adjacent cells at ip0 (even), read when any is set, with L2 policy pol; BORDER:
// the row crosses a y / z face (rb: its border, border pulls; both cells share its mapping, so the
// pulls with c_x = 0 stay one aligned 32-bit word)
// BORDER 1: the pair's row crosses a y / z face and neither cell is a bulk cell on an x face: both take
// the row's border rb[0].  BORDER 2: rb[0] the row's border, by which the c_x = 0 pulls of every cell
// of the row go (one word for the pair), rb[1 + v] the border of cell v, by which its other pulls go.
// XF: a cell of the pair is on an x face of a row crossing no other face (xf bit 0: cell 0 on the
// low face, bit 1: cell 0 on the high face, bit 2: cell 1 on the high face).
template <int S, bool HINT, int Q = 19, int BORDER = 0, bool XF = false>
__device__ __forceinline__ void pair_adj_load(const StepArgs& a, int ip0, bool any, [[maybe_unused]] uint64_t pol,
                                              F2 (&ft)[Q], [[maybe_unused]] const BorderCell* rb = nullptr,
                                              [[maybe_unused]] int xf = 0)
{
    using T = typename Codec<S>::T;
    static_assert(sizeof(T) == 2, "2-byte storage");
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const T* p;
        if constexpr (BORDER != 0) p = static_cast<const T*>(a.f_in) + border_pull<Q>(a, rb[0], q, ip0);
        else p = static_cast<const T*>(a.fin_s[q]) + ip0;
        if (lat_c(Q, q, 0) == 0) {
            uint32_t wd = 0u;
            if constexpr (HINT) wd = any ? ld_hint_b32(p, pol) : 0u;
            else wd = any ? __ldg(reinterpret_cast<const unsigned int*>(p)) : 0u;
            ft[q] = held_unpack(T{}, wd);
        } else {
            const T* p1 = p + 1;
            if constexpr (BORDER == 2) {
                p = static_cast<const T*>(a.f_in) + border_pull<Q>(a, rb[1], q, ip0);
                p1 = static_cast<const T*>(a.f_in) + border_pull<Q>(a, rb[2], q, ip0 + 1);
            }
            if constexpr (XF) {
                p = static_cast<const T*>(xface_base<Q>(a, q, xf & 1, xf & 2)) + ip0;
                p1 = static_cast<const T*>(xface_base<Q>(a, q, false, xf & 4)) + ip0 + 1;
            }
            float x0, x1;
            if constexpr (HINT) {
                x0 = any ? held_bits(T{}, ld_hint_b16(p, pol)) : 0.f;
                x1 = any ? held_bits(T{}, ld_hint_b16(p1, pol)) : 0.f;
            } else {
                x0 = any ? Codec<S>::load_held(p) : 0.f;
                x1 = any ? Codec<S>::load_held(p1) : 0.f;
            }
            ft[q] = pk(x0, x1);
        }
    }
}

// the results of two adjacent cells at ip0: one packed 32-bit store per direction when both are
// active, else each active cell's own element
template <int S, bool HINT, int Q = 19>
__device__ __forceinline__ void pair_adj_store(const StepArgs& a, const F2 (&ft)[Q], const bool (&act)[2], int ip0,
                                               [[maybe_unused]] uint64_t pol)
{
    using T = typename Codec<S>::T;
    if (act[0] && act[1]) {
#pragma unroll
        for (int q = 0; q < Q; q++) {
            T* p = static_cast<T*>(a.fout_q[q]) + ip0;
            const uint32_t wd = held_pack(T{}, lane0(ft[q]), lane1(ft[q]));
            if constexpr (HINT) st_hint_b32(p, wd, pol);
            else *reinterpret_cast<uint32_t*>(p) = wd;
        }
    } else {
#pragma unroll
        for (int q = 0; q < Q; q++) {
            T* p = static_cast<T*>(a.fout_q[q]) + ip0;
            if (act[0]) Codec<S>::store_held(p, lane0(ft[q]));
            if (act[1]) Codec<S>::store_held(p + 1, lane1(ft[q]));
        }
    }
}

// bulk_pair for two adjacent cells of 2-byte storage (ip0 even, cell ip0 + 1 the second): the
// pulls with c_x = 0 of both cells are one aligned 32-bit word (the pull offset c_y px + c_z pxy is
// even), and when both cells are active their results leave as one packed 32-bit store.  Both
// cells' pulls are read when either is active (the row is padded by a ghost cell on each side).
template <int S, bool LES, int XM = 0>
__device__ __forceinline__ void bulk_pair_adj(const StepArgs& a, const uint8_t (&fl)[2], const bool (&act)[2],
                                              const int (&ci)[2], const int (&cj)[2], const int (&ck)[2],
                                              const int (&ic)[2], int ip0, bool plain = false)
{
    F2 ft[19];
    const bool xcell = XM != 0 && (xface_cell(a, ci[0]) || xface_cell(a, ci[1]));
    if (row_crosses(a, cj[0], ck[0]) || xcell) {
        if constexpr (XM != 0) {
            const BorderCell rb[3] = {row_border(a, cj[0], ck[0]), border_cell(a, ci[0], cj[0], ck[0]),
                                      border_cell(a, ci[1], cj[1], ck[1])};
            pair_adj_load<S, false, 19, 2>(a, ip0, act[0] || act[1], 0, ft, rb);
        } else {
            const BorderCell rb = row_border(a, cj[0], ck[0]);
            pair_adj_load<S, false, 19, 1>(a, ip0, act[0] || act[1], 0, ft, &rb);
        }
        bulk_collide2<S, LES>(a, ft, fl, act, ci, cj, ck, ic, plain);
        pair_adj_store<S, false>(a, ft, act, ip0, 0);
    } else if (LBFFS_BULK_EVICT && a.l2_policy != 0) {
        const uint64_t pol = a.l2_policy == 1 ? l2_policy_evict_first() : l2_policy_evict_normal();
        pair_adj_load<S, true>(a, ip0, act[0] || act[1], pol, ft);
        bulk_collide2<S, LES>(a, ft, fl, act, ci, cj, ck, ic, plain);
        pair_adj_store<S, true>(a, ft, act, ip0, pol);
    } else {
        pair_adj_load<S, false>(a, ip0, act[0] || act[1], 0, ft);
        bulk_collide2<S, LES>(a, ft, fl, act, ci, cj, ck, ic, plain);
        pair_adj_store<S, false>(a, ft, act, ip0, 0);
    }
}

// 2-byte D3Q19 storage: L2 prefetch of the rows the CTA LBFFS_BULK_PREFETCH launches ahead will
// pull (one bulk prefetch per direction, issued by the first Q threads; the range is shrunk to
// whole 16-byte units inside the pulled elements, so it never leaves the population planes).  The
// 2-byte kernel is latency-bound with half the bytes in flight of FP32; for the bandwidth-bound
// FP32 and D3Q27 kernels the extra requests measured slower.
template <int Q, int S, int V>
__device__ __forceinline__ void bulk_prefetch(const StepArgs& a)
{
#if LBFFS_BULK_PREFETCH > 0
    using T = typename Codec<S>::T;
    if (Q == 19 && S != ST_FP32 && threadIdx.x < Q) {
        const long long nb = (long long)gridDim.x * gridDim.y * gridDim.z;
        const long long fb = (long long)blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z) +
                             LBFFS_BULK_PREFETCH;
        if (fb < nb) {
            const int fx = (int)(fb % gridDim.x), fr = (int)(fb / gridDim.x);
            const int fj = fr % a.ny, fk = fr / a.ny;
            const int x0 = fx * BULK_BX * V, n = min(BULK_BX * V, a.nx - x0);
            const uintptr_t base = reinterpret_cast<uintptr_t>(a.fin_s[threadIdx.x]);
            const uintptr_t lo = base + (uintptr_t)pidx(a, x0, fj, fk) * sizeof(T);
            const uintptr_t b0 = (lo + 15) & ~(uintptr_t)15, b1 = (lo + (uintptr_t)n * sizeof(T)) & ~(uintptr_t)15;
            if (b1 > b0)
                asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(b0), "r"((unsigned)(b1 - b0)) : "memory");
        }
    }
#endif
}

// The adjacent pair of a bulk_block lane with its pulls issued together with its flag loads
// (one memory round trip before the collision instead of two): the pair's pulls are read whenever
// its first cell is in the row, active or not (a solid cell's values are read and dropped).
template <int S, bool LES, int Q = 19, int XM = 0>
__device__ __forceinline__ void bulk_pair_adj_eager(const StepArgs& a, int i0, int j, int k, int row, int prow,
                                                    bool inrange = true)
{
    const bool valid = inrange && i0 < a.nx;
    uint8_t fl[2];
    fl[0] = valid ? __ldg(a.flags + row + i0) : FL_SOLID;
    fl[1] = valid && i0 + 1 < a.nx ? __ldg(a.flags + row + i0 + 1) : FL_SOLID;
    const bool hint = LBFFS_BULK_EVICT && a.l2_policy != 0;
    [[maybe_unused]] uint64_t pol = 0;
    F2 ft[Q];
    const bool cross = row_crosses(a, j, k);
    // the pair's x-face cells in a row crossing no y / z face
    const int xf = XM != 0 && valid && !cross ? xface_bits(a, i0, i0 + 1) : 0;
    bool xany = false;
    if constexpr (XM == 1) xany = __any_sync(0xffffffffu, xf != 0);
    if (cross) {
        if constexpr (XM != 0) {
            const BorderCell rb[3] = {row_border(a, j, k), border_cell(a, i0, j, k), border_cell(a, i0 + 1, j, k)};
            pair_adj_load<S, false, Q, 2>(a, prow + i0, valid, 0, ft, rb);
        } else {
            const BorderCell rb = row_border(a, j, k);
            pair_adj_load<S, false, Q, 1>(a, prow + i0, valid, 0, ft, &rb);
        }
    } else if (xany) {
        if constexpr (XM == 1) pair_adj_load<S, false, Q, 0, true>(a, prow + i0, valid, 0, ft, nullptr, xf);
    } else if (hint) {
        pol = a.l2_policy == 1 ? l2_policy_evict_first() : l2_policy_evict_normal();
        pair_adj_load<S, true, Q>(a, prow + i0, valid, pol, ft);
    } else {
        pair_adj_load<S, false, Q>(a, prow + i0, valid, 0, ft);
    }
    const int ic[2] = {row + i0, row + i0 + 1};
    const PairSide side = pair_side<LES>(a, fl, ic);
    const bool act[2] = {!(fl[0] & (FL_SOLID | FL_SPECIAL)), !(fl[1] & (FL_SOLID | FL_SPECIAL))};
    const bool plain = __all_sync(0xffffffffu, plain_pair(a, fl, act, i0, i0 + 1, j, k));
    // XM 2 D3Q27 writes the ghost slots with the whole warp: every lane stays
    constexpr bool WARP_PUSH = XM == 2 && Q == 27;
    if constexpr (!WARP_PUSH) {
        if (!(act[0] || act[1])) return;
    }
    const int ci[2] = {i0, i0 + 1}, cj[2] = {j, j}, ck[2] = {k, k};
    const bool any = WARP_PUSH ? (act[0] || act[1]) : true;
    if (any) bulk_collide2<S, LES, Q>(a, ft, fl, act, ci, cj, ck, ic, plain, &side);
    // the ghost slots of the x-face cells of the row's first and last warp, before the row stores (the
    // populations are live until then anyway)
    if constexpr (WARP_PUSH) {
        if (__any_sync(0xffffffffu, xf != 0)) xface_push_pairs<Q, S>(a, ft, xf, act, prow);
    } else if constexpr (XM == 2) {
        if (xf != 0) xface_push_lane<Q, S>(a, ft, xf, act, prow + i0, prow + i0 + 1);
    }
    if (any) {
        if (hint) pair_adj_store<S, true, Q>(a, ft, act, prow + i0, pol);
        else pair_adj_store<S, false, Q>(a, ft, act, prow + i0, 0);
    }
}

// bulk_pair (cells i0 and i0 + 32) with the pulls issued together with the flag loads; a cell's
// pulls are read whenever it is in the row, active or not
template <int S, bool LES, int Q = 19, int XM = 0>
__device__ __forceinline__ void bulk_pair_eager(const StepArgs& a, int i0, int j, int k, int row, int prow)
{
    using T = typename Codec<S>::T;
    const bool valid[2] = {i0 < a.nx, i0 + 32 < a.nx};
    uint8_t fl[2];
    F2 ft[Q];
#pragma unroll
    for (int v = 0; v < 2; v++) fl[v] = valid[v] ? __ldg(a.flags + row + i0 + 32 * v) : FL_SOLID;
    const bool cross = row_crosses(a, j, k);
    // the pair's x-face cells in a row crossing no y / z face
    const int xf = XM != 0 && !cross ? xface_bits(a, valid[0] ? i0 : -1, valid[1] ? i0 + 32 : -1) : 0;
    bool xany = false;
    if constexpr (XM == 1) xany = __any_sync(0xffffffffu, xf != 0);
    if (cross) {
        // the c_x = 0 pulls by the row's border (one mapping for the row), the others by the cell's own
        // (x-face kernels) or the row's
        const BorderCell rb[3] = {row_border(a, j, k), XM ? border_cell(a, i0, j, k) : row_border(a, j, k),
                                  XM ? border_cell(a, i0 + 32, j, k) : row_border(a, j, k)};
        const T* f = static_cast<const T*>(a.f_in);
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const bool cx0 = XM == 0 || lat_c(Q, q, 0) == 0;
            const T* p = f + border_pull<Q>(a, cx0 ? rb[0] : rb[1], q, prow + i0);
            const T* p1 = cx0 ? p + 32 : f + border_pull<Q>(a, rb[2], q, prow + i0 + 32);
            const float x0 = valid[0] ? Codec<S>::load_held(p) : 0.f;
            const float x1 = valid[1] ? Codec<S>::load_held(p1) : 0.f;
            ft[q] = pk(x0, x1);
        }
    } else if (XM == 1 && xany) {
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const T* p = static_cast<const T*>(xface_base<Q>(a, q, xf & 1, xf & 2)) + prow + i0;
            const T* p1 = static_cast<const T*>(xface_base<Q>(a, q, false, xf & 4)) + prow + i0 + 32;
            const float x0 = valid[0] ? Codec<S>::load_held(p) : 0.f;
            const float x1 = valid[1] ? Codec<S>::load_held(p1) : 0.f;
            ft[q] = pk(x0, x1);
        }
    } else {
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const T* p = static_cast<const T*>(a.fin_s[q]) + prow + i0;
            const float x0 = valid[0] ? Codec<S>::load_held(p) : 0.f;
            const float x1 = valid[1] ? Codec<S>::load_held(p + 32) : 0.f;
            ft[q] = pk(x0, x1);
        }
    }
    const int ic[2] = {row + i0, row + i0 + 32};
    const PairSide side = pair_side<LES>(a, fl, ic);
    const bool act[2] = {!(fl[0] & (FL_SOLID | FL_SPECIAL)), !(fl[1] & (FL_SOLID | FL_SPECIAL))};
    const bool plain = __all_sync(0xffffffffu, plain_pair(a, fl, act, i0, i0 + 32, j, k));
    constexpr bool WARP_PUSH = XM == 2 && Q == 27;  // as in bulk_pair_adj_eager
    if constexpr (!WARP_PUSH) {
        if (!(act[0] || act[1])) return;
    }
    const int ci[2] = {i0, i0 + 32}, cj[2] = {j, j}, ck[2] = {k, k};
    const bool any = WARP_PUSH ? (act[0] || act[1]) : true;
    if (any) bulk_collide2<S, LES, Q>(a, ft, fl, act, ci, cj, ck, ic, plain, &side);
    // the ghost slots of the x-face cells of the row's first and last warp, as in bulk_pair_adj_eager
    if constexpr (WARP_PUSH) {
        if (__any_sync(0xffffffffu, xf != 0)) xface_push_pairs<Q, S>(a, ft, xf, act, prow);
    } else if constexpr (XM == 2) {
        if (xf != 0) xface_push_lane<Q, S>(a, ft, xf, act, prow + i0, prow + i0 + 32);
    }
    if (any) {
#pragma unroll
        for (int q = 0; q < Q; q++) {
            T* p = static_cast<T*>(a.fout_q[q]) + prow + i0;
            if (act[0]) Codec<S>::store_held(p, lane0(ft[q]));
            if (act[1]) Codec<S>::store_held(p + 32, lane1(ft[q]));
        }
    }
}

// One thread per BULK_V cells of a row, 32 apart (lane, lane + 32, ...), so each load and store
// instruction of a warp covers 32 consecutive cells.  Every population is pulled from the same
// offset for every cell: cells on the domain border read the ghost layer (filled by k_halo with the
// reference's face streaming before the step, or, for the x-face slots of XM 2, by the x-face cells
// in the previous step), except where border pulls read across the border directly (rows on a y / z
// face, and the x-face cells of XM 1).
// One CTA tile: BULK_BX * bulk_v<Q>() cells of row (j, k) starting at x-block xb.  PF: the tile is
// CTA (xb, j, k) of a k_bulk grid, so the L2 prefetch of the tiles launched later may run.  XM: the
// kernel's x-face handling (k_bulk).
template <int Q, int S, int COLL, int SGS, bool LES, bool PF = true, int XM = 0>
__device__ __forceinline__ void bulk_block(const StepArgs& a, int xb, int j, int k)
{
    using T = typename Codec<S>::T;
    constexpr bool HELD = (Q == 19);
    constexpr int V = bulk_v<Q, COLL, SGS>();
    // 2-byte D3Q19 pair path: a lane owns two adjacent cells (bulk_pair_adj); otherwise cells
    // lane + 32 v
    constexpr bool ADJ = Q == 19 && SGS != SGS_WALE && V == 2 && S != ST_FP32 && LBFFS_BULK_ADJ;
    // D3Q27 recursive regularised collision on cell pairs (packed FP32x2): adjacent cells for 2-byte
    // storage, cells 32 apart for FP32
    constexpr bool PAIR27 = Q == 27 && V == 2;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int base = (xb * (BULK_BX / 32) + warp) * (32 * V);
    const int i0 = ADJ ? base + 2 * lane : base + lane;
    constexpr int DV = ADJ ? 1 : 32;  // x distance of a lane's consecutive cells
    const int row = (k * a.ny + j) * a.nx;
    const int prow = pidx(a, 0, j, k);
    if constexpr (PF) bulk_prefetch<Q, S, V>(a);
    if constexpr (PAIR27) {
        if constexpr (S != ST_FP32) bulk_pair_adj_eager<S, LES, 27, XM>(a, base + 2 * lane, j, k, row, prow);
        else bulk_pair_eager<S, LES, 27, XM>(a, base + lane, j, k, row, prow);
        return;
    }
    if constexpr (ADJ && LBFFS_BULK_EAGER) {
        bulk_pair_adj_eager<S, LES, 19, XM>(a, i0, j, k, row, prow);
        return;
    } else if constexpr (Q == 19 && SGS != SGS_WALE && V == 2 && !ADJ && LBFFS_BULK_EAGER32) {
        bulk_pair_eager<S, LES, 19, XM>(a, i0, j, k, row, prow);
        return;
    }
    uint8_t fl[V];
    bool act[V];
    bool any = false;
#pragma unroll
    for (int v = 0; v < V; v++) {
        const int i = i0 + DV * v;
        fl[v] = (i < a.nx) ? __ldg(a.flags + row + i) : FL_SOLID;
        act[v] = !(fl[v] & (FL_SOLID | FL_SPECIAL));
        any |= act[v];
    }
    bool plain = false;
    if constexpr (Q == 19 && SGS != SGS_WALE && V == 2) plain = __all_sync(0xffffffffu, plain_pair(a, fl, act));
    if (!any) return;
    if constexpr (ADJ) {
        const int ci[2] = {i0, i0 + 1}, cj[2] = {j, j}, ck[2] = {k, k};
        const int ic[2] = {row + i0, row + i0 + 1};
        bulk_pair_adj<S, LES, XM>(a, fl, act, ci, cj, ck, ic, prow + i0, plain);
    } else if constexpr (Q == 19 && SGS != SGS_WALE && V == 2) {
        const int ci[2] = {i0, i0 + 32}, cj[2] = {j, j}, ck[2] = {k, k};
        const int ic[2] = {row + i0, row + i0 + 32}, ip[2] = {prow + i0, prow + i0 + 32};
        bulk_pair<S, LES, XM>(a, fl, act, ci, cj, ck, ic, ip, plain);
    } else {
        float ft[V][Q];
        const bool cross = row_crosses(a, j, k);
#pragma unroll
        for (int v = 0; v < V; v++) {
            if (!act[v]) continue;
            const int ip = prow + i0 + DV * v;
            if (cross || (XM != 0 && xface_cell(a, i0 + DV * v))) {
                const BorderCell rb = XM ? border_cell(a, i0 + DV * v, j, k) : row_border(a, j, k);
#pragma unroll
                for (int q = 0; q < Q; q++) {
                    const T* p = static_cast<const T*>(a.f_in) + border_pull<Q>(a, rb, q, ip);
                    ft[v][q] = HELD ? Codec<S>::load_held(p) : Codec<S>::load(p, lat_w(Q, q));
                }
            } else {
#pragma unroll
                for (int q = 0; q < Q; q++) {
                    const T* p = static_cast<const T*>(a.fin_s[q]) + ip;
                    ft[v][q] = HELD ? Codec<S>::load_held(p) : Codec<S>::load(p, lat_w(Q, q));
                }
            }
        }
#pragma unroll
        for (int v = 0; v < V; v++) {
            if (!act[v]) continue;
            const int i = i0 + DV * v;
            bulk_cell<Q, S, COLL, SGS, LES>(a, ft[v], fl[v], i, j, k, row + i, prow + i);
        }
    }
}

// Segment mapping of the same per-cell work, for lattices with narrow rows: a row is cut into
// ceil(nx / 32) segments of 32 cells, segments are numbered row after row ((j, k) order), and warp
// w of the CTA takes segments g0 + BULK_V * w + v.  A 24-cell row then keeps 24 of 32 lanes busy
// where a BULK_BX * BULK_V-cell row tile keeps 24 of 256.  spr = segments per row, nseg = all;
// dspr / dny divide by spr and ny.
template <int Q, int S, int COLL, int SGS, bool LES>
__device__ __forceinline__ void bulk_segments(const StepArgs& a, int g0, int spr, int nseg, FastDiv dspr, FastDiv dny)
{
    using T = typename Codec<S>::T;
    constexpr bool HELD = (Q == 19);
    // 2-byte D3Q19 pair path: lanes 0-15 own adjacent cell pairs of the warp's first segment,
    // lanes 16-31 of its second (bulk_pair_adj); otherwise lane l takes cell l of both segments
    constexpr bool ADJ = Q == 19 && SGS != SGS_WALE && BULK_V == 2 && S != ST_FP32 && LBFFS_BULK_ADJ;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if constexpr (ADJ && LBFFS_BULK_EAGER) {
        const int g = g0 + warp * BULK_V + (lane >> 4);
        const bool inrange = g < nseg;
        const int row = inrange ? fdiv(g, dspr) : 0;
        const int i0 = (g - row * spr) * 32 + 2 * (lane & 15);
        const int k = fdiv(row, dny), j = row - k * a.ny;
        bulk_pair_adj_eager<S, LES>(a, inrange ? i0 : a.nx, j, k, row * a.nx, pidx(a, 0, j, k), inrange);
        return;
    } else if constexpr (Q == 19 && SGS != SGS_WALE && BULK_V == 2 && LBFFS_BULK_EAGER32) {
        // FP32: lane l takes cell l of both segments, its pulls issued together with the flag loads
        // (as bulk_pair_eager does for a row tile)
        int ci[2], cj[2], ck[2], ic[2], ip[2];
        bool valid[2];
        uint8_t fl[2];
#pragma unroll
        for (int v = 0; v < 2; v++) {
            const int g = g0 + warp * 2 + v;
            const int row = g < nseg ? fdiv(g, dspr) : 0;
            ci[v] = (g - row * spr) * 32 + lane;
            valid[v] = g < nseg && ci[v] < a.nx;
            ck[v] = fdiv(row, dny);
            cj[v] = row - ck[v] * a.ny;
            ic[v] = row * a.nx + ci[v];
            ip[v] = pidx(a, ci[v], cj[v], ck[v]);
            fl[v] = valid[v] ? __ldg(a.flags + ic[v]) : FL_SOLID;
        }
        F2 ft[19];
        if (row_crosses(a, cj[0], ck[0]) || row_crosses(a, cj[1], ck[1])) {
            const BorderCell rb[2] = {row_border(a, cj[0], ck[0]), row_border(a, cj[1], ck[1])};
            const T* f = static_cast<const T*>(a.f_in);
#pragma unroll
            for (int q = 0; q < 19; q++) {
                const float x0 = valid[0] ? Codec<S>::load_held(f + border_pull<19>(a, rb[0], q, ip[0])) : 0.f;
                const float x1 = valid[1] ? Codec<S>::load_held(f + border_pull<19>(a, rb[1], q, ip[1])) : 0.f;
                ft[q] = pk(x0, x1);
            }
        } else {
#pragma unroll
            for (int q = 0; q < 19; q++) {
                const T* p = static_cast<const T*>(a.fin_s[q]);
                const float x0 = valid[0] ? Codec<S>::load_held(p + ip[0]) : 0.f;
                const float x1 = valid[1] ? Codec<S>::load_held(p + ip[1]) : 0.f;
                ft[q] = pk(x0, x1);
            }
        }
        const PairSide side = pair_side<LES>(a, fl, ic);
        const bool act[2] = {!(fl[0] & (FL_SOLID | FL_SPECIAL)), !(fl[1] & (FL_SOLID | FL_SPECIAL))};
        const bool plain = __all_sync(0xffffffffu, plain_pair(a, fl, act));
        if (!(act[0] || act[1])) return;
        bulk_collide2<S, LES>(a, ft, fl, act, ci, cj, ck, ic, plain, &side);
#pragma unroll
        for (int q = 0; q < 19; q++) {
            T* p = static_cast<T*>(a.fout_q[q]);
            if (act[0]) Codec<S>::store_held(p + ip[0], lane0(ft[q]));
            if (act[1]) Codec<S>::store_held(p + ip[1], lane1(ft[q]));
        }
        return;
    }
    int ci[BULK_V], cj[BULK_V], ck[BULK_V];
    uint8_t fl[BULK_V];
    bool act[BULK_V];
    bool any = false;
#pragma unroll
    for (int v = 0; v < BULK_V; v++) {
        const int g = ADJ ? g0 + warp * BULK_V + (lane >> 4) : g0 + warp * BULK_V + v;
        const int row = fdiv(g, dspr);
        ci[v] = ADJ ? (g - row * spr) * 32 + 2 * (lane & 15) + v : (g - row * spr) * 32 + lane;
        ck[v] = fdiv(row, dny);
        cj[v] = row - ck[v] * a.ny;
        fl[v] = (g < nseg && ci[v] < a.nx) ? __ldg(a.flags + (long long)row * a.nx + ci[v]) : FL_SOLID;
        act[v] = !(fl[v] & (FL_SOLID | FL_SPECIAL));
        any |= act[v];
    }
    bool plain = false;
    if constexpr (Q == 19 && SGS != SGS_WALE && BULK_V == 2) plain = __all_sync(0xffffffffu, plain_pair(a, fl, act));
    if (!any) return;
    if constexpr (ADJ) {
        const int ic[2] = {(ck[0] * a.ny + cj[0]) * a.nx + ci[0], (ck[0] * a.ny + cj[0]) * a.nx + ci[0] + 1};
        bulk_pair_adj<S, LES>(a, fl, act, ci, cj, ck, ic, pidx(a, ci[0], cj[0], ck[0]), plain);
    } else if constexpr (Q == 19 && SGS != SGS_WALE && BULK_V == 2) {
        const int ic[2] = {(ck[0] * a.ny + cj[0]) * a.nx + ci[0], (ck[1] * a.ny + cj[1]) * a.nx + ci[1]};
        const int ip[2] = {pidx(a, ci[0], cj[0], ck[0]), pidx(a, ci[1], cj[1], ck[1])};
        bulk_pair<S, LES>(a, fl, act, ci, cj, ck, ic, ip, plain);
    } else {
        float ft[BULK_V][Q];
#pragma unroll
        for (int v = 0; v < BULK_V; v++) {
            if (!act[v]) continue;
            const int ip = pidx(a, ci[v], cj[v], ck[v]);
            if (row_crosses(a, cj[v], ck[v])) {
                const BorderCell rb = row_border(a, cj[v], ck[v]);
#pragma unroll
                for (int q = 0; q < Q; q++) {
                    const T* p = static_cast<const T*>(a.f_in) + border_pull<Q>(a, rb, q, ip);
                    ft[v][q] = HELD ? Codec<S>::load_held(p) : Codec<S>::load(p, lat_w(Q, q));
                }
            } else {
#pragma unroll
                for (int q = 0; q < Q; q++) {
                    const T* p = static_cast<const T*>(a.fin_s[q]) + ip;
                    ft[v][q] = HELD ? Codec<S>::load_held(p) : Codec<S>::load(p, lat_w(Q, q));
                }
            }
        }
#pragma unroll
        for (int v = 0; v < BULK_V; v++) {
            if (!act[v]) continue;
            const int ic = (ck[v] * a.ny + cj[v]) * a.nx + ci[v];
            bulk_cell<Q, S, COLL, SGS, LES>(a, ft[v], fl[v], ci[v], cj[v], ck[v], ic, pidx(a, ci[v], cj[v], ck[v]));
        }
    }
}

// Resident CTAs per SM the D3Q19 / D3Q27 bulk kernels may be compiled for (register budget 65536 /
// (128 x this)); build-time tuning values.  1 leaves the register count to the compiler.
#ifndef LBFFS_BULK_MINB19
#define LBFFS_BULK_MINB19 8
#endif
#ifndef LBFFS_BULK_MINB27
#define LBFFS_BULK_MINB27 6
#endif
// D3Q27 with the eddy viscosity on (the LES step, C3): 7 measured 7.7 % faster than 6 on the
// 768x192x192 step (FP16S), where 6 is 0.8 % faster on the plain cavity
#ifndef LBFFS_BULK_MINB27_LES
#define LBFFS_BULK_MINB27_LES 7
#endif
#define LBFFS_BULK_BOUNDS(Q, LES) \
    __launch_bounds__(BULK_BX, (Q) == 19 ? LBFFS_BULK_MINB19 : (LES) ? LBFFS_BULK_MINB27_LES : LBFFS_BULK_MINB27)

// XM: bulk cells on the x faces pull across them from per-context plane bases (1, border_pulls 2)
// or through ghost slots they write themselves (2, border_pulls 3); 0: no bulk cell on an x face
// pulls across it from where it lies (border_pulls 0 and 1)
template <int Q, int S, int COLL, int SGS, bool LES, int XM>
__global__ void LBFFS_BULK_BOUNDS(Q, LES) k_bulk(const StepArgs a)
{
    bulk_block<Q, S, COLL, SGS, LES, true, XM>(a, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ---- a lane group per boundary cell (special_cell with G lanes) ----
// Lane q < Q of the warp does the per-direction memory work of direction q: its pull, its own
// previous value, the outlet's inner value and the STL link's reads, all issued in one round trip
// after the cell index; the values are exchanged by shuffles and the operators run on the full
// population set in every lane, so the cell's arithmetic is the thread version's.

// velocity, opposite direction and weight of direction q (q at run time)
template <int Q>
struct LaneDir {
    int c[3];
    int opp;
    float w;
};
template <int Q>
__device__ __forceinline__ LaneDir<Q> lane_dir(int q)
{
    LaneDir<Q> r{{0, 0, 0}, 0, 0.f};
#pragma unroll
    for (int p = 0; p < Q; p++)
        if (q == p) {
            r.c[0] = lat_c(Q, p, 0);
            r.c[1] = lat_c(Q, p, 1);
            r.c[2] = lat_c(Q, p, 2);
            r.opp = lat_opp(Q, p);
            r.w = lat_w(Q, p);
        }
    return r;
}

// upwind<Q> for a direction given by its velocity c (run time)
__device__ __forceinline__ long long upwind_c(const int (&c)[3], const int (&x)[3], const int (&N)[3], const int (&b)[3],
                                              bool face)
{
    int n[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        n[d] = x[d] - c[d];
        if (n[d] < 0) {
            if (face && is_wall_code(b[d])) return -1;
            n[d] += N[d];
        } else if (n[d] >= N[d]) {
            if (face && is_wall_code(b[d])) return -1;
            n[d] -= N[d];
        }
    }
    return ((long long)n[2] * N[1] + n[1]) * N[0] + n[0];
}

// border_pull<Q> for direction q with velocity c and missing direction m given at run time
__device__ __forceinline__ long long border_pull_c(const StepArgs& a, const BorderCell& g, const int (&c)[3], int q,
                                                   int m, int ip)
{
    int shift = 0;
    bool out = false, wall = false;
#pragma unroll
    for (int e = 0; e < 3; e++) {
        if (c[e] > 0 && g.lo[e]) {
            out = true;
            shift += g.wrap[e];
            wall |= is_wall_code(g.b[e]);
        } else if (c[e] < 0 && g.hi[e]) {
            out = true;
            shift -= g.wrap[e];
            wall |= is_wall_code(g.b[e]);
        }
    }
    const long long pull = (long long)q * a.pE + (ip - (c[0] + c[1] * a.px + c[2] * a.pxy));
    if (!out) return pull;
    if (!(g.face && wall)) return pull + shift;
    return (long long)m * a.pE + ip;
}

// The general boundary path of entry t of the special list: one thread per cell (G = 1), or a group
// of G lanes per cell (G = 8, 16 or 32, aligned within the warp), every lane of the group calling
// with the same t; lane g of the group does the reads of directions g, g + G, ...
template <int Q, int S, int COLL, int G = 1>
__device__ __forceinline__ void special_cell(const StepArgs& a, long long t)
{
    using T = typename Codec<S>::T;
    constexpr bool GRP = G > 1;
    constexpr int K = GRP ? (Q + G - 1) / G : 1;  // directions per lane
    static_assert(G == 1 || G == 8 || G == 16 || G == 32, "lanes per cell");
    const long long ic = a.special[t];
    const int N[3] = {a.nx, a.ny, a.nz};
    const long long nxny = (long long)a.nx * a.ny;
    const int x[3] = {(int)(ic % a.nx), (int)((ic / a.nx) % a.ny), (int)(ic / nxny)};
    auto id = [&](int ii, int jj, int kk) { return ((long long)kk * a.ny + jj) * a.nx + ii; };
    // the cell one step inside the face along axis d (clamped into the grid for axes of 1-2 cells)
    auto inner = [&](int d, int side) {
        int y[3] = {x[0], x[1], x[2]};
        y[d] = side < 0 ? min(1, N[d] - 1) : max(N[d] - 2, 0);
        return id(y[0], y[1], y[2]);
    };
    auto inner_p = [&](int d, int side) {
        int y[3] = {x[0], x[1], x[2]};
        y[d] = side < 0 ? min(1, N[d] - 1) : max(N[d] - 2, 0);
        return pidx(a, y[0], y[1], y[2]);
    };
    const int ip = pidx(a, x[0], x[1], x[2]);
    const uint16_t bw = a.bc[ic];
    const int b[3] = {bw & 7, (bw >> 3) & 7, (bw >> 6) & 7};
    const bool face = (bw >> 9) & 1;
    // population q of the padded cell pcell (previous step)
    auto F = [&](int q, int pcell) {
        return Codec<S>::load(static_cast<const T*>(a.fin_q[q]) + pcell, lat_w(Q, q));
    };

    // streaming: upwind value, or the face rule's value (upwindID_B + reflectOrMirrorQ): from the
    // ghost that holds it (filled by k_halo), or, with border pulls, read where the rule takes it
    float ft[Q];
    [[maybe_unused]] const int lane = GRP ? (int)(threadIdx.x & (G - 1)) : 0;
    [[maybe_unused]] const unsigned gmask =
        G == 32 ? 0xffffffffu : (((1u << (G & 31)) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    [[maybe_unused]] LaneDir<Q> ld[K];
    // groups: this lane's outlet values and STL-link results with their momentum-exchange sums
    // fb + f_q, for its directions lane + G k (the rest direction and q >= Q have none)
    [[maybe_unused]] float v_out[K], v_link[K], v_fw[K];
    [[maybe_unused]] bool has_out[K], link[K];
    if constexpr (GRP) {
        const T* fin = static_cast<const T*>(a.f_in);
        const bool border = a.border_pulls && (x[0] == 0 || x[0] == N[0] - 1 || x[1] == 0 || x[1] == N[1] - 1 ||
                                               x[2] == 0 || x[2] == N[2] - 1);
        const BorderCell g = border_cell(a, x[0], x[1], x[2]);
        const bool nei = a.nei_solid[ic] == 1;
        const bool outlet = face && (b[0] == BC_OUTLET || b[1] == BC_OUTLET || b[2] == BC_OUTLET);
        float fs[K], fo[K], f_in_cell[K], fb[K], sdf1[K], ufc[K][3];
        int out_axis[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int qk = lane + G * k;
            const bool okq = qk < Q;
            const int lq = okq ? qk : 0;  // lanes past Q stand in for direction 0
            ld[k] = lane_dir<Q>(lq);
            long long el;
            if (border) {
                int m = 0;
#pragma unroll
                for (int p = 0; p < Q; p++)
                    if (lq == p) m = missing_dir<Q>(p, g.b);
                el = border_pull_c(a, g, ld[k].c, lq, m, ip);
            } else {
                el = (long long)lq * a.pE + (ip - (ld[k].c[0] + ld[k].c[1] * a.px + ld[k].c[2] * a.pxy));
            }
            fs[k] = Codec<S>::load(fin + el, ld[k].w);
            fo[k] = Codec<S>::load(fin + (long long)lq * a.pE + ip, ld[k].w);  // the cell's own previous f_q
            // outflowBC's inner value (the last outlet face of the cell whose inward direction q is)
            f_in_cell[k] = 0.f;
            out_axis[k] = 0;
            has_out[k] = false;
            if (outlet) {
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    if (b[d] != BC_OUTLET) continue;
#pragma unroll
                    for (int side = -1; side <= 1; side += 2) {
                        if (!((side < 0 && x[d] == 0) || (side > 0 && x[d] == N[d] - 1))) continue;
                        if (qk >= 1 && okq && ld[k].c[d] == -side) {
                            f_in_cell[k] = Codec<S>::load(fin + (long long)lq * a.pE + inner_p(d, side), ld[k].w);
                            has_out[k] = true;
                            out_axis[k] = d;
                        }
                    }
                }
            }
            // STL link of direction q (internalWallBC): its reads, before the link test resolves
            link[k] = false;
            fb[k] = sdf1[k] = 0.f;
            ufc[k][0] = ufc[k][1] = ufc[k][2] = 0.f;
            if (nei && qk >= 1 && okq) {
                const long long up = upwind_c(ld[k].c, x, N, b, face);
                link[k] = up >= 0 && a.solid[up] == 1;
                // F(opposite of q, ip); opposite directions have equal weights
                fb[k] = Codec<S>::load(fin + (long long)ld[k].opp * a.pE + ip, ld[k].w);
                if (a.wall != WALL_BB) {
                    sdf1[k] = up >= 0 ? a.sdf[up] : 0.f;
                    const int cb[3] = {-ld[k].c[0], -ld[k].c[1], -ld[k].c[2]};
                    const long long fl = upwind_c(cb, x, N, b, face);
                    const long long fc = fl < 0 ? ic : fl;
                    ufc[k][0] = a.u_p[fc];
                    ufc[k][1] = a.v_p[fc];
                    ufc[k][2] = a.w_p[fc];
                }
            }
        }
#pragma unroll
        for (int q = 0; q < Q; q++) ft[q] = __shfl_sync(gmask, fs[q / G], q % G, G);
        const float uo_[3] = {a.u_p[ic], a.v_p[ic], a.w_p[ic]};
#pragma unroll
        for (int k = 0; k < K; k++) {
            v_out[k] = v_link[k] = v_fw[k] = 0.f;
            if (has_out[k]) {
                const float gq = 0.57735026919f - (out_axis[k] == 0 ? uo_[0] : out_axis[k] == 1 ? uo_[1] : uo_[2]);
                v_out[k] = gq * f_in_cell[k] + (1.f - gq) * fo[k];
            }
            if (link[k]) {
                if (a.wall == WALL_BB) {
                    v_link[k] = fb[k];
                } else {
                    const float omega_l = a.omega[ic], rho_o = a.rho_p[ic], tau_o = a.tau_p[ic];
                    const float usq = uo_[0] * uo_[0] + uo_[1] * uo_[1] + uo_[2] * uo_[2];
                    const float sdf0 = a.sdf[ic];
                    const float qf = fabsf(sdf0) / (fabsf(sdf0) + fabsf(sdf1[k]));
                    const float we = 1.f / (1.f / omega_l + tau_o);
                    const float uc =
                        -uo_[0] * (float)ld[k].c[0] - uo_[1] * (float)ld[k].c[1] - uo_[2] * (float)ld[k].c[2];
                    float feq, chi;
                    if (qf <= 0.5f) {
                        const float uf = -ufc[k][0] * (float)ld[k].c[0] - ufc[k][1] * (float)ld[k].c[1] -
                                         ufc[k][2] * (float)ld[k].c[2];
                        feq = (rho_o + 3.f * uf + 4.5f * uc * uc - 1.5f * usq) * ld[k].w;
                        chi = we * (2.f * qf - 1.f) / (1.f - 2.f * we);
                    } else {
                        feq = (rho_o + 3.f * (1.f - 1.f / qf) * uc + 4.5f * uc * uc - 1.5f * usq) * ld[k].w;
                        chi = we * (2.f * qf - 1.f);
                    }
                    v_link[k] = (1.f - chi) * fb[k] + chi * feq;
                }
                v_fw[k] = fb[k] + v_link[k];
            }
        }
    } else if (a.border_pulls && (x[0] == 0 || x[0] == N[0] - 1 || x[1] == 0 || x[1] == N[1] - 1 || x[2] == 0 ||
                                  x[2] == N[2] - 1)) {
        const BorderCell g = border_cell(a, x[0], x[1], x[2]);
#pragma unroll
        for (int q = 0; q < Q; q++)
            ft[q] = Codec<S>::load(static_cast<const T*>(a.f_in) + border_pull<Q>(a, g, q, ip), lat_w(Q, q));
    } else {
#pragma unroll
        for (int q = 0; q < Q; q++) ft[q] = Codec<S>::load(static_cast<const T*>(a.fin_s[q]) + ip, lat_w(Q, q));
    }

    const float uo[3] = {a.u_p[ic], a.v_p[ic], a.w_p[ic]};
    const float omega_c = a.omega[ic];
    if (face) {
        float fts[Q];  // the streamed values (the bounce-back momentum of the wall function uses them)
#pragma unroll
        for (int q = 0; q < Q; q++) fts[q] = ft[q];
        // cornerFlag (kernel.cl:1346-1397)
        const bool on0 = x[0] == 0 || x[0] == N[0] - 1, on1 = x[1] == 0 || x[1] == N[1] - 1,
                   on2 = x[2] == 0 || x[2] == N[2] - 1;
        const bool corner = (N[2] - 1 == 0 || b[2] == 0) ? (on0 && on1) : ((int)on0 + (int)on1 + (int)on2 >= 2);
        if (!corner) {
            // fixedVelocityBC (kernel.cl:1399-1512): Ladd correction with wall density
            const float uw[3] = {a.u0[ic], a.v0[ic], a.w0[ic]};
#pragma unroll
            for (int d = 0; d < 3; d++) {
                if (b[d] != BC_FIXVEL) continue;
                int side;
                if (x[d] == 0) side = -1;
                else if (x[d] == N[d] - 1) side = 1;
                else continue;
                float tang = 0.f, outg = 0.f;
#pragma unroll
                for (int q = 0; q < Q; q++) {
                    if (lat_c(Q, q, d) == 0) tang += ft[q];
                    else if (lat_c(Q, q, d) == side) outg += ft[q];
                }
                float rhow = (tang + 2.f * outg) / (1.f + (float)side * uw[d]);
                if ((side < 0 && uw[d] < 0.f) || (side > 0 && uw[d] > 0.f)) {
                    // x-max reads its own cell (kernel.cl:1425-1429)
                    rhow = a.rho_p[(side > 0 && d == 0) ? ic : inner(d, side)];
                }
#pragma unroll
                for (int q = 0; q < Q; q++) {
                    if (lat_c(Q, q, d) != -side) continue;
                    const float mult = (Q == 27 && d == 2 && side > 0 && lat_n2(Q, q) == 3) ? 4.f : 1.f;
                    const float cu = (float)lat_c(Q, q, 0) * uw[0] + (float)lat_c(Q, q, 1) * uw[1] + (float)lat_c(Q, q, 2) * uw[2];
                    ft[q] += mult * 6.f * lat_w(Q, q) * rhow * cu;
                }
            }
            // fixedDensityBC (kernel.cl:1514-1611), rho_w = 1
#pragma unroll
            for (int d = 0; d < 3; d++) {
                if (b[d] != BC_FIXDEN) continue;
                const long long in = inner(d, x[d] == 0 ? -1 : 1);
                const float uw[3] = {uo[0] + 0.5f * (uo[0] - a.u_p[in]), uo[1] + 0.5f * (uo[1] - a.v_p[in]),
                                     uo[2] + 0.5f * (uo[2] - a.w_p[in])};
                const float usq = uw[0] * uw[0] + uw[1] * uw[1] + uw[2] * uw[2];
#pragma unroll
                for (int side = -1; side <= 1; side += 2) {
                    if (!((side < 0 && x[d] == 0) || (side > 0 && x[d] == N[d] - 1))) continue;
#pragma unroll
                    for (int q = 0; q < Q; q++) {
                        if (lat_c(Q, q, d) != -side) continue;
                        const float cu = (float)lat_c(Q, q, 0) * uw[0] + (float)lat_c(Q, q, 1) * uw[1] + (float)lat_c(Q, q, 2) * uw[2];
                        ft[q] = -ft[q] + 2.f * lat_w(Q, q) * (1.f + 4.5f * cu * cu - 1.5f * usq);
                    }
                }
            }
        }
        if (!corner) {
            // wallFunctionBC (D3Q19 kernel.cl:1657-1924, D3Q27 1524-): a stationary wall whose
            // tangential slip velocity comes from the log-law shear stress of the cell 1 inward,
            // minus the momentum the face's bounce-back exchanged in this step's streaming (which
            // the reference's streaming() leaves in Fw before internalWallBC resets it), applied as
            // a moving-wall correction to the populations entering from the face.  Per axis the low
            // face wins over the high one (if / else if).
            const float nu = (1.f / omega_c - 0.5f) / 3.f;
            float fwc[3] = {0.f, 0.f, 0.f};
            if (b[0] == BC_WALLFN || b[1] == BC_WALLFN || b[2] == BC_WALLFN) {
#pragma unroll
                for (int q = 1; q < Q; q++) {
                    if (upwind<Q>(q, x, N, b, face) >= 0) continue;
#pragma unroll
                    for (int dd = 0; dd < 3; dd++)
                        if (lat_c(Q, q, dd)) fwc[dd] += -2.f * fts[q] * (float)lat_c(Q, q, dd);
                }
            }
#pragma unroll
            for (int d = 0; d < 3; d++) {
                if (b[d] != BC_WALLFN) continue;
                int side;
                if (x[d] == 0) side = -1;
                else if (x[d] == N[d] - 1) side = 1;
                else continue;
                const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;  // tangential axes, in order
                float tang = 0.f, outg = 0.f;
#pragma unroll
                for (int q = 0; q < Q; q++) {
                    if (lat_c(Q, q, d) == 0) tang += ft[q];
                    else if (lat_c(Q, q, d) == side) outg += ft[q];
                }
                const float rhow = tang + 2.f * outg;
                // the probe 1 cell inward (a 1-cell axis: the cell itself; the reference's z-max face
                // reads k + 1, outside the grid: here k - 1)
                const long long pr = (d == 2 && N[2] == 1) ? ic : inner(d, side);
                const float up[3] = {a.u_p[pr], a.v_p[pr], a.w_p[pr]};
                float mag = sqrtf(up[t1] * up[t1] + up[t2] * up[t2]);
                float tw[3] = {0.f, 0.f, 0.f};  // wall velocity (normal component stays 0)
                if (mag != 0.f) {
                    const float tauw = calc_tauw(rhow, mag, nu);
                    mag = sqrtf(uo[t1] * uo[t1] + uo[t2] * uo[t2]);
                    // the z-min face of the reference does not test the cell's own speed
                    if (mag != 0.f || (d == 2 && side < 0)) {
                        tw[t1] = -3.f * (tauw * (uo[t1] / mag) - fwc[t1]) / rhow;
                        tw[t2] = -3.f * (tauw * (uo[t2] / mag) - fwc[t2]) / rhow;
                    }
                }
                const int n = -side;  // inward direction along d
#pragma unroll
                for (int q = 1; q < Q; q++) {
                    if (lat_c(Q, q, d) != n || lat_n2(Q, q) == 1) continue;  // axis term: rho_w * 0
                    float s = 0.f;  // the wall's normal speed, then the tangential terms
                    if (lat_c(Q, q, t1)) s += (float)(lat_c(Q, q, t1) * n) * tw[t1];
                    if (lat_c(Q, q, t2)) s += (float)(lat_c(Q, q, t2) * n) * tw[t2];
                    const float den = lat_n2(Q, q) == 2 ? (Q == 19 ? 6.f : 9.f) : 36.f;
                    ft[q] += (float)n * (rhow * s) / den;
                }
            }
        }
        // outflowBC (Geier et al. 2015 App. F; kernel.cl:2005-2097)
        if constexpr (GRP) {
            // the lanes' outlet values (computed from the same reads as below)
#pragma unroll
            for (int q = 1; q < Q; q++) {
                const float vq = __shfl_sync(gmask, v_out[q / G], q % G, G);
                if (__shfl_sync(gmask, (int)has_out[q / G], q % G, G)) ft[q] = vq;
            }
        } else if (b[0] == BC_OUTLET || b[1] == BC_OUTLET || b[2] == BC_OUTLET) {
            const float cs = 0.57735026919f;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                if (b[d] != BC_OUTLET) continue;
#pragma unroll
                for (int side = -1; side <= 1; side += 2) {
                    if (!((side < 0 && x[d] == 0) || (side > 0 && x[d] == N[d] - 1))) continue;
                    const int in = inner_p(d, side);
                    const float g = cs - uo[d];
#pragma unroll
                    for (int q = 1; q < Q; q++) {
                        if (lat_c(Q, q, d) != -side) continue;
                        ft[q] = g * F(q, in) + (1.f - g) * F(q, ip);
                    }
                }
            }
        }
    }

    // internalWallBC: STL links (kernel.cl:1926-2003 / D3Q27 1823-1897)
    float fw[3] = {0.f, 0.f, 0.f};
    const float omega = a.omega[ic];
    if constexpr (GRP) {
        // the lanes' link results, and the momentum exchange summed in direction order
        bool any_link = false;
#pragma unroll
        for (int k = 0; k < K; k++) any_link |= link[k];
        if (__any_sync(gmask, any_link)) {
#pragma unroll
            for (int q = 1; q < Q; q++) {
                const float vq = __shfl_sync(gmask, v_link[q / G], q % G, G);
                const float sq = __shfl_sync(gmask, v_fw[q / G], q % G, G);
                if (__shfl_sync(gmask, (int)link[q / G], q % G, G)) {
                    ft[q] = vq;
#pragma unroll
                    for (int d = 0; d < 3; d++)
                        if (lat_c(Q, q, d)) fw[d] += -sq * (float)lat_c(Q, q, d);
                }
            }
        }
    } else if (a.nei_solid[ic] == 1) {
        const float rho_o = a.rho_p[ic], tau_o = a.tau_p[ic];
        const float usq = uo[0] * uo[0] + uo[1] * uo[1] + uo[2] * uo[2];
#pragma unroll
        for (int q = 1; q < Q; q++) {
            const long long up = upwind<Q>(q, x, N, b, face);
            if (up < 0 || a.solid[up] != 1) continue;
            const int qb = lat_opp(Q, q);
            const float fb = F(qb, ip);
            if (a.wall == WALL_BB) {
                ft[q] = fb;
            } else {
                const float sdf0 = a.sdf[ic], sdf1 = a.sdf[up];
                const float qf = fabsf(sdf0) / (fabsf(sdf0) + fabsf(sdf1));
                const float we = 1.f / (1.f / omega + tau_o);
                const float uc = -uo[0] * (float)lat_c(Q, q, 0) - uo[1] * (float)lat_c(Q, q, 1) - uo[2] * (float)lat_c(Q, q, 2);
                float feq, chi;
                if (qf <= 0.5f) {
                    const long long fl = upwind<Q>(qb, x, N, b, face);
                    const long long fc = fl < 0 ? ic : fl;
                    const float ufc = -a.u_p[fc] * (float)lat_c(Q, q, 0) - a.v_p[fc] * (float)lat_c(Q, q, 1) -
                                      a.w_p[fc] * (float)lat_c(Q, q, 2);
                    feq = (rho_o + 3.f * ufc + 4.5f * uc * uc - 1.5f * usq) * lat_w(Q, q);
                    chi = we * (2.f * qf - 1.f) / (1.f - 2.f * we);
                } else {
                    feq = (rho_o + 3.f * (1.f - 1.f / qf) * uc + 4.5f * uc * uc - 1.5f * usq) * lat_w(Q, q);
                    chi = we * (2.f * qf - 1.f);
                }
                ft[q] = (1.f - chi) * fb + chi * feq;
            }
#pragma unroll
            for (int d = 0; d < 3; d++)
                if (lat_c(Q, q, d)) fw[d] += -(fb + ft[q]) * (float)lat_c(Q, q, d);
        }
    }
    if (!GRP || lane == 0) {
        a.fwx[ic] = fw[0];
        a.fwy[ic] = fw[1];
        a.fwz[ic] = fw[2];
    }

    float rho, u, v, w, tsgs = 0.f;
    Mom19 m19;
    if constexpr (Q == 19) {
        m19 = moments19<false>(ft);
        rho = m19.rho;
        const float ir = 1.f / rho;
        u = m19.j[0] * ir + 0.5f * a.dpdx * ir;
        v = m19.j[1] * ir;
        w = m19.j[2] * ir;
    } else {
        macroscopics<Q>(ft, a.dpdx, rho, u, v, w);
    }
    if (a.sgs == SGS_WALE) {
        const float own[3] = {u, v, w};
        tsgs = wale_general(a, x[0], x[1], x[2], ic, own);
    } else if (a.les != 0.f) {
        if constexpr (Q == 19) tsgs = smagorinsky19(m19, u, v, w, omega, a.les, a.cs);
        else tsgs = smagorinsky<Q>(ft, rho, u, v, w, omega, a.les, a.cs);
        tsgs = damping(a, tsgs, a.sdf[ic], u, v, w, omega);
    }
    if (!GRP || lane == 0) {
        a.rho_n[ic] = rho;
        a.u_n[ic] = u;
        a.v_n[ic] = v;
        a.w_n[ic] = w;
        a.tau_n[ic] = tsgs;
        if (a.err && !(rho == rho)) atomicOr(a.err, 1);
    }
    const float tau = sponge_tau(a, 1.f / omega, tsgs, x[0], x[1], x[2]);
    if constexpr (Q == 19) {
        const float U[3] = {u - 0.5f * a.dpdx / rho, v, w};
        collide_rr19m(ft, m19, U, 1.f / (tau + tsgs), 1.f / rho, a.omega_b, a.dpdx);
    } else {
        collide<Q, COLL>(ft, rho, u, v, w, 1.f / (tau + tsgs), a);
    }
    if constexpr (GRP) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int qk = lane + G * k;
            float mine = ft[0];
#pragma unroll
            for (int q = 1; q < Q; q++)
                if (qk == q) mine = ft[q];
            if (qk < Q) Codec<S>::store(static_cast<T*>(a.f_out) + (long long)qk * a.pE + ip, mine, ld[k].w);
        }
    } else {
#pragma unroll
        for (int q = 0; q < Q; q++) Codec<S>::store(static_cast<T*>(a.fout_q[q]) + ip, ft[q], lat_w(Q, q));
    }
}

template <int Q, int S, int COLL>
__global__ void __launch_bounds__(SPECIAL_BS) k_special(const StepArgs a)
{
    const long long t = (long long)blockIdx.x * SPECIAL_BS + threadIdx.x;
    if (t < a.n_special) special_cell<Q, S, COLL>(a, t);
}

// a group of LBFFS_SPECIAL_LANES lanes per listed cell (special_cell with G lanes): for short lists,
// where one thread per cell leaves most SMs idle and each thread's chain of dependent reads sets the
// kernel's time.  16 lanes (two cells per warp) measured 4 % faster on the 1024x256x4 channel than
// 32 and 13 % faster than 8; a build-time tuning value
#ifndef LBFFS_SPECIAL_LANES
#define LBFFS_SPECIAL_LANES 16
#endif
template <int Q, int S, int COLL>
__global__ void __launch_bounds__(SPECIAL_BS) k_special_warp(const StepArgs a)
{
    constexpr int G = LBFFS_SPECIAL_LANES;
    const long long t = (long long)blockIdx.x * (SPECIAL_BS / G) + (threadIdx.x / G);
    if (t < a.n_special) special_cell<Q, S, COLL, G>(a, t);
}

// ---- ghost layer: the reference's face streaming for populations that cross the grid edge ----
// Every population q of a cell P whose upwind neighbour P - c_q lies outside the grid is pulled
// from the ghost P - c_q.  The ghost holds the value upwindID_B / reflectOrMirrorQ would pull
// (D3Q19 kernel.cl:114-575, D3Q27 kernel.cl:1133-1146): the periodically wrapped upwind cell's
// value, or, when a crossed face of P carries a wall code, P's own value of the bounce-back /
// mirror direction.  The fill runs over the six faces of the grid: each thread takes one face cell
// and the directions that cross its face outward-in (5 for D3Q19, 9 for D3Q27).  A diagonal
// crossing two faces at an edge is written by both faces' threads with the same value.  Raw
// element copies (W: the element's bit pattern): no rounding.
template <int Q>
__host__ __device__ constexpr int side_count()
{
    return Q == 19 ? 5 : 9;
}

__host__ __device__ constexpr int side_count_rt(int Q) { return Q == 19 ? 5 : 9; }

// Direction tables of the ghost fill, read per block from constant memory (one short code path
// for every face and direction instead of one unrolled variant each, which keeps the kernel in
// the instruction cache): velocity, the bounce-back and the three mirror directions.
struct HaloDir {
    signed char c[3];
    signed char opp, mx, my, mz;  // reflection; mirror across x / y / z (the reflection where c_d = 0)
    signed char nonzero;          // number of nonzero components
};

template <int Q>
struct HaloTable {
    HaloDir d[27];
    signed char side[3][2][9];  // [axis][low / high face][n]: the directions crossing that face inward
    constexpr HaloTable() : d{}, side{}
    {
        for (int q = 0; q < Q; q++) {
            const int c0 = lat_c(Q, q, 0), c1 = lat_c(Q, q, 1), c2 = lat_c(Q, q, 2);
            const int r = lat_opp(Q, q);
            d[q].c[0] = (signed char)c0;
            d[q].c[1] = (signed char)c1;
            d[q].c[2] = (signed char)c2;
            d[q].opp = (signed char)r;
            d[q].mx = (signed char)(c0 ? lat_find(Q, -c0, c1, c2) : r);
            d[q].my = (signed char)(c1 ? lat_find(Q, c0, -c1, c2) : r);
            d[q].mz = (signed char)(c2 ? lat_find(Q, c0, c1, -c2) : r);
            d[q].nonzero = (signed char)((c0 != 0) + (c1 != 0) + (c2 != 0));
        }
        for (int ax = 0; ax < 3; ax++)
            for (int hi = 0; hi < 2; hi++) {
                int m = 0;
                for (int q = 1; q < Q; q++)
                    if (lat_c(Q, q, ax) == (hi ? -1 : 1)) side[ax][hi][m++] = (signed char)q;
            }
    }
};

__constant__ const HaloTable<19> kHalo19{};
__constant__ const HaloTable<27> kHalo27{};

template <int Q>
__device__ __forceinline__ const HaloTable<Q>& halo_table()
{
    if constexpr (Q == 19) return kHalo19;
    else return kHalo27;
}

// reflectOrMirrorQ with the run-time direction dq and the cell's face codes b (missing_dir)
template <int Q>
__device__ __forceinline__ int halo_missing(const HaloDir& dq, const int (&b)[3])
{
    if (Q == 19) {
        if (dq.nonzero < 2) return dq.opp;
        if (dq.c[0] != 0 && b[0] == BC_SYM) return dq.mx;  // first Symmetry axis among the nonzero components
        if (dq.c[1] != 0 && b[1] == BC_SYM) return dq.my;
        if (dq.c[2] != 0 && b[2] == BC_SYM) return dq.mz;
        return dq.opp;
    }
    int out = dq.opp;  // the last Symmetry axis wins; a zero component falls back to reflection
    if (b[0] == BC_SYM) out = dq.mx;
    if (b[1] == BC_SYM) out = dq.my;
    if (b[2] == BC_SYM) out = dq.mz;
    return out;
}

// Ghost fill work of one lattice: for each axis, its two faces in blocks of HALO_BS face cells.
// Block b of the flattened grid: axis, face (low / high) and run of cells; thread: one face cell,
// which fills the ghosts of all NQ directions it pulls across that face (its flags and boundary
// word are read once; the NQ source values are gathered before the ghosts are written).
constexpr int HALO_BS = 128;

__host__ __device__ inline long long halo_face_cells(const PadGeom& g, int axis)
{
    return axis == 0 ? (long long)g.ny * g.nz : axis == 1 ? (long long)g.nx * g.nz : (long long)g.nx * g.ny;
}

__host__ __device__ inline long long halo_blocks(const PadGeom& g, int /*Q*/, int axis)
{
    return 2LL * ((halo_face_cells(g, axis) + HALO_BS - 1) / HALO_BS);
}

// The ghosts one face cell x (on face HI of axis AX) fills: the directions that cross that face
// inward, known at compile time, so every lattice constant of the loop folds.
template <int Q, typename W, int AX, int HI>
__device__ __forceinline__ void halo_cell(W* f, const PadGeom& g, const int (&x)[3], uint16_t bw)
{
    constexpr int NQ = side_count<Q>();
    constexpr HaloTable<Q> T{};
    const int bcode[3] = {bw & 7, (bw >> 3) & 7, (bw >> 6) & 7};
    const bool face = (bw >> 9) & 1;
    const int N[3] = {g.nx, g.ny, g.nz};
    const int ip = g.porg + x[2] * g.pxy + x[1] * g.px + x[0];
    W v[NQ];
#pragma unroll
    for (int n = 0; n < NQ; n++) {
        const int q = T.side[AX][HI][n];
        const HaloDir dq = T.d[q];
        int up[3];
        bool miss = false;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            up[d] = x[d] - dq.c[d];
            if (up[d] < 0) {
                miss |= face && is_wall_code(bcode[d]);
                up[d] += N[d];
            } else if (up[d] >= N[d]) {
                miss |= face && is_wall_code(bcode[d]);
                up[d] -= N[d];
            }
        }
        const int src_q = miss ? halo_missing<Q>(dq, bcode) : q;
        const int src_i = miss ? ip : g.porg + up[2] * g.pxy + up[1] * g.px + up[0];
        v[n] = __ldg(f + (long long)src_q * g.pE + src_i);
    }
    // an x ghost sits alone in the padding sector before / after its row: writing the whole
    // 32-byte sector avoids a read-modify-write of a partly written sector
    constexpr int A = 32 / (int)sizeof(W);
    const bool whole = AX == 0 && (!HI || (g.nx % A) == 0);
#pragma unroll
    for (int n = 0; n < NQ; n++) {
        const int q = T.side[AX][HI][n];
        const long long dst =
            (long long)q * g.pE + (ip - (T.d[q].c[0] + T.d[q].c[1] * g.px + T.d[q].c[2] * g.pxy));
        if (whole) {
            W* sec = f + (HI ? dst : dst - (A - 1));
            const uint32_t w32 = sizeof(W) == 4 ? (uint32_t)v[n] : ((uint32_t)v[n] | ((uint32_t)v[n] << 16));
            const uint4 quad = make_uint4(w32, w32, w32, w32);
            reinterpret_cast<uint4*>(sec)[0] = quad;
            reinterpret_cast<uint4*>(sec)[1] = quad;
        } else {
            f[dst] = v[n];
        }
    }
}

// halo_cell with the axis and side at run time and the direction table in constant memory (one
// short code path for all six faces)
template <int Q, typename W>
__device__ __forceinline__ void halo_cell_rt(W* f, const PadGeom& g, const int (&x)[3], uint16_t bw, int AX, int HI)
{
    constexpr int NQ = side_count<Q>();
    const HaloTable<Q>& T = halo_table<Q>();
    const int bcode[3] = {bw & 7, (bw >> 3) & 7, (bw >> 6) & 7};
    const bool face = (bw >> 9) & 1;
    const int N[3] = {g.nx, g.ny, g.nz};
    const int ip = g.porg + x[2] * g.pxy + x[1] * g.px + x[0];
    W v[NQ];
#pragma unroll
    for (int n = 0; n < NQ; n++) {
        const int q = T.side[AX][HI][n];
        const HaloDir dq = T.d[q];
        int up[3];
        bool miss = false;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            up[d] = x[d] - dq.c[d];
            if (up[d] < 0) {
                miss |= face && is_wall_code(bcode[d]);
                up[d] += N[d];
            } else if (up[d] >= N[d]) {
                miss |= face && is_wall_code(bcode[d]);
                up[d] -= N[d];
            }
        }
        const int src_q = miss ? halo_missing<Q>(dq, bcode) : q;
        const int src_i = miss ? ip : g.porg + up[2] * g.pxy + up[1] * g.px + up[0];
        v[n] = __ldg(f + (long long)src_q * g.pE + src_i);
    }
    // an x ghost sits alone in the padding sector before / after its row: writing the whole
    // 32-byte sector avoids a read-modify-write of a partly written sector
    constexpr int A = 32 / (int)sizeof(W);
    const bool whole = AX == 0 && (!HI || (g.nx % A) == 0);
#pragma unroll
    for (int n = 0; n < NQ; n++) {
        const int q = T.side[AX][HI][n];
        const long long dst =
            (long long)q * g.pE + (ip - (T.d[q].c[0] + T.d[q].c[1] * g.px + T.d[q].c[2] * g.pxy));
        if (whole) {
            W* sec = f + (HI ? dst : dst - (A - 1));
            const uint32_t w32 = sizeof(W) == 4 ? (uint32_t)v[n] : ((uint32_t)v[n] | ((uint32_t)v[n] << 16));
            const uint4 quad = make_uint4(w32, w32, w32, w32);
            reinterpret_cast<uint4*>(sec)[0] = quad;
            reinterpret_cast<uint4*>(sec)[1] = quad;
        } else {
            f[dst] = v[n];
        }
    }
}

// SPEC: one code path per face (halo_cell) or one for all faces (halo_cell_rt).  The per-face
// paths fold every constant but are six cold code paths when the faces are of similar size (a
// 256^3 cavity: the run-time path fills the ghosts 6 % faster); when one axis holds most face
// cells (a 1024x256x4 channel, 98 % on the z faces) the per-face path is 13 % faster.
template <int Q, typename W, bool SPEC = true>
__device__ __forceinline__ void halo_block(W* f, const uint8_t* __restrict__ flags, const uint16_t* __restrict__ bc,
                                           const PadGeom& g, long long b, int tid)
{
    int axis = 0;
    long long blk = b;
    long long nb = halo_blocks(g, Q, 0);
    if (blk >= nb) {
        blk -= nb;
        axis = 1;
        nb = halo_blocks(g, Q, 1);
        if (blk >= nb) {
            blk -= nb;
            axis = 2;
        }
    }
    // every count below is < 2^31 (the padded plane size is, by construction of the context), so
    // the face-cell decode runs in 32-bit arithmetic
    const unsigned cells = (unsigned)halo_face_cells(g, axis);
    const unsigned per = (cells + HALO_BS - 1) / HALO_BS;
    const int hi = (unsigned)blk >= per ? 1 : 0;
    const unsigned p = ((unsigned)blk - (unsigned)hi * per) * HALO_BS + (unsigned)tid;
    if (p >= cells) return;
    const int N[3] = {g.nx, g.ny, g.nz};
    // face cell: the face coordinate on axis, the other two from p in row-major order
    const int a0 = axis == 0 ? 1 : 0, a1 = axis == 2 ? 1 : 2;
    int x[3];
    x[axis] = hi ? N[axis] - 1 : 0;
    const unsigned q0 = p / (unsigned)N[a0];
    x[a0] = (int)(p - q0 * (unsigned)N[a0]);
    x[a1] = (int)q0;
    const int ic = (x[2] * g.ny + x[1]) * g.nx + x[0];
    const uint8_t fl = __ldg(flags + ic);  // both loads in flight together
    const uint16_t bw = __ldg(bc + ic);
    if (fl & FL_SOLID) return;  // nobody pulls through a solid cell's ghosts
    if constexpr (!SPEC) {
        halo_cell_rt<Q, W>(f, g, x, bw, axis, hi);
        return;
    }
    // axis and side are uniform over the block: one specialised path each
    switch (axis * 2 + hi) {
        case 0: halo_cell<Q, W, 0, 0>(f, g, x, bw); break;
        case 1: halo_cell<Q, W, 0, 1>(f, g, x, bw); break;
        case 2: halo_cell<Q, W, 1, 0>(f, g, x, bw); break;
        case 3: halo_cell<Q, W, 1, 1>(f, g, x, bw); break;
        case 4: halo_cell<Q, W, 2, 0>(f, g, x, bw); break;
        default: halo_cell<Q, W, 2, 1>(f, g, x, bw); break;
    }
}

}  // namespace lbffs

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
#include "collide.cuh"
#include "lbffs_common.cuh"

namespace lbffs {

constexpr int BULK_BX = 128;
constexpr int SPECIAL_BS = 128;

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

__device__ __forceinline__ float damping(float t, float sdf, float cs)
{
    if (sdf != 10000.f && sdf > 0.f) {
        const float d = fminf(1.f, 0.41f * sdf / cs);
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

// ------------------------------------------------------------------------------------------
__device__ __forceinline__ bool is_wall_code(int b) { return b == 1 || b == 4 || b == 5 || b == 6 || b == 7; }

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

// bounce-back / mirror direction for a missing link on a domain face (reflectOrMirrorQ, D3Q19
// kernel.cl:114-326; D3Q27 kernel.cl:1133-1146 with mirrorQx/y/z)
template <int Q>
__device__ __forceinline__ int missing_dir(int q, const int (&b)[3])
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

// Face-aware pull for the bulk kernel: per axis, the index correction of a periodic wrap and the
// "missing link" flag of a wall are computed once per cell; each direction then only adds the
// corrections of its nonzero components (the selection is resolved at compile time).
struct FaceAxes {
    long long wlo[3], whi[3];  // index correction when pulling across the low / high face (wrap)
    bool mlo[3], mhi[3];       // pulling across the low / high face hits a wall (bounce-back / mirror)
    bool sym[3];               // Symmetry code on that axis
};

__device__ __forceinline__ FaceAxes face_axes(const int (&x)[3], const int (&N)[3], const long long (&st)[3],
                                              uint16_t bw)
{
    FaceAxes fa;
    const bool face = (bw >> 9) & 1;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int b = (bw >> (3 * d)) & 7;
        const bool wall = face && is_wall_code(b);
        fa.wlo[d] = (x[d] == 0) ? (long long)N[d] * st[d] : 0;
        fa.whi[d] = (x[d] == N[d] - 1) ? -(long long)N[d] * st[d] : 0;
        fa.mlo[d] = (x[d] == 0) && wall;
        fa.mhi[d] = (x[d] == N[d] - 1) && wall;
        fa.sym[d] = b == BC_SYM;
    }
    return fa;
}

template <int Q>
__device__ __forceinline__ int missing_dir_sym(int q, const bool (&sym)[3])
{
    const int c0 = lat_c(Q, q, 0), c1 = lat_c(Q, q, 1), c2 = lat_c(Q, q, 2);
    const int r = lat_opp(Q, q);
    if (Q == 19) {
        if ((c0 != 0) + (c1 != 0) + (c2 != 0) < 2) return r;
        const int fa = c0 ? lat_find(Q, -c0, c1, c2) : lat_find(Q, c0, -c1, c2);  // first nonzero axis
        const int fb = c2 ? lat_find(Q, c0, c1, -c2) : lat_find(Q, c0, -c1, c2);  // second nonzero axis
        const bool sa = c0 ? sym[0] : sym[1];
        const bool sb = c2 ? sym[2] : sym[1];
        return sa ? fa : (sb ? fb : r);
    }
    int out = r;
    if (sym[0]) out = c0 ? lat_find(Q, -c0, c1, c2) : r;
    if (sym[1]) out = c1 ? lat_find(Q, c0, -c1, c2) : r;
    if (sym[2]) out = c2 ? lat_find(Q, c0, c1, -c2) : r;
    return out;
}

// plane and cell that population q of cell ic is pulled from
template <int Q>
__device__ __forceinline__ int pull_src(int q, long long ic, const long long (&st)[3], const FaceAxes& fa, int& plane)
{
    long long idx = ic;
    bool miss = false;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int c = lat_c(Q, q, d);
        if (c == 1) {
            idx += fa.wlo[d] - st[d];
            miss |= fa.mlo[d];
        } else if (c == -1) {
            idx += fa.whi[d] + st[d];
            miss |= fa.mhi[d];
        }
    }
    plane = miss ? missing_dir_sym<Q>(q, fa.sym) : q;
    return miss ? (int)ic : (int)idx;
}

// ------------------------------------------------------------------------------------------
template <int Q, int S, int COLL, int SGS, bool LES>
__global__ void __launch_bounds__(BULK_BX) k_bulk(const StepArgs a)
{
    using T = typename Codec<S>::T;
    const int i = blockIdx.x * BULK_BX + threadIdx.x;
    if (i >= a.nx) return;
    const int j = blockIdx.y, k = blockIdx.z;
    const long long ic = ((long long)k * a.ny + j) * a.nx + i;
    const uint8_t fl = __ldg(a.flags + ic);
    if (fl & (FL_SOLID | FL_SPECIAL)) return;

    const T* fin = static_cast<const T*>(a.f_in);
    T* fout = static_cast<T*>(a.f_out);
    // D3Q19 holds f (FP32 storage) or f - w (shifted storage) through the whole step; D3Q27 holds f
    constexpr bool HELD = (Q == 19);
    auto ld = [&](int plane, int cell, int q) {
        const T* p = static_cast<const T*>(a.fin_q[plane]) + cell;
        return HELD ? Codec<S>::load_held(p) : Codec<S>::load(p, lat_w(Q, q));
    };
    const int ic32 = (int)ic;
    float ft[Q];
    if (__any_sync(__activemask(), (fl & FL_FACE) != 0)) {
        // a warp with a domain-face cell (walls, periodic wrap, symmetry only: upwindID_B with
        // bounce-back or mirror, kernel.cl:328-575 / 114-326); interior lanes get zero corrections
        const long long st[3] = {1, a.nx, (a.nz > 1) ? (long long)a.nx * a.ny : 0};
        const int x[3] = {i, j, k}, N[3] = {a.nx, a.ny, a.nz};
        const FaceAxes fa = face_axes(x, N, st, __ldg(a.bc + ic));
#pragma unroll
        for (int q = 0; q < Q; q++) {
            int plane;
            const int cell = pull_src<Q>(q, ic, st, fa, plane);
            ft[q] = ld(plane, cell, q);
        }
    } else {
#pragma unroll
        for (int q = 0; q < Q; q++) ft[q] = ld(q, ic32 - a.pull_off[q], q);
    }
    const float omega = (fl & FL_OMEGA) ? __ldg(a.omega + ic) : a.omega0;
    float rho, u, v, w, tsgs = 0.f;
    if constexpr (Q == 19) {
        const Mom19 m = moments19<Codec<S>::DEV>(ft);
        rho = m.rho;
        const float ir = 1.f / rho;
        u = m.j[0] * ir + 0.5f * a.dpdx * ir;  // updateRhoUVW (kernel.cl:3509-3523)
        v = m.j[1] * ir;
        w = m.j[2] * ir;
        if constexpr (SGS == SGS_WALE) {
            const float own[3] = {u, v, w};
            tsgs = wale_general(a, i, j, k, ic, own);
        } else if constexpr (LES) {
            tsgs = smagorinsky19(m, u, v, w, omega, a.les, a.cs);
            if (fl & FL_SDF) tsgs = damping(tsgs, __ldg(a.sdf + ic), a.cs);
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
        const float U[3] = {u - 0.5f * a.dpdx * ir, v, w};
        collide_rr19m(ft, m, U, we, a.omega_b, a.dpdx);
    } else {
        macroscopics<Q>(ft, a.dpdx, rho, u, v, w);
        if constexpr (SGS == SGS_WALE) {
            const float own[3] = {u, v, w};
            tsgs = wale_general(a, i, j, k, ic, own);
        } else if constexpr (LES) {
            tsgs = smagorinsky<Q>(ft, rho, u, v, w, omega, a.les, a.cs);
            if (fl & FL_SDF) tsgs = damping(tsgs, __ldg(a.sdf + ic), a.cs);
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
        collide<Q, COLL>(ft, rho, u, v, w, we, a);
    }
#pragma unroll
    for (int q = 0; q < Q; q++) {
        T* p = static_cast<T*>(a.fout_q[q]) + ic32;
        if constexpr (HELD) Codec<S>::store_held(p, ft[q]);
        else Codec<S>::store(p, ft[q], lat_w(Q, q));
    }
}

template <int Q, int S, int COLL>
__global__ void __launch_bounds__(SPECIAL_BS) k_special(const StepArgs a)
{
    using T = typename Codec<S>::T;
    const long long t = (long long)blockIdx.x * SPECIAL_BS + threadIdx.x;
    if (t >= a.n_special) return;
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
    const uint16_t bw = a.bc[ic];
    const int b[3] = {bw & 7, (bw >> 3) & 7, (bw >> 6) & 7};
    const bool face = (bw >> 9) & 1;
    const T* fin = static_cast<const T*>(a.f_in);
    T* fout = static_cast<T*>(a.f_out);
    const long long E = a.E;
    auto F = [&](int q, long long cell) { return Codec<S>::load(fin + (long long)q * E + cell, lat_w(Q, q)); };

    float ft[Q];
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const long long up = (q == 0) ? ic : upwind<Q>(q, x, N, b, face);
        ft[q] = (up >= 0) ? F(q, up) : F(missing_dir<Q>(q, b), ic);
    }

    const float uo[3] = {a.u_p[ic], a.v_p[ic], a.w_p[ic]};
    if (face) {
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
        // outflowBC (Geier et al. 2015 App. F; kernel.cl:2005-2097)
        if (b[0] == BC_OUTLET || b[1] == BC_OUTLET || b[2] == BC_OUTLET) {
            const float cs = 0.57735026919f;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                if (b[d] != BC_OUTLET) continue;
#pragma unroll
                for (int side = -1; side <= 1; side += 2) {
                    if (!((side < 0 && x[d] == 0) || (side > 0 && x[d] == N[d] - 1))) continue;
                    const long long in = inner(d, side);
                    const float g = cs - uo[d];
#pragma unroll
                    for (int q = 1; q < Q; q++) {
                        if (lat_c(Q, q, d) != -side) continue;
                        ft[q] = g * F(q, in) + (1.f - g) * F(q, ic);
                    }
                }
            }
        }
    }

    // internalWallBC: STL links (kernel.cl:1926-2003 / D3Q27 1823-1897)
    float fw[3] = {0.f, 0.f, 0.f};
    const float omega = a.omega[ic];
    if (a.nei_solid[ic] == 1) {
        const float rho_o = a.rho_p[ic], tau_o = a.tau_p[ic];
        const float usq = uo[0] * uo[0] + uo[1] * uo[1] + uo[2] * uo[2];
#pragma unroll
        for (int q = 1; q < Q; q++) {
            const long long up = upwind<Q>(q, x, N, b, face);
            if (up < 0 || a.solid[up] != 1) continue;
            const int qb = lat_opp(Q, q);
            const float fb = F(qb, ic);
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
    a.fwx[ic] = fw[0];
    a.fwy[ic] = fw[1];
    a.fwz[ic] = fw[2];

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
        tsgs = damping(tsgs, a.sdf[ic], a.cs);
    }
    a.rho_n[ic] = rho;
    a.u_n[ic] = u;
    a.v_n[ic] = v;
    a.w_n[ic] = w;
    a.tau_n[ic] = tsgs;
    if (a.err && !(rho == rho)) atomicOr(a.err, 1);
    const float tau = sponge_tau(a, 1.f / omega, tsgs, x[0], x[1], x[2]);
    if constexpr (Q == 19) {
        const float U[3] = {u - 0.5f * a.dpdx / rho, v, w};
        collide_rr19m(ft, m19, U, 1.f / (tau + tsgs), a.omega_b, a.dpdx);
    } else {
        collide<Q, COLL>(ft, rho, u, v, w, 1.f / (tau + tsgs), a);
    }
#pragma unroll
    for (int q = 0; q < Q; q++) Codec<S>::store(fout + (long long)q * E + ic, ft[q], lat_w(Q, q));
}

}  // namespace lbffs

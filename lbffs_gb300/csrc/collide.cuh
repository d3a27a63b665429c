// Device collision operators of the fused step.  All loops run over compile-time
// bounds and are fully unrolled, so the populations and moments live in registers.
//
//  collide_rr<19>   recursive-regularised collision of D3Q19_opencl/kernel.cl:3156-3309:
//                   second-order Hermite moments, bulk/shear split of the diagonal
//                   (omega_P / omega_M from omega_B), recursive third (c_a^2 c_b) and
//                   fourth (c_a^2 c_b^2) order non-equilibrium terms, D3Q19 raw-moment
//                   inverse, first-order pressure-gradient source rho w_q 3 c_qx dpdx.
//  collide_rr<27>   the same closure on the full D3Q27 tensor Hermite basis (no reference
//                   counterpart; defined with the CPU oracle): every coefficient of order
//                   >= 3 is u-products + (1 - omega) * its recursive non-equilibrium part.
//  collide_cumulant the parametrised cumulant operator (Geier et al. 2015) as run by
//                   D3Q27_opencl/kernel.cl:2352-2691, including its clim limiter and its
//                   fifth-order back-conversion products.
#pragma once
#include "lbffs_common.cuh"
#include "pair.cuh"

namespace lbffs {

// c_a^{n} for n in 0..2 with c in {-1,0,1}, evaluated at compile time after unrolling
__device__ __forceinline__ float ipow(float x, int n) { return n == 0 ? 1.f : n == 1 ? x : x * x; }

// N2 (second-order non-equilibrium moments / rho) and R2 (their relaxed values plus u u) of the
// recursive regularised collision from M2[a][b] = sum_q (c_a c_b - delta_ab / 3) f_q (upper triangle)
__device__ __forceinline__ void rr_second_from(float (&M2)[3][3], float rho, const float (&U)[3], float we,
                                               float omega_b, float (&N2)[3][3], float (&R2)[3][3])
{
    const float ir = 1.f / rho;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = a; b < 3; b++) {
            M2[a][b] *= ir;
            N2[a][b] = M2[a][b] - U[a] * U[b];
            N2[b][a] = N2[a][b];
        }
    const float wm = (omega_b - we) * (1.f / 3.f), wp = wm + we;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float r = M2[a][a];
#pragma unroll
        for (int b = 0; b < 3; b++) r -= (a == b ? wp : wm) * N2[b][b];
        R2[a][a] = r;
#pragma unroll
        for (int b = a + 1; b < 3; b++) {
            R2[a][b] = M2[a][b] - we * N2[a][b];
            R2[b][a] = R2[a][b];
        }
    }
}

template <int Q>
__device__ __forceinline__ void rr_second_order(const float (&ft)[Q], float rho, const float (&U)[3], float we,
                                                float omega_b, float (&N2)[3][3], float (&R2)[3][3])
{
    float M2[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) M2[a][b] = 0.f;
#pragma unroll
    for (int q = 0; q < Q; q++) {
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = a; b < 3; b++) {
                const int cc = lat_c(Q, q, a) * lat_c(Q, q, b);
                if (a == b) M2[a][b] += ((float)cc - 1.f / 3.f) * ft[q];
                else if (cc != 0) M2[a][b] += (float)cc * ft[q];
            }
    }
    rr_second_from(M2, rho, U, we, omega_b, N2, R2);
}

// D3Q19 recursive regularised collision; U is the velocity with the half-force shift removed.
__device__ __forceinline__ void collide_rr19(float (&f)[19], float rho, const float (&U)[3], float we, float omega_b,
                                             float dpdx)
{
    float N2[3][3], R2[3][3];
    rr_second_order<19>(f, rho, U, we, omega_b, N2, R2);
    const float third = 1.f / 3.f, ninth = 1.f / 9.f, k1 = 1.f - we;
    float T3[3][3], Q4[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
            if (a == b) continue;
            const float n3 = U[b] * N2[a][a] + 2.f * U[a] * N2[a][b];
            T3[a][b] = U[a] * U[a] * U[b] + k1 * n3 + third * U[b];
            const float n4 = U[b] * U[b] * N2[a][a] + U[a] * U[a] * N2[b][b] + 4.f * U[a] * U[b] * N2[a][b];
            Q4[a][b] = U[a] * U[a] * U[b] * U[b] + k1 * n4 + third * (R2[a][a] + R2[b][b]) + ninth;
        }
    const float RM[3] = {R2[0][0] + third, R2[1][1] + third, R2[2][2] + third};
    const float src = rho * 3.f * dpdx;
#pragma unroll
    for (int q = 0; q < 19; q++) {
        const int cx = lat_c(19, q, 0), cy = lat_c(19, q, 1), cz = lat_c(19, q, 2);
        const int n2 = lat_n2(19, q);
        float val;
        if (n2 == 0) {
            val = rho * (1.f - RM[0] - RM[1] - RM[2] + Q4[0][1] + Q4[0][2] + Q4[1][2]);
        } else if (n2 == 1) {
            const int a = cx ? 0 : cy ? 1 : 2, b = (a + 1) % 3, d = (a + 2) % 3;
            const float s = (float)(a == 0 ? cx : a == 1 ? cy : cz);
            val = 0.5f * rho * (s * U[a] + RM[a] - s * T3[b][a] - s * T3[d][a] - Q4[a][b] - Q4[a][d]);
        } else {
            const int a = cx ? 0 : 1, b = cz ? 2 : 1;
            const float sa = (float)(a == 0 ? cx : cy), sb = (float)(b == 2 ? cz : cy);
            val = 0.25f * rho * (sa * sb * R2[a][b] + sb * T3[a][b] + sa * T3[b][a] + Q4[a][b]);
        }
        if (cx != 0) val += lat_w(19, q) * (float)cx * src;
        f[q] = val;
    }
}

// ---- D3Q19 in moment form: all moments from the 9 opposite pairs (a = f_q + f_qbar, d = f_q - f_qbar) ----
// The populations may be held as f_q (FP32 storage) or as deviations g_q = f_q - w_q (shifted storage,
// DEV = true); every formula below is written in terms of r = sum_q (held value), which is rho or
// rho - 1, so both forms share it and the large constant parts never cancel in FP32.
// Moments of the held values.  With a held scale HS (2^15 for FP16S storage) r, j and s are HS
// times the moments of f (f form) or of f - w (deviation form); rho is unscaled.
// The value type V is float (one cell) or F2 (two cells in packed FP32x2 lanes); the expressions
// are the same for both.
template <class V>
struct Mom19T {
    V r;        // sum of the held values: rho (f form) or rho - 1 (deviation form)
    V rho;
    V j[3];     // sum_q c_q f_q
    V s[3][3];  // sum_q c_a c_b (held value); diagonal: sum c_a^2 f_q - 1/3 in deviation form
};
using Mom19 = Mom19T<float>;

template <bool DEV, int HS = 1, class V = float>
__device__ __forceinline__ Mom19T<V> moments19(const V (&f)[19])
{
    const V a1 = f[1] + f[2], d1 = f[1] - f[2], a3 = f[3] + f[4], d3 = f[3] - f[4];
    const V a5 = f[5] + f[6], d5 = f[5] - f[6], a7 = f[7] + f[8], d7 = f[7] - f[8];
    const V a9 = f[9] + f[10], d9 = f[9] - f[10], a11 = f[11] + f[12], d11 = f[11] - f[12];
    const V a13 = f[13] + f[14], d13 = f[13] - f[14], a15 = f[15] + f[16], d15 = f[15] - f[16];
    const V a17 = f[17] + f[18], d17 = f[17] - f[18];
    Mom19T<V> m;
    m.s[0][0] = (a1 + a7) + (a9 + a11) + a13;
    m.s[1][1] = (a3 + a7) + (a9 + a15) + a17;
    m.s[2][2] = (a5 + a11) + (a13 + a15) + a17;
    m.r = (f[0] + a1) + (a3 + a5) + ((a7 + a9) + (a11 + a13)) + (a15 + a17);
    if constexpr (HS == 1) {
        if constexpr (DEV) m.rho = 1.f + m.r;
        else m.rho = m.r;
    } else {
        if constexpr (DEV) m.rho = 1.f + m.r * (1.f / HS);
        else m.rho = m.r * (1.f / HS);
    }
    m.j[0] = (d1 + d7) + (d9 + d11) + d13;
    m.j[1] = (d3 + d7) - d9 + (d15 + d17);
    m.j[2] = (d5 + d11) - d13 + (d15 - d17);
    m.s[0][1] = m.s[1][0] = a7 - a9;
    m.s[0][2] = m.s[2][0] = a11 - a13;
    m.s[1][2] = m.s[2][1] = a15 - a17;
    return m;
}

// sum over the components of the non-equilibrium stress squared, Pi_neq : Pi_neq, of
// smagorinskyTauSGS, with sum_q c_a c_b feq_q = rho delta_ab / 3 + u_a u_b for the reference's
// feq = (rho + 3 c.u + 4.5 (c.u)^2 - 1.5 u^2) w_q (fourth-order isotropy of D3Q19); s_aa - r/3 is
// sum c_a^2 f - rho/3 in either form
template <int HS = 1, class V = float>
__device__ __forceinline__ V smag_pp19(const Mom19T<V>& m, V u, V v, V w)
{
    // each component is formed with its sign flipped (u_a u_b minus the moment), which the squares
    // below do not see; the products are fused explicitly
    const V r3 = m.r * (1.f / 3.f);
    V pxx, pyy, pzz, pxy, pxz, pyz;
    if constexpr (HS == 1) {
        pxx = mad(u, u, r3 - m.s[0][0]), pyy = mad(v, v, r3 - m.s[1][1]), pzz = mad(w, w, r3 - m.s[2][2]);
        pxy = mad(u, v, neg(m.s[0][1])), pxz = mad(u, w, neg(m.s[0][2])), pyz = mad(v, w, neg(m.s[1][2]));
    } else {
        constexpr float is = 1.f / HS;
        pxx = mad(u, u, (r3 - m.s[0][0]) * is), pyy = mad(v, v, (r3 - m.s[1][1]) * is);
        pzz = mad(w, w, (r3 - m.s[2][2]) * is);
        pxy = mad(u, v, m.s[0][1] * (-is)), pxz = mad(u, w, m.s[0][2] * (-is)), pyz = mad(v, w, m.s[1][2] * (-is));
    }
    V t = mad(pyz, pyz, mad(pxz, pxz, pxy * pxy));
    t = t + t;
    return mad(pxx, pxx, mad(pyy, pyy, mad(pzz, pzz, t)));
}

// the eddy relaxation time of smagorinskyTauSGS (without damping) from Pi_neq : Pi_neq
__device__ __forceinline__ float smag_tau(float pp, float rho, float omega, float les, float cs)
{
    const float tau = 1.f / omega;
    return les * 0.5f * (sqrtf(fmaf(tau, tau, 18.f * 1.41421356237f * cs * cs * sqrtf(pp) / rho)) - tau);
}

template <int HS = 1>
__device__ __forceinline__ float smagorinsky19(const Mom19& m, float u, float v, float w, float omega, float les,
                                               float cs)
{
    return smag_tau(smag_pp19<HS>(m, u, v, w), m.rho, omega, les, cs);
}

// recursive regularised collision (D3Q19 kernel.cl:3156-3309) from the moments; U without the half-force
// shift.  Each output is written w_q * r + rho * (deviation), i.e. f_q or f_q - w_q as held, times the
// held scale HS (a power of two, so the scaled results are the unscaled ones times HS exactly).
// ir1 = 1 / rho (one division per cell, computed by the caller).
template <int HS = 1, class V = float>
__device__ __forceinline__ void collide_rr19m(V (&f)[19], const Mom19T<V>& m, const V (&U)[3], V we, V ir1,
                                              float omega_b, float dpdx)
{
    // every multiply that feeds an add is fused explicitly (mad)
    const float third = 1.f / 3.f;
    const V k1 = 1.f - we, rho = m.rho, nwe = neg(we);
    V ir;
    if constexpr (HS == 1) ir = ir1;
    else ir = ir1 * (1.f / HS);
    const V r3 = m.r * third;
    const V NU[3] = {neg(U[0]), neg(U[1]), neg(U[2])};
    const V UU[3] = {U[0] * U[0], U[1] * U[1], U[2] * U[2]};
    const V U2[3] = {U[0] + U[0], U[1] + U[1], U[2] + U[2]};
    const V TU[3] = {U[0] * third, U[1] * third, U[2] * third};
    V N2[3][3], R2[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = a; b < 3; b++) {
            const V m2 = (a == b) ? (m.s[a][a] - r3) * ir : m.s[a][b] * ir;
            N2[a][b] = N2[b][a] = mad(NU[a], U[b], m2);
            R2[a][b] = R2[b][a] = m2;
        }
    const V wm = (omega_b - we) * third;
    const V wn = wm * (N2[0][0] + N2[1][1] + N2[2][2]);
#pragma unroll
    for (int a = 0; a < 3; a++) {
        R2[a][a] = R2[a][a] - mad(we, N2[a][a], wn);  // omega_P on the own axis, omega_M on the others
#pragma unroll
        for (int b = a + 1; b < 3; b++) R2[a][b] = R2[b][a] = mad(nwe, N2[a][b], R2[a][b]);
    }
    // T3[a][b]: c_a^2 c_b moment; Q4[a][b]: c_a^2 c_b^2 moment minus its constant 1/9
    V T3[3][3], Q4[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
            if (a == b) continue;
            const V n3 = mad(U[b], N2[a][a], U2[a] * N2[a][b]);
            T3[a][b] = mad(UU[a], U[b], mad(k1, n3, TU[b]));
            if (b > a) {
                const V n4 = mad(UU[b], N2[a][a], mad(UU[a], N2[b][b], (U2[a] * U2[b]) * N2[a][b]));
                Q4[a][b] = Q4[b][a] = mad(UU[a], UU[b], mad(k1, n4, (R2[a][a] + R2[b][b]) * third));
            }
        }
    const V h = rho * (0.5f * HS), qr = rho * (0.25f * HS);
    const V base1 = m.r * (1.f / 18.f), base2 = m.r * (1.f / 36.f);
    const V src1 = rho * (3.f * dpdx * (1.f / 18.f) * HS), src2 = rho * (3.f * dpdx * (1.f / 36.f) * HS);
    // axis pairs (q+, q-) = (1,2) (3,4) (5,6)
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int b = (a + 1) % 3, d = (a + 2) % 3;
        const V A = mad(h, R2[a][a] - Q4[a][b] - Q4[a][d], base1);
        const V B = h * (U[a] - T3[b][a] - T3[d][a]);
        if (a == 0) {
            f[1] = A + B + src1;
            f[2] = A - B - src1;
        } else {
            f[1 + 2 * a] = A + B;
            f[2 + 2 * a] = A - B;
        }
    }
    // diagonal planes (a,b) = (x,y) q7-10, (x,z) q11-14, (y,z) q15-18: (+,+) (-,-) (+,-) (-,+)
#pragma unroll
    for (int p = 0; p < 3; p++) {
        const int a = p < 2 ? 0 : 1, b = p == 0 ? 1 : 2;
        const V P = mad(qr, Q4[a][b], base2), Rr = qr * R2[a][b], X = qr * T3[a][b], Y = qr * T3[b][a];
        const V pp = P + Rr, pm = P - Rr, xp = X + Y, xm = Y - X;
        if (a == 0) {
            f[7 + 4 * p] = pp + xp + src2;
            f[8 + 4 * p] = pp - xp - src2;
            f[9 + 4 * p] = pm + xm + src2;
            f[10 + 4 * p] = pm - xm - src2;
        } else {
            f[7 + 4 * p] = pp + xp;
            f[8 + 4 * p] = pp - xp;
            f[9 + 4 * p] = pm + xm;
            f[10 + 4 * p] = pm - xm;
        }
    }
    // rest population last: it absorbs the rounding of the other 18, so each cell's mass is kept to
    // within one unbiased rounding (the collision conserves mass exactly in real arithmetic)
    f[0] = m.r - (((f[1] + f[2]) + (f[3] + f[4]) + (f[5] + f[6])) +
                  (((f[7] + f[8]) + (f[9] + f[10])) + ((f[11] + f[12]) + (f[13] + f[14]))) + ((f[15] + f[16]) + (f[17] + f[18])));
}

// 1-D backward chimera step (central moments about u -> populations at c = -1, 0, +1)
__device__ __forceinline__ void chimera_back(float k0, float k1, float k2, float u, float& fm, float& f0, float& fp)
{
    f0 = k0 * (1.f - u * u) - 2.f * u * k1 - k2;
    fm = 0.5f * (k0 * (u * u - u) + k1 * (2.f * u - 1.f) + k2);
    fp = 0.5f * (k0 * (u * u + u) + k1 * (2.f * u + 1.f) + k2);
}

__device__ __forceinline__ void moments_to_pop27(float (&M)[3][3][3], float u, float v, float w, float (&f)[27])
{
    float P[3][3][3];
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int c = 0; c < 3; c++) chimera_back(M[0][b][c], M[1][b][c], M[2][b][c], u, P[0][b][c], P[1][b][c], P[2][b][c]);
#pragma unroll
    for (int s = 0; s < 3; s++)
#pragma unroll
        for (int c = 0; c < 3; c++) chimera_back(P[s][0][c], P[s][1][c], P[s][2][c], v, M[s][0][c], M[s][1][c], M[s][2][c]);
#pragma unroll
    for (int s = 0; s < 3; s++)
#pragma unroll
        for (int t = 0; t < 3; t++) chimera_back(M[s][t][0], M[s][t][1], M[s][t][2], w, P[s][t][0], P[s][t][1], P[s][t][2]);
#pragma unroll
    for (int q = 0; q < 27; q++) f[q] = P[lat_c(27, q, 0) + 1][lat_c(27, q, 1) + 1][lat_c(27, q, 2) + 1];
}

// ---- D3Q27 recursive regularised collision in moment form (bulk cells) ----
// The populations are held as in collide_rr19m (f_q, or g_q = HS (f_q - w_q) for shifted storage), one
// cell (float) or two (F2).  The moments come from the 13 opposite pairs (q, q + 1 for odd q) into the
// same Mom19T record the D3Q19 path uses, always in deviation form: r = sum of (f_q - w_q) (times HS),
// that is rho - 1, and s = sum c_a c_b (f_q - w_q), from which the second-order stress follows without
// the cancellation of two O(1/3) terms.  Held f (DEV = false, FP32 storage) is shifted per opposite
// pair (a_p - 2 w_p, exact when a_p lies within a factor two of 2 w_p); rho itself is the direct sum.
template <bool DEV, int HS = 1, class V = float>
__device__ __forceinline__ Mom19T<V> moments27p(const V (&f)[27])
{
    V a[14], d[14];
#pragma unroll
    for (int p = 1; p < 14; p++) {
        a[p] = f[2 * p - 1] + f[2 * p];
        d[p] = f[2 * p - 1] - f[2 * p];
    }
    Mom19T<V> m;
    // rest, axis pairs, edge pairs, corner pairs
    const V tot = ((f[0] + (a[1] + a[2])) + (a[3] + (a[4] + a[5]))) +
                  (((a[6] + a[7]) + (a[8] + a[9])) + ((a[10] + a[11]) + (a[12] + a[13])));
    if constexpr (DEV) {
        m.r = tot;
        if constexpr (HS == 1) m.rho = 1.f + m.r;
        else m.rho = 1.f + m.r * (1.f / HS);
    } else {
        static_assert(HS == 1, "f held unscaled");
        m.rho = tot;
        m.r = tot - 1.f;
#pragma unroll
        for (int p = 1; p < 14; p++) a[p] = a[p] - 2.f * lat_w(27, 2 * p - 1);
    }
#pragma unroll
    for (int x = 0; x < 3; x++) {
        V jx = d[x + 1];  // the axis pair of x comes first (q = 2x + 1)
#pragma unroll
        for (int p = 4; p < 14; p++) {
            const int c = lat_c(27, 2 * p - 1, x);
            if (c > 0) jx = jx + d[p];
            else if (c < 0) jx = jx - d[p];
        }
        m.j[x] = jx;
#pragma unroll
        for (int y = x; y < 3; y++) {
            V s;
            bool first = true;
#pragma unroll
            for (int p = 1; p < 14; p++) {
                const int cc = lat_c(27, 2 * p - 1, x) * lat_c(27, 2 * p - 1, y);
                if (cc == 0) continue;
                if (first) {
                    s = cc > 0 ? a[p] : neg(a[p]);
                    first = false;
                } else if (cc > 0) {
                    s = s + a[p];
                } else {
                    s = s - a[p];
                }
            }
            m.s[x][y] = m.s[y][x] = s;
        }
    }
    return m;
}

// The D3Q27 recursive regularised collision (the same operator as collide_rr27) from the moments, for
// held populations: U without the half-force shift, ir1 = 1 / rho.  FOUT: the results are f_q (FP32
// storage), else HS (f_q - w_q).  Post-collision populations are the tensor Hermite expansion
// f_q = w_q rho sum_{abc} H_abc h_a(c_x) h_b(c_y) h_c(c_z) with the 1-D basis h = (1, 3c, 9/2 (c^2 - 1/3))
// and weights (1/6, 2/3, 1/6): H_000 = 1, H_1 = U (the pressure-gradient source 3 rho w_q c_x dpdx is
// dpdx added to H_100), H_2 = R2 (bulk / shear split), every higher coefficient = its u-products +
// (1 - omega) times its recursive non-equilibrium part.  The held output HS (f_q - w_q) takes rho - 1 = r
// in place of rho H_000.  Each coefficient is scaled by rho HS and by (1/6, 1/2, 1/2) per axis for its
// order (0, 1, 2) along the axis, so that each 1-D pass of the expansion is P(+-1) = T_0 + T_2 +- T_1,
// P(0) = 4 T_0 - 2 T_2.
template <int HS = 1, bool FOUT = false, class V = float>
__device__ __forceinline__ void collide_rr27p(V (&f)[27], const Mom19T<V>& m, const V (&U)[3], V we, V ir1,
                                              float omega_b, float dpdx)
{
    const float third = 1.f / 3.f;
    const V k1 = 1.f - we, nwe = neg(we);
    V ir;
    if constexpr (HS == 1) ir = ir1;
    else ir = ir1 * (1.f / HS);
    const V r3 = m.r * third;
    const V NU[3] = {neg(U[0]), neg(U[1]), neg(U[2])};
    V N2[3][3], R2[3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = a; b < 3; b++) {
            const V m2 = (a == b) ? (m.s[a][a] - r3) * ir : m.s[a][b] * ir;
            N2[a][b] = N2[b][a] = mad(NU[a], U[b], m2);
            R2[a][b] = R2[b][a] = m2;
        }
    const V wm = (omega_b - we) * third;
    const V wn = wm * (N2[0][0] + N2[1][1] + N2[2][2]);
#pragma unroll
    for (int a = 0; a < 3; a++) {
        R2[a][a] = R2[a][a] - mad(we, N2[a][a], wn);
#pragma unroll
        for (int b = a + 1; b < 3; b++) R2[a][b] = R2[b][a] = mad(nwe, N2[a][b], R2[a][b]);
    }
    const V u = U[0], v = U[1], w = U[2];
    const V uu = u * u, vv = v * v, ww = w * w, uv = u * v, uw = u * w, vw = v * w;
    // A = (1 - omega) N2, D = 2 A (off-diagonal), B_aa = u_a^2 + A_aa
    const V Axy = k1 * N2[0][1], Axz = k1 * N2[0][2], Ayz = k1 * N2[1][2];
    const V Dxy = Axy + Axy, Dxz = Axz + Axz, Dyz = Ayz + Ayz;
    const V Ayy = k1 * N2[1][1], Azz = k1 * N2[2][2];
    const V Bxx = mad(k1, N2[0][0], uu), Byy = mad(k1, N2[1][1], vv), Bzz = mad(k1, N2[2][2], ww);
    // third order (x^2 y, ...; xyz)
    const V H210 = mad(Bxx, v, Dxy * u), H201 = mad(Bxx, w, Dxz * u);
    const V H120 = mad(Byy, u, Dxy * v), H021 = mad(Byy, w, Dyz * v);
    const V H102 = mad(Bzz, u, Dxz * w), H012 = mad(Bzz, v, Dyz * w);
    const V H111 = mad(uv + Axy, w, mad(Axz, v, Ayz * u));
    // fourth order
    const V H220 = mad(Bxx, vv, mad(Ayy, uu, (Dxy + Dxy) * uv));
    const V H202 = mad(Bxx, ww, mad(Azz, uu, (Dxz + Dxz) * uw));
    const V H022 = mad(Byy, ww, mad(Azz, vv, (Dyz + Dyz) * vw));
    const V H211 = mad(Bxx, vw, mad(Dxy, uw, mad(Dxz, uv, Ayz * uu)));
    const V H121 = mad(Byy, uw, mad(Dxy, vw, mad(Dyz, uv, Axz * vv)));
    const V H112 = mad(Bzz, uv, mad(Dxz, vw, mad(Dyz, uw, Axy * ww)));
    // fifth and sixth order
    const V H221 = mad(w, H220, mad(Dxz, u * vv, Dyz * (uu * v)));
    const V H212 = mad(v, H202, mad(Dxy, u * ww, Dyz * (uu * w)));
    const V H122 = mad(u, H022, mad(Dxy, v * ww, Dxz * (vv * w)));
    const V H222 = mad(ww, H220, uv * mad(Azz, uv, (mad(Dxz, vw, Dyz * uw)) * 2.f));
    // scaled coefficients T[a][b][c]
    const V rho = m.rho;
    const V s2 = rho * (HS / 72.f), s1 = rho * (HS / 24.f), s0 = rho * (HS / 8.f);
    V T[3][3][3];
    if constexpr (FOUT) T[0][0][0] = m.rho * (1.f / 216.f);
    else T[0][0][0] = m.r * (1.f / 216.f);
    T[1][0][0] = (u + dpdx) * s2;
    T[0][1][0] = v * s2;
    T[0][0][1] = w * s2;
    T[2][0][0] = R2[0][0] * s2;
    T[0][2][0] = R2[1][1] * s2;
    T[0][0][2] = R2[2][2] * s2;
    T[1][1][0] = R2[0][1] * s1;
    T[1][0][1] = R2[0][2] * s1;
    T[0][1][1] = R2[1][2] * s1;
    T[2][1][0] = H210 * s1;
    T[2][0][1] = H201 * s1;
    T[1][2][0] = H120 * s1;
    T[0][2][1] = H021 * s1;
    T[1][0][2] = H102 * s1;
    T[0][1][2] = H012 * s1;
    T[2][2][0] = H220 * s1;
    T[2][0][2] = H202 * s1;
    T[0][2][2] = H022 * s1;
    T[1][1][1] = H111 * s0;
    T[2][1][1] = H211 * s0;
    T[1][2][1] = H121 * s0;
    T[1][1][2] = H112 * s0;
    T[2][2][1] = H221 * s0;
    T[2][1][2] = H212 * s0;
    T[1][2][2] = H122 * s0;
    T[2][2][2] = H222 * s0;
    // the three 1-D passes; index 0 / 1 / 2 of a finished axis is c = 0 / +1 / -1
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const V e = T[0][b][c] + T[2][b][c];
            const V p0 = mad(T[0][b][c], 4.f, T[2][b][c] * (-2.f));
            const V p1 = e + T[1][b][c];
            T[2][b][c] = e - T[1][b][c];
            T[1][b][c] = p1;
            T[0][b][c] = p0;
        }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const V e = T[a][0][c] + T[a][2][c];
            const V p0 = mad(T[a][0][c], 4.f, T[a][2][c] * (-2.f));
            const V p1 = e + T[a][1][c];
            T[a][2][c] = e - T[a][1][c];
            T[a][1][c] = p1;
            T[a][0][c] = p0;
        }
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) {
            const V e = T[a][b][0] + T[a][b][2];
            const V p0 = mad(T[a][b][0], 4.f, T[a][b][2] * (-2.f));
            const V p1 = e + T[a][b][1];
            T[a][b][2] = e - T[a][b][1];
            T[a][b][1] = p1;
            T[a][b][0] = p0;
        }
#pragma unroll
    for (int q = 0; q < 27; q++) {
        const int cx = lat_c(27, q, 0), cy = lat_c(27, q, 1), cz = lat_c(27, q, 2);
        f[q] = T[cx < 0 ? 2 : cx][cy < 0 ? 2 : cy][cz < 0 ? 2 : cz];
    }
}

// D3Q27 recursive regularised collision on the tensor Hermite basis; U without the half-force shift.
__device__ __forceinline__ void rr27_closure(float (&f)[27], float rho, const float (&U)[3], float we, float dpdx,
                                             const float (&N2)[3][3], const float (&R2)[3][3]);

__device__ __forceinline__ void collide_rr27(float (&f)[27], float rho, const float (&U)[3], float we, float omega_b,
                                             float dpdx)
{
    float N2[3][3], R2[3][3];
    rr_second_order<27>(f, rho, U, we, omega_b, N2, R2);
    rr27_closure(f, rho, U, we, dpdx, N2, R2);
}

// D3Q27 moments from the 13 opposite pairs (q, q + 1 for odd q): rho, j = sum c f and
// S[a][b] = sum c_a c_b f (all components)
struct Mom27 {
    float rho;
    float j[3];
    float s[3][3];
};

__device__ __forceinline__ Mom27 moments27(const float (&f)[27])
{
    float a[14], d[14];
#pragma unroll
    for (int p = 1; p < 14; p++) {
        a[p] = f[2 * p - 1] + f[2 * p];
        d[p] = f[2 * p - 1] - f[2 * p];
    }
    Mom27 m;
    float r = f[0];
#pragma unroll
    for (int p = 1; p < 14; p++) r += a[p];
    m.rho = r;
#pragma unroll
    for (int x = 0; x < 3; x++) {
        float jx = 0.f;
#pragma unroll
        for (int p = 1; p < 14; p++) {
            const int c = lat_c(27, 2 * p - 1, x);
            if (c > 0) jx += d[p];
            else if (c < 0) jx -= d[p];
        }
        m.j[x] = jx;
#pragma unroll
        for (int y = x; y < 3; y++) {
            float sxy = 0.f;
#pragma unroll
            for (int p = 1; p < 14; p++) {
                const int cc = lat_c(27, 2 * p - 1, x) * lat_c(27, 2 * p - 1, y);
                if (cc > 0) sxy += a[p];
                else if (cc < 0) sxy -= a[p];
            }
            m.s[x][y] = m.s[y][x] = sxy;
        }
    }
    return m;
}

// Pi_neq : Pi_neq of smagorinskyTauSGS from the raw second moments: sum_q c_a c_b feq_q =
// rho delta_ab / 3 + u_a u_b for the reference's second-order equilibrium (fourth-order isotropy
// of the velocity set)
__device__ __forceinline__ float smag_pp_raw(const float (&S)[3][3], float rho, float u, float v, float w)
{
    const float r3 = rho * (1.f / 3.f);
    const float pxx = S[0][0] - r3 - u * u, pyy = S[1][1] - r3 - v * v, pzz = S[2][2] - r3 - w * w;
    const float pxy = S[0][1] - u * v, pxz = S[0][2] - u * w, pyz = S[1][2] - v * w;
    return pxx * pxx + pyy * pyy + pzz * pzz + 2.f * (pxy * pxy + pxz * pxz + pyz * pyz);
}

// collide_rr27 with the second moments already summed (moments27)
__device__ __forceinline__ void collide_rr27m(float (&f)[27], const Mom27& m, const float (&U)[3], float we,
                                              float omega_b, float dpdx)
{
    float M2[3][3];
    const float r3 = m.rho * (1.f / 3.f);
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) M2[a][b] = (a == b) ? m.s[a][a] - r3 : m.s[a][b];
    float N2[3][3], R2[3][3];
    rr_second_from(M2, m.rho, U, we, omega_b, N2, R2);
    rr27_closure(f, m.rho, U, we, dpdx, N2, R2);
}

// everything of the D3Q27 recursive regularised collision after the second-order moments
__device__ __forceinline__ void rr27_closure(float (&f)[27], float rho, const float (&U)[3], float we, float dpdx,
                                             const float (&N2)[3][3], const float (&R2)[3][3])
{
    const float third = 1.f / 3.f, k1 = 1.f - we;
    float H[3][3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int n = a + b + c;
                if (n == 0) {
                    H[a][b][c] = 1.f;
                } else if (n == 1) {
                    H[a][b][c] = a ? U[0] : b ? U[1] : U[2];
                } else if (n == 2) {
                    const int p = a ? 0 : 1, r = c ? 2 : (b ? 1 : 0);
                    const int pp = (a == 2) ? 0 : (b == 2) ? 1 : (c == 2) ? 2 : p;
                    const int rr = (a == 2) ? 0 : (b == 2) ? 1 : (c == 2) ? 2 : r;
                    H[a][b][c] = R2[pp][rr];
                } else {
                    const float eq = ipow(U[0], a) * ipow(U[1], b) * ipow(U[2], c);
                    float neq = 0.f;
                    if (a == 2) neq += N2[0][0] * ipow(U[1], b) * ipow(U[2], c);
                    if (b == 2) neq += N2[1][1] * ipow(U[0], a) * ipow(U[2], c);
                    if (c == 2) neq += N2[2][2] * ipow(U[0], a) * ipow(U[1], b);
                    if (a && b) neq += (float)(a * b) * N2[0][1] * ipow(U[0], a - 1) * ipow(U[1], b - 1) * ipow(U[2], c);
                    if (a && c) neq += (float)(a * c) * N2[0][2] * ipow(U[0], a - 1) * ipow(U[1], b) * ipow(U[2], c - 1);
                    if (b && c) neq += (float)(b * c) * N2[1][2] * ipow(U[0], a) * ipow(U[1], b - 1) * ipow(U[2], c - 1);
                    H[a][b][c] = eq + k1 * neq;
                }
            }
    float M[3][3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                float s = 0.f;
#pragma unroll
                for (int ta = 0; ta < 2; ta++)
#pragma unroll
                    for (int tb = 0; tb < 2; tb++)
#pragma unroll
                        for (int tc = 0; tc < 2; tc++) {
                            if ((ta && a != 2) || (tb && b != 2) || (tc && c != 2)) continue;
                            const float coef = (ta ? third : 1.f) * (tb ? third : 1.f) * (tc ? third : 1.f);
                            s += coef * H[ta ? 0 : a][tb ? 0 : b][tc ? 0 : c];
                        }
                M[a][b][c] = rho * s;
            }
    moments_to_pop27(M, 0.f, 0.f, 0.f, f);
    const float src = rho * 3.f * dpdx;
#pragma unroll
    for (int q = 0; q < 27; q++)
        if (lat_c(27, q, 0) != 0) f[q] += lat_w(27, q) * (float)lat_c(27, q, 0) * src;
}

// Cumulant collision (D3Q27_opencl/kernel.cl:2352-2691); u is the velocity including the half-force shift.
__device__ __forceinline__ void collide_cumulant(float (&f)[27], float rho, float u, float v, float w, float we,
                                                 float omega_b, float clim)
{
    float K[3][3][3];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++)
#pragma unroll
            for (int c = 0; c < 3; c++) K[a][b][c] = 0.f;
#pragma unroll
    for (int q = 0; q < 27; q++) {
        const float dx = (float)lat_c(27, q, 0) - u, dy = (float)lat_c(27, q, 1) - v, dz = (float)lat_c(27, q, 2) - w;
        const float px[3] = {1.f, dx, dx * dx}, py[3] = {1.f, dy, dy * dy}, pz[3] = {1.f, dz, dz * dz};
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++)
#pragma unroll
                for (int c = 0; c < 3; c++)
                    if (a + b + c > 0) K[a][b][c] += px[a] * py[b] * pz[c] * f[q];
    }
    K[0][0][0] = rho;
    const float ir = 1.f / rho;
    const float C200 = K[2][0][0], C020 = K[0][2][0], C002 = K[0][0][2];
    const float C110 = K[1][1][0], C101 = K[1][0][1], C011 = K[0][1][1];
    const float C210 = K[2][1][0], C201 = K[2][0][1], C021 = K[0][2][1], C120 = K[1][2][0], C102 = K[1][0][2],
                C012 = K[0][1][2], C111 = K[1][1][1];
    // the fourth-order cumulants C211..C022, the fifth-order C122..C221 and C222 relax to their
    // equilibrium with rate 1 (omega6..omega10 = 1, D3Q27 kernel.cl:2474-2478), so they are not formed

    const float w1 = we, w2 = omega_b;
    const float w3 = 8.f * (w1 - 2.f) * (w2 * (3.f * w1 - 1.f) - 5.f * w1) /
                     (8.f * (5.f - 2.f * w1) * w1 + w2 * (8.f + w1 * (9.f * w1 - 26.f)));
    const float w4 = 8.f * (w1 - 2.f) * (w1 + w2 * (3.f * w1 - 7.f)) / (w2 * (56.f - 42.f * w1 + 9.f * w1 * w1) - 8.f * w1);
    const float w5 = 24.f * (w1 - 2.f) * (4.f * w1 * w1 + w1 * w2 * (18.f - 13.f * w1) + w2 * w2 * (2.f + w1 * (6.f * w1 - 11.f))) /
                     (16.f * w1 * w1 * (w1 - 6.f) - 2.f * w1 * w2 * (216.f + 5.f * w1 * (9.f * w1 - 46.f)) +
                      w2 * w2 * (w1 * (3.f * w1 - 10.f) * (15.f * w1 - 28.f) - 48.f));
    auto lim = [&](float wr, float x) {
        const float ax = fabsf(x);
        return ax > 0.f ? wr + (1.f - wr) * ax / (ax + clim * rho) : 1.f;
    };
    const float w3a = lim(w3, C120 + C102), w3b = lim(w3, C210 + C012), w3c = lim(w3, C201 + C021);
    const float w4a = lim(w4, C120 - C102), w4b = lim(w4, C210 - C012), w4c = lim(w4, C201 - C021);
    const float w5l = lim(w5, C111);
    float A = (4.f * w1 * w1 + 2.f * w1 * w2 * (w1 - 6.f) + w2 * w2 * (w1 * (10.f - 3.f * w1) - 4.f)) /
              ((w1 - w2) * (w2 * (2.f + 3.f * w1) - 8.f * w1));
    float B = (4.f * w1 * w2 * (9.f * w1 - 16.f) - 4.f * w1 * w1 - 2.f * w2 * w2 * (2.f + 9.f * w1 * (w1 - 2.f))) /
              (3.f * (w1 - w2) * (w2 * (2.f + 3.f * w1) - 8.f * w1));
    A = fmaxf(A, 0.f);
    B = fmaxf(B, 0.f);

    const float K000 = rho;
    const float Dxu = -0.5f * (w1 * (2.f * C200 - C020 - C002) + w2 * (C200 + C020 + C002 - K000)) * ir;
    const float Dyv = Dxu + 1.5f * w1 * (C200 - C020) * ir;
    const float Dzw = Dxu + 1.5f * w1 * (C200 - C002) * ir;
    const float Dxv = -3.f * w1 * C110 * ir, Dxw = -3.f * w1 * C101 * ir, Dyw = -3.f * w1 * C011 * ir;
    float X1 = (1.f - w1) * (C200 - C020) - 3.f * rho * (1.f - 0.5f * w1) * (u * u * Dxu - v * v * Dyv);
    float X2 = (1.f - w1) * (C200 - C002) - 3.f * rho * (1.f - 0.5f * w1) * (u * u * Dxu - w * w * Dzw);
    float X3 = K000 * w2 + (1.f - w2) * (C200 + C020 + C002) - 3.f * rho * (1.f - 0.5f * w2) * (u * u * Dxu + v * v * Dyv + w * w * Dzw);
    float M[3][3][3];
    M[0][0][0] = K000;
    M[1][0][0] = -K[1][0][0];
    M[0][1][0] = -K[0][1][0];
    M[0][0][1] = -K[0][0][1];
    M[2][0][0] = (X1 + X2 + X3) * (1.f / 3.f);
    M[0][2][0] = M[2][0][0] - X1;
    M[0][0][2] = M[2][0][0] - X2;
    M[1][1][0] = (1.f - w1) * C110;
    M[1][0][1] = (1.f - w1) * C101;
    M[0][1][1] = (1.f - w1) * C011;
    X1 = (1.f - w3a) * (C120 + C102);
    X2 = (1.f - w4a) * (C120 - C102);
    M[1][2][0] = 0.5f * (X1 + X2);
    M[1][0][2] = 0.5f * (X1 - X2);
    X1 = (1.f - w3b) * (C210 + C012);
    X2 = (1.f - w4b) * (C210 - C012);
    M[2][1][0] = 0.5f * (X1 + X2);
    M[0][1][2] = 0.5f * (X1 - X2);
    X1 = (1.f - w3c) * (C201 + C021);
    X2 = (1.f - w4c) * (C201 - C021);
    M[2][0][1] = 0.5f * (X1 + X2);
    M[0][2][1] = 0.5f * (X1 - X2);
    M[1][1][1] = (1.f - w5l) * C111;
    const float tw = 1.f / w1 - 0.5f;
    // omega6..omega10 = 1 (kernel.cl:2474-2478): the fourth- to sixth-order cumulants relax to equilibrium
    X1 = 2.f * tw * A * rho * (Dxu - 2.f * Dyv + Dzw) * (1.f / 3.f);
    X2 = 2.f * tw * A * rho * (Dxu + Dyv - 2.f * Dzw) * (1.f / 3.f);
    X3 = -4.f * tw * A * rho * (Dxu + Dyv + Dzw) * (1.f / 3.f);
    const float Cs220 = (X1 + X2 + X3) * (1.f / 3.f), Cs202 = -(X1 - X3) * (1.f / 3.f), Cs022 = -(X2 - X3) * (1.f / 3.f);
    const float Cs211 = -tw * B * rho * Dyw * (1.f / 3.f);
    const float Cs121 = -tw * B * rho * Dxw * (1.f / 3.f);
    const float Cs112 = -tw * B * rho * Dxv * (1.f / 3.f);
    M[2][1][1] = Cs211 + (M[2][0][0] * M[0][1][1] + 2.f * M[1][1][0] * M[1][0][1]) * ir;
    M[1][2][1] = Cs121 + (M[0][2][0] * M[1][0][1] + 2.f * M[0][1][1] * M[1][1][0]) * ir;
    M[1][1][2] = Cs112 + (M[0][0][2] * M[1][1][0] + 2.f * M[1][0][1] * M[0][1][1]) * ir;
    M[2][2][0] = Cs220 + (M[2][0][0] * M[0][2][0] + 2.f * M[1][1][0] * M[1][1][0]) * ir;
    M[2][0][2] = Cs202 + (M[0][0][2] * M[2][0][0] + 2.f * M[1][0][1] * M[1][0][1]) * ir;
    M[0][2][2] = Cs022 + (M[0][2][0] * M[0][0][2] + 2.f * M[0][1][1] * M[0][1][1]) * ir;
    M[1][2][2] = (M[0][2][2] * M[1][2][0] + M[0][2][0] * M[1][0][2] + 4.f * M[0][1][1] * M[1][1][1] +
                  2.f * (M[1][0][1] * M[0][2][1] + M[1][1][0] * M[0][1][2])) * ir;
    M[2][1][2] = (M[2][0][2] * M[0][1][2] + M[0][0][2] * M[2][1][0] + 4.f * M[1][0][1] * M[1][1][1] +
                  2.f * (M[1][1][0] * M[1][0][2] + M[0][1][1] * M[2][0][1])) * ir;
    M[2][2][1] = (M[2][2][0] * M[2][0][1] + M[2][0][0] * M[0][2][1] + 4.f * M[1][1][0] * M[1][1][1] +
                  2.f * (M[0][1][1] * M[2][1][0] + M[1][0][1] * M[1][2][0])) * ir;
    M[2][2][2] = (4.f * M[1][1][1] * M[1][1][1] + M[2][0][0] * M[0][2][2] + M[0][2][0] * M[2][0][2] + M[0][0][2] * M[2][2][0] +
                  4.f * (M[0][1][1] * M[2][1][1] + M[1][0][1] * M[1][2][1] + M[1][1][0] * M[1][1][2]) +
                  2.f * (M[1][2][0] * M[1][0][2] + M[2][1][0] * M[0][1][2] + M[2][0][1] * M[0][2][1])) * ir -
                 (16.f * M[1][1][0] * M[1][0][1] * M[0][1][1] +
                  4.f * (M[1][0][1] * M[1][0][1] * M[0][2][0] + M[0][1][1] * M[0][1][1] * M[2][0][0] + M[1][1][0] * M[1][1][0] * M[0][0][2]) +
                  2.f * M[2][0][0] * M[0][2][0] * M[0][0][2]) * ir * ir;
    moments_to_pop27(M, u, v, w, f);
}

}  // namespace lbffs

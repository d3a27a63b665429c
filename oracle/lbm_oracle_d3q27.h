/*
 * Test infrastructure only.  D3Q27 collision operators of the CPU oracle
 * (included by lbm_oracle.c).
 *
 * collide_cumulant27: the parametrised cumulant operator of Geier et al.,
 *   Comput. Math. Appl. 70 (2015), as the reference runs it
 *   (D3Q27_opencl/kernel.cl:2352-2691): central moments about the local
 *   velocity, cumulants up to sixth order, relaxation rates omega3-5 and the
 *   A/B fourth-order corrections of the paper, the clim limiter on the third
 *   order, and the chimera back-transform x -> y -> z.  The reference's
 *   back-conversion of the fifth-order cumulants uses Ks022, Ks202, Ks220 in
 *   the first products of Ks122, Ks212, Ks221 (kernel.cl:2575-2577) where the
 *   forward conversion uses K002, K200, K020; that is reproduced.
 *
 * collide_rr27: recursive-regularised collision on the full D3Q27 tensor
 *   Hermite basis (Malaspinas 2015; Coreixas et al. 2017).  The reference has
 *   no D3Q27 RR operator; this is the FP64-checkable definition the CUDA
 *   kernel is held to.  Non-equilibrium Hermite coefficients of order >= 3
 *   follow the recursion a_neq(S) = sum over index pairs {p,q} of S of
 *   N2[s_p][s_q] * prod_{r != p,q} u_{s_r}, which reduces to the D3Q19
 *   operator's third/fourth-order terms; all orders >= 3 relax with omega_eff,
 *   second order with the same bulk/shear split as D3Q19.
 */

/* 1-D backward chimera step: central moments (k0,k1,k2) about velocity u -> populations at c=-1,0,+1 */
static inline void chimera_back(real k0, real k1, real k2, real u, real* fm, real* f0, real* fp)
{
    *f0 = k0 * ((real)1 - u * u) - (real)2 * u * k1 - k2;
    *fm = (real)0.5 * (k0 * (u * u - u) + k1 * ((real)2 * u - (real)1) + k2);
    *fp = (real)0.5 * (k0 * (u * u + u) + k1 * ((real)2 * u + (real)1) + k2);
}

/* populations from central moments M[a][b][c] (orders along x,y,z) about (u,v,w) */
static void moments_to_pop27(const lat* L, real M[3][3][3], real u, real v, real w, real* out)
{
    real Px[3][3][3]; /* [sx][b][c], sx index 0:-1 1:0 2:+1 */
    for (int b = 0; b < 3; b++)
        for (int c = 0; c < 3; c++) chimera_back(M[0][b][c], M[1][b][c], M[2][b][c], u, &Px[0][b][c], &Px[1][b][c], &Px[2][b][c]);
    real Py[3][3][3];
    for (int s = 0; s < 3; s++)
        for (int c = 0; c < 3; c++) chimera_back(Px[s][0][c], Px[s][1][c], Px[s][2][c], v, &Py[s][0][c], &Py[s][1][c], &Py[s][2][c]);
    real P[3][3][3];
    for (int s = 0; s < 3; s++)
        for (int t = 0; t < 3; t++) chimera_back(Py[s][t][0], Py[s][t][1], Py[s][t][2], w, &P[s][t][0], &P[s][t][1], &P[s][t][2]);
    for (int q = 0; q < L->Q; q++) out[q] = P[L->c[q][0] + 1][L->c[q][1] + 1][L->c[q][2] + 1];
}

void collide_cumulant27(const ctx* X, real* out, const real* ft, real rho, real u, real v, real w, real tau,
                        real tau_sgs)
{
    const lat* L = &X->L;
    const real clim = X->p->clim;
    real K[3][3][3];
    memset(K, 0, sizeof(K));
    for (int q = 0; q < L->Q; q++) {
        real d[3] = {(real)L->c[q][0] - u, (real)L->c[q][1] - v, (real)L->c[q][2] - w};
        real px[3] = {1, d[0], d[0] * d[0]}, py[3] = {1, d[1], d[1] * d[1]}, pz[3] = {1, d[2], d[2] * d[2]};
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                for (int c = 0; c < 3; c++)
                    if (a + b + c > 0) K[a][b][c] += px[a] * py[b] * pz[c] * ft[q];
    }
    K[0][0][0] = rho;
    const real ir = (real)1 / rho;
#define Kx(a, b, c) K[a][b][c]
    /* cumulants (central moments up to third order are cumulants) */
    const real C200 = Kx(2, 0, 0), C020 = Kx(0, 2, 0), C002 = Kx(0, 0, 2);
    const real C110 = Kx(1, 1, 0), C101 = Kx(1, 0, 1), C011 = Kx(0, 1, 1);
    const real C210 = Kx(2, 1, 0), C201 = Kx(2, 0, 1), C021 = Kx(0, 2, 1), C120 = Kx(1, 2, 0), C102 = Kx(1, 0, 2),
               C012 = Kx(0, 1, 2), C111 = Kx(1, 1, 1);
    const real C211 = Kx(2, 1, 1) - (Kx(2, 0, 0) * Kx(0, 1, 1) + (real)2 * Kx(1, 1, 0) * Kx(1, 0, 1)) * ir;
    const real C121 = Kx(1, 2, 1) - (Kx(0, 2, 0) * Kx(1, 0, 1) + (real)2 * Kx(1, 1, 0) * Kx(0, 1, 1)) * ir;
    const real C112 = Kx(1, 1, 2) - (Kx(0, 0, 2) * Kx(1, 1, 0) + (real)2 * Kx(1, 0, 1) * Kx(0, 1, 1)) * ir;
    const real C220 = Kx(2, 2, 0) - (Kx(2, 0, 0) * Kx(0, 2, 0) + (real)2 * Kx(1, 1, 0) * Kx(1, 1, 0)) * ir;
    const real C202 = Kx(2, 0, 2) - (Kx(0, 0, 2) * Kx(2, 0, 0) + (real)2 * Kx(1, 0, 1) * Kx(1, 0, 1)) * ir;
    const real C022 = Kx(0, 2, 2) - (Kx(0, 2, 0) * Kx(0, 0, 2) + (real)2 * Kx(0, 1, 1) * Kx(0, 1, 1)) * ir;
    const real C122 = Kx(1, 2, 2) - (Kx(0, 0, 2) * Kx(1, 2, 0) + Kx(0, 2, 0) * Kx(1, 0, 2) + (real)4 * Kx(0, 1, 1) * Kx(1, 1, 1) +
                                     (real)2 * (Kx(1, 0, 1) * Kx(0, 2, 1) + Kx(1, 1, 0) * Kx(0, 1, 2))) * ir;
    const real C212 = Kx(2, 1, 2) - (Kx(2, 0, 0) * Kx(0, 1, 2) + Kx(0, 0, 2) * Kx(2, 1, 0) + (real)4 * Kx(1, 0, 1) * Kx(1, 1, 1) +
                                     (real)2 * (Kx(1, 1, 0) * Kx(1, 0, 2) + Kx(0, 1, 1) * Kx(2, 0, 1))) * ir;
    const real C221 = Kx(2, 2, 1) - (Kx(0, 2, 0) * Kx(2, 0, 1) + Kx(2, 0, 0) * Kx(0, 2, 1) + (real)4 * Kx(1, 1, 0) * Kx(1, 1, 1) +
                                     (real)2 * (Kx(0, 1, 1) * Kx(2, 1, 0) + Kx(1, 0, 1) * Kx(1, 2, 0))) * ir;
    const real C222 =
        Kx(2, 2, 2) -
        ((real)4 * Kx(1, 1, 1) * Kx(1, 1, 1) + Kx(2, 0, 0) * Kx(0, 2, 2) + Kx(0, 2, 0) * Kx(2, 0, 2) + Kx(0, 0, 2) * Kx(2, 2, 0) +
         (real)4 * (Kx(0, 1, 1) * Kx(2, 1, 1) + Kx(1, 0, 1) * Kx(1, 2, 1) + Kx(1, 1, 0) * Kx(1, 1, 2)) +
         (real)2 * (Kx(1, 2, 0) * Kx(1, 0, 2) + Kx(2, 1, 0) * Kx(0, 1, 2) + Kx(2, 0, 1) * Kx(0, 2, 1))) * ir +
        ((real)16 * Kx(1, 1, 0) * Kx(1, 0, 1) * Kx(0, 1, 1) +
         (real)4 * (Kx(1, 0, 1) * Kx(1, 0, 1) * Kx(0, 2, 0) + Kx(0, 1, 1) * Kx(0, 1, 1) * Kx(2, 0, 0) + Kx(1, 1, 0) * Kx(1, 1, 0) * Kx(0, 0, 2)) +
         (real)2 * Kx(2, 0, 0) * Kx(0, 2, 0) * Kx(0, 0, 2)) * ir * ir;

    /* relaxation rates (Geier et al. 2015, eqs. for omega3-5, A, B) */
    const real w1 = (real)1 / (tau + tau_sgs), w2 = X->p->omegaB;
    const real w3 = (real)8 * (w1 - (real)2) * (w2 * ((real)3 * w1 - (real)1) - (real)5 * w1) /
                    ((real)8 * ((real)5 - (real)2 * w1) * w1 + w2 * ((real)8 + w1 * ((real)9 * w1 - (real)26)));
    const real w4 = (real)8 * (w1 - (real)2) * (w1 + w2 * ((real)3 * w1 - (real)7)) /
                    (w2 * ((real)56 - (real)42 * w1 + (real)9 * w1 * w1) - (real)8 * w1);
    const real w5 = (real)24 * (w1 - (real)2) *
                    ((real)4 * w1 * w1 + w1 * w2 * ((real)18 - (real)13 * w1) + w2 * w2 * ((real)2 + w1 * ((real)6 * w1 - (real)11))) /
                    ((real)16 * w1 * w1 * (w1 - (real)6) - (real)2 * w1 * w2 * ((real)216 + (real)5 * w1 * ((real)9 * w1 - (real)46)) +
                     w2 * w2 * (w1 * ((real)3 * w1 - (real)10) * ((real)15 * w1 - (real)28) - (real)48));
#define LIM(wr, x) ((real)fabs((double)(x)) > 0 ? (wr) + ((real)1 - (wr)) * (real)fabs((double)(x)) / ((real)fabs((double)(x)) + clim * rho) : (real)1)
    const real w3a = LIM(w3, C120 + C102), w3b = LIM(w3, C210 + C012), w3c = LIM(w3, C201 + C021);
    const real w4a = LIM(w4, C120 - C102), w4b = LIM(w4, C210 - C012), w4c = LIM(w4, C201 - C021);
    const real w5l = LIM(w5, C111);
#undef LIM
    const real w6 = 1, w7 = 1, w8 = 1, w9 = 1, w10 = 1;
    real A = ((real)4 * w1 * w1 + (real)2 * w1 * w2 * (w1 - (real)6) + w2 * w2 * (w1 * ((real)10 - (real)3 * w1) - (real)4)) /
             ((w1 - w2) * (w2 * ((real)2 + (real)3 * w1) - (real)8 * w1));
    real B = ((real)4 * w1 * w2 * ((real)9 * w1 - (real)16) - (real)4 * w1 * w1 - (real)2 * w2 * w2 * ((real)2 + (real)9 * w1 * (w1 - (real)2))) /
             ((real)3 * (w1 - w2) * (w2 * ((real)2 + (real)3 * w1) - (real)8 * w1));
    A = (A > 0) ? A : 0; /* fmax semantics: NaN -> 0 */
    B = (B > 0) ? B : 0;

    const real K000 = K[0][0][0];
    const real Cs110 = ((real)1 - w1) * C110, Cs101 = ((real)1 - w1) * C101, Cs011 = ((real)1 - w1) * C011;
    const real Dxu = -(real)0.5 * (w1 * ((real)2 * C200 - C020 - C002) + w2 * (C200 + C020 + C002 - K000)) * ir;
    const real Dyv = Dxu + (real)1.5 * w1 * (C200 - C020) * ir;
    const real Dzw = Dxu + (real)1.5 * w1 * (C200 - C002) * ir;
    const real Dxv = -(real)3 * w1 * C110 * ir, Dxw = -(real)3 * w1 * C101 * ir, Dyw = -(real)3 * w1 * C011 * ir;
    real X1 = ((real)1 - w1) * (C200 - C020) - (real)3 * rho * ((real)1 - (real)0.5 * w1) * (u * u * Dxu - v * v * Dyv);
    real X2 = ((real)1 - w1) * (C200 - C002) - (real)3 * rho * ((real)1 - (real)0.5 * w1) * (u * u * Dxu - w * w * Dzw);
    real X3 = K000 * w2 + ((real)1 - w2) * (C200 + C020 + C002) -
              (real)3 * rho * ((real)1 - (real)0.5 * w2) * (u * u * Dxu + v * v * Dyv + w * w * Dzw);
    const real Cs200 = (X1 + X2 + X3) / (real)3, Cs020 = Cs200 - X1, Cs002 = Cs200 - X2;
    X1 = ((real)1 - w3a) * (C120 + C102);
    X2 = ((real)1 - w4a) * (C120 - C102);
    const real Cs120 = (real)0.5 * (X1 + X2), Cs102 = (real)0.5 * (X1 - X2);
    X1 = ((real)1 - w3b) * (C210 + C012);
    X2 = ((real)1 - w4b) * (C210 - C012);
    const real Cs210 = (real)0.5 * (X1 + X2), Cs012 = (real)0.5 * (X1 - X2);
    X1 = ((real)1 - w3c) * (C201 + C021);
    X2 = ((real)1 - w4c) * (C201 - C021);
    const real Cs201 = (real)0.5 * (X1 + X2), Cs021 = (real)0.5 * (X1 - X2);
    const real Cs111 = ((real)1 - w5l) * C111;
    const real tw = (real)1 / w1 - (real)0.5;
    X1 = ((real)1 - w6) * (C220 - (real)2 * C202 + C022) + (real)2 * tw * w6 * A * rho * (Dxu - (real)2 * Dyv + Dzw) / (real)3;
    X2 = ((real)1 - w6) * (C220 + C202 - (real)2 * C022) + (real)2 * tw * w6 * A * rho * (Dxu + Dyv - (real)2 * Dzw) / (real)3;
    X3 = ((real)1 - w7) * (C220 + C202 + C022) - (real)4 * tw * w7 * A * rho * (Dxu + Dyv + Dzw) / (real)3;
    const real Cs220 = (X1 + X2 + X3) / (real)3, Cs202 = -(X1 - X3) / (real)3, Cs022 = -(X2 - X3) / (real)3;
    const real Cs211 = ((real)1 - w8) * C211 - tw * w8 * B * rho * Dyw / (real)3;
    const real Cs121 = ((real)1 - w8) * C121 - tw * w8 * B * rho * Dxw / (real)3;
    const real Cs112 = ((real)1 - w8) * C112 - tw * w8 * B * rho * Dxv / (real)3;
    const real Cs221 = ((real)1 - w9) * C221, Cs212 = ((real)1 - w9) * C212, Cs122 = ((real)1 - w9) * C122;
    const real Cs222 = ((real)1 - w10) * C222;

    /* post-collision central moments */
    real M[3][3][3];
    M[0][0][0] = K000;
    M[1][0][0] = -K[1][0][0];
    M[0][1][0] = -K[0][1][0];
    M[0][0][1] = -K[0][0][1];
    M[2][0][0] = Cs200; M[0][2][0] = Cs020; M[0][0][2] = Cs002;
    M[1][1][0] = Cs110; M[1][0][1] = Cs101; M[0][1][1] = Cs011; M[1][1][1] = Cs111;
    M[2][1][0] = Cs210; M[2][0][1] = Cs201; M[0][2][1] = Cs021; M[1][2][0] = Cs120; M[1][0][2] = Cs102; M[0][1][2] = Cs012;
    M[2][1][1] = Cs211 + (M[2][0][0] * M[0][1][1] + (real)2 * M[1][1][0] * M[1][0][1]) * ir;
    M[1][2][1] = Cs121 + (M[0][2][0] * M[1][0][1] + (real)2 * M[0][1][1] * M[1][1][0]) * ir;
    M[1][1][2] = Cs112 + (M[0][0][2] * M[1][1][0] + (real)2 * M[1][0][1] * M[0][1][1]) * ir;
    M[2][2][0] = Cs220 + (M[2][0][0] * M[0][2][0] + (real)2 * M[1][1][0] * M[1][1][0]) * ir;
    M[2][0][2] = Cs202 + (M[0][0][2] * M[2][0][0] + (real)2 * M[1][0][1] * M[1][0][1]) * ir;
    M[0][2][2] = Cs022 + (M[0][2][0] * M[0][0][2] + (real)2 * M[0][1][1] * M[0][1][1]) * ir;
    M[1][2][2] = Cs122 + (M[0][2][2] * M[1][2][0] + M[0][2][0] * M[1][0][2] + (real)4 * M[0][1][1] * M[1][1][1] +
                          (real)2 * (M[1][0][1] * M[0][2][1] + M[1][1][0] * M[0][1][2])) * ir;
    M[2][1][2] = Cs212 + (M[2][0][2] * M[0][1][2] + M[0][0][2] * M[2][1][0] + (real)4 * M[1][0][1] * M[1][1][1] +
                          (real)2 * (M[1][1][0] * M[1][0][2] + M[0][1][1] * M[2][0][1])) * ir;
    M[2][2][1] = Cs221 + (M[2][2][0] * M[2][0][1] + M[2][0][0] * M[0][2][1] + (real)4 * M[1][1][0] * M[1][1][1] +
                          (real)2 * (M[0][1][1] * M[2][1][0] + M[1][0][1] * M[1][2][0])) * ir;
    M[2][2][2] = Cs222 +
                 ((real)4 * M[1][1][1] * M[1][1][1] + M[2][0][0] * M[0][2][2] + M[0][2][0] * M[2][0][2] + M[0][0][2] * M[2][2][0] +
                  (real)4 * (M[0][1][1] * M[2][1][1] + M[1][0][1] * M[1][2][1] + M[1][1][0] * M[1][1][2]) +
                  (real)2 * (M[1][2][0] * M[1][0][2] + M[2][1][0] * M[0][1][2] + M[2][0][1] * M[0][2][1])) * ir -
                 ((real)16 * M[1][1][0] * M[1][0][1] * M[0][1][1] +
                  (real)4 * (M[1][0][1] * M[1][0][1] * M[0][2][0] + M[0][1][1] * M[0][1][1] * M[2][0][0] + M[1][1][0] * M[1][1][0] * M[0][0][2]) +
                  (real)2 * M[2][0][0] * M[0][2][0] * M[0][0][2]) * ir * ir;
#undef Kx
    moments_to_pop27(L, M, u, v, w, out);
}

/* Hermite coefficient of the multiset S (axis indices, length n <= 6), non-equilibrium part, from the
 * second-order non-equilibrium tensor N2 by the recursive-regularisation closure. */
static real rr_neq(const int* S, int n, real N2[3][3], const real* U)
{
    real s = 0;
    for (int p = 0; p < n; p++)
        for (int q = p + 1; q < n; q++) {
            real t = N2[S[p]][S[q]];
            for (int r = 0; r < n; r++)
                if (r != p && r != q) t *= U[S[r]];
            s += t;
        }
    return s;
}

void collide_rr27(const ctx* X, real* out, const real* ft, real rho, real u, real v, real w, real tau, real tau_sgs)
{
    const lat* L = &X->L;
    const real third = (real)1 / (real)3;
    const real we = (real)1 / (tau + tau_sgs);
    const real U[3] = {u, v, w};
    /* second-order Hermite coefficients / rho */
    real M2[3][3] = {{0}};
    for (int q = 0; q < L->Q; q++)
        for (int a = 0; a < 3; a++)
            for (int b = a; b < 3; b++) M2[a][b] += ((real)(L->c[q][a] * L->c[q][b]) - (a == b ? third : (real)0)) * ft[q];
    const real ir = (real)1 / rho;
    real N2[3][3], R2[3][3];
    for (int a = 0; a < 3; a++)
        for (int b = a; b < 3; b++) {
            M2[a][b] *= ir;
            N2[a][b] = N2[b][a] = M2[a][b] - U[a] * U[b];
        }
    const real wm = (X->p->omegaB - we) / (real)3, wp = wm + we;
    for (int a = 0; a < 3; a++) {
        R2[a][a] = M2[a][a];
        for (int b = 0; b < 3; b++) R2[a][a] -= (a == b ? wp : wm) * N2[b][b];
        for (int b = a + 1; b < 3; b++) R2[a][b] = R2[b][a] = M2[a][b] - we * N2[a][b];
    }
    /* post-collision Hermite coefficients H[nx][ny][nz] (per rho) */
    real H[3][3][3];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++)
            for (int c = 0; c < 3; c++) {
                const int ord[3] = {a, b, c};
                int S[6], n = 0;
                real eq = 1;
                for (int ax = 0; ax < 3; ax++)
                    for (int r = 0; r < ord[ax]; r++) {
                        S[n++] = ax;
                        eq *= U[ax];
                    }
                if (n == 0) H[a][b][c] = 1;
                else if (n == 1) H[a][b][c] = U[S[0]];
                else if (n == 2) H[a][b][c] = R2[S[0]][S[1]];
                else H[a][b][c] = eq + ((real)1 - we) * rr_neq(S, n, N2, U);
            }
    /* raw moments: an axis of order 2 carries c^2 = H2 + 1/3 */
    real Mr[3][3][3];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++)
            for (int c = 0; c < 3; c++) {
                real s = 0;
                for (int ta = 0; ta <= (a == 2); ta++)
                    for (int tb = 0; tb <= (b == 2); tb++)
                        for (int tc = 0; tc <= (c == 2); tc++) {
                            real coef = 1;
                            if (ta) coef *= third;
                            if (tb) coef *= third;
                            if (tc) coef *= third;
                            s += coef * H[ta ? 0 : a][tb ? 0 : b][tc ? 0 : c];
                        }
                Mr[a][b][c] = rho * s;
            }
    moments_to_pop27(L, Mr, (real)0, (real)0, (real)0, out);
    for (int q = 0; q < L->Q; q++) out[q] += rho * L->w[q] * (real)3 * (real)L->c[q][0] * X->p->dpdx;
}

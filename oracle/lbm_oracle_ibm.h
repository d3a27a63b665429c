/*
 * Test infrastructure only.  Immersed-boundary sub-step of the CPU oracle
 * (included by lbm_oracle.c): the intended mathematics of the reference's
 * k_Gwall / k_Gibm / k_Force (D3Q19_opencl/kernel.cl:3648-3806,
 * ns.cpp:542-601) -- direct forcing with trilinear interpolation and the
 * same trilinear spreading, markers advanced after spreading.
 *
 * Deliberate differences from the reference text, each a reference defect:
 *  - the spread accumulates (kernel.cl:3760-3762 store the pre-add value);
 *  - the rotation projection uses OX.e0 (kernel.cl:1213/1256 use OX_x*e0_z
 *    for the z term); identical to the reference when the rotation rate is 0;
 *  - k_Force reads the u8 solid flags (kernel.cl:3784 types them float);
 *  - a marker on the rotation axis gets zero rotation velocity instead of NaN.
 * Added motion (no reference counterpart): a sinusoidal displacement
 * A*sin(2*pi*t/T) on top of the constant translation; the per-step target
 * velocity is the per-step displacement, so positions follow the sine exactly.
 *
 * The oracle accumulates the spread in double whatever REAL is, matching the
 * FP64 Lagrangian accumulation of the CUDA path.
 */

typedef struct or_motion {
    real ampX, ampY, ampZ, period; /* sinusoidal displacement; period <= 0 disables it */
    long step;                     /* step counter t, advanced by the oracle */
} or_motion;

static void rot_frame(const or_ibm* m, real X, real Y, real Z, real* OOp, real* e1, real* e2, real* r)
{
    const real e0[3] = {m->axX, m->axY, m->axZ};
    const real OX[3] = {X - m->rotX, Y - m->rotY, Z - m->rotZ};
    const real d = OX[0] * e0[0] + OX[1] * e0[1] + OX[2] * e0[2];
    real OpX[3];
    for (int a = 0; a < 3; a++) {
        OOp[a] = d * e0[a];
        OpX[a] = OX[a] - OOp[a];
    }
    const real mag = (real)sqrt((double)(OpX[0] * OpX[0] + OpX[1] * OpX[1] + OpX[2] * OpX[2]));
    *r = mag;
    if (mag == 0) {
        e1[0] = e1[1] = e1[2] = e2[0] = e2[1] = e2[2] = 0;
        return;
    }
    for (int a = 0; a < 3; a++) e1[a] = OpX[a] / mag;
    e2[0] = e0[1] * e1[2] - e0[2] * e1[1];
    e2[1] = e0[2] * e1[0] - e0[0] * e1[2];
    e2[2] = e0[0] * e1[1] - e0[1] * e1[0];
}

/* trilinear box of marker (x,y,z): the cell (int)x,(int)y,(int)z and its +1 neighbours inside the domain
 * (icBox, kernel.cl:1112-1155). Returns the number of cells written to cells[]/wts[]. */
static int ibm_box(const ctx* X, real x, real y, real z, long* cells, real* wts)
{
    const int i = (int)x, j = (int)y, k = (int)z;
    if (!(i >= 0 && i < X->N[0] && j >= 0 && j < X->N[1] && k >= 0 && k < X->N[2])) return 0;
    int n = 0;
    for (int dk = 0; dk <= 1; dk++)
        for (int dj = 0; dj <= 1; dj++)
            for (int di = 0; di <= 1; di++) {
                int ii = i + di, jj = j + dj, kk = k + dk;
                if (ii >= X->N[0] || jj >= X->N[1] || kk >= X->N[2]) continue;
                cells[n] = idx(X, ii, jj, kk);
                wts[n] = ((real)1 - (real)fabs((double)((real)ii - x))) * ((real)1 - (real)fabs((double)((real)jj - y))) *
                         ((real)1 - (real)fabs((double)((real)kk - z)));
                n++;
            }
    return n;
}

static or_motion* g_motion; /* set by oracle_step_motion for the duration of one call */

static void ibm_substep(const ctx* X, const or_ibm* m)
{
    or_fields* A = X->a;
    const long E = X->E;
    const lat* L = &X->L;
    real d[3] = {0, 0, 0};
    if (g_motion && g_motion->period > 0) {
        const double T = (double)g_motion->period, t = (double)g_motion->step;
        const double s = sin(2.0 * M_PI * (t + 1.0) / T) - sin(2.0 * M_PI * t / T);
        d[0] = (real)((double)g_motion->ampX * s);
        d[1] = (real)((double)g_motion->ampY * s);
        d[2] = (real)((double)g_motion->ampZ * s);
    }
    const real uT[3] = {m->uT + d[0], m->vT + d[1], m->wT + d[2]};
    double* G = (double*)calloc((size_t)(3 * E), sizeof(double));
    for (int n = 0; n < m->n; n++) {
        real* P = m->markers + 3 * n;
        real OOp[3], e1[3], e2[3], r;
        rot_frame(m, P[0], P[1], P[2], OOp, e1, e2, &r);
        real ut[3];
        for (int a = 0; a < 3; a++) ut[a] = uT[a] + r * m->rotOmega * e2[a];
        long cells[8];
        real wts[8];
        int nb = ibm_box(X, P[0], P[1], P[2], cells, wts);
        real ui[3] = {0, 0, 0};
        for (int b = 0; b < nb; b++) {
            ui[0] += A->u[cells[b]] * wts[b];
            ui[1] += A->v[cells[b]] * wts[b];
            ui[2] += A->w[cells[b]] * wts[b];
        }
        m->Gmx[n] = ut[0] - ui[0];
        m->Gmy[n] = ut[1] - ui[1];
        m->Gmz[n] = ut[2] - ui[2];
    }
    for (int n = 0; n < m->n; n++) {
        real* P = m->markers + 3 * n;
        long cells[8];
        real wts[8];
        int nb = ibm_box(X, P[0], P[1], P[2], cells, wts);
        for (int b = 0; b < nb; b++) {
            G[cells[b]] += (double)(m->Gmx[n] * wts[b]);
            G[E + cells[b]] += (double)(m->Gmy[n] * wts[b]);
            G[2 * E + cells[b]] += (double)(m->Gmz[n] * wts[b]);
        }
        for (int a = 0; a < 3; a++) P[a] += uT[a];
        real OOp[3], e1[3], e2[3], r;
        rot_frame(m, P[0], P[1], P[2], OOp, e1, e2, &r);
        if (r > 0) {
            const real c = (real)cos((double)m->rotOmega), s = (real)sin((double)m->rotOmega);
            const real rc[3] = {m->rotX, m->rotY, m->rotZ};
            for (int a = 0; a < 3; a++) P[a] = rc[a] + OOp[a] + r * (c * e1[a] + s * e2[a]);
        }
    }
    for (long ic = 0; ic < E; ic++) {
        A->Gx[ic] = (real)G[ic];
        A->Gy[ic] = (real)G[E + ic];
        A->Gz[ic] = (real)G[2 * E + ic];
        if (A->solid[ic] != 0) continue;
        const real g[3] = {A->Gx[ic], A->Gy[ic], A->Gz[ic]};
        if (g[0] == 0 && g[1] == 0 && g[2] == 0) continue;
        for (int q = 0; q < L->Q; q++) {
            real gc = g[0] * (real)L->c[q][0] + g[1] * (real)L->c[q][1] + g[2] * (real)L->c[q][2];
            A->fTmp[(long)q * E + ic] += A->rho[ic] * L->w[q] * (real)3 * gc;
        }
    }
    free(G);
    if (g_motion) g_motion->step++;
}

int oracle_step(const or_config* cfg, or_fields* a, const or_params* p, const or_ibm* ibm, int nsteps);

/* oracle_step with the sinusoidal marker motion; motion->step is advanced per step. */
int oracle_step_motion(const or_config* cfg, or_fields* a, const or_params* p, const or_ibm* ibm, or_motion* motion,
                       int nsteps)
{
    g_motion = motion;
    int rc = oracle_step(cfg, a, p, ibm, nsteps);
    g_motion = 0;
    return rc;
}

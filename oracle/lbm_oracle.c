/*
 * Test infrastructure only -- never linked into the product library.
 *
 * CPU restatement of the LBFFS lattice-Boltzmann step (one
 * k_streamingCollision launch + handle swap, D3Q19_opencl/ns.cpp:509-603),
 * written from the reference's algorithm, not from its text.  It is the
 * checker for the CUDA path: GPU results are compared with it at small sizes.
 *
 * Built twice: REAL=float (the reference's FP32 arithmetic) and REAL=double
 * (the FP64 oracle the storage-precision error budgets are stated against).
 *
 * Semantics pinned by the tests against the reference compiled from source:
 *  - neighbour reads of rho/u/v/w see the previous step (the reference reads
 *    them while other work-items overwrite them, D3Q19 kernel.cl:3518-3522);
 *  - an upwind index of -1 (domain wall) never forms an STL link;
 *  - cells with boundary==0 wrap periodically (the reference assumes every
 *    domain-face cell has boundary==1, ns.cpp:164-177).
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#ifndef REAL
#define REAL float
#endif
typedef REAL real;

/* ---- lattices (D3Q19 kernel.cl:3555-3560, D3Q27 kernel.cl:2742-2747) ---- */
static const int C19[19][3] = {{0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},   {0, -1, 0}, {0, 0, 1},  {0, 0, -1},
                               {1, 1, 0},  {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0},  {1, 0, 1},  {-1, 0, -1}, {1, 0, -1},
                               {-1, 0, 1}, {0, 1, 1},  {0, -1, -1}, {0, 1, -1}, {0, -1, 1}};
static const int C27[27][3] = {{0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 1, 0},   {0, -1, 0}, {0, 0, 1},  {0, 0, -1},
                               {1, 1, 0},   {-1, -1, 0}, {1, -1, 0},  {-1, 1, 0},  {1, 0, 1},  {-1, 0, -1}, {1, 0, -1},
                               {-1, 0, 1},  {0, 1, 1},   {0, -1, -1}, {0, 1, -1},  {0, -1, 1}, {1, 1, 1},  {-1, -1, -1},
                               {-1, 1, 1},  {1, -1, -1}, {1, -1, 1},  {-1, 1, -1}, {1, 1, -1}, {-1, -1, 1}};

enum { BC_CYCLIC = 0, BC_BB = 1, BC_OUTLET = 3, BC_SYM = 4, BC_FIXVEL = 5, BC_FIXDEN = 6, BC_WALLFN = 7 };
enum { SGS_SMAG = 0, SGS_WALE = 1 };
enum { WALL_BB = 0, WALL_IBB = 1 };
enum { COLL_RR = 0, COLL_CUMULANT = 1 };

/* Same memory layout as ref_driver.c's structs so one Python wrapper drives both. */
typedef struct or_fields {
    real *f, *fTmp;
    int *boundary, *boundary1, *boundary2, *boundary3;
    real* sdf;
    unsigned char *solid, *neiSolid;
    real *u0, *v0, *w0;
    real *Fwx, *Fwy, *Fwz;
    real *tauSGS, *rho, *u, *v, *w, *omega;
    real *Gx, *Gy, *Gz;
    real *rhoPrev, *uPrev, *vPrev, *wPrev;
} or_fields;

typedef struct or_params {
    int nx, ny, nz;
    real dpdx, rho_av, LES;
    int isReadMovingWalls;
    real omegaB, spzWidth, clim;
    int nthreads;
} or_params;

typedef struct or_ibm {
    real *markers, *Gmx, *Gmy, *Gmz;
    int n;
    real uT, vT, wT, rotX, rotY, rotZ, axX, axY, axZ, rotOmega;
} or_ibm;

typedef struct or_config {
    int q;         /* 19 or 27 */
    int sgs;       /* SGS_SMAG (honours LES) or SGS_WALE (as shipped, ignores LES) */
    int wall;      /* WALL_BB or WALL_IBB */
    int collision; /* COLL_RR or COLL_CUMULANT */
    real cs;       /* Smagorinsky constant */
    int damping;   /* DAMP_WALL (the reference's live factor), DAMP_VAN_DRIEST or DAMP_NONE */
} or_config;

enum { DAMP_WALL = 0, DAMP_VAN_DRIEST = 1, DAMP_NONE = 2 };

typedef struct lat {
    int Q;
    int c[27][3];
    real w[27];
    int opp[27];
} lat;

static void make_lat(lat* L, int Q)
{
    L->Q = Q;
    for (int q = 0; q < Q; q++) {
        const int* cq = (Q == 19) ? C19[q] : C27[q];
        int n2 = 0;
        for (int a = 0; a < 3; a++) {
            L->c[q][a] = cq[a];
            n2 += cq[a] * cq[a];
        }
        double w;
        if (Q == 19) w = n2 == 0 ? 1.0 / 3.0 : n2 == 1 ? 1.0 / 18.0 : 1.0 / 36.0;
        else w = n2 == 0 ? 8.0 / 27.0 : n2 == 1 ? 2.0 / 27.0 : n2 == 2 ? 1.0 / 54.0 : 1.0 / 216.0;
        L->w[q] = (real)w;
    }
    for (int q = 0; q < Q; q++)
        for (int p = 0; p < Q; p++)
            if (L->c[p][0] == -L->c[q][0] && L->c[p][1] == -L->c[q][1] && L->c[p][2] == -L->c[q][2]) L->opp[q] = p;
}

static int find_q(const lat* L, int x, int y, int z)
{
    for (int q = 0; q < L->Q; q++)
        if (L->c[q][0] == x && L->c[q][1] == y && L->c[q][2] == z) return q;
    return -1;
}

typedef struct ctx {
    const or_config* cfg;
    const or_params* p;
    or_fields* a;
    lat L;
    long E;
    int N[3];
    int sponge[6]; /* face-centre cell of x-/x+/y-/y+/z-/z+ is Outlet or FixedDensity (kernel.cl:2447-2501) */
} ctx;

static inline long idx(const ctx* X, int i, int j, int k) { return ((long)k * X->N[1] + j) * X->N[0] + i; }
static inline int is_wall_code(int b) { return b == 1 || b == 4 || b == 5 || b == 6 || b == 7; }

/* upwindID_B (D3Q19 kernel.cl:328-575, D3Q27 kernel.cl:530-549): per-axis periodic wrap unless the
 * face code of that axis is a wall, in which case the link is missing (-1). */
static long upwind_face(const ctx* X, int q, const int x[3], const int b[3])
{
    int n[3];
    for (int a = 0; a < 3; a++) {
        n[a] = x[a] - X->L.c[q][a];
        if (n[a] == -1) {
            if (is_wall_code(b[a])) return -1;
            n[a] = X->N[a] - 1;
        } else if (n[a] == X->N[a]) {
            if (is_wall_code(b[a])) return -1;
            n[a] = 0;
        }
    }
    return idx(X, n[0], n[1], n[2]);
}

/* interior pull (streamingInternal / streaming2D): periodic wrap in every axis. */
static long upwind_wrap(const ctx* X, int q, const int x[3])
{
    int n[3];
    for (int a = 0; a < 3; a++) {
        n[a] = x[a] - X->L.c[q][a];
        if (n[a] < 0) n[a] += X->N[a];
        if (n[a] >= X->N[a]) n[a] -= X->N[a];
    }
    return idx(X, n[0], n[1], n[2]);
}

/* Direction whose own-cell population replaces a missing link on a domain face:
 * D3Q19 reflectOrMirrorQ (kernel.cl:114-326) -- first Symmetry axis among the direction's
 * nonzero axes (x before y before z) mirrors that component, otherwise full reflection;
 * D3Q27 (kernel.cl:1133-1146 with mirrorQx/y/z 187-527) -- the last Symmetry axis (z over y over x)
 * wins; it mirrors that component when the direction has one, otherwise reflects. */
static int missing_dir(const ctx* X, int q, const int b[3])
{
    const lat* L = &X->L;
    int r = L->opp[q];
    if (L->Q == 19) {
        int nz_axes = 0;
        for (int a = 0; a < 3; a++) nz_axes += L->c[q][a] != 0;
        if (nz_axes < 2) return r;
        for (int a = 0; a < 3; a++) {
            if (L->c[q][a] != 0 && b[a] == BC_SYM) {
                int m[3] = {L->c[q][0], L->c[q][1], L->c[q][2]};
                m[a] = -m[a];
                return find_q(L, m[0], m[1], m[2]);
            }
        }
        return r;
    }
    int out = r;
    for (int a = 0; a < 3; a++) {
        if (b[a] == BC_SYM) {
            if (L->c[q][a] != 0) {
                int m[3] = {L->c[q][0], L->c[q][1], L->c[q][2]};
                m[a] = -m[a];
                out = find_q(L, m[0], m[1], m[2]);
            } else {
                out = r;
            }
        }
    }
    return out;
}

/* cornerFlag (D3Q19 kernel.cl:1346-1397) */
static int corner_flag(const ctx* X, int b3, const int x[3])
{
    int on[3];
    for (int a = 0; a < 3; a++) on[a] = (x[a] == 0 || x[a] == X->N[a] - 1);
    if (X->N[2] - 1 == 0 || b3 == 0) return on[0] && on[1];
    return (on[0] + on[1] + on[2]) >= 2;
}

/* fixedVelocityBC (D3Q19 kernel.cl:1399-1512, D3Q27 kernel.cl:1243-1384): Ladd moving-wall correction
 * ft_q += 6 w_q rho_w (c_q . u_w) on the incoming directions, with the wall density from the known
 * populations (or the inner cell's previous density for inflow-reversed walls).  D3Q27 applies four
 * times the corner weight on the z-max face (kernel.cl:1372-1375); that is kept. */
static void fixed_velocity(const ctx* X, real* ft, const real uw[3], const int b[3], long ic, const int x[3])
{
    const lat* L = &X->L;
    for (int a = 0; a < 3; a++) {
        if (b[a] != BC_FIXVEL) continue;
        int side;
        if (x[a] == 0) side = -1;
        else if (x[a] == X->N[a] - 1) side = +1;
        else continue;
        real tang = 0, out = 0;
        for (int q = 0; q < L->Q; q++) {
            if (L->c[q][a] == 0) tang += ft[q];
            else if (L->c[q][a] == side) out += ft[q];
        }
        real rhow = (tang + (real)2 * out) / ((real)1 + (real)side * uw[a]);
        if ((side < 0 && uw[a] < 0) || (side > 0 && uw[a] > 0)) {
            long inner;
            if (side > 0 && a == 0) {
                inner = ic; /* the reference reads its own cell here (kernel.cl:1425-1429) */
            } else {
                int y[3] = {x[0], x[1], x[2]};
                y[a] = side < 0 ? 1 : X->N[a] - 2;
                inner = idx(X, y[0], y[1], y[2]);
            }
            rhow = X->a->rhoPrev[inner];
        }
        for (int q = 0; q < L->Q; q++) {
            if (L->c[q][a] != -side) continue;
            int n2 = L->c[q][0] * L->c[q][0] + L->c[q][1] * L->c[q][1] + L->c[q][2] * L->c[q][2];
            real mult = (L->Q == 27 && a == 2 && side > 0 && n2 == 3) ? (real)4 : (real)1;
            real cu = (real)L->c[q][0] * uw[0] + (real)L->c[q][1] * uw[1] + (real)L->c[q][2] * uw[2];
            ft[q] += mult * (real)6 * L->w[q] * rhow * cu;
        }
    }
}

/* fixedDensityBC (D3Q19 kernel.cl:1514-1611, D3Q27 kernel.cl:1385-1486): anti-bounce-back with
 * rho_w = 1 and the wall velocity extrapolated from the own and inner cells' previous velocity. */
static void fixed_density(const ctx* X, real* ft, const int b[3], long ic, const int x[3])
{
    const lat* L = &X->L;
    const or_fields* A = X->a;
    for (int a = 0; a < 3; a++) {
        if (b[a] != BC_FIXDEN) continue;
        int y[3] = {x[0], x[1], x[2]};
        y[a] = (x[a] == 0) ? 1 : X->N[a] - 2;
        long in = idx(X, y[0], y[1], y[2]);
        real uw[3] = {A->uPrev[ic] + (real)0.5 * (A->uPrev[ic] - A->uPrev[in]),
                      A->vPrev[ic] + (real)0.5 * (A->vPrev[ic] - A->vPrev[in]),
                      A->wPrev[ic] + (real)0.5 * (A->wPrev[ic] - A->wPrev[in])};
        real usq = uw[0] * uw[0] + uw[1] * uw[1] + uw[2] * uw[2];
        for (int side = -1; side <= 1; side += 2) {
            if (!((side < 0 && x[a] == 0) || (side > 0 && x[a] == X->N[a] - 1))) continue;
            for (int q = 0; q < L->Q; q++) {
                if (L->c[q][a] != -side) continue;
                real cu = (real)L->c[q][0] * uw[0] + (real)L->c[q][1] * uw[1] + (real)L->c[q][2] * uw[2];
                ft[q] = -ft[q] + (real)2 * L->w[q] * (real)1 * ((real)1 + (real)4.5 * cu * cu - (real)1.5 * usq);
            }
        }
    }
}

/* calcTauw (D3Q19 kernel.cl:1621-1655, D3Q27 kernel.cl:1487-1522): Newton iterations on
 * Spalding's law for the friction velocity 1.5 cells from the wall.  The reference's loop updates a
 * y+ declared inside the loop body, so its convergence test always compares with the first y+. */
static real calc_tauw(real rhow, real magUp, real nu)
{
    const real y = (real)1.5, kappa = (real)0.42, Ek = (real)9.1;
    real ut = sqrt(nu * magUp);
    const real yPlus = y * ut / nu;
    int iter = 0;
    real err;
    do {
        real kUu = fmin(kappa * magUp / ut, (real)50);
        real fkUu = exp(kUu) - (real)1 - kUu * ((real)1 + (real)0.5 * kUu);
        real func = -ut * y / nu + magUp / ut + (fkUu - kUu * kUu * kUu / (real)6) / Ek;
        real dfunc = y / nu + magUp / (ut * ut) + (kUu * fkUu / ut) / Ek;
        ut = ut + func / dfunc;
        err = fabs(yPlus - y * ut / nu);
    } while (err > (real)0.005 && ++iter < 100);
    ut = fmax(ut, (real)0);
    return rhow * ut * ut;
}

/* wallFunctionBC (D3Q19 kernel.cl:1657-1924, D3Q27 kernel.cl:1524-): on a face with code 7 the
 * populations entering from the wall get a moving-wall correction whose tangential velocity is
 * -3 (tau_w e_t - Fw_t) / rho_w, tau_w from the previous-step tangential speed one cell inward and
 * e_t the direction of the cell's own previous-step tangential velocity.  Fw is the momentum the
 * face's bounce-back exchanged in this step's streaming (streaming(), D3Q19 kernel.cl:1281-1312,
 * writes it before internalWallBC resets the field).  Per axis the low face takes precedence
 * (if / else if); the z-max face probes k - 1 (the reference reads k + 1, outside the grid); the
 * z-min face does not test the own speed for zero, as in the reference. */
static void wall_function(const ctx* X, real* ft, const int b[3], long ic, const int x[3], real omega,
                          const real fw[3])
{
    const lat* L = &X->L;
    const or_fields* A = X->a;
    const real nu = ((real)1 / omega - (real)0.5) / (real)3;
    const real uo[3] = {A->uPrev[ic], A->vPrev[ic], A->wPrev[ic]};
    for (int a = 0; a < 3; a++) {
        if (b[a] != BC_WALLFN) continue;
        int side;
        if (x[a] == 0) side = -1;
        else if (x[a] == X->N[a] - 1) side = 1;
        else continue;
        const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
        real tang = 0, outg = 0;
        for (int q = 0; q < L->Q; q++) {
            if (L->c[q][a] == 0) tang += ft[q];
            else if (L->c[q][a] == side) outg += ft[q];
        }
        const real rhow = tang + (real)2 * outg;
        int y[3] = {x[0], x[1], x[2]};
        if (!(a == 2 && X->N[2] == 1)) y[a] = side < 0 ? (X->N[a] > 1 ? 1 : 0) : (X->N[a] > 1 ? X->N[a] - 2 : 0);
        const long pr = idx(X, y[0], y[1], y[2]);
        const real up[3] = {A->uPrev[pr], A->vPrev[pr], A->wPrev[pr]};
        real mag = sqrt(up[t1] * up[t1] + up[t2] * up[t2]);
        real tw[3] = {0, 0, 0};
        if (mag != (real)0) {
            const real tauw = calc_tauw(rhow, mag, nu);
            mag = sqrt(uo[t1] * uo[t1] + uo[t2] * uo[t2]);
            if (mag != (real)0 || (a == 2 && side < 0)) {
                tw[t1] = (real)-3 * (tauw * (uo[t1] / mag) - fw[t1]) / rhow;
                tw[t2] = (real)-3 * (tauw * (uo[t2] / mag) - fw[t2]) / rhow;
            }
        }
        const int n = -side;
        for (int q = 1; q < L->Q; q++) {
            const int nz = (L->c[q][0] != 0) + (L->c[q][1] != 0) + (L->c[q][2] != 0);
            if (L->c[q][a] != n || nz == 1) continue;
            real sum = 0;
            if (L->c[q][t1]) sum += (real)(L->c[q][t1] * n) * tw[t1];
            if (L->c[q][t2]) sum += (real)(L->c[q][t2] * n) * tw[t2];
            const real den = nz == 2 ? (L->Q == 19 ? (real)6 : (real)9) : (real)36;
            ft[q] += (real)n * (rhow * sum) / den;
        }
    }
}

/* outflowBC (Geier et al. 2015 App. F; D3Q19 kernel.cl:2005-2097, D3Q27 kernel.cl:1900-1991):
 * incoming populations blend the inner and own previous post-collision values with the own
 * previous velocity component of that axis.  Later faces overwrite earlier ones. */
static void outflow(const ctx* X, real* ft, const real* f, const real uo[3], const int b[3], long ic,
                    const int x[3])
{
    const lat* L = &X->L;
    if (!(b[0] == BC_OUTLET || b[1] == BC_OUTLET || b[2] == BC_OUTLET)) return;
    const real cs = (real)(1.0 / sqrt(3.0));
    for (int a = 0; a < 3; a++) {
        if (b[a] != BC_OUTLET) continue;
        for (int side = -1; side <= 1; side += 2) {
            if (!((side < 0 && x[a] == 0) || (side > 0 && x[a] == X->N[a] - 1))) continue;
            int y[3] = {x[0], x[1], x[2]};
            y[a] = side < 0 ? 1 : X->N[a] - 2;
            long in = idx(X, y[0], y[1], y[2]);
            real g = cs - uo[a];
            for (int q = 1; q < L->Q; q++) {
                if (L->c[q][a] != -side) continue;
                ft[q] = g * f[(long)q * X->E + in] + ((real)1 - g) * f[(long)q * X->E + ic];
            }
        }
    }
}

/* internalWallBC: simple bounce-back (D3Q19 kernel.cl:1926-2003) or Filippova-Hanel with the
 * Mei-Luo-Shyy variant for q_f <= 1/2 (D3Q27 kernel.cl:1823-1897).  Returns the link force. */
static void internal_wall(const ctx* X, real* ft, const real* f, const long* up, long ic, real omega,
                          real tau_sgs_prev, real Fw[3])
{
    const lat* L = &X->L;
    const or_fields* A = X->a;
    Fw[0] = Fw[1] = Fw[2] = 0;
    if (A->neiSolid[ic] != 1) return;
    const real u = A->uPrev[ic], v = A->vPrev[ic], w = A->wPrev[ic], rho = A->rhoPrev[ic];
    for (int q = 1; q < L->Q; q++) {
        if (up[q] < 0 || A->solid[up[q]] != 1) continue;
        int qb = L->opp[q];
        real fb = f[(long)qb * X->E + ic];
        if (X->cfg->wall == WALL_BB) {
            ft[q] = fb;
        } else {
            real sdf0 = A->sdf[ic], sdf1 = A->sdf[up[q]];
            real qf = (real)fabs((double)sdf0) / ((real)fabs((double)sdf0) + (real)fabs((double)sdf1));
            real tau = (real)1 / omega;
            real we = (real)1 / (tau + tau_sgs_prev);
            real usq = u * u + v * v + w * w;
            real uc = -u * (real)L->c[q][0] - v * (real)L->c[q][1] - w * (real)L->c[q][2];
            real feq, chi;
            if (qf <= (real)0.5) {
                long fl = up[qb];
                real ufc = -A->uPrev[fl] * (real)L->c[q][0] - A->vPrev[fl] * (real)L->c[q][1] -
                           A->wPrev[fl] * (real)L->c[q][2];
                feq = (rho + (real)3 * ufc + (real)4.5 * uc * uc - (real)1.5 * usq) * L->w[q];
                chi = we * ((real)2 * qf - (real)1) / ((real)1 - (real)2 * we);
            } else {
                feq = (rho + (real)3 * ((real)1 - (real)1 / qf) * uc + (real)4.5 * uc * uc - (real)1.5 * usq) * L->w[q];
                chi = we * ((real)2 * qf - (real)1);
            }
            ft[q] = ((real)1 - chi) * fb + chi * feq;
        }
        for (int a = 0; a < 3; a++) Fw[a] += -(fb + ft[q]) * (real)L->c[q][a];
    }
}

/* Van Driest damped mixing length kappa * y * (1 - exp(-y+ / A+)) of the block the reference keeps
 * commented out in smagorinskyTauSGS (D3Q19 kernel.cl:2178-2197, D3Q27 kernel.cl:2072-2091): y+ from
 * the log law u+ = ln(E y+) / kappa with the cell's own speed |u| at wall distance y, by the
 * reference's fixed-point iteration y+ <- (kappa |u| y / nu + y+) / (1 + ln(E y+)) from y+ = 1, at
 * most 10 iterations, stopping when y+ changes by at most 0.001; kappa 0.41, A+ 26, E 9.8.  The
 * eddy viscosity is scaled by min(1, length / Cs)^2; this returns length / Cs. */
static real van_driest_ratio(real y, real umag, real nu, real cs)
{
    const real kappa = (real)0.41, Aplus = (real)26, Ek = (real)9.8;
    real yp = 1, ypn;
    int it = 0;
    do {
        ypn = yp;
        yp = (kappa * umag * y / nu + yp) / ((real)1 + (real)log((double)(Ek * yp)));
        it++;
    } while ((real)fabs((double)(yp - ypn)) > (real)0.001 && it < 10);
    return (kappa / cs) * (((real)1 + (real)1e-10) - (real)exp((double)(-yp / Aplus))) * y;
}

/* smagorinskyTauSGS (D3Q19 kernel.cl:2133-2201): eddy relaxation time from |Pi_neq| with the
 * min(1, kappa y / Cs)^2 near-wall damping (y = sdf when one is set), or the Van Driest damping
 * above, or none. */
static real smagorinsky(const ctx* X, const real* ft, real rho, real u, real v, real w, real omega, real sdf)
{
    const lat* L = &X->L;
    real tau = (real)1 / omega;
    real P[3][3] = {{0}};
    real usq = u * u + v * v + w * w;
    for (int q = 0; q < L->Q; q++) {
        real cu = u * (real)L->c[q][0] + v * (real)L->c[q][1] + w * (real)L->c[q][2];
        real feq = (rho + (real)3 * cu + (real)4.5 * cu * cu - (real)1.5 * usq) * L->w[q];
        real d = ft[q] - feq;
        for (int a = 0; a < 3; a++)
            for (int b = a; b < 3; b++) P[a][b] += (real)(L->c[q][a] * L->c[q][b]) * d;
    }
    real pp = P[0][0] * P[0][0] + P[1][1] * P[1][1] + P[2][2] * P[2][2] +
              (real)2 * (P[0][1] * P[0][1] + P[0][2] * P[0][2] + P[1][2] * P[1][2]);
    real spp = (real)sqrt((double)pp);
    real cs = X->cfg->cs;
    real t = X->p->LES * (real)0.5 *
             (-tau + (real)sqrt((double)(tau * tau + (real)18 * (real)sqrt(2.0) * cs * cs * spp / rho)));
    if (sdf != (real)10000 && sdf > 0 && X->cfg->damping != DAMP_NONE) {
        real d;
        if (X->cfg->damping == DAMP_VAN_DRIEST) {
            d = van_driest_ratio(sdf, (real)sqrt((double)usq), (tau - (real)0.5) / (real)3, cs);
        } else {
            d = (real)0.41 * sdf / cs;
        }
        if (d > 1) d = 1;
        t *= d * d;
    }
    return t;
}

/* waleTauSGS (D3Q19 kernel.cl:2267-2365) with central differences (one-sided on the faces; the
 * k == 0 one-sided z difference is identically zero in the reference and stays so). */
static real wale(const ctx* X, int i, int j, int k, long ic)
{
    const or_fields* A = X->a;
    const int nx = X->N[0], ny = X->N[1], nz = X->N[2];
    const real* cur[3] = {A->u, A->v, A->w};
    const real* prev[3] = {A->uPrev, A->vPrev, A->wPrev};
#define VAL(c, ii, jj, kk) ((idx(X, ii, jj, kk) == ic) ? cur[c][ic] : prev[c][idx(X, ii, jj, kk)])
    real g[3][3]; /* g[c][d] = d u_c / d x_d */
    for (int c = 0; c < 3; c++) {
        g[c][0] = (i > 0 && i < nx - 1) ? (real)0.5 * (VAL(c, i + 1, j, k) - VAL(c, i - 1, j, k))
                  : (i == 0)            ? VAL(c, 1, j, k) - VAL(c, 0, j, k)
                                        : VAL(c, nx - 1, j, k) - VAL(c, nx - 2, j, k);
        g[c][1] = (j > 0 && j < ny - 1) ? (real)0.5 * (VAL(c, i, j + 1, k) - VAL(c, i, j - 1, k))
                  : (j == 0)            ? VAL(c, i, 1, k) - VAL(c, i, 0, k)
                                        : VAL(c, i, ny - 1, k) - VAL(c, i, ny - 2, k);
        g[c][2] = (k > 0 && k < nz - 1) ? (real)0.5 * (VAL(c, i, j, k + 1) - VAL(c, i, j, k - 1))
                  : (nz - 1 == 0)       ? (real)0
                  : (k == 0)            ? (real)0
                                        : VAL(c, i, j, nz - 1) - VAL(c, i, j, nz - 2);
    }
#undef VAL
    real S[3][3], SS = 0, gg[3][3], tr = 0, SdSd = 0;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            S[a][b] = (real)0.5 * (g[a][b] + g[b][a]);
            SS += S[a][b] * S[a][b];
        }
    /* (grad u . grad u)_ab = sum_c du_c/dx_a du_b/dx_c  with the reference's index convention */
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            gg[a][b] = 0;
            for (int c = 0; c < 3; c++) gg[a][b] += g[c][a] * g[b][c];
        }
    for (int a = 0; a < 3; a++) tr += gg[a][a];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            real sd = (real)0.5 * (gg[a][b] + gg[b][a]) - (a == b ? tr / (real)3 : (real)0);
            SdSd += sd * sd;
        }
    const real cw = (real)0.325;
    if (SS > (real)1e-24 && SdSd > (real)1e-24)
        return (real)3 * (cw * cw * (real)pow((double)SdSd, 1.5) /
                          ((real)pow((double)SS, 2.5) + (real)pow((double)SdSd, 1.25))) * (real)3;
    return 0;
}

/* tauSpongeZone (D3Q19 kernel.cl:2444-2503) */
static real sponge(const ctx* X, real omega, real tau_sgs, int i, int j, int k)
{
    real tau = (real)1 / omega;
    const real sw = X->p->spzWidth;
    const int x[3] = {i, j, k};
    for (int a = 0; a < 3; a++) {
        real n = (real)X->N[a];
        if (X->sponge[2 * a] && (real)x[a] < n * sw) {
            real fx = (real)x[a] / (n * sw);
            tau = ((real)1 - fx) * ((real)1 - tau_sgs) + fx * tau;
        }
        if (X->sponge[2 * a + 1] && (real)x[a] > n * ((real)1 - sw)) {
            real fx = (real)(X->N[a] - x[a]) / (n * sw);
            tau = ((real)1 - fx) * ((real)1 - tau_sgs) + fx * tau;
        }
    }
    return tau;
}

/* collisionRecursiveRegularized (D3Q19 kernel.cl:3156-3309): regularised Hermite moments up to the
 * fourth order built recursively from the second-order non-equilibrium part, bulk/shear split of
 * the diagonal second-order moments, then the D3Q19 raw-moment inverse.  Written per axis / axis
 * pair: T3[a][b] is the c_a^2 c_b moment, Q4[a][b] the c_a^2 c_b^2 moment. */
static void collide_rr19(const ctx* X, real* out, const real* ft, real rho, real u0, real u1, real u2, real tau,
                         real tau_sgs)
{
    const lat* L = &X->L;
    const real third = (real)1 / (real)3, ninth = (real)1 / (real)9;
    const real we = (real)1 / (tau + tau_sgs);
    const real U[3] = {u0, u1, u2};
    real M2[3][3] = {{0}};
    for (int q = 0; q < L->Q; q++)
        for (int a = 0; a < 3; a++)
            for (int b = a; b < 3; b++) {
                real h = (real)(L->c[q][a] * L->c[q][b]) - (a == b ? third : (real)0);
                M2[a][b] += h * ft[q];
            }
    const real ir = (real)1 / rho;
    real N2[3][3], R2[3][3];
    for (int a = 0; a < 3; a++)
        for (int b = a; b < 3; b++) {
            M2[a][b] *= ir;
            N2[a][b] = M2[a][b] - U[a] * U[b];
            N2[b][a] = N2[a][b];
        }
    const real wm = (X->p->omegaB - we) / (real)3, wp = wm + we;
    for (int a = 0; a < 3; a++) {
        R2[a][a] = M2[a][a];
        for (int b = 0; b < 3; b++) R2[a][a] -= (a == b ? wp : wm) * N2[b][b];
        for (int b = a + 1; b < 3; b++) R2[a][b] = R2[b][a] = M2[a][b] - we * N2[a][b];
    }
    real RM2[3][3], T3[3][3], Q4[3][3];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            RM2[a][b] = R2[a][b] + (a == b ? third : (real)0);
            if (a == b) continue;
            real n3 = U[b] * N2[a][a] + (real)2 * U[a] * N2[a][b];
            T3[a][b] = U[a] * U[a] * U[b] + ((real)1 - we) * n3 + third * U[b];
            real n4 = U[b] * U[b] * N2[a][a] + U[a] * U[a] * N2[b][b] + (real)4 * U[a] * U[b] * N2[a][b];
            Q4[a][b] = U[a] * U[a] * U[b] * U[b] + ((real)1 - we) * n4 + third * (R2[a][a] + R2[b][b]) + ninth;
        }
    for (int q = 0; q < L->Q; q++) {
        const int* c = L->c[q];
        int n2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
        real val;
        if (n2 == 0) {
            val = rho * ((real)1 - RM2[0][0] - RM2[1][1] - RM2[2][2] + Q4[0][1] + Q4[0][2] + Q4[1][2]);
        } else if (n2 == 1) {
            int a = c[0] ? 0 : c[1] ? 1 : 2, b = (a + 1) % 3, d = (a + 2) % 3;
            real s = (real)(c[a]);
            val = (real)0.5 * rho * (s * U[a] + RM2[a][a] - s * T3[b][a] - s * T3[d][a] - Q4[a][b] - Q4[a][d]);
        } else {
            int a = c[0] ? 0 : 1, b = c[2] ? 2 : 1;
            real sa = (real)c[a], sb = (real)c[b];
            val = (real)0.25 * rho * (sa * sb * RM2[a][b] + sb * T3[a][b] + sa * T3[b][a] + Q4[a][b]);
        }
        out[q] = val + rho * L->w[q] * (real)3 * (real)c[0] * X->p->dpdx;
    }
}

void collide_cumulant27(const ctx* X, real* out, const real* ft, real rho, real u, real v, real w, real tau,
                        real tau_sgs);
void collide_rr27(const ctx* X, real* out, const real* ft, real rho, real u, real v, real w, real tau,
                  real tau_sgs);

static void cell_step(const ctx* X, long ic)
{
    or_fields* A = X->a;
    const lat* L = &X->L;
    const long E = X->E;
    if (A->solid[ic] != 0) return;
    const int i = (int)(ic % X->N[0]), j = (int)((ic / X->N[0]) % X->N[1]), k = (int)(ic / ((long)X->N[0] * X->N[1]));
    const int x[3] = {i, j, k};
    const int b[3] = {A->boundary1[ic], A->boundary2[ic], A->boundary3[ic]};
    const real uo[3] = {A->uPrev[ic], A->vPrev[ic], A->wPrev[ic]};
    const real uw[3] = {A->u0[ic], A->v0[ic], A->w0[ic]};
    const real omega = A->omega[ic];
    const real tsgs_prev = A->tauSGS[ic];
    const real* f = A->f;
    real ft[27];
    long up[27];
    ft[0] = f[ic];
    up[0] = ic;
    if (A->boundary[ic] == 1) {
        real fws[3] = {0, 0, 0};  /* bounce-back momentum of the face (streaming(), kernel.cl:1281-1312) */
        for (int q = 1; q < L->Q; q++) {
            up[q] = upwind_face(X, q, x, b);
            if (up[q] >= 0) {
                ft[q] = f[(long)q * E + up[q]];
            } else {
                ft[q] = f[(long)missing_dir(X, q, b) * E + ic];
                for (int a = 0; a < 3; a++) fws[a] += (real)-2 * ft[q] * (real)L->c[q][a];
            }
        }
        if (!corner_flag(X, b[2], x)) {
            fixed_velocity(X, ft, uw, b, ic, x);
            fixed_density(X, ft, b, ic, x);
            wall_function(X, ft, b, ic, x, omega, fws);
        }
        outflow(X, ft, f, uo, b, ic, x);
    } else {
        for (int q = 1; q < L->Q; q++) {
            up[q] = upwind_wrap(X, q, x);
            ft[q] = f[(long)q * E + up[q]];
        }
    }
    real Fw[3];
    internal_wall(X, ft, f, up, ic, omega, tsgs_prev, Fw);
    A->Fwx[ic] = Fw[0];
    A->Fwy[ic] = Fw[1];
    A->Fwz[ic] = Fw[2];

    real rho = 0, m[3] = {0, 0, 0};
    for (int q = 0; q < L->Q; q++) {
        rho += ft[q];
        for (int a = 0; a < 3; a++) m[a] += ft[q] * (real)L->c[q][a];
    }
    real u = m[0] / rho, v = m[1] / rho, w = m[2] / rho;
    u += (real)0.5 * X->p->dpdx / rho;
    A->rho[ic] = rho;
    A->u[ic] = u;
    A->v[ic] = v;
    A->w[ic] = w;
    A->Gx[ic] = A->Gy[ic] = A->Gz[ic] = 0;

    real tsgs = (X->cfg->sgs == SGS_WALE) ? wale(X, i, j, k, ic) : smagorinsky(X, ft, rho, u, v, w, omega, A->sdf[ic]);
    A->tauSGS[ic] = tsgs;
    real tau = sponge(X, omega, tsgs, i, j, k);

    real out[27];
    if (L->Q == 19) collide_rr19(X, out, ft, rho, u - (real)0.5 * X->p->dpdx / rho, v, w, tau, tsgs);
    else if (X->cfg->collision == COLL_CUMULANT) collide_cumulant27(X, out, ft, rho, u, v, w, tau, tsgs);
    else collide_rr27(X, out, ft, rho, u - (real)0.5 * X->p->dpdx / rho, v, w, tau, tsgs);
    for (int q = 0; q < L->Q; q++) A->fTmp[(long)q * E + ic] = out[q];
}

#include "lbm_oracle_d3q27.h"
#include "lbm_oracle_ibm.h"

static void init_ctx(ctx* X, const or_config* cfg, const or_params* p, or_fields* a)
{
    X->cfg = cfg;
    X->p = p;
    X->a = a;
    make_lat(&X->L, cfg->q);
    X->N[0] = p->nx;
    X->N[1] = p->ny;
    X->N[2] = p->nz;
    X->E = (long)p->nx * p->ny * p->nz;
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    long c[6] = {idx(X, 0, ny / 2, nz / 2), idx(X, nx - 1, ny / 2, nz / 2), idx(X, nx / 2, 0, nz / 2),
                 idx(X, nx / 2, ny - 1, nz / 2), idx(X, nx / 2, ny / 2, 0), idx(X, nx / 2, ny / 2, nz - 1)};
    const int* bl[3] = {a->boundary1, a->boundary2, a->boundary3};
    for (int s = 0; s < 6; s++) {
        int code = bl[s / 2][c[s]];
        X->sponge[s] = (code == BC_OUTLET || code == BC_FIXDEN);
    }
}

int oracle_q_real_bytes(void) { return (int)sizeof(real); }

/* One collision of one cell, for the tests that check the collision operators on their own:
 * ft -> out with the cell's rho and velocity (u including the half-force shift, as the step passes
 * it), molecular relaxation time tau and eddy part tau_sgs.  collision: COLL_RR or COLL_CUMULANT
 * (D3Q27 only). */
int oracle_collide(int q, int collision, const real* ft, real rho, real u, real v, real w, real tau, real tau_sgs,
                   real omegaB, real dpdx, real clim, real* out)
{
    if (q != 19 && q != 27) return -1;
    if (q == 19 && collision != COLL_RR) return -1;
    or_config cfg = {q, SGS_SMAG, WALL_BB, collision, (real)0.1, DAMP_WALL};
    or_params p;
    memset(&p, 0, sizeof p);
    p.nx = p.ny = p.nz = 1;
    p.dpdx = dpdx;
    p.omegaB = omegaB;
    p.clim = clim;
    ctx X;
    memset(&X, 0, sizeof X);
    X.cfg = &cfg;
    X.p = &p;
    make_lat(&X.L, q);
    if (q == 19) collide_rr19(&X, out, ft, rho, u - (real)0.5 * dpdx / rho, v, w, tau, tau_sgs);
    else if (collision == COLL_CUMULANT) collide_cumulant27(&X, out, ft, rho, u, v, w, tau, tau_sgs);
    else collide_rr27(&X, out, ft, rho, u - (real)0.5 * dpdx / rho, v, w, tau, tau_sgs);
    return 0;
}

/* Runs nsteps steps; on return a->f points at the newest populations. */
int oracle_step(const or_config* cfg, or_fields* a, const or_params* p, const or_ibm* ibm, int nsteps)
{
    if (cfg->q != 19 && cfg->q != 27) return -1;
    ctx X;
    init_ctx(&X, cfg, p, a);
    const long E = X.E;
    const int nt = p->nthreads > 0 ? p->nthreads : omp_get_max_threads();
    for (int s = 0; s < nsteps; s++) {
        memcpy(a->rhoPrev, a->rho, sizeof(real) * E);
        memcpy(a->uPrev, a->u, sizeof(real) * E);
        memcpy(a->vPrev, a->v, sizeof(real) * E);
        memcpy(a->wPrev, a->w, sizeof(real) * E);
#pragma omp parallel for schedule(static) num_threads(nt)
        for (long ic = 0; ic < E; ic++) cell_step(&X, ic);
        if (ibm && ibm->n > 1) ibm_substep(&X, ibm);
        real* t = a->f;
        a->f = a->fTmp;
        a->fTmp = t;
    }
    return 0;
}

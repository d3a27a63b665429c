/*
 * Test infrastructure only: host driver for the reference's step kernels
 * compiled as C (see build_ref.py).  One call of k_streamingCollision per
 * cell, split over OpenMP threads, exactly as one OpenCL NDRange launch of
 * D3Q19_opencl/ns.cpp:514-536 followed by the handle swap at ns.cpp:602.
 * The IBM sub-step (ns.cpp:542-601) runs k_Gwall per marker, the patched
 * k_Gibm serially (the spread accumulates) and k_Force per cell.
 *
 * The file is built once per variant; with -Dfloat=double every "float"
 * below (and in the included kernel) is double.
 */
#include "ref_shim.h"
#ifndef REF_CS
#define REF_CS 0.1f
#endif

__thread int lbffs_ref_gid;

#include REF_KERNEL_FILE

#include <string.h>
#include <omp.h>

typedef struct ref_fields {
    float *f, *fTmp;
    int *boundary, *boundary1, *boundary2, *boundary3;
    float *sdf;
    unsigned char *solid, *neiSolid;
    float *u0, *v0, *w0;
    float *Fwx, *Fwy, *Fwz;
    float *tauSGS, *rho, *u, *v, *w, *omega;
    float *Gx, *Gy, *Gz;
    float *rhoPrev, *uPrev, *vPrev, *wPrev; /* snapshot scratch, E each */
} ref_fields;

typedef struct ref_params {
    int nx, ny, nz;
    float dpdx, rho_av, LES;
    int isReadMovingWalls;
    float omegaB, spzWidth, clim;
    int nthreads;
} ref_params;

typedef struct ref_ibm {
    float *markers; /* 3 * n, x y z in lattice units, advanced in place */
    float *Gmx, *Gmy, *Gmz; /* per-marker forcing, n each */
    int n;
    float uT, vT, wT, rotX, rotY, rotZ, axX, axY, axZ, rotOmega;
} ref_ibm;

int ref_q(void) { return REF_Q; }
int ref_real_bytes(void) { return (int)sizeof(float); }

static void one_step(ref_fields* a, const ref_params* p, const ref_ibm* ibm)
{
    const unsigned E = (unsigned)p->nx * (unsigned)p->ny * (unsigned)p->nz;
    memcpy(a->rhoPrev, a->rho, sizeof(float) * E);
    memcpy(a->uPrev, a->u, sizeof(float) * E);
    memcpy(a->vPrev, a->v, sizeof(float) * E);
    memcpy(a->wPrev, a->w, sizeof(float) * E);
    int nt = p->nthreads > 0 ? p->nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nt)
    for (long ic = 0; ic < (long)E; ic++) {
        lbffs_ref_gid = (int)ic;
        k_streamingCollision(a->rhoPrev, a->uPrev, a->vPrev, a->wPrev, a->f, a->fTmp, a->boundary, a->boundary1,
                             a->boundary2, a->boundary3, a->sdf, a->solid, a->neiSolid, a->u0, a->v0, a->w0, a->Fwx,
                             a->Fwy, a->Fwz, a->tauSGS, a->rho, a->u, a->v, a->w, a->omega, a->Gx, a->Gy, a->Gz, E,
                             p->dpdx, p->rho_av, p->nx, p->ny, p->nz, p->LES, p->isReadMovingWalls, p->omegaB,
                             p->spzWidth
#if REF_Q == 27
                             ,
                             p->clim
#endif
        );
    }
    if (ibm && ibm->n > 1) {
#pragma omp parallel for schedule(static) num_threads(nt)
        for (int m = 0; m < ibm->n; m++) {
            lbffs_ref_gid = m;
            k_Gwall(a->rho, a->u, a->v, a->w, ibm->markers, ibm->Gmx, ibm->Gmy, ibm->Gmz, ibm->n, p->nx, p->ny, p->nz,
                    ibm->uT, ibm->vT, ibm->wT, ibm->rotX, ibm->rotY, ibm->rotZ, ibm->axX, ibm->axY, ibm->axZ,
                    ibm->rotOmega);
        }
        for (int m = 0; m < ibm->n; m++) {
            lbffs_ref_gid = m;
            k_Gibm(a->rho, a->Gx, a->Gy, a->Gz, ibm->markers, ibm->Gmx, ibm->Gmy, ibm->Gmz, ibm->n, p->nx, p->ny,
                   p->nz, ibm->uT, ibm->vT, ibm->wT, ibm->rotX, ibm->rotY, ibm->rotZ, ibm->axX, ibm->axY, ibm->axZ,
                   ibm->rotOmega);
        }
#pragma omp parallel for schedule(static) num_threads(nt)
        for (long ic = 0; ic < (long)E; ic++) {
            lbffs_ref_gid = (int)ic;
            k_Force(a->fTmp, a->solid, a->rho, a->Gx, a->Gy, a->Gz, E);
        }
    }
    float* t = a->f;
    a->f = a->fTmp;
    a->fTmp = t;
}

/* Runs nsteps steps; on return a->f points at the newest populations. */
int ref_step(ref_fields* a, const ref_params* p, const ref_ibm* ibm, int nsteps)
{
    for (int s = 0; s < nsteps; s++) one_step(a, p, ibm);
    return 0;
}

// Immersed-boundary sub-step: argument block and launchers (ibm.cu).
#pragma once
#include "lbffs_common.cuh"

namespace lbffs {

struct IbmMotion {
    float trans[3];  // per-step translation (uMovingTrans.., walls.hpp:606-626)
    float rot[3];    // rotation centre
    float axis[3];   // unit rotation axis
    float rot_omega; // rotation angle per step
    float amp[3];    // sinusoidal displacement amplitude
    float period;    // steps; <= 0 disables the sinusoid
};

struct IbmArgs {
    float* markers;       // 3n
    float* gm;            // 3n per-marker forcing of the last step
    double* acc;          // 3E FP64 spread accumulator (zero outside the current box)
    double* lag;          // 3 FP64 Lagrangian force accumulated since the last reset
    int* box;             // [0..5] current box lo/hi, [6..11] previous box lo/hi
    long long* t;         // step counter of the motion
    IbmMotion motion;
    int n, nx, ny, nz;
    long long E;
    const float *u, *v, *w, *rho;  // this step's macroscopics
    const uint8_t* flags;
    void* f_out;                   // this step's post-collision populations (padded planes)
    int px, pxy, porg;             // padded plane geometry: cell (i,j,k) at porg + k*pxy + j*px + i
    long long pE;
    float *gx, *gy, *gz;           // Eulerian forcing field (GxIBM..)
};

cudaError_t ibm_init_box(const IbmArgs& a, cudaStream_t st);
cudaError_t ibm_substep(const IbmArgs& a, int storage, int Q, int nsm, cudaStream_t st);

}  // namespace lbffs

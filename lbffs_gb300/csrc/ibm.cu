// Immersed-boundary sub-step (direct forcing), the intended mathematics of
// k_Gwall / k_Gibm / k_Force (D3Q19_opencl/kernel.cl:3648-3806, ns.cpp:542-601):
//   1. zero the Eulerian forcing G over the previous step's marker box
//   2. per marker: trilinear interpolation of this step's velocity over its 8-cell box,
//      G_m = u_target - u_interp, spread G_m with the same weights (FP64 atomics),
//      FP64 accumulation of sum_m G_m * sum(weights) (the Lagrangian force)
//   3. over the current marker box: G = spread, f_out += rho w_q 3 (G . c_q) on fluid cells
//   4. advance the markers (translation + sinusoidal displacement + rotation) and compute
//      the next marker box on the device
// The marker box lives in device memory (int[12]: current lo/hi, previous lo/hi) so a step
// never waits for the host; the bulk kernel reads it to decide which cells store their
// macroscopics for step 2.  Differences from the reference text are reference defects:
// the spread accumulates (kernel.cl:3760-3762 store the pre-add value), the rotation
// projection uses OX.e0 (kernel.cl:1213 uses OX_x*e0_z), k_Force reads u8 solid flags.
#include "ibm.h"

namespace lbffs {

__device__ __forceinline__ long long cidx(int i, int j, int k, int nx, int ny) { return ((long long)k * ny + j) * nx + i; }

// 8-cell box of a marker (icBox, kernel.cl:1112-1155); returns the count
__device__ __forceinline__ int marker_box(float x, float y, float z, int nx, int ny, int nz, long long (&cells)[8],
                                          float (&w)[8])
{
    const int i = (int)x, j = (int)y, k = (int)z;
    if (!(i >= 0 && i < nx && j >= 0 && j < ny && k >= 0 && k < nz)) return 0;
    int n = 0;
#pragma unroll
    for (int dk = 0; dk <= 1; dk++)
#pragma unroll
        for (int dj = 0; dj <= 1; dj++)
#pragma unroll
            for (int di = 0; di <= 1; di++) {
                const int ii = i + di, jj = j + dj, kk = k + dk;
                if (ii >= nx || jj >= ny || kk >= nz) continue;
                cells[n] = cidx(ii, jj, kk, nx, ny);
                w[n] = (1.f - fabsf((float)ii - x)) * (1.f - fabsf((float)jj - y)) * (1.f - fabsf((float)kk - z));
                n++;
            }
    return n;
}

struct RotFrame {
    float oop[3], e1[3], e2[3], r;
};

__device__ __forceinline__ RotFrame rot_frame(const IbmMotion& m, float X, float Y, float Z)
{
    RotFrame f;
    const float e0[3] = {m.axis[0], m.axis[1], m.axis[2]};
    const float ox[3] = {X - m.rot[0], Y - m.rot[1], Z - m.rot[2]};
    const float d = ox[0] * e0[0] + ox[1] * e0[1] + ox[2] * e0[2];
    float opx[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        f.oop[a] = d * e0[a];
        opx[a] = ox[a] - f.oop[a];
    }
    f.r = sqrtf(opx[0] * opx[0] + opx[1] * opx[1] + opx[2] * opx[2]);
    if (f.r == 0.f) {
#pragma unroll
        for (int a = 0; a < 3; a++) f.e1[a] = f.e2[a] = 0.f;
        return f;
    }
#pragma unroll
    for (int a = 0; a < 3; a++) f.e1[a] = opx[a] / f.r;
    f.e2[0] = e0[1] * f.e1[2] - e0[2] * f.e1[1];
    f.e2[1] = e0[2] * f.e1[0] - e0[0] * f.e1[2];
    f.e2[2] = e0[0] * f.e1[1] - e0[1] * f.e1[0];
    return f;
}

// per-step translation including the sinusoidal displacement of step t
__device__ __forceinline__ void step_translation(const IbmMotion& m, long long t, float (&d)[3])
{
    double s = 0.0;
    if (m.period > 0.f) {
        const double T = (double)m.period;
        s = sin(2.0 * 3.14159265358979323846 * ((double)t + 1.0) / T) - sin(2.0 * 3.14159265358979323846 * (double)t / T);
    }
    d[0] = m.trans[0] + (float)((double)m.amp[0] * s);
    d[1] = m.trans[1] + (float)((double)m.amp[1] * s);
    d[2] = m.trans[2] + (float)((double)m.amp[2] * s);
}

// cells of a box stored in device memory: count and the t-th cell
struct BoxIter {
    int lo[3], bx, by;
    long long n;
};

__device__ __forceinline__ BoxIter box_iter(const int* box)
{
    BoxIter b;
    const int bz = box[5] - box[2] + 1;
    b.bx = box[3] - box[0] + 1;
    b.by = box[4] - box[1] + 1;
    b.lo[0] = box[0];
    b.lo[1] = box[1];
    b.lo[2] = box[2];
    b.n = (b.bx > 0 && b.by > 0 && bz > 0) ? (long long)b.bx * b.by * bz : 0;
    return b;
}

__device__ __forceinline__ long long box_cell(const BoxIter& b, long long t, int nx, int ny)
{
    const int ii = b.lo[0] + (int)(t % b.bx), jj = b.lo[1] + (int)((t / b.bx) % b.by),
              kk = b.lo[2] + (int)(t / ((long long)b.bx * b.by));
    return cidx(ii, jj, kk, nx, ny);
}

__global__ void k_ibm_zero(IbmArgs a)
{
    const BoxIter b = box_iter(a.box + 6);  // previous box
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < b.n; t += (long long)gridDim.x * blockDim.x) {
        const long long ic = box_cell(b, t, a.nx, a.ny);
        a.gx[ic] = 0.f;
        a.gy[ic] = 0.f;
        a.gz[ic] = 0.f;
    }
}

__global__ void k_ibm_interp_spread(IbmArgs a)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    float d[3];
    step_translation(a.motion, *a.t, d);
    double lag[3] = {0.0, 0.0, 0.0};
    if (m < a.n) {
        const float X = a.markers[3 * m], Y = a.markers[3 * m + 1], Z = a.markers[3 * m + 2];
        const RotFrame fr = rot_frame(a.motion, X, Y, Z);
        float ut[3];
#pragma unroll
        for (int c = 0; c < 3; c++) ut[c] = d[c] + fr.r * a.motion.rot_omega * fr.e2[c];
        long long cells[8];
        float w[8];
        const int nb = marker_box(X, Y, Z, a.nx, a.ny, a.nz, cells, w);
        float ui[3] = {0.f, 0.f, 0.f};
        for (int b = 0; b < nb; b++) {
            ui[0] += a.u[cells[b]] * w[b];
            ui[1] += a.v[cells[b]] * w[b];
            ui[2] += a.w[cells[b]] * w[b];
        }
        const float G[3] = {ut[0] - ui[0], ut[1] - ui[1], ut[2] - ui[2]};
        a.gm[3 * m] = G[0];
        a.gm[3 * m + 1] = G[1];
        a.gm[3 * m + 2] = G[2];
        for (int b = 0; b < nb; b++) {
            atomicAdd(a.acc + cells[b], (double)(G[0] * w[b]));
            atomicAdd(a.acc + a.E + cells[b], (double)(G[1] * w[b]));
            atomicAdd(a.acc + 2 * a.E + cells[b], (double)(G[2] * w[b]));
            lag[0] += (double)(G[0] * w[b]);
            lag[1] += (double)(G[1] * w[b]);
            lag[2] += (double)(G[2] * w[b]);
        }
    }
    // Lagrangian force of this step, FP64 (warp reduce then one atomic per warp)
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double v = lag[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(a.lag + c, v);
    }
}

template <int S, int Q>
__global__ void k_ibm_force(IbmArgs a)
{
    using T = typename Codec<S>::T;
    T* f = static_cast<T*>(a.f_out);
    const BoxIter bi = box_iter(a.box);
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < bi.n; t += (long long)gridDim.x * blockDim.x) {
        const long long ic = box_cell(bi, t, a.nx, a.ny);
        const int ip = a.porg + (bi.lo[2] + (int)(t / ((long long)bi.bx * bi.by))) * a.pxy +
                       (bi.lo[1] + (int)((t / bi.bx) % bi.by)) * a.px + bi.lo[0] + (int)(t % bi.bx);
        const float g[3] = {(float)a.acc[ic], (float)a.acc[a.E + ic], (float)a.acc[2 * a.E + ic]};
        a.acc[ic] = 0.0;
        a.acc[a.E + ic] = 0.0;
        a.acc[2 * a.E + ic] = 0.0;
        a.gx[ic] = g[0];
        a.gy[ic] = g[1];
        a.gz[ic] = g[2];
        if (!(a.flags[ic] & FL_SOLID) && (g[0] != 0.f || g[1] != 0.f || g[2] != 0.f)) {
            const float r3 = a.rho[ic] * 3.f;
#pragma unroll
            for (int q = 0; q < Q; q++) {
                const float gc = g[0] * (float)lat_c(Q, q, 0) + g[1] * (float)lat_c(Q, q, 1) + g[2] * (float)lat_c(Q, q, 2);
                T* p = f + (long long)q * a.pE + ip;
                const float w = lat_w(Q, q);
                float v;
                if constexpr (S == ST_FP32) v = *p;
                else if constexpr (S == ST_FP16S) v = fmaf(__half2float(*p), FP16S_INV, w);
                else v = __bfloat162float(*p) + w;
                v += r3 * w * gc;
                if constexpr (S == ST_FP32) *p = v;
                else if constexpr (S == ST_FP16S) *p = __float2half_rn((v - w) * FP16S_SCALE);
                else *p = __float2bfloat16_rn(v - w);
            }
        }
    }
}

// single block: advance markers, compute the next box, rotate box buffers, advance t
__global__ void k_ibm_move(IbmArgs a)
{
    __shared__ int lo[3], hi[3];
    if (threadIdx.x < 3) {
        lo[threadIdx.x] = 0x7fffffff;
        hi[threadIdx.x] = -1;
    }
    __syncthreads();
    float d[3];
    step_translation(a.motion, *a.t, d);
    const float c = cosf(a.motion.rot_omega), s = sinf(a.motion.rot_omega);
    for (int m = threadIdx.x; m < a.n; m += blockDim.x) {
        float P[3] = {a.markers[3 * m] + d[0], a.markers[3 * m + 1] + d[1], a.markers[3 * m + 2] + d[2]};
        const RotFrame fr = rot_frame(a.motion, P[0], P[1], P[2]);
        if (fr.r > 0.f) {
#pragma unroll
            for (int q = 0; q < 3; q++) P[q] = a.motion.rot[q] + fr.oop[q] + fr.r * (c * fr.e1[q] + s * fr.e2[q]);
        }
        a.markers[3 * m] = P[0];
        a.markers[3 * m + 1] = P[1];
        a.markers[3 * m + 2] = P[2];
        const int N[3] = {a.nx, a.ny, a.nz};
        const int ci[3] = {(int)P[0], (int)P[1], (int)P[2]};
        if (ci[0] >= 0 && ci[0] < N[0] && ci[1] >= 0 && ci[1] < N[1] && ci[2] >= 0 && ci[2] < N[2]) {
#pragma unroll
            for (int q = 0; q < 3; q++) {
                atomicMin(&lo[q], ci[q]);
                atomicMax(&hi[q], min(ci[q] + 1, N[q] - 1));
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 3; q++) {
            a.box[6 + q] = a.box[q];
            a.box[9 + q] = a.box[3 + q];
            a.box[q] = (hi[q] >= 0) ? lo[q] : 1;
            a.box[3 + q] = (hi[q] >= 0) ? hi[q] : 0;
        }
        *a.t += 1;
    }
}

// initial box of freshly set markers (current box; previous box empty)
__global__ void k_ibm_init_box(IbmArgs a)
{
    __shared__ int lo[3], hi[3];
    if (threadIdx.x < 3) {
        lo[threadIdx.x] = 0x7fffffff;
        hi[threadIdx.x] = -1;
    }
    __syncthreads();
    for (int m = threadIdx.x; m < a.n; m += blockDim.x) {
        const int N[3] = {a.nx, a.ny, a.nz};
        const int ci[3] = {(int)a.markers[3 * m], (int)a.markers[3 * m + 1], (int)a.markers[3 * m + 2]};
        if (ci[0] >= 0 && ci[0] < N[0] && ci[1] >= 0 && ci[1] < N[1] && ci[2] >= 0 && ci[2] < N[2]) {
#pragma unroll
            for (int q = 0; q < 3; q++) {
                atomicMin(&lo[q], ci[q]);
                atomicMax(&hi[q], min(ci[q] + 1, N[q] - 1));
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 0; q < 3; q++) {
            a.box[q] = (hi[q] >= 0) ? lo[q] : 1;
            a.box[3 + q] = (hi[q] >= 0) ? hi[q] : 0;
            a.box[6 + q] = 1;
            a.box[9 + q] = 0;
        }
        *a.t = 0;
    }
}

cudaError_t ibm_init_box(const IbmArgs& a, cudaStream_t st)
{
    k_ibm_init_box<<<1, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t ibm_substep(const IbmArgs& a, int storage, int Q, int nsm, cudaStream_t st)
{
    const int nb_box = nsm * 4;
    k_ibm_zero<<<nb_box, 256, 0, st>>>(a);
    k_ibm_interp_spread<<<(a.n + 127) / 128, 128, 0, st>>>(a);
#define LBFFS_FORCE(S)                                                            \
    if (Q == 19) k_ibm_force<S, 19><<<nb_box, 256, 0, st>>>(a);                   \
    else k_ibm_force<S, 27><<<nb_box, 256, 0, st>>>(a);
    switch (storage) {
        case ST_FP32: LBFFS_FORCE(ST_FP32); break;
        case ST_FP16S: LBFFS_FORCE(ST_FP16S); break;
        case ST_BF16S: LBFFS_FORCE(ST_BF16S); break;
        default: return cudaErrorInvalidValue;
    }
#undef LBFFS_FORCE
    k_ibm_move<<<1, 1024, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace lbffs

// lbffs_mass_noalloc: FP64 fluid mass of float32 populations that the caller already holds on
// the device, computed without allocating anything.
//
// Who needs this.  Some callers cannot allocate device memory at the moment they want a mass
// check: a serving loop that has admitted its cases against a fixed HBM budget (an allocation
// after admission can fail, and cudaMalloc / cudaFree wait for the whole device, stalling every
// case in flight), and a driver that owns its population buffers itself and only wants a
// conservation check between steps without building a full lattice context (lbffs_create
// allocates the whole lattice).  lbffs_mass needs a context and its reduction buffer; this entry
// point needs neither.
//
// How.  The per-block FP64 partial sums live in one file-scope __device__ array of fixed size,
// which every GPU that loads this library keeps until the process exits.  The first call on a
// device looks up that array's device address with cudaGetSymbolAddress (this may load the
// library's device code on that device) and caches it; make that first call before any stream
// capture.  Every later call reuses the cached address and only launches two kernels on the
// caller's stream: one writes a partial per block of 8192 cells, one adds the partials in block
// order and writes the result to the caller's device address.  No slot needs clearing between
// calls: the second kernel reads only slots the first kernel of the same call has just written.
// All calls on a device share the array, so two calls whose kernels overlap on the GPU (on
// different streams without ordering between them) race and both results are undefined.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/lbffs_cuda.h"
#include "launch.h"

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_CELLS_PER_THREAD = 32;
constexpr long long NA_CELLS_PER_BLOCK = (long long)NA_THREADS * NA_CELLS_PER_THREAD;  // 8192
constexpr int NA_MAX_BLOCKS = LBFFS_NOALLOC_MAX_CELLS / (int)NA_CELLS_PER_BLOCK;         // 32768

// The shared scratch: one double per block, 256 KiB per device.  In host code this name is only
// a handle for cudaGetSymbolAddress, never a device address.
static __device__ __align__(256) double g_mass_partials[NA_MAX_BLOCKS];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_setup_mutex;
double* g_partials_addr[NA_MAX_DEVICES] = {};

__device__ __forceinline__ double na_block_sum(double v, double* sh)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < NA_THREADS / 32; w++) s += sh[w];
    return s;
}

// Block b sums cells [b * 8192, (b + 1) * 8192); a cell's density is its Q populations added in
// order q = 0..Q-1 in FP32, the same per-cell arithmetic as lbffs_mass.
template <int Q>
__global__ void __launch_bounds__(NA_THREADS) k_mass_partials(const float* __restrict__ f,
                                                              const unsigned char* __restrict__ solid,
                                                              long long E, double* __restrict__ partials)
{
    __shared__ double sh[NA_THREADS / 32];
    const long long base = (long long)blockIdx.x * NA_CELLS_PER_BLOCK;
    double acc = 0.0;
    for (int k = 0; k < NA_CELLS_PER_THREAD; k++) {
        const long long ic = base + (long long)k * NA_THREADS + threadIdx.x;
        if (ic >= E || solid[ic]) continue;
        float r = 0.f;
#pragma unroll
        for (int q = 0; q < Q; q++) r += __ldg(f + (long long)q * E + ic);
        acc += (double)r;
    }
    acc = na_block_sum(acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// One warp adds the partials in block order (lane-strided, then a fixed shuffle tree).
__global__ void k_mass_finish(const double* __restrict__ partials, int nblocks, double* __restrict__ out)
{
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += 32) s += partials[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) *out = s;
}

int na_fail(int code, const std::string& msg)
{
    lbffs::set_thread_error(msg);
    return code;
}

// makes `device` current for the call and gives the caller's current device back on every return
struct DeviceScope {
    int saved = -1;
    cudaError_t enter(int device)
    {
        cudaError_t e = cudaGetDevice(&saved);
        if (e != cudaSuccess) {
            saved = -1;
            return e;
        }
        return saved == device ? cudaSuccess : cudaSetDevice(device);
    }
    ~DeviceScope()
    {
        int cur = -1;
        if (saved >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != saved) cudaSetDevice(saved);
    }
};

}  // namespace

extern "C" int lbffs_mass_noalloc(int device, const float* f, const unsigned char* solid, int q, long long n_cells,
                                  double* out, void* stream)
{
    if (!f || !solid || !out) return na_fail(LBFFS_E_ARG, "lbffs_mass_noalloc: null pointer");
    if (q != 19 && q != 27) return na_fail(LBFFS_E_ARG, "lbffs_mass_noalloc: q must be 19 or 27");
    if (n_cells < 0) return na_fail(LBFFS_E_ARG, "lbffs_mass_noalloc: n_cells must be >= 0");
    if (n_cells > LBFFS_NOALLOC_MAX_CELLS)
        return na_fail(LBFFS_E_ARG, "lbffs_mass_noalloc: n_cells " + std::to_string(n_cells) +
                                        " exceeds the maximum of " + std::to_string(LBFFS_NOALLOC_MAX_CELLS) +
                                        " cells (fixed scratch of " + std::to_string(NA_MAX_BLOCKS) +
                                        " block partials)");
    if (device < 0 || device >= NA_MAX_DEVICES)
        return na_fail(LBFFS_E_ARG, "lbffs_mass_noalloc: device ordinal out of range");

    DeviceScope scope;
    cudaError_t e = scope.enter(device);
    if (e != cudaSuccess) return na_fail(LBFFS_E_CUDA, std::string("lbffs_mass_noalloc: cudaSetDevice: ") +
                                                           cudaGetErrorString(e));
    double* partials;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_partials_addr[device]) {
            double* p = nullptr;
            e = cudaGetSymbolAddress((void**)&p, g_mass_partials);
            if (e != cudaSuccess || !p)
                return na_fail(LBFFS_E_CUDA, std::string("lbffs_mass_noalloc: cudaGetSymbolAddress: ") +
                                                 cudaGetErrorString(e));
            g_partials_addr[device] = p;
        }
        partials = g_partials_addr[device];
    }

    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nblocks = (int)((n_cells + NA_CELLS_PER_BLOCK - 1) / NA_CELLS_PER_BLOCK);
    if (nblocks > 0) {
        if (q == 19)
            k_mass_partials<19><<<nblocks, NA_THREADS, 0, st>>>(f, solid, n_cells, partials);
        else
            k_mass_partials<27><<<nblocks, NA_THREADS, 0, st>>>(f, solid, n_cells, partials);
    }
    k_mass_finish<<<1, 32, 0, st>>>(partials, nblocks, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail(LBFFS_E_CUDA, std::string("lbffs_mass_noalloc: launch: ") +
                                                           cudaGetErrorString(e));
    return LBFFS_OK;
}

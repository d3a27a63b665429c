// The context behind the C ABI (include/lbffs_cuda.h), shared by the single-lattice entry points
// and the server: device buffers of one lattice, its geometry lists and its step state.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/lbffs_cuda.h"
#include "arena.h"
#include "ibm.h"
#include "launch.h"

namespace lbffs {
struct OutputState;  // output.cu: fields of lbffs_output and the asynchronous file writer
}

// host <-> device copies of FP32 populations in flight at once (one direction plane per copy); a
// build-time tuning value
#ifndef LBFFS_COPY_STREAMS
#define LBFFS_COPY_STREAMS 4
#endif

struct lbffs_ctx {
    lbffs_desc d{};
    int Q = 19;
    long long E = 0;
    size_t tsize = 4;
    int nsm = 0;
    long long l2_bytes = 0;  // the device's L2 size
    cudaStream_t stream = nullptr;
    std::string err = "no error";

    void* f[2] = {nullptr, nullptr};
    int fcur = 0;
    int* iarr[4] = {nullptr, nullptr, nullptr, nullptr};  // boundary, boundary1..3 as uploaded
    uint8_t *solid = nullptr, *nei = nullptr, *flags = nullptr;
    uint16_t* bc = nullptr;
    float *u0 = nullptr, *v0 = nullptr, *w0 = nullptr, *omega = nullptr, *sdf = nullptr;
    float* macro[2][5] = {{nullptr}};
    int mcur = 0;
    float* fw[3] = {nullptr, nullptr, nullptr};
    float* g[3] = {nullptr, nullptr, nullptr};
    uint32_t* special = nullptr;
    long long n_special = 0;
    lbffs::PadGeom pg{};
    long long counts[4] = {0, 0, 0, 0};
    float omega0 = 1.f;
    int sponge_mask = 0;
    bool dirty = true;
    // pulls across the grid's border: face_ok when every face carries one boundary code per axis
    // (face_codes, StepArgs layout) and the face flag is set on exactly the border cells.  pull_mode
    // (StepArgs::border_pulls) 1 when moreover both x faces carry boundary-kernel codes (inlet /
    // outlet / fixed density / wall function), so bulk rows cross only y / z faces; with bulk cells on
    // the x faces (nz > 1) 3 when neither x face is Cyclic (those cells write the x ghost slots they
    // pull from next step themselves), else 2 (they pull across the x face from per-context plane
    // bases) where that kernel is built; 0 otherwise.  Modes 1 and 2 run without a ghost fill; mode
    // 3 fills the ghost layer once, before its first step from a state the pushes did not write
    // (xghost_ok false).
    int face_codes = 0;
    bool face_ok = false;
    bool pull_ok = false;
    int pull_mode = 0;
    bool xghost_ok = false;
    bool pulls_on = true;  // lbffs_set_border_pulls
    int* d_err = nullptr;
    float* stage = nullptr;
    size_t stage_elems = 0;
    double* partial = nullptr;
    int partial_blocks = 0;

    // IBM
    int n_markers = 0;
    float* markers = nullptr;
    float* gm = nullptr;
    double* ibm_acc = nullptr;
    double* ibm_lag = nullptr;
    int* ibm_box = nullptr;
    long long* ibm_t = nullptr;
    lbffs::IbmMotion motion{};

    // server cases: device memory from the server's arena, the server's stream and staging
    lbffs::Arena* arena = nullptr;
    bool own_stream = true, own_stage = true;

    // the boundary kernel runs beside the bulk kernel on a second stream (lbffs_step)
    cudaStream_t side = nullptr;     // boundary kernel, one thread per cell: launched first, higher priority
    cudaStream_t side_lo = nullptr;  // boundary kernel, a lane group per cell: launched after the bulk kernel
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    // FP32 population transfers: the direction planes' copies spread over these streams (created on
    // the first transfer), with one event each to join them back into the context's stream
    cudaStream_t copy_st[LBFFS_COPY_STREAMS] = {};
    cudaEvent_t copy_ev[LBFFS_COPY_STREAMS + 1] = {};

    // output step and asynchronous writes (output.cu)
    lbffs::OutputState* out = nullptr;

    // timing
    bool timing = false;
    int bulk_kind = 0;  // D3Q19 bulk kernel variant (lbffs_set_bulk_kernel)
    int special_kind = -1;  // boundary kernel mapping (lbffs_set_special_kernel): -1 by list length
    struct Ev {
        cudaEvent_t a, b;
        int kind;
    };
    std::vector<Ev> pending;
    std::vector<cudaEvent_t> pool;
    double ms[4] = {0, 0, 0, 0};
    long long launches[4] = {0, 0, 0, 0};
};

namespace lbffs {

// record msg as the context's (and this thread's) last error and return code
int ctx_fail(lbffs_ctx* c, int code, const std::string& msg);
// zero-filled device allocation from the context's arena (server cases) or cudaMalloc
cudaError_t ctx_alloc_bytes(lbffs_ctx* c, void** p, size_t bytes);
template <class T>
inline cudaError_t ctx_alloc(lbffs_ctx* c, T** p, size_t n)
{
    return ctx_alloc_bytes(c, reinterpret_cast<void**>(p), n * sizeof(T) + 16);
}
void ctx_free(lbffs_ctx* c, void* p);
// join the asynchronous file writer, if one runs; its error, if any, becomes the context's
int ctx_io_wait(lbffs_ctx* c);
// join the writer and free the output state
void ctx_output_release(lbffs_ctx* c);
// device array of an output field (LBFFS_OUT_* or LBFFS_*MEAN); create: allocate a missing one
// (zero-filled).  nullptr when absent (or on allocation failure with create).
float* ctx_output_field(lbffs_ctx* c, int field, bool create);
// create a context; arena / stream / stage are the server's (nullptr: the context owns its own)
int ctx_create(const lbffs_desc* d, Arena* arena, cudaStream_t stream, float* stage, size_t stage_elems,
               lbffs_ctx** out);
// condense the uploaded geometry into flags, boundary words and the special list
int ctx_commit(lbffs_ctx* c);
// device bytes a context allocates for lattice d (its special list, at most 4 bytes per cell,
// included), rounded up per block as the server's arena does
size_t ctx_footprint(const lbffs_desc& d);
// kernel arguments of one step reading population copy src and macroscopic copy msrc
void ctx_step_args(const lbffs_ctx* c, const lbffs_step_params* p, int src, int msrc, StepArgs& a);

}  // namespace lbffs

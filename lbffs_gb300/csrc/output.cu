// Output step of the reference driver (D3Q19_opencl/write.hpp, identical for D3Q27 but for the
// population count) on the device, and its files written off the critical path.
//
// lbffs_output    cal_rhoUVW (D3Q19.hpp:647-666) of every cell from the current populations,
//                 in the host function's float order, into output-owned rho / u / v / w fields;
//                 rho_av, rhoMax / rhoMin, uAve, the wall and IBM force sums and the time-mean
//                 accumulation of write.hpp:16-76.  The reference downloads all populations
//                 (19 or 27 floats per cell) to do this on the host; here nothing leaves the
//                 device but the scalars.
// lbffs_write_vtk / lbffs_write_restart
//                 the VTK file (write.hpp:78-600, including asciiToBinary's byte order) and the
//                 restart file data.dat (write.hpp:603-631).  The call snapshots what the file
//                 needs on the device, enqueues the copies on an I/O stream and returns; a host
//                 thread fetches the fields through a pinned buffer, formats and writes them while
//                 the next steps run.  lbffs_io_wait joins it.
// lbffs_read_restart
//                 restart.hpp: data.dat back into the populations.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "ctx.h"

namespace lbffs {

struct OutputState {
    float* fld[4] = {nullptr, nullptr, nullptr, nullptr};  // rho, u, v, w of the last lbffs_output
    float* tau = nullptr;                                   // tauSGS at the last lbffs_output
    float* g[3] = {nullptr, nullptr, nullptr};              // IBM forcing at the last lbffs_output
    bool g_valid = false;                                   // forceCoeffs: G fields were captured
    float* mean[3] = {nullptr, nullptr, nullptr};           // uMean, vMean, wMean
    float time_mean = 0.f;
    bool have_output = false;
    void* f_snap = nullptr;  // populations for an asynchronous restart write
    double* partial = nullptr;
    int nblocks = 0;
    float* d_uave = nullptr;
    // asynchronous writer
    cudaStream_t io = nullptr;
    cudaEvent_t ready = nullptr;
    float* stage = nullptr;  // device staging of decoded population rows
    float* pinned = nullptr;
    size_t chunk = 0;  // floats per staging / pinned chunk
    std::thread th;
    bool running = false;
    int rc = LBFFS_OK;
    std::string msg;
};

namespace {

constexpr int OUT_BS = 256;
// partial results per block: sum(rho - 1) over fluid, fluid count, max, min, Fw xyz, G xyz
constexpr int OUT_NP = 10;

template <int Q, int S>
__global__ void __launch_bounds__(OUT_BS) k_output(const void* __restrict__ f, PadGeom g, const uint8_t* __restrict__ solid,
                                                   float dpdx, int interval, float* __restrict__ rho_o,
                                                   float* __restrict__ u_o, float* __restrict__ v_o,
                                                   float* __restrict__ w_o, float* __restrict__ um,
                                                   float* __restrict__ vm, float* __restrict__ wm, const float* fwx,
                                                   const float* fwy, const float* fwz, const float* gx, const float* gy,
                                                   const float* gz, double* __restrict__ partial)
{
    using T = typename Codec<S>::T;
    const long long E = (long long)g.nx * g.ny * g.nz;
    double s_rho = 0.0, s_n = 0.0, s_f[3] = {0.0, 0.0, 0.0}, s_g[3] = {0.0, 0.0, 0.0};
    float mx = -INFINITY, mn = INFINITY;
    for (long long ic = (long long)blockIdx.x * blockDim.x + threadIdx.x; ic < E; ic += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(ic % g.nx), j = (int)((ic / g.nx) % g.ny), k = (int)(ic / ((long long)g.nx * g.ny));
        const long long ip = (long long)g.porg + (long long)k * g.pxy + (long long)j * g.px + i;
        float rho = 0.f, u = 0.f, v = 0.f, w = 0.f;
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const float fq = Codec<S>::load(static_cast<const T*>(f) + (long long)q * g.pE + ip, lat_w(Q, q));
            rho = __fadd_rn(rho, fq);
            // f * c_q with c_q in {-1, 0, 1}: the product is exact, and a zero term leaves the sum
            if (lat_c(Q, q, 0)) u = lat_c(Q, q, 0) > 0 ? __fadd_rn(u, fq) : __fsub_rn(u, fq);
            if (lat_c(Q, q, 1)) v = lat_c(Q, q, 1) > 0 ? __fadd_rn(v, fq) : __fsub_rn(v, fq);
            if (lat_c(Q, q, 2)) w = lat_c(Q, q, 2) > 0 ? __fadd_rn(w, fq) : __fsub_rn(w, fq);
        }
        u = __fdiv_rn(u, rho);
        v = __fdiv_rn(v, rho);
        w = __fdiv_rn(w, rho);
        u = __fadd_rn(u, __fdiv_rn(__fmul_rn(0.5f, dpdx), rho));
        rho_o[ic] = rho;
        u_o[ic] = u;
        v_o[ic] = v;
        w_o[ic] = w;
        if (interval > 0) {
            const float iv = (float)interval;
            um[ic] = __fadd_rn(um[ic], __fmul_rn(u, iv));
            vm[ic] = __fadd_rn(vm[ic], __fmul_rn(v, iv));
            wm[ic] = __fadd_rn(wm[ic], __fmul_rn(w, iv));
        }
        mx = fmaxf(mx, rho);
        mn = fminf(mn, rho);
        if (solid[ic] == 0) {
            s_rho += (double)rho - 1.0;
            s_n += 1.0;
            if (fwx) {
                s_f[0] += (double)fwx[ic];
                s_f[1] += (double)fwy[ic];
                s_f[2] += (double)fwz[ic];
            }
            if (gx) {
                s_g[0] += (double)gx[ic];
                s_g[1] += (double)gy[ic];
                s_g[2] += (double)gz[ic];
            }
        }
    }
    double vals[OUT_NP] = {s_rho, s_n, (double)mx, (double)mn, s_f[0], s_f[1], s_f[2], s_g[0], s_g[1], s_g[2]};
    __shared__ double red[OUT_NP][OUT_BS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int p = 0; p < OUT_NP; p++) {
        double x = vals[p];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_down_sync(0xffffffffu, x, o);
            x = p == 2 ? fmax(x, y) : p == 3 ? fmin(x, y) : x + y;
        }
        if (lane == 0) red[p][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < OUT_NP) {
        const int p = threadIdx.x;
        double x = red[p][0];
        for (int q = 1; q < OUT_BS / 32; q++) x = p == 2 ? fmax(x, red[p][q]) : p == 3 ? fmin(x, red[p][q]) : x + red[p][q];
        partial[(long long)blockIdx.x * OUT_NP + p] = x;
    }
}

// uAve of write.hpp:51-60: u * c of the x = 0 plane added in the reference's order (j outer,
// k inner) by one thread, the products staged through shared memory in chunks
__global__ void __launch_bounds__(1024) k_uave(const float* __restrict__ u, int nx, int ny, int nz, float c,
                                               float* __restrict__ out)
{
    __shared__ float buf[1024];
    const long long n = (long long)ny * nz;
    float s = 0.f;
    for (long long base = 0; base < n; base += 1024) {
        const long long t = base + threadIdx.x;
        if (t < n) {
            const int j = (int)(t / nz), k = (int)(t % nz);
            buf[threadIdx.x] = __fmul_rn(u[((long long)k * ny + j) * nx], c);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int m = (int)min(1024LL, n - base);
            for (int x = 0; x < m; x++) s = __fadd_rn(s, buf[x]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = __fdiv_rn(s, (float)(ny * nz));
}

cudaError_t launch_output(lbffs_ctx* c, OutputState* o, float dpdx, int interval, const float* const* fw,
                          const float* const* gg)
{
    const void* f = c->f[c->fcur];
#define LBFFS_OUT(Q, S)                                                                                            \
    k_output<Q, S><<<o->nblocks, OUT_BS, 0, c->stream>>>(f, c->pg, c->solid, dpdx, interval, o->fld[0], o->fld[1], \
                                                         o->fld[2], o->fld[3], o->mean[0], o->mean[1], o->mean[2],  \
                                                         fw[0], fw[1], fw[2], gg[0], gg[1], gg[2], o->partial)
    const int Q = c->Q, S = c->d.storage;
    if (Q == 19 && S == ST_FP32) LBFFS_OUT(19, ST_FP32);
    else if (Q == 19 && S == ST_FP16S) LBFFS_OUT(19, ST_FP16S);
    else if (Q == 19 && S == ST_BF16S) LBFFS_OUT(19, ST_BF16S);
    else if (Q == 27 && S == ST_FP32) LBFFS_OUT(27, ST_FP32);
    else if (Q == 27 && S == ST_FP16S) LBFFS_OUT(27, ST_FP16S);
    else LBFFS_OUT(27, ST_BF16S);
#undef LBFFS_OUT
    return cudaGetLastError();
}

#define OCK(x)                                                                                                 \
    do {                                                                                                       \
        cudaError_t e_ = (x);                                                                                  \
        if (e_ != cudaSuccess) return ctx_fail(c, LBFFS_E_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

OutputState* state(lbffs_ctx* c)
{
    if (!c->out) c->out = new OutputState();
    return c->out;
}

// the pinned and device staging of the writer thread, its stream and event
cudaError_t ensure_io(lbffs_ctx* c, OutputState* o)
{
    if (o->io) return cudaSuccess;
    cudaError_t e = cudaStreamCreateWithFlags(&o->io, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&o->ready, cudaEventDisableTiming);
    const long long nx = c->d.nx;
    const long long rows = std::max(1LL, (long long)(4 << 20) / nx);  // about 16 MB per chunk
    o->chunk = (size_t)(rows * nx);
    if (e == cudaSuccess) e = cudaMallocHost(&o->pinned, o->chunk * sizeof(float));
    if (e == cudaSuccess) e = ctx_alloc_bytes(c, (void**)&o->stage, o->chunk * sizeof(float));
    return e;
}

// asciiToBinary (src/base.hpp:35-43): bytes 3, 2, 1 and again 3 of the float
inline void put_binary(std::string& s, float x)
{
    unsigned char b[4];
    std::memcpy(b, &x, 4);
    s.push_back((char)b[3]);
    s.push_back((char)b[2]);
    s.push_back((char)b[1]);
    s.push_back((char)b[3]);
}

// operator<< of a float on a default-formatted stream: "%g", six significant digits
inline void put_ascii(std::string& s, double x)
{
    char buf[40];
    const int n = std::snprintf(buf, sizeof buf, "%g\n", x);
    s.append(buf, (size_t)n);
}
inline void put_ascii_int(std::string& s, int x)
{
    char buf[24];
    const int n = std::snprintf(buf, sizeof buf, "%d\n", x);
    s.append(buf, (size_t)n);
}

struct VtkField {
    const char* name;
    const void* dev;  // device array (float, int or uint8), nullptr: zeros
    int kind;         // 0 float, 1 int, 2 uint8
    int op;           // 0 x, 1 x * c, 2 3 * (3 x L c) (nuSGS), 3 x * L, 4 x * c / timeMean
};

struct VtkJob {
    std::string path;
    bool binary;
    float c, L, time_mean;
    int nx, ny, nz;
    std::vector<VtkField> fields;
};

struct RestartJob {
    std::string path;
    int nt, nx, ny, nz, Q, storage;
    PadGeom pg;
};

// n elements (elem bytes each) of a device field from element off into host memory
bool fetch(OutputState* o, const void* dev, size_t elem, size_t off, size_t n, void* host)
{
    if (cudaMemcpyAsync(o->pinned, static_cast<const char*>(dev) + off * elem, n * elem, cudaMemcpyDeviceToHost,
                        o->io) != cudaSuccess)
        return false;
    if (cudaStreamSynchronize(o->io) != cudaSuccess) return false;
    std::memcpy(host, o->pinned, n * elem);
    return true;
}

void vtk_thread(int device, OutputState* o, VtkJob job)
{
    cudaSetDevice(device);
    FILE* fp = std::fopen(job.path.c_str(), "wb");
    if (!fp) {
        o->rc = LBFFS_E_ARG;
        o->msg = "lbffs_write_vtk: cannot open " + job.path;
        return;
    }
    const size_t E = (size_t)job.nx * job.ny * job.nz;
    std::string head;
    char buf[256];
    head += "# vtk DataFile Version 3.0\n";
    head += "vtk output\n";
    head += job.binary ? "BINARY\n" : "ASCII\n";
    head += "DATASET STRUCTURED_POINTS\n";
    std::snprintf(buf, sizeof buf, "DIMENSIONS %d %d %d\n", job.nx, job.ny, job.nz);
    head += buf;
    head += "ORIGIN 0 0 0\n";
    std::snprintf(buf, sizeof buf, "SPACING %g %g %g\n\n", (double)job.L, (double)job.L, (double)job.L);
    head += buf;
    std::snprintf(buf, sizeof buf, "POINT_DATA %zu\n", E);
    head += buf;
    bool ok = std::fwrite(head.data(), 1, head.size(), fp) == head.size();
    const size_t chunk = o->chunk;
    std::vector<unsigned char> raw(chunk * 4);
    std::string out;
    out.reserve(job.binary ? chunk * 4 : chunk * 14);
    for (const VtkField& fd : job.fields) {
        if (!ok) break;
        const std::string h = std::string("SCALARS ") + fd.name + " float\nLOOKUP_TABLE default\n";
        ok = std::fwrite(h.data(), 1, h.size(), fp) == h.size();
        const size_t elem = fd.kind == 2 ? 1 : 4;
        for (size_t off = 0; off < E && ok; off += chunk) {
            const size_t n = std::min(chunk, E - off);
            if (fd.dev) {
                if (!fetch(o, fd.dev, elem, off, n, raw.data())) {
                    ok = false;
                    o->rc = LBFFS_E_CUDA;
                    o->msg = "lbffs_write_vtk: device copy failed";
                    break;
                }
            } else {
                std::memset(raw.data(), 0, n * elem);
            }
            out.clear();
            for (size_t t = 0; t < n; t++) {
                if (fd.kind == 1) {
                    int x;
                    std::memcpy(&x, raw.data() + 4 * t, 4);
                    if (job.binary) put_binary(out, (float)x);
                    else put_ascii_int(out, x);
                    continue;
                }
                float x;
                if (fd.kind == 2) x = (float)raw[t];
                else std::memcpy(&x, raw.data() + 4 * t, 4);
                float y;
                switch (fd.op) {
                    case 1: y = x * job.c; break;
                    case 2: {
                        const float nu_sgs = 3.f * x * job.L * job.c;
                        y = 3.f * nu_sgs;
                        break;
                    }
                    case 3: y = x * job.L; break;
                    case 4: y = x * job.c / job.time_mean; break;
                    default: y = x;
                }
                if (job.binary) put_binary(out, y);
                else put_ascii(out, (double)y);
            }
            ok = std::fwrite(out.data(), 1, out.size(), fp) == out.size();
        }
        if (ok) ok = std::fputc('\n', fp) != EOF;
    }
    if (std::fclose(fp) != 0) ok = false;
    if (!ok && o->rc == LBFFS_OK) {
        o->rc = LBFFS_E_ARG;
        o->msg = "lbffs_write_vtk: write to " + job.path + " failed";
    }
}

void restart_thread(int device, OutputState* o, RestartJob job)
{
    cudaSetDevice(device);
    FILE* fp = std::fopen(job.path.c_str(), "wb");
    if (!fp) {
        o->rc = LBFFS_E_ARG;
        o->msg = "lbffs_write_restart: cannot open " + job.path;
        return;
    }
    const int head[4] = {job.nt, job.nx, job.ny, job.nz};
    bool ok = std::fwrite(head, sizeof(int), 4, fp) == 4;
    const long long nx = job.nx, rows = (long long)job.Q * job.ny * job.nz;
    const long long crow = (long long)(o->chunk / (size_t)nx);
    for (long long r = 0; r < rows && ok; r += crow) {
        const long long n = std::min(crow, rows - r);
        const size_t cnt = (size_t)(n * nx);
        if (decode_f(job.storage, job.Q, o->f_snap, o->stage, r, n, job.pg, o->io) != cudaSuccess ||
            cudaMemcpyAsync(o->pinned, o->stage, cnt * sizeof(float), cudaMemcpyDeviceToHost, o->io) != cudaSuccess ||
            cudaStreamSynchronize(o->io) != cudaSuccess) {
            o->rc = LBFFS_E_CUDA;
            o->msg = "lbffs_write_restart: device copy failed";
            ok = false;
            break;
        }
        ok = std::fwrite(o->pinned, sizeof(float), cnt, fp) == cnt;
    }
    if (std::fclose(fp) != 0) ok = false;
    if (!ok && o->rc == LBFFS_OK) {
        o->rc = LBFFS_E_ARG;
        o->msg = "lbffs_write_restart: write to " + job.path + " failed";
    }
}

}  // namespace

int ctx_io_wait(lbffs_ctx* c)
{
    OutputState* o = c->out;
    if (!o || !o->running) return LBFFS_OK;
    o->th.join();
    o->running = false;
    const int rc = o->rc;
    o->rc = LBFFS_OK;
    if (rc != LBFFS_OK) return ctx_fail(c, rc, o->msg);
    return LBFFS_OK;
}

float* ctx_output_field(lbffs_ctx* c, int field, bool create)
{
    if (!c->out && !create) return nullptr;
    OutputState* o = state(c);
    float** p = nullptr;
    if (field >= LBFFS_OUT_RHO && field <= LBFFS_OUT_W) p = &o->fld[field - LBFFS_OUT_RHO];
    else if (field >= LBFFS_UMEAN && field <= LBFFS_WMEAN) p = &o->mean[field - LBFFS_UMEAN];
    if (!p) return nullptr;
    if (!*p && create && ctx_alloc(c, p, (size_t)c->E) != cudaSuccess) *p = nullptr;
    return *p;
}

void ctx_output_release(lbffs_ctx* c)
{
    OutputState* o = c->out;
    if (!o) return;
    if (o->running) o->th.join();
    for (float* p : o->fld) ctx_free(c, p);
    for (float* p : o->g) ctx_free(c, p);
    for (float* p : o->mean) ctx_free(c, p);
    ctx_free(c, o->tau);
    ctx_free(c, o->f_snap);
    ctx_free(c, o->partial);
    ctx_free(c, o->d_uave);
    ctx_free(c, o->stage);
    if (o->pinned) cudaFreeHost(o->pinned);
    if (o->ready) cudaEventDestroy(o->ready);
    if (o->io) cudaStreamDestroy(o->io);
    delete o;
    c->out = nullptr;
}

}  // namespace lbffs

using namespace lbffs;

extern "C" int lbffs_output(lbffs_ctx* c, const lbffs_output_params* p, lbffs_output_result* r)
{
    if (!c || !p || !r) return ctx_fail(c, LBFFS_E_ARG, "lbffs_output: null argument");
    if (p->out_interval < 0) return ctx_fail(c, LBFFS_E_ARG, "lbffs_output: out_interval must be >= 0");
    int rc = ctx_io_wait(c);  // the writer may still read the previous output's fields
    if (rc != LBFFS_OK) return rc;
    OCK(cudaSetDevice(c->d.device));
    OutputState* o = state(c);
    const size_t E = (size_t)c->E;
    for (auto& fp : o->fld)
        if (!fp) OCK(ctx_alloc(c, &fp, E));
    if (!o->tau) OCK(ctx_alloc(c, &o->tau, E));
    if (p->out_interval > 0)
        for (auto& mp : o->mean)
            if (!mp) OCK(ctx_alloc(c, &mp, E));
    if (!o->partial) {
        o->nblocks = std::max(1, c->nsm) * 8;
        OCK(ctx_alloc(c, &o->partial, (size_t)o->nblocks * OUT_NP));
        OCK(ctx_alloc(c, &o->d_uave, 1));
    }
    const bool gf = p->force_coeffs && c->g[0];
    if (gf)
        for (auto& gp : o->g)
            if (!gp) OCK(ctx_alloc(c, &gp, E));
    const float* fw[3] = {nullptr, nullptr, nullptr};
    const float* gg[3] = {nullptr, nullptr, nullptr};
    if (p->force_coeffs)
        for (int a = 0; a < 3; a++) {
            fw[a] = c->fw[a];
            gg[a] = c->g[a];
        }
    OCK(launch_output(c, o, p->dpdx, p->out_interval, fw, gg));
    OCK(cudaMemcpyAsync(o->tau, c->macro[c->mcur][4], E * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    if (gf)
        for (int a = 0; a < 3; a++)
            OCK(cudaMemcpyAsync(o->g[a], c->g[a], E * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    o->g_valid = gf;
    k_uave<<<1, 1024, 0, c->stream>>>(o->fld[1], c->d.nx, c->d.ny, c->d.nz, p->c, o->d_uave);
    OCK(cudaGetLastError());
    std::vector<double> part((size_t)o->nblocks * OUT_NP);
    float uave = 0.f;
    OCK(cudaMemcpyAsync(part.data(), o->partial, part.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    OCK(cudaMemcpyAsync(&uave, o->d_uave, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    OCK(cudaStreamSynchronize(c->stream));
    double s[OUT_NP] = {0, 0, -INFINITY, INFINITY, 0, 0, 0, 0, 0, 0};
    for (int b = 0; b < o->nblocks; b++)
        for (int k = 0; k < OUT_NP; k++) {
            const double x = part[(size_t)b * OUT_NP + k];
            s[k] = k == 2 ? std::max(s[k], x) : k == 3 ? std::min(s[k], x) : s[k] + x;
        }
    // rho_av = rho_av_tmp / float(eleFluid) + 1.f, stored as float (write.hpp:47)
    const long long nf = (long long)s[1];
    r->n_fluid = nf;
    r->rho_av = (float)(s[0] / (double)(float)nf + 1.0);
    r->rho_max = (float)s[2];
    r->rho_min = (float)s[3];
    r->u_ave = uave;
    for (int a = 0; a < 3; a++) {
        r->fw[a] = s[4 + a];
        r->g_ibm[a] = s[7 + a];
    }
    if (p->out_interval > 0) o->time_mean += (float)p->out_interval;
    r->time_mean = o->time_mean;
    o->have_output = true;
    return LBFFS_OK;
}

extern "C" int lbffs_write_vtk(lbffs_ctx* c, const char* path, int binary, const lbffs_output_params* p)
{
    if (!c || !path || !p) return ctx_fail(c, LBFFS_E_ARG, "lbffs_write_vtk: null argument");
    int rc = ctx_io_wait(c);
    if (rc != LBFFS_OK) return rc;
    OutputState* o = c->out;
    if (!o || !o->have_output) return ctx_fail(c, LBFFS_E_STATE, "lbffs_write_vtk: call lbffs_output first");
    OCK(cudaSetDevice(c->d.device));
    OCK(ensure_io(c, o));
    VtkJob job;
    job.path = path;
    job.binary = binary != 0;
    job.c = p->c;
    job.L = p->L;
    job.time_mean = o->time_mean;
    job.nx = c->d.nx;
    job.ny = c->d.ny;
    job.nz = c->d.nz;
    const void* g0 = o->g_valid ? o->g[0] : nullptr;
    const void* g1 = o->g_valid ? o->g[1] : nullptr;
    const void* g2 = o->g_valid ? o->g[2] : nullptr;
    job.fields = {{"u", o->fld[1], 0, 1},          {"v", o->fld[2], 0, 1},          {"w", o->fld[3], 0, 1},
                  {"rho", o->fld[0], 0, 0},        {"nuSGS", o->tau, 0, 2},         {"boundary1", c->iarr[1], 1, 0},
                  {"boundary2", c->iarr[2], 1, 0}, {"boundary3", c->iarr[3], 1, 0}, {"sdf", c->sdf, 0, 3},
                  {"solid", c->solid, 2, 0},       {"neiSolid", c->nei, 2, 0},      {"GxIBM", g0, 0, 0},
                  {"GyIBM", g1, 0, 0},             {"GzIBM", g2, 0, 0},             {"omega", c->omega, 0, 0},
                  {"uMean", o->mean[0], 0, 4},     {"vMean", o->mean[1], 0, 4},     {"wMean", o->mean[2], 0, 4}};
    // the I/O stream's copies start after the work already queued on the compute stream
    OCK(cudaEventRecord(o->ready, c->stream));
    OCK(cudaStreamWaitEvent(o->io, o->ready, 0));
    o->rc = LBFFS_OK;
    o->th = std::thread(vtk_thread, c->d.device, o, std::move(job));
    o->running = true;
    return LBFFS_OK;
}

extern "C" int lbffs_write_restart(lbffs_ctx* c, const char* path, int nt)
{
    if (!c || !path) return ctx_fail(c, LBFFS_E_ARG, "lbffs_write_restart: null argument");
    int rc = ctx_io_wait(c);
    if (rc != LBFFS_OK) return rc;
    OCK(cudaSetDevice(c->d.device));
    OutputState* o = state(c);
    OCK(ensure_io(c, o));
    const size_t bytes = (size_t)c->pg.pE * c->tsize * (size_t)c->Q;
    if (!o->f_snap) OCK(ctx_alloc_bytes(c, &o->f_snap, bytes));
    // the populations of this step, copied on the compute stream before a later step overwrites them
    OCK(cudaMemcpyAsync(o->f_snap, c->f[c->fcur], bytes, cudaMemcpyDeviceToDevice, c->stream));
    OCK(cudaEventRecord(o->ready, c->stream));
    OCK(cudaStreamWaitEvent(o->io, o->ready, 0));
    RestartJob job{path, nt, c->d.nx, c->d.ny, c->d.nz, c->Q, c->d.storage, c->pg};
    o->rc = LBFFS_OK;
    o->th = std::thread(restart_thread, c->d.device, o, std::move(job));
    o->running = true;
    return LBFFS_OK;
}

extern "C" int lbffs_read_restart(lbffs_ctx* c, const char* path, int* nt)
{
    if (!c || !path || !nt) return ctx_fail(c, LBFFS_E_ARG, "lbffs_read_restart: null argument");
    int rc = ctx_io_wait(c);
    if (rc != LBFFS_OK) return rc;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return ctx_fail(c, LBFFS_E_ARG, std::string("lbffs_read_restart: cannot open ") + path);
    int head[4];
    if (std::fread(head, sizeof(int), 4, fp) != 4) {
        std::fclose(fp);
        return ctx_fail(c, LBFFS_E_ARG, "lbffs_read_restart: short header");
    }
    if (head[1] != c->d.nx || head[2] != c->d.ny || head[3] != c->d.nz) {
        std::fclose(fp);
        return ctx_fail(c, LBFFS_E_ARG, "lbffs_read_restart: grid " + std::to_string(head[1]) + "x" +
                                            std::to_string(head[2]) + "x" + std::to_string(head[3]) +
                                            " does not match the context");
    }
    std::vector<float> f((size_t)c->E * c->Q);
    const size_t got = std::fread(f.data(), sizeof(float), f.size(), fp);
    std::fclose(fp);
    if (got != f.size()) return ctx_fail(c, LBFFS_E_ARG, "lbffs_read_restart: short population data");
    rc = lbffs_upload(c, LBFFS_F, f.data(), f.size() * sizeof(float));
    if (rc != LBFFS_OK) return rc;
    *nt = head[0];
    return LBFFS_OK;
}

extern "C" int lbffs_io_wait(lbffs_ctx* c)
{
    if (!c) return ctx_fail(c, LBFFS_E_ARG, "lbffs_io_wait: null argument");
    return ctx_io_wait(c);
}

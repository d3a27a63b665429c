// C-ABI implementation (include/lbffs_cuda.h): context lifetime, field transfer,
// geometry commit, the step loop and reductions.  Host code only; kernels live in
// step_inst.cu / step_dispatch.cu, setup.cu and ibm.cu.
#include <climits>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"

using namespace lbffs;

namespace {

thread_local std::string g_thread_error = "no error";

enum FieldKind { K_F, K_INT, K_U8, K_FLOAT, K_MACRO };

struct FieldInfo {
    FieldKind kind;
    int macro;  // index into the macro buffers for K_MACRO
};

FieldInfo field_info(int f)
{
    switch (f) {
        case LBFFS_F: return {K_F, -1};
        case LBFFS_BOUNDARY:
        case LBFFS_BOUNDARY1:
        case LBFFS_BOUNDARY2:
        case LBFFS_BOUNDARY3: return {K_INT, -1};
        case LBFFS_SOLID:
        case LBFFS_NEISOLID: return {K_U8, -1};
        case LBFFS_RHO: return {K_MACRO, 0};
        case LBFFS_U: return {K_MACRO, 1};
        case LBFFS_V: return {K_MACRO, 2};
        case LBFFS_W: return {K_MACRO, 3};
        case LBFFS_TAUSGS: return {K_MACRO, 4};
        default: return {K_FLOAT, -1};
    }
}

}  // namespace

static int fail(lbffs_ctx* c, int code, const std::string& msg)
{
    if (c) c->err = msg;
    g_thread_error = msg;
    return code;
}

void lbffs::set_thread_error(const std::string& msg) { g_thread_error = msg; }

int lbffs::ctx_fail(lbffs_ctx* c, int code, const std::string& msg) { return fail(c, code, msg); }

#define CK(call)                                                                                      \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return fail(c, LBFFS_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));         \
    } while (0)

cudaError_t lbffs::ctx_alloc_bytes(lbffs_ctx* c, void** p, size_t bytes)
{
    *p = nullptr;
    if (c->arena) {
        *p = c->arena->alloc(bytes);
        if (!*p) return cudaErrorMemoryAllocation;
        return cudaMemsetAsync(*p, 0, bytes, c->stream);
    }
    // zeroed on the context's stream: the context's streams are non-blocking, so a memset on the
    // legacy default stream would not be ordered before the kernels that fill the buffer next
    // (a special list built right after its allocation was intermittently zeroed under it)
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, bytes, c->stream);
    return e;
}

void lbffs::ctx_free(lbffs_ctx* c, void* p)
{
    if (!p) return;
    if (c->arena && c->arena->owns(p)) c->arena->release(p);
    else cudaFree(p);
}

template <class T>
static cudaError_t dalloc(lbffs_ctx* c, T** p, size_t n)
{
    return ctx_alloc(c, p, n);
}

static size_t field_bytes(const lbffs_ctx* c, int f)
{
    FieldInfo fi = field_info(f);
    switch (fi.kind) {
        case K_F: return sizeof(float) * (size_t)c->Q * (size_t)c->E;
        case K_U8: return (size_t)c->E;
        default: return 4 * (size_t)c->E;
    }
}

static void* field_ptr(lbffs_ctx* c, int f)
{
    switch (f) {
        case LBFFS_BOUNDARY: return c->iarr[0];
        case LBFFS_BOUNDARY1: return c->iarr[1];
        case LBFFS_BOUNDARY2: return c->iarr[2];
        case LBFFS_BOUNDARY3: return c->iarr[3];
        case LBFFS_SOLID: return c->solid;
        case LBFFS_NEISOLID: return c->nei;
        case LBFFS_SDF: return c->sdf;
        case LBFFS_U0: return c->u0;
        case LBFFS_V0: return c->v0;
        case LBFFS_W0: return c->w0;
        case LBFFS_OMEGA: return c->omega;
        case LBFFS_FWX: return c->fw[0];
        case LBFFS_FWY: return c->fw[1];
        case LBFFS_FWZ: return c->fw[2];
        case LBFFS_GXIBM: return c->g[0];
        case LBFFS_GYIBM: return c->g[1];
        case LBFFS_GZIBM: return c->g[2];
        case LBFFS_OUT_RHO:
        case LBFFS_OUT_U:
        case LBFFS_OUT_V:
        case LBFFS_OUT_W:
        case LBFFS_UMEAN:
        case LBFFS_VMEAN:
        case LBFFS_WMEAN: return ctx_output_field(c, f, false);
        default: return nullptr;
    }
}

static bool geometry_field(int f)
{
    return f == LBFFS_BOUNDARY || f == LBFFS_BOUNDARY1 || f == LBFFS_BOUNDARY2 || f == LBFFS_BOUNDARY3 ||
           f == LBFFS_SOLID || f == LBFFS_NEISOLID || f == LBFFS_SDF || f == LBFFS_OMEGA;
}

extern "C" const char* lbffs_last_error(const lbffs_ctx* c) { return c ? c->err.c_str() : g_thread_error.c_str(); }

extern "C" int lbffs_destroy(lbffs_ctx* c)
{
    if (!c) return LBFFS_OK;
    cudaSetDevice(c->d.device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    ctx_output_release(c);
    void* ptrs[] = {c->f[0], c->f[1], c->iarr[0], c->iarr[1], c->iarr[2], c->iarr[3], c->solid, c->nei, c->flags,
                    c->bc, c->u0, c->v0, c->w0, c->omega, c->sdf, c->fw[0], c->fw[1], c->fw[2], c->g[0], c->g[1],
                    c->g[2], c->special, c->d_err, c->partial, c->markers, c->gm, c->ibm_acc,
                    c->ibm_lag, c->ibm_box, c->ibm_t};
    for (void* p : ptrs) ctx_free(c, p);
    if (c->own_stage) ctx_free(c, c->stage);
    for (auto& row : c->macro)
        for (float* p : row) ctx_free(c, p);
    for (auto& e : c->pending) {
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    for (auto e : c->pool) cudaEventDestroy(e);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->side_lo) cudaStreamDestroy(c->side_lo);
    for (auto s : c->copy_st)
        if (s) cudaStreamDestroy(s);
    for (auto e : c->copy_ev)
        if (e) cudaEventDestroy(e);
    if (c->fork_ev) cudaEventDestroy(c->fork_ev);
    if (c->join_ev) cudaEventDestroy(c->join_ev);
    if (c->stream && c->own_stream) cudaStreamDestroy(c->stream);
    delete c;
    return LBFFS_OK;
}

int lbffs::ctx_create(const lbffs_desc* desc, Arena* arena, cudaStream_t stream, float* stage, size_t stage_elems,
                      lbffs_ctx** out)
{
    lbffs_ctx* c = nullptr;
    if (!desc || !out) return fail(c, LBFFS_E_ARG, "lbffs_create: null argument");
    *out = nullptr;
    const lbffs_desc& d = *desc;
    if (d.nx < 1 || d.ny < 1 || d.nz < 1 || d.ny > 65535 || d.nz > 65535)
        return fail(c, LBFFS_E_ARG, "lbffs_create: grid extents must be >= 1 and ny, nz <= 65535");
    if (d.q != 19 && d.q != 27) return fail(c, LBFFS_E_ARG, "lbffs_create: q must be 19 or 27");
    if (d.storage < LBFFS_FP32 || d.storage > LBFFS_BF16S) return fail(c, LBFFS_E_ARG, "lbffs_create: bad storage");
    if (d.collision != LBFFS_COLL_RR && d.collision != LBFFS_COLL_CUMULANT)
        return fail(c, LBFFS_E_ARG, "lbffs_create: bad collision");
    if (d.q == 19 && d.collision == LBFFS_COLL_CUMULANT)
        return fail(c, LBFFS_E_ARG, "lbffs_create: the cumulant operator is D3Q27 only");
    if (d.sgs != LBFFS_SGS_SMAGORINSKY && d.sgs != LBFFS_SGS_WALE) return fail(c, LBFFS_E_ARG, "lbffs_create: bad sgs");
    if (d.wall != LBFFS_WALL_BB && d.wall != LBFFS_WALL_IBB) return fail(c, LBFFS_E_ARG, "lbffs_create: bad wall");
    if (!(d.cs > 0.f)) return fail(c, LBFFS_E_ARG, "lbffs_create: cs must be > 0");
    if (d.damping < LBFFS_DAMP_WALL || d.damping > LBFFS_DAMP_NONE)
        return fail(c, LBFFS_E_ARG, "lbffs_create: bad damping");
    const long long E = (long long)d.nx * d.ny * d.nz;
    if (E >= (1LL << 31)) return fail(c, LBFFS_E_ARG, "lbffs_create: more than 2^31 - 1 cells");
    // padded planes: one ghost cell on every side, rows starting on 32-byte sectors
    const int tsize = d.storage == LBFFS_FP32 ? 4 : 2;
    const long long A = 32 / tsize;
    const long long px = ((A + d.nx + 1 + A - 1) / A) * A;
    const long long pxy = px * (d.ny + 2), pE = pxy * (d.nz + 2);
    if (pE >= (1LL << 31))
        return fail(c, LBFFS_E_ARG, "lbffs_create: more than 2^31 - 1 cells including the ghost layer");

    c = new lbffs_ctx();
    c->d = d;
    c->Q = d.q;
    c->E = E;
    c->tsize = tsize;
    c->pg = PadGeom{d.nx, d.ny, d.nz, (int)px, (int)pxy, (int)(pxy + px + A), pE};
    c->arena = arena;
    cudaError_t e = cudaSetDevice(d.device);
    if (e != cudaSuccess) {
        int r = fail(c, LBFFS_E_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
        lbffs_destroy(c);
        return r;
    }
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, d.device);
    c->nsm = nsm > 0 ? nsm : 1;
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, d.device);
    c->l2_bytes = l2;
#define CKC(call)                                                                                          \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess) {                                                                           \
            int r_ = fail(c, LBFFS_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));            \
            g_thread_error = c->err;                                                                       \
            lbffs_destroy(c);                                                                              \
            return r_;                                                                                     \
        }                                                                                                  \
    } while (0)
    if (stream) {
        c->stream = stream;
        c->own_stream = false;
    } else {
        CKC(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    }
    const size_t qe = (size_t)c->Q * (size_t)E;
    const size_t qpe = (size_t)c->Q * (size_t)pE;
    for (int b = 0; b < 2; b++) CKC(ctx_alloc_bytes(c, &c->f[b], qpe * c->tsize + 16));
    for (int b = 0; b < 4; b++) CKC(dalloc(c, &c->iarr[b], E));
    CKC(dalloc(c, &c->solid, E));
    CKC(dalloc(c, &c->nei, E));
    CKC(dalloc(c, &c->flags, E));
    CKC(dalloc(c, &c->bc, E));
    CKC(dalloc(c, &c->u0, E));
    CKC(dalloc(c, &c->v0, E));
    CKC(dalloc(c, &c->w0, E));
    CKC(dalloc(c, &c->omega, E));
    CKC(dalloc(c, &c->sdf, E));
    for (auto& row : c->macro)
        for (float*& p : row) CKC(dalloc(c, &p, E));
    for (int a = 0; a < 3; a++) CKC(dalloc(c, &c->fw[a], E));
    CKC(dalloc(c, &c->d_err, 1));
    if (stage) {
        c->stage = stage;
        c->stage_elems = stage_elems;
        c->own_stage = false;
    } else {
        c->stage_elems = (size_t)16 << 20;  // 64 MB float staging for population conversion, whole rows
        if (c->stage_elems < (size_t)d.nx) c->stage_elems = (size_t)d.nx;
        if (c->stage_elems > qe) c->stage_elems = qe;
        CKC(dalloc(c, &c->stage, c->stage_elems));
    }
    c->partial_blocks = 4 * c->nsm;
    CKC(dalloc(c, &c->partial, (size_t)3 * c->partial_blocks));
    CKC(fill_f32(c->sdf, 10000.f, E, c->stream));
    CKC(fill_f32(c->omega, 1.f, E, c->stream));
    CKC(cudaStreamSynchronize(c->stream));
#undef CKC
    *out = c;
    return LBFFS_OK;
}

size_t lbffs::ctx_footprint(const lbffs_desc& d)
{
    const size_t E = (size_t)d.nx * d.ny * d.nz;
    const size_t tsize = d.storage == LBFFS_FP32 ? 4 : 2;
    const size_t A = 32 / tsize;
    const size_t px = ((A + d.nx + 1 + A - 1) / A) * A;
    const size_t pE = px * (d.ny + 2) * (d.nz + 2);
    auto blk = [](size_t b) { return (b + 16 + Arena::kAlign - 1) / Arena::kAlign * Arena::kAlign; };
    size_t t = 2 * blk((size_t)d.q * pE * tsize);
    t += 4 * blk(4 * E);                       // boundary codes
    t += 3 * blk(E) + blk(2 * E);              // solid, neiSolid, flags, bc
    t += 5 * blk(4 * E);                       // u0, v0, w0, omega, sdf
    t += 10 * blk(4 * E) + 3 * blk(4 * E);     // macroscopics x 2, Fw
    t += blk(4 * E) + blk(E);                  // special list (worst case), classify scratch
    t += blk(64 * 1024);                       // error word, partial sums, compaction counters
    return t;
}

extern "C" int lbffs_create(const lbffs_desc* desc, lbffs_ctx** out)
{
    return ctx_create(desc, nullptr, nullptr, nullptr, 0, out);
}

// IBM forcing fields (GxIBM..), allocated when markers or an upload first need them
static cudaError_t ensure_g(lbffs_ctx* c)
{
    for (int a = 0; a < 3; a++)
        if (!c->g[a]) {
            cudaError_t e = dalloc(c, &c->g[a], c->E);
            if (e != cudaSuccess) return e;
        }
    return cudaSuccess;
}

// Compact list (ascending cell order) of the fluid cells whose flags intersect mask.
static int build_list(lbffs_ctx* c, uint8_t mask, uint32_t** list, long long* n)
{
    const long long E = c->E;
    const long long nb = (E + SETUP_CHUNK - 1) / SETUP_CHUNK;
    unsigned* d_counts = nullptr;
    unsigned long long* d_off = nullptr;
    CK(ctx_alloc_bytes(c, (void**)&d_counts, sizeof(unsigned) * nb));
    cudaError_t e = setup_count_special(c->flags, E, mask, d_counts, c->stream);
    std::vector<unsigned> counts(nb);
    std::vector<unsigned long long> off(nb);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(counts.data(), d_counts, sizeof(unsigned) * nb, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    unsigned long long total = 0;
    for (long long b = 0; b < nb; b++) {
        off[b] = total;
        total += counts[b];
    }
    if (e == cudaSuccess) e = ctx_alloc_bytes(c, (void**)&d_off, sizeof(unsigned long long) * nb);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_off, off.data(), sizeof(unsigned long long) * nb, cudaMemcpyHostToDevice, c->stream);
    if (*list) {
        ctx_free(c, *list);
        *list = nullptr;
    }
    if (e == cudaSuccess) e = ctx_alloc_bytes(c, (void**)list, sizeof(uint32_t) * (total + 1));
    if (e == cudaSuccess) e = setup_scatter_special(c->flags, E, mask, d_off, *list, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    ctx_free(c, d_counts);
    ctx_free(c, d_off);
    CK(e);
    *n = (long long)total;
    return LBFFS_OK;
}

static int commit(lbffs_ctx* c)
{
    const int nx = c->d.nx, ny = c->d.ny, nz = c->d.nz;
    c->xghost_ok = false;
    const long long E = c->E;
    // validate boundary codes on the device
    {
        int* chk = nullptr;
        CK(ctx_alloc_bytes(c, (void**)&chk, 2 * sizeof(int)));
        int init[2] = {0, INT_MIN}, res[2];
        cudaError_t e = cudaMemcpyAsync(chk, init, sizeof(init), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = setup_check_codes(c->iarr[1], c->iarr[2], c->iarr[3], E, chk, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(res, chk, sizeof(res), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        ctx_free(c, chk);
        CK(e);
        if (res[0] & 2) return fail(c, LBFFS_E_ARG, "invalid boundary code " + std::to_string(res[1]));
    }
    // sponge zone face-centre codes (tauSpongeZone, kernel.cl:2447-2501)
    for (int b = 1; b <= 3; b++) {
        const long long cen[2] = {b == 1   ? ((long long)(nz / 2) * ny + ny / 2) * nx + 0
                                  : b == 2 ? ((long long)(nz / 2) * ny + 0) * nx + nx / 2
                                           : ((long long)0 * ny + ny / 2) * nx + nx / 2,
                                  b == 1   ? ((long long)(nz / 2) * ny + ny / 2) * nx + nx - 1
                                  : b == 2 ? ((long long)(nz / 2) * ny + ny - 1) * nx + nx / 2
                                           : ((long long)(nz - 1) * ny + ny / 2) * nx + nx / 2};
        for (int s = 0; s < 2; s++) {
            int v = 0;
            CK(cudaMemcpyAsync(&v, c->iarr[b] + cen[s], sizeof(int), cudaMemcpyDeviceToHost, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            const int bit = 2 * (b - 1) + s;
            if (v == BC_OUTLET || v == BC_FIXDEN) c->sponge_mask |= (1 << bit);
            else c->sponge_mask &= ~(1 << bit);
            c->face_codes = (c->face_codes & ~(7 << (3 * bit))) | ((v & 7) << (3 * bit));
        }
    }
    // one boundary code per face and axis (the codes just read) and the face flag on exactly the
    // border cells: the step kernels can then pull across the border without a ghost layer
    {
        int* bad = nullptr;
        CK(ctx_alloc_bytes(c, (void**)&bad, sizeof(int)));
        int h = 0;
        cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(int), c->stream);
        if (e == cudaSuccess)
            e = setup_check_faces(c->iarr[0], c->iarr[1], c->iarr[2], c->iarr[3], c->face_codes, nx, ny, nz, bad,
                                  c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h, bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        ctx_free(c, bad);
        CK(e);
        c->face_ok = h == 0;
        // mode 1: both x faces are boundary-kernel faces and the bulk kernels cross only y / z faces;
        // modes 3 and 2: x-face bulk cells take their x-crossing pulls through ghost slots they write
        // themselves (no Cyclic x face: the value is the cell's own) or from per-context plane bases
        // (where that kernel is built).  A 2D grid with a wall code on its z faces keeps the ghost
        // layer: there its x-face cells are face cells for the z-crossing directions where their row
        // neighbours are not, so a pair's shared c_x = 0 pull would not hold; with Cyclic (or outlet)
        // z codes every cell of a row takes those directions alike.
        auto kernel_face = [](int code) {
            return code == BC_OUTLET || code == BC_FIXVEL || code == BC_FIXDEN || code == BC_WALLFN;
        };
        const bool x_kernel = kernel_face(c->face_codes & 7) && kernel_face((c->face_codes >> 3) & 7);
        const bool x_cyclic = (c->face_codes & 7) == BC_CYCLIC || ((c->face_codes >> 3) & 7) == BC_CYCLIC;
        const bool x_pulls = xface_pulls_built(c->Q, c->d.storage == LBFFS_FP32 ? ST_FP32 : ST_FP16S);
        const bool z_wall = is_wall_code((c->face_codes >> 12) & 7) || is_wall_code((c->face_codes >> 15) & 7);
        c->pull_mode = !(LBFFS_BORDER_PULLS && c->face_ok) ? 0
                       : x_kernel                            ? 1
                       : nz <= 1 && z_wall                   ? 0
                       : !x_cyclic                           ? 3
                       : x_pulls                             ? 2
                                                             : 0;
        c->pull_ok = c->pull_mode != 0;
    }
    // uniform relaxation rate: the value at the domain centre
    const long long centre = ((long long)(nz / 2) * ny + ny / 2) * nx + nx / 2;
    CK(cudaMemcpyAsync(&c->omega0, c->omega + centre, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));

    CK(setup_pack_bc(c->iarr[0], c->iarr[1], c->iarr[2], c->iarr[3], c->bc, nx, ny, nz, c->stream));
    uint8_t* scratch = nullptr;
    CK(ctx_alloc_bytes(c, (void**)&scratch, E));
    cudaError_t e = setup_classify(c->Q, c->bc, c->solid, c->nei, c->sdf, c->omega, c->omega0, c->d.cs,
                                   c->d.damping, c->flags, scratch, nx, ny, nz, c->stream);
    cudaStreamSynchronize(c->stream);
    ctx_free(c, scratch);
    CK(e);

    {
        int r = build_list(c, FL_SPECIAL, &c->special, &c->n_special);
        if (r != LBFFS_OK) return r;
    }

    // per-class counts (on the device) and zeroed link forces
    {
        unsigned long long* cnt = nullptr;
        CK(ctx_alloc_bytes(c, (void**)&cnt, 4 * sizeof(unsigned long long)));
        unsigned long long h[4] = {0, 0, 0, 0};
        cudaError_t e = cudaMemsetAsync(cnt, 0, 4 * sizeof(unsigned long long), c->stream);
        if (e == cudaSuccess) e = setup_count_flags(c->flags, E, cnt, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        ctx_free(c, cnt);
        CK(e);
        for (int k = 0; k < 4; k++) c->counts[k] = (long long)h[k];
    }
    for (int a = 0; a < 3; a++) CK(cudaMemsetAsync(c->fw[a], 0, sizeof(float) * E, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->dirty = false;
    return LBFFS_OK;
}

// Population q of an FP32 context between the reference's dense host layout (f[q * E + ic]) and
// the padded device planes of the current copy (upload: into copy 0), as one pitched 3-D copy:
// rows of nx floats, the device rows px apart and its planes pxy apart.
static cudaError_t copy_plane_f32(lbffs_ctx* c, int q, const float* host_in, bool upload, cudaStream_t st)
{
    const PadGeom& g = c->pg;
    float* dev = static_cast<float*>(upload ? c->f[0] : c->f[c->fcur]) + (size_t)q * (size_t)g.pE + g.porg;
    float* h = const_cast<float*>(host_in) + (size_t)q * (size_t)c->E;
    cudaMemcpy3DParms p = {};
    const cudaPitchedPtr dp = make_cudaPitchedPtr(dev, (size_t)g.px * sizeof(float), (size_t)g.nx, (size_t)g.ny + 2);
    const cudaPitchedPtr hp = make_cudaPitchedPtr(h, (size_t)g.nx * sizeof(float), (size_t)g.nx, (size_t)g.ny);
    p.srcPtr = upload ? hp : dp;
    p.dstPtr = upload ? dp : hp;
    p.extent = make_cudaExtent((size_t)g.nx * sizeof(float), (size_t)g.ny, (size_t)g.nz);
    p.kind = upload ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    return cudaMemcpy3DAsync(&p, st);
}

// The Q plane copies of an FP32 population transfer, LBFFS_COPY_STREAMS of them in flight at once
// (each copy engine moves one pitched copy at a time), ordered after and joined back into the
// context's stream.
static cudaError_t copy_planes_f32(lbffs_ctx* c, const float* host, bool upload)
{
    cudaError_t e = cudaSuccess;
    if (LBFFS_COPY_STREAMS > 1 && !c->copy_st[0]) {
        for (int k = 0; k < LBFFS_COPY_STREAMS && e == cudaSuccess; k++)
            e = cudaStreamCreateWithFlags(&c->copy_st[k], cudaStreamNonBlocking);
        for (int k = 0; k <= LBFFS_COPY_STREAMS && e == cudaSuccess; k++)
            e = cudaEventCreateWithFlags(&c->copy_ev[k], cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
    }
    if (LBFFS_COPY_STREAMS <= 1) {
        for (int q = 0; q < c->Q && e == cudaSuccess; q++) e = copy_plane_f32(c, q, host, upload, c->stream);
        return e;
    }
    e = cudaEventRecord(c->copy_ev[LBFFS_COPY_STREAMS], c->stream);
    for (int k = 0; k < LBFFS_COPY_STREAMS && e == cudaSuccess; k++)
        e = cudaStreamWaitEvent(c->copy_st[k], c->copy_ev[LBFFS_COPY_STREAMS], 0);
    for (int q = 0; q < c->Q && e == cudaSuccess; q++)
        e = copy_plane_f32(c, q, host, upload, c->copy_st[q % LBFFS_COPY_STREAMS]);
    for (int k = 0; k < LBFFS_COPY_STREAMS && e == cudaSuccess; k++) {
        e = cudaEventRecord(c->copy_ev[k], c->copy_st[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->copy_ev[k], 0);
    }
    return e;
}

// The device address of page-locked host memory (cudaHostAlloc / cudaHostRegister), through which
// the conversion kernels read or write the reference's packed population layout in one pass over
// the host link; null for pageable memory, which goes through copies.
static const void* pinned_device_ptr(const void* host)
{
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

extern "C" int lbffs_upload(lbffs_ctx* c, int field, const void* host, size_t bytes)
{
    if (!c || !host) return fail(c, LBFFS_E_ARG, "lbffs_upload: null argument");
    if (field < 0 || field >= LBFFS_NFIELDS) return fail(c, LBFFS_E_ARG, "lbffs_upload: bad field id");
    if (bytes != field_bytes(c, field))
        return fail(c, LBFFS_E_ARG, "lbffs_upload: field " + std::to_string(field) + " expects " +
                                         std::to_string(field_bytes(c, field)) + " bytes, got " + std::to_string(bytes));
    {
        const int rc = ctx_io_wait(c);  // an asynchronous file write may still read the fields
        if (rc != LBFFS_OK) return rc;
    }
    CK(cudaSetDevice(c->d.device));
    FieldInfo fi = field_info(field);
    if (fi.kind == K_F) {
        c->xghost_ok = false;
        const long long nx = c->d.nx;
        const long long rows = (long long)c->Q * c->d.ny * c->d.nz, chunk = (long long)c->stage_elems / nx;
        const float* h = static_cast<const float*>(host);
        // both population copies get the uploaded values: initialization.hpp fills f and fTmp alike, and
        // cells that are never written (solid cells) must read the same values from either copy
        if (const void* hd = pinned_device_ptr(host)) {
            // pinned host memory: one kernel reads the packed rows over the host link and writes both
            // padded copies (with the storage conversion)
            CK(encode_f(c->d.storage, c->Q, static_cast<const float*>(hd), c->f[0], c->f[1], 0, rows, c->pg,
                        c->stream));
            CK(cudaStreamSynchronize(c->stream));
            return LBFFS_OK;
        }
        if (c->d.storage == LBFFS_FP32) {
            // FP32 is stored as is: one pitched copy per direction into the padded planes, then the
            // second copy device to device (no staging, no conversion kernel)
            CK(copy_planes_f32(c, h, true));
            CK(cudaMemcpyAsync(c->f[1], c->f[0], (size_t)c->Q * (size_t)c->pg.pE * sizeof(float),
                               cudaMemcpyDeviceToDevice, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            return LBFFS_OK;
        }
        for (long long r = 0; r < rows; r += chunk) {
            const long long n = (rows - r < chunk) ? rows - r : chunk;
            CK(cudaMemcpyAsync(c->stage, h + r * nx, (size_t)(n * nx) * sizeof(float), cudaMemcpyHostToDevice,
                               c->stream));
            CK(encode_f(c->d.storage, c->Q, c->stage, c->f[0], c->f[1], r, n, c->pg, c->stream));
        }
        CK(cudaStreamSynchronize(c->stream));
        return LBFFS_OK;
    }
    if (fi.kind == K_MACRO) {
        for (int b = 0; b < 2; b++)
            CK(cudaMemcpyAsync(c->macro[b][fi.macro], host, bytes, cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        return LBFFS_OK;
    }
    if (field == LBFFS_GXIBM || field == LBFFS_GYIBM || field == LBFFS_GZIBM) CK(ensure_g(c));
    if (field >= LBFFS_OUT_RHO && field <= LBFFS_OUT_W)
        return fail(c, LBFFS_E_ARG, "lbffs_upload: the output fields are written by lbffs_output only");
    if (field >= LBFFS_UMEAN && field <= LBFFS_WMEAN && !ctx_output_field(c, field, true))
        return fail(c, LBFFS_E_CUDA, "lbffs_upload: cannot allocate the time-mean field");
    void* p = field_ptr(c, field);
    CK(cudaMemcpyAsync(p, host, bytes, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (geometry_field(field)) c->dirty = true;
    return LBFFS_OK;
}

extern "C" int lbffs_download(lbffs_ctx* c, int field, void* host, size_t bytes)
{
    if (!c || !host) return fail(c, LBFFS_E_ARG, "lbffs_download: null argument");
    if (field < 0 || field >= LBFFS_NFIELDS) return fail(c, LBFFS_E_ARG, "lbffs_download: bad field id");
    if (bytes != field_bytes(c, field)) return fail(c, LBFFS_E_ARG, "lbffs_download: size mismatch");
    CK(cudaSetDevice(c->d.device));
    FieldInfo fi = field_info(field);
    if (fi.kind == K_F) {
        const long long nx = c->d.nx;
        const long long rows = (long long)c->Q * c->d.ny * c->d.nz, chunk = (long long)c->stage_elems / nx;
        float* h = static_cast<float*>(host);
        if (const void* hd = pinned_device_ptr(host)) {
            // pinned host memory: one kernel reads the padded planes and writes the packed rows over
            // the host link (with the storage conversion)
            CK(decode_f(c->d.storage, c->Q, c->f[c->fcur], static_cast<float*>(const_cast<void*>(hd)), 0, rows,
                        c->pg, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            return LBFFS_OK;
        }
        if (c->d.storage == LBFFS_FP32) {
            CK(copy_planes_f32(c, h, false));
            CK(cudaStreamSynchronize(c->stream));
            return LBFFS_OK;
        }
        for (long long r = 0; r < rows; r += chunk) {
            const long long n = (rows - r < chunk) ? rows - r : chunk;
            CK(decode_f(c->d.storage, c->Q, c->f[c->fcur], c->stage, r, n, c->pg, c->stream));
            CK(cudaMemcpyAsync(h + r * nx, c->stage, (size_t)(n * nx) * sizeof(float), cudaMemcpyDeviceToHost,
                               c->stream));
            CK(cudaStreamSynchronize(c->stream));
        }
        return LBFFS_OK;
    }
    const void* p = fi.kind == K_MACRO ? c->macro[c->mcur][fi.macro] : field_ptr(c, field);
    if (!p) {  // IBM forcing fields before any marker was set: zero
        memset(host, 0, bytes);
        return LBFFS_OK;
    }
    CK(cudaMemcpyAsync(host, p, bytes, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return LBFFS_OK;
}

static cudaEvent_t get_event(lbffs_ctx* c)
{
    if (!c->pool.empty()) {
        cudaEvent_t e = c->pool.back();
        c->pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

static void harvest_timing(lbffs_ctx* c)
{
    for (auto& ev : c->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ev.a, ev.b) == cudaSuccess) {
            c->ms[ev.kind] += ms;
            c->launches[ev.kind] += 1;
        }
        c->pool.push_back(ev.a);
        c->pool.push_back(ev.b);
    }
    c->pending.clear();
}

int lbffs::ctx_commit(lbffs_ctx* c) { return commit(c); }

void lbffs::ctx_step_args(const lbffs_ctx* c, const lbffs_step_params* p, int src, int msrc, StepArgs& a)
{
    a = StepArgs{};
    a.flags = c->flags;
    a.bc = c->bc;
    a.solid = c->solid;
    a.nei_solid = c->nei;
    a.u0 = c->u0;
    a.v0 = c->v0;
    a.w0 = c->w0;
    a.omega = c->omega;
    a.sdf = c->sdf;
    a.fwx = c->fw[0];
    a.fwy = c->fw[1];
    a.fwz = c->fw[2];
    a.gx = c->g[0];
    a.gy = c->g[1];
    a.gz = c->g[2];
    a.special = c->special;
    a.n_special = c->n_special;
    a.E = c->E;
    a.nx = c->d.nx;
    a.ny = c->d.ny;
    a.nz = c->d.nz;
    a.omega0 = c->omega0;
    a.dpdx = p->dpdx;
    a.les = p->les;
    a.omega_b = p->omega_b;
    a.spz = p->spz_width;
    a.clim = p->clim;
    a.cs = c->d.cs;
    a.damping = c->d.damping;
    a.border_pulls = 0;
    a.face_codes = c->face_codes;
    a.sponge_mask = c->sponge_mask;
    a.sgs = c->d.sgs;
    a.wall = c->d.wall;
    a.px = c->pg.px;
    a.pxy = c->pg.pxy;
    a.porg = c->pg.porg;
    a.pE = c->pg.pE;
    a.ibm_box = c->n_markers > 1 ? c->ibm_box : nullptr;
    a.err = c->d_err;
    a.f_in = c->f[src];
    a.f_out = c->f[1 - src];
    for (int q = 0; q < c->Q; q++) {
        const long long pull =
            lat_c(c->Q, q, 0) + (long long)lat_c(c->Q, q, 1) * a.px + (long long)lat_c(c->Q, q, 2) * a.pxy;
        const size_t plane = (size_t)q * (size_t)a.pE * c->tsize;
        a.fin_q[q] = static_cast<const char*>(a.f_in) + plane;
        // plane base moved back by the pull offset; every address formed from it is inside the plane
        a.fin_s[q] = reinterpret_cast<const void*>(reinterpret_cast<uintptr_t>(a.fin_q[q]) -
                                                   (uintptr_t)(pull * (long long)c->tsize));
        a.fout_q[q] = static_cast<char*>(a.f_out) + plane;
    }
    // x-face pull bases (border_pulls 2): a cell on the low / high x face of a row that crosses no
    // other face, its border codes (the x face's code, 0, 0) and face flag set (border_pull)
    {
        const int nx = c->d.nx;
        const int code_lo = c->face_codes & 7;
        const int code_hi = nx == 1 ? code_lo : (c->face_codes >> 3) & 7;
        for (int q = 0; q < c->Q; q++) {
            a.fin_xlo[q] = a.fin_s[q];
            a.fin_xhi[q] = a.fin_s[q];
            const int cx = lat_c(c->Q, q, 0);
            if (cx == 0) continue;
            const int code = cx > 0 ? code_lo : code_hi;
            const void*& base = cx > 0 ? a.fin_xlo[q] : a.fin_xhi[q];
            if (is_wall_code(code)) {
                const int b[3] = {code, 0, 0};
                base = a.fin_q[c->Q == 19 ? missing_dir<19>(q, b) : missing_dir<27>(q, b)];
            } else {
                // the periodic image: nx elements further (low face) or back (high face)
                const long long sh = (cx > 0 ? nx : -nx) * (long long)c->tsize;
                base = reinterpret_cast<const void*>(reinterpret_cast<uintptr_t>(a.fin_s[q]) + (uintptr_t)sh);
            }
        }
    }
    float* const* mp = c->macro[msrc];
    float* const* mn = c->macro[1 - msrc];
    a.rho_p = mp[0];
    a.u_p = mp[1];
    a.v_p = mp[2];
    a.w_p = mp[3];
    a.tau_p = mp[4];
    a.rho_n = mn[0];
    a.u_n = mn[1];
    a.v_n = mn[2];
    a.w_n = mn[3];
    a.tau_n = mn[4];
    a.store_all = p->store_fields == 2;
    a.bulk_kind = c->Q == 19 ? c->bulk_kind : 0;
    // the warp mapping is built for D3Q19
    a.special_kind = c->Q != 19                ? 0
                     : c->special_kind >= 0    ? c->special_kind
                     : c->n_special <= LBFFS_SPECIAL_WARP_MAX ? 1
                                                              : 0;
    a.l2_policy = 2LL * c->Q * c->pg.pE * c->tsize <= c->l2_bytes ? 1 : 0;
}

extern "C" int lbffs_step(lbffs_ctx* c, const lbffs_step_params* p, int nsteps)
{
    if (!c || !p) return fail(c, LBFFS_E_ARG, "lbffs_step: null argument");
    if (nsteps < 0) return fail(c, LBFFS_E_ARG, "lbffs_step: nsteps < 0");
    CK(cudaSetDevice(c->d.device));
    if (c->dirty) {
        int r = commit(c);
        if (r != LBFFS_OK) return r;
    }
    StepConfig cfg{c->d.storage, c->d.collision, c->d.sgs, c->d.wall,
                   c->d.sgs == LBFFS_SGS_SMAGORINSKY && p->les != 0.f};
    auto launch = (c->Q == 19) ? launch_q19 : launch_q27;
    // the boundary kernel and the bulk kernel write disjoint cells and read only this step's source
    // copy: the boundary kernel runs on a second stream, forked after the ghost fill and joined
    // before anything that reads the step's results
    if (c->n_special > 0 && !c->side) {
        // one thread per listed cell: launched before the bulk kernel on a higher-priority stream, so
        // the small kernel takes SMs as the bulk kernel's CTAs retire instead of waiting behind all of
        // them.  A lane group per cell: launched after the bulk kernel at the same priority, so its many
        // register-heavy warps do not crowd out the bulk kernel's first wave (the 1024x256x4 channel:
        // 2.7 % faster; the long lists of the D3Q27 step: 1.6 % slower that way, hence the split)
        int lo = 0, hi = 0;
        CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        CK(cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, hi));
        CK(cudaStreamCreateWithPriority(&c->side_lo, cudaStreamNonBlocking, lo));
        CK(cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming));
    }
    // pulls across the grid's border: straight from where the face streaming takes them when the faces
    // allow it (pull_ok) and the bulk kernel is the per-thread one; otherwise from the ghost layer,
    // filled before every step.  The IBM forcing pass changes populations after the step: the pulls
    // of modes 1 and 2 read them where the pass left them, as the ghost fill does, but the x-face
    // cells of mode 3 would have written their ghost slots before it, so with markers mode 3 gives
    // way to the ghost fill.
    const bool pulls = c->pull_ok && c->pulls_on && c->bulk_kind == 0 && (c->n_markers <= 1 || c->pull_mode != 3);
    const int pull_mode = pulls ? c->pull_mode : 0;
    for (int s = 0; s < nsteps; s++) {
        StepArgs a;
        ctx_step_args(c, p, c->fcur, c->mcur, a);
        a.store_all = (p->store_fields == 2) || (p->store_fields == 1 && s == nsteps - 1);
        a.border_pulls = pull_mode;
        // ghost layer of this step's source populations: the face streaming of the six faces (mode 3:
        // once, when the x-face cells did not write their slots in the step that made the source)
        if (pull_mode == 0 || (pull_mode == 3 && !c->xghost_ok)) {
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (c->timing) {
                e0 = get_event(c);
                e1 = get_event(c);
                cudaEventRecord(e0, c->stream);
            }
            cudaError_t e = halo_fill(c->Q, (int)c->tsize, c->f[c->fcur], c->flags, c->bc, c->pg, c->stream);
            if (c->timing) {
                cudaEventRecord(e1, c->stream);
                c->pending.push_back({e0, e1, 3});
            }
            if (e != cudaSuccess) return fail(c, LBFFS_E_CUDA, std::string("halo launch: ") + cudaGetErrorString(e));
        }
        float** mn = c->macro[1 - c->mcur];
        const bool fork = c->n_special > 0;
        const bool side_first = a.special_kind != 1;
        cudaStream_t side = side_first ? c->side : c->side_lo;
        if (fork) {
            CK(cudaEventRecord(c->fork_ev, c->stream));
            CK(cudaStreamWaitEvent(side, c->fork_ev, 0));
        }
        for (int h = 0; h < 2; h++) {
            const int half = side_first ? 1 - h : h;
            const bool bulk = half == 0;
            if (!bulk && !fork) continue;
            cudaStream_t st = bulk ? c->stream : side;
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (c->timing) {
                e0 = get_event(c);
                e1 = get_event(c);
                cudaEventRecord(e0, st);
            }
            cudaError_t e = launch(a, cfg, bulk, st);
            if (c->timing) {
                cudaEventRecord(e1, st);
                c->pending.push_back({e0, e1, bulk ? 0 : 1});
            }
            if (e != cudaSuccess) return fail(c, LBFFS_E_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
        }
        if (fork) {
            CK(cudaEventRecord(c->join_ev, side));
            CK(cudaStreamWaitEvent(c->stream, c->join_ev, 0));
        }
        if (c->n_markers > 1) {
            IbmArgs ia{};
            ia.markers = c->markers;
            ia.gm = c->gm;
            ia.acc = c->ibm_acc;
            ia.lag = c->ibm_lag;
            ia.box = c->ibm_box;
            ia.t = c->ibm_t;
            ia.motion = c->motion;
            ia.n = c->n_markers;
            ia.nx = a.nx;
            ia.ny = a.ny;
            ia.nz = a.nz;
            ia.E = c->E;
            ia.u = mn[1];
            ia.v = mn[2];
            ia.w = mn[3];
            ia.rho = mn[0];
            ia.flags = c->flags;
            ia.f_out = a.f_out;
            ia.px = a.px;
            ia.pxy = a.pxy;
            ia.porg = a.porg;
            ia.pE = a.pE;
            ia.gx = c->g[0];
            ia.gy = c->g[1];
            ia.gz = c->g[2];
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (c->timing) {
                e0 = get_event(c);
                e1 = get_event(c);
                cudaEventRecord(e0, c->stream);
            }
            cudaError_t e = ibm_substep(ia, c->d.storage, c->Q, c->nsm, c->stream);
            if (c->timing) {
                cudaEventRecord(e1, c->stream);
                c->pending.push_back({e0, e1, 2});
            }
            if (e != cudaSuccess) return fail(c, LBFFS_E_CUDA, std::string("ibm launch: ") + cudaGetErrorString(e));
        }
        c->fcur = 1 - c->fcur;
        c->mcur = 1 - c->mcur;
        c->xghost_ok = pull_mode == 3;
    }
    return LBFFS_OK;
}

extern "C" int lbffs_synchronize(lbffs_ctx* c)
{
    if (!c) return fail(c, LBFFS_E_ARG, "lbffs_synchronize: null context");
    CK(cudaSetDevice(c->d.device));
    CK(cudaStreamSynchronize(c->stream));
    if (c->timing) harvest_timing(c);
    int h = 0;
    CK(cudaMemcpy(&h, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h & 2) return fail(c, LBFFS_E_CUDA, "a bulk-copy wait of the row-staged step kernel ran out");
    if (h) return fail(c, LBFFS_E_NONFINITE, "non-finite density produced by the step (divergence)");
    return LBFFS_OK;
}

extern "C" int lbffs_force_sum(lbffs_ctx* c, double out[3])
{
    if (!c || !out) return fail(c, LBFFS_E_ARG, "lbffs_force_sum: null argument");
    CK(cudaSetDevice(c->d.device));
    out[0] = out[1] = out[2] = 0.0;
    if (c->dirty || c->n_special == 0) return LBFFS_OK;
    const int nb = c->partial_blocks;
    CK(reduce_force(c->special, c->n_special, c->fw[0], c->fw[1], c->fw[2], c->partial, nb, c->stream));
    std::vector<double> h((size_t)3 * nb);
    CK(cudaMemcpyAsync(h.data(), c->partial, sizeof(double) * 3 * nb, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int b = 0; b < nb; b++)
        for (int a = 0; a < 3; a++) out[a] += h[(size_t)3 * b + a];
    return LBFFS_OK;
}

extern "C" int lbffs_mass(lbffs_ctx* c, double* out)
{
    if (!c || !out) return fail(c, LBFFS_E_ARG, "lbffs_mass: null argument");
    CK(cudaSetDevice(c->d.device));
    if (c->dirty) {
        int r = commit(c);
        if (r != LBFFS_OK) return r;
    }
    const int nb = c->partial_blocks;
    CK(reduce_mass(c->d.storage, c->Q, c->f[c->fcur], c->flags, c->E, c->pg, c->partial, nb, c->stream));
    std::vector<double> h(nb);
    CK(cudaMemcpyAsync(h.data(), c->partial, sizeof(double) * nb, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    double s = 0.0;
    for (int b = 0; b < nb; b++) s += h[b];
    *out = s;
    return LBFFS_OK;
}

extern "C" int lbffs_links(lbffs_ctx* c, long long* cells, unsigned* masks, long long capacity, long long* n)
{
    if (!c || !n) return fail(c, LBFFS_E_ARG, "lbffs_links: null argument");
    CK(cudaSetDevice(c->d.device));
    if (c->dirty) {
        int r = commit(c);
        if (r != LBFFS_OK) return r;
    }
    *n = 0;
    if (c->n_special == 0) return LBFFS_OK;
    uint32_t* d_masks = nullptr;
    CK(ctx_alloc_bytes(c, (void**)&d_masks, sizeof(uint32_t) * c->n_special + 16));
    cudaError_t e = setup_link_masks(c->Q, c->special, c->n_special, c->bc, c->solid, c->nei, c->d.nx, c->d.ny,
                                     c->d.nz, d_masks, c->stream);
    std::vector<uint32_t> hm(c->n_special), hc(c->n_special);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hm.data(), d_masks, sizeof(uint32_t) * c->n_special, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hc.data(), c->special, sizeof(uint32_t) * c->n_special, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    ctx_free(c, d_masks);
    CK(e);
    long long k = 0;
    for (long long t = 0; t < c->n_special; t++) {
        if (!hm[t]) continue;
        if (k < capacity && cells && masks) {
            cells[k] = hc[t];
            masks[k] = hm[t];
        }
        k++;
    }
    *n = k;
    return LBFFS_OK;
}

extern "C" int lbffs_set_markers(lbffs_ctx* c, const float* xyz, int n)
{
    if (!c || (n > 0 && !xyz) || n < 0) return fail(c, LBFFS_E_ARG, "lbffs_set_markers: bad argument");
    CK(cudaSetDevice(c->d.device));
    CK(cudaStreamSynchronize(c->stream));
    ctx_free(c, c->markers);
    ctx_free(c, c->gm);
    c->markers = c->gm = nullptr;
    c->n_markers = n;
    if (n == 0) return LBFFS_OK;
    CK(ensure_g(c));
    CK(dalloc(c, &c->markers, (size_t)3 * n));
    CK(dalloc(c, &c->gm, (size_t)3 * n));
    CK(cudaMemcpyAsync(c->markers, xyz, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    if (!c->ibm_acc) CK(dalloc(c, &c->ibm_acc, (size_t)3 * c->E));
    if (!c->ibm_lag) CK(dalloc(c, &c->ibm_lag, 3));
    if (!c->ibm_box) CK(dalloc(c, &c->ibm_box, 12));
    if (!c->ibm_t) CK(dalloc(c, &c->ibm_t, 1));
    IbmArgs ia{};
    ia.markers = c->markers;
    ia.box = c->ibm_box;
    ia.t = c->ibm_t;
    ia.n = n;
    ia.nx = c->d.nx;
    ia.ny = c->d.ny;
    ia.nz = c->d.nz;
    CK(ibm_init_box(ia, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return LBFFS_OK;
}

extern "C" int lbffs_get_markers(lbffs_ctx* c, float* xyz, int n)
{
    if (!c || !xyz || n != c->n_markers) return fail(c, LBFFS_E_ARG, "lbffs_get_markers: bad argument");
    if (n == 0) return LBFFS_OK;
    CK(cudaSetDevice(c->d.device));
    CK(cudaMemcpyAsync(xyz, c->markers, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return LBFFS_OK;
}

extern "C" int lbffs_set_motion(lbffs_ctx* c, const lbffs_motion* m)
{
    if (!c || !m) return fail(c, LBFFS_E_ARG, "lbffs_set_motion: null argument");
    c->motion.trans[0] = m->u_trans;
    c->motion.trans[1] = m->v_trans;
    c->motion.trans[2] = m->w_trans;
    c->motion.rot[0] = m->rot_x;
    c->motion.rot[1] = m->rot_y;
    c->motion.rot[2] = m->rot_z;
    c->motion.axis[0] = m->axis_x;
    c->motion.axis[1] = m->axis_y;
    c->motion.axis[2] = m->axis_z;
    c->motion.rot_omega = m->rot_omega;
    c->motion.amp[0] = m->amp_x;
    c->motion.amp[1] = m->amp_y;
    c->motion.amp[2] = m->amp_z;
    c->motion.period = m->period;
    if (c->ibm_t) {
        CK(cudaSetDevice(c->d.device));
        CK(cudaMemsetAsync(c->ibm_t, 0, sizeof(long long), c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    return LBFFS_OK;
}

extern "C" int lbffs_ibm_force_sum(lbffs_ctx* c, double out[3])
{
    if (!c || !out) return fail(c, LBFFS_E_ARG, "lbffs_ibm_force_sum: null argument");
    out[0] = out[1] = out[2] = 0.0;
    if (!c->ibm_lag) return LBFFS_OK;
    CK(cudaSetDevice(c->d.device));
    CK(cudaMemcpyAsync(out, c->ibm_lag, sizeof(double) * 3, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemsetAsync(c->ibm_lag, 0, sizeof(double) * 3, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return LBFFS_OK;
}

extern "C" int lbffs_get_stream(lbffs_ctx* c, void** stream)
{
    if (!c || !stream) return fail(c, LBFFS_E_ARG, "lbffs_get_stream: null argument");
    *stream = (void*)c->stream;
    return LBFFS_OK;
}

extern "C" int lbffs_set_timing(lbffs_ctx* c, int enabled)
{
    if (!c) return fail(c, LBFFS_E_ARG, "lbffs_set_timing: null context");
    CK(cudaSetDevice(c->d.device));
    CK(cudaStreamSynchronize(c->stream));
    harvest_timing(c);
    c->timing = enabled != 0;
    for (int k = 0; k < 3; k++) {
        c->ms[k] = 0;
        c->launches[k] = 0;
    }
    return LBFFS_OK;
}

extern "C" int lbffs_kernel_time(lbffs_ctx* c, const char* name, double* total_ms, long long* launches)
{
    if (!c || !name || !total_ms || !launches) return fail(c, LBFFS_E_ARG, "lbffs_kernel_time: null argument");
    int k = !strcmp(name, "bulk")      ? 0
            : !strcmp(name, "special") ? 1
            : !strcmp(name, "ibm")     ? 2
            : !strcmp(name, "halo")    ? 3
                                       : -1;
    if (k < 0) return fail(c, LBFFS_E_ARG, "lbffs_kernel_time: unknown kernel name");
    CK(cudaSetDevice(c->d.device));
    CK(cudaStreamSynchronize(c->stream));
    harvest_timing(c);
    *total_ms = c->ms[k];
    *launches = c->launches[k];
    return LBFFS_OK;
}

extern "C" int lbffs_cell_counts(lbffs_ctx* c, long long out[4])
{
    if (!c || !out) return fail(c, LBFFS_E_ARG, "lbffs_cell_counts: null argument");
    CK(cudaSetDevice(c->d.device));
    if (c->dirty) {
        int r = commit(c);
        if (r != LBFFS_OK) return r;
    }
    for (int k = 0; k < 4; k++) out[k] = c->counts[k];
    return LBFFS_OK;
}

extern "C" int lbffs_init_rest(lbffs_ctx* c)
{
    if (!c) return fail(c, LBFFS_E_ARG, "lbffs_init_rest: null context");
    CK(cudaSetDevice(c->d.device));
    c->xghost_ok = false;
    const size_t plane_bytes = (size_t)c->pg.pE * c->tsize;
    for (int b = 0; b < 2; b++) {
        if (c->d.storage == LBFFS_FP32) {
            for (int q = 0; q < c->Q; q++)
                CK(fill_f32(reinterpret_cast<float*>(static_cast<char*>(c->f[b]) + q * plane_bytes), lat_w(c->Q, q),
                            c->pg.pE, c->stream));
        } else {
            // shifted storage holds f - w = 0
            CK(cudaMemsetAsync(c->f[b], 0, plane_bytes * c->Q, c->stream));
        }
    }
    CK(cudaStreamSynchronize(c->stream));
    return LBFFS_OK;
}

extern "C" int lbffs_set_bulk_kernel(lbffs_ctx* c, int kind)
{
    if (!c || kind < 0 || kind > 1) return fail(c, LBFFS_E_ARG, "lbffs_set_bulk_kernel: kind must be 0 or 1");
    c->bulk_kind = kind;
    return LBFFS_OK;
}

extern "C" int lbffs_set_border_pulls(lbffs_ctx* c, int enabled)
{
    if (!c || enabled < 0 || enabled > 1) return fail(c, LBFFS_E_ARG, "lbffs_set_border_pulls: enabled must be 0 or 1");
    c->pulls_on = enabled != 0;
    c->xghost_ok = false;
    return LBFFS_OK;
}

extern "C" int lbffs_set_special_kernel(lbffs_ctx* c, int kind)
{
    if (!c || kind < -1 || kind > 1)
        return fail(c, LBFFS_E_ARG, "lbffs_set_special_kernel: kind must be -1, 0 or 1");
    c->special_kind = kind;
    return LBFFS_OK;
}

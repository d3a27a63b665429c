// lbffs_server_*: continuous batching of many lattice solves on one GPU.
//
// An admission thread brings queued cases in while slots and the HBM arena allow: a case becomes
// an ordinary context whose buffers are carved from the arena, gets its arrays uploaded and its
// geometry committed on the set-up stream (while the batch computes), and is handed over ready at
// step 0.  A loop thread owns the batched GPU work.  Each round it
//   1. moves the ready cases into the batch;
//   2. when the resident set changed, rebuilds the batch tables (per group of storage format and
//      LES switch: the cases' kernel arguments for both parities, the prefix sums of bulk tiles
//      and special cells) and captures steps_per_round steps into a CUDA graph;
//   3. replays the graph once: every step is one batched ghost-layer, bulk and special launch per
//      group (the special launches on a parallel branch beside the bulk ones) plus a counter tick,
//      so all resident cases advance together, each case's device
//      step counter choosing its ping-pong parity and stopping it at exactly its nsteps;
//   4. reads back the counters and retires finished cases: their final fields are downloaded and
//      their arena blocks released, which lets the next round admit more.
// Requests that arrive while a round runs are admitted at the next round boundary, so their work
// overlaps with the cases already on the device.
#include <algorithm>
#include <chrono>
#include <string>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "batch.h"
#include "ctx.h"
#include "step_kernels.cuh"

using namespace lbffs;

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
    long long id = 0;
    lbffs_desc desc{};
    lbffs_step_params params{};
    long long nsteps = 0;
    int want_f = 0;
    std::vector<int> bnd[4];
    std::vector<unsigned char> solid, nei;
    std::vector<float> sdf, u0, v0, w0, omega, f;
    double t_submit = 0, t_admit = 0, t_done = 0;
    int state = LBFFS_CASE_QUEUED;
    std::string err;
    lbffs_ctx* ctx = nullptr;
    int slot = -1;
    bool in_graph = false;  // part of the captured batch (its counter is read back each round)
    std::vector<float> res[5];  // rho, u, v, w, f
};

struct Group {
    int storage = 0;
    bool les = false;
    std::vector<Request*> members;
    BatchCase* d_cases = nullptr;
    int2* d_ctas = nullptr;  // (case, run) of each bulk CTA: the segment launch's, then the row-tile launch's
    size_t ctas_cap = 0;
    long long* d_sp = nullptr;
    size_t cap = 0;
    int ntiles = 0, ntiles_rows = 0;
    long long nspecial = 0, nhalo = 0;
};

template <class T>
cudaError_t grow(T** p, size_t& cap, size_t n)
{
    if (n <= cap && *p) return cudaSuccess;
    if (*p) cudaFree(*p);
    *p = nullptr;
    cap = n < 16 ? 16 : n * 2;
    return cudaMalloc(p, sizeof(T) * cap);
}

}  // namespace

struct lbffs_server {
    lbffs_server_desc d{};
    cudaStream_t stream = nullptr;         // batched steps (graph replay)
    cudaStream_t setup_stream = nullptr;   // admission: per-case uploads and commits
    cudaStream_t result_stream = nullptr;  // retirement: result downloads
    cudaStream_t branch = nullptr;         // captured graph: the boundary kernels' parallel branch
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    void* arena_mem = nullptr;
    std::unique_ptr<Arena> arena;
    float* stage = nullptr;   // admission staging
    float* stage2 = nullptr;  // retirement staging
    size_t stage_elems = 0;
    long long* d_done = nullptr;
    long long* h_done = nullptr;  // pinned
    std::vector<int> free_slots;

    std::vector<Group> groups;
    int* d_tick_slots = nullptr;
    long long* d_tick_nsteps = nullptr;
    size_t tick_cap = 0, tick_cap2 = 0;
    int ntick = 0;
    cudaGraphExec_t exec = nullptr;
    bool rebuild = true;

    std::thread loop, admitter;
    std::mutex mu;
    std::condition_variable cv;       // wakes the loop (cases ready / stop)
    std::condition_variable admit_cv; // wakes the admitter (submission / memory or slot freed / stop)
    std::condition_variable done_cv;  // wakes waiters (a case finished)
    std::vector<Request*> ready;      // admitted and set up, not yet in the batch
    bool stop = false;
    std::deque<Request*> queue;
    std::vector<Request*> resident;
    std::vector<Request*> to_retire;  // finished, out of the batch tables, results not yet read
    std::map<long long, std::unique_ptr<Request>> all;
    long long next_id = 1;
    std::string err = "no error";
    bool admit_poke = true;  // a submission or a change the admitter has not looked at yet

    // statistics
    long long submitted = 0, completed = 0, failed = 0, rounds = 0, graph_builds = 0;
    double cell_updates = 0, t_first = -1, t_last = 0;
    double gpu_busy_s = 0, build_s = 0, resident_sum = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<double> latency, queue_wait;
};

namespace {

int srv_fail(lbffs_server* s, int code, const std::string& msg)
{
    if (s) s->err = msg;
    set_thread_error(msg);
    return code;
}

// one case: create its context in the arena and bring it to step 0; false when it does not fit
bool admit_one(lbffs_server* s, Request* r)
{
    lbffs_ctx* c = nullptr;
    if (ctx_create(&r->desc, s->arena.get(), s->setup_stream, s->stage, s->stage_elems, &c) != LBFFS_OK) {
        const std::string m = lbffs_last_error(nullptr);
        if (m.find("memory") != std::string::npos) return false;  // retry when blocks free up
        r->err = m;
        r->state = LBFFS_CASE_FAILED;
        return true;
    }
    const size_t E = (size_t)c->E;
    auto up = [&](int field, const void* p, size_t bytes) { return p ? lbffs_upload(c, field, p, bytes) : LBFFS_OK; };
    int rc = LBFFS_OK;
    const int ids[4] = {LBFFS_BOUNDARY, LBFFS_BOUNDARY1, LBFFS_BOUNDARY2, LBFFS_BOUNDARY3};
    for (int b = 0; b < 4 && rc == LBFFS_OK; b++) rc = up(ids[b], r->bnd[b].data(), 4 * E);
    if (rc == LBFFS_OK) rc = up(LBFFS_SOLID, r->solid.data(), E);
    if (rc == LBFFS_OK) rc = up(LBFFS_NEISOLID, r->nei.data(), E);
    if (rc == LBFFS_OK && !r->sdf.empty()) rc = up(LBFFS_SDF, r->sdf.data(), 4 * E);
    if (rc == LBFFS_OK && !r->u0.empty()) rc = up(LBFFS_U0, r->u0.data(), 4 * E);
    if (rc == LBFFS_OK && !r->v0.empty()) rc = up(LBFFS_V0, r->v0.data(), 4 * E);
    if (rc == LBFFS_OK && !r->w0.empty()) rc = up(LBFFS_W0, r->w0.data(), 4 * E);
    if (rc == LBFFS_OK && !r->omega.empty()) rc = up(LBFFS_OMEGA, r->omega.data(), 4 * E);
    if (rc == LBFFS_OK) rc = r->f.empty() ? lbffs_init_rest(c) : up(LBFFS_F, r->f.data(), 4 * E * c->Q);
    if (rc == LBFFS_OK) rc = ctx_commit(c);
    if (rc == LBFFS_OK && cudaStreamSynchronize(s->setup_stream) != cudaSuccess) rc = LBFFS_E_CUDA;
    if (rc != LBFFS_OK) {
        const bool memory = c->err.find("memory") != std::string::npos;
        if (!memory) r->err = c->err;
        lbffs_destroy(c);
        if (!memory) {
            r->state = LBFFS_CASE_FAILED;
            return true;  // consumed (failed), not retried
        }
        return false;
    }
    c->fcur = c->mcur = 0;
    c->xghost_ok = false;
    r->ctx = c;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        r->slot = s->free_slots.back();
        s->free_slots.pop_back();
    }
    // the slot is in no captured graph (it was freed only after a rebuild dropped its last case).
    // The counter is cleared on the device: the pinned read-back buffer h_done belongs to the loop
    // thread, whose asynchronous copy of all counters may be landing in it right now.
    if (cudaMemsetAsync(s->d_done + r->slot, 0, sizeof(long long), s->setup_stream) != cudaSuccess ||
        cudaStreamSynchronize(s->setup_stream) != cudaSuccess) {
        r->err = "step counter reset failed";
        r->state = LBFFS_CASE_FAILED;
        lbffs_destroy(c);
        r->ctx = nullptr;
        std::lock_guard<std::mutex> lock(s->mu);
        s->free_slots.push_back(r->slot);
        r->slot = -1;
        return true;
    }
    r->t_admit = now_s();
    r->state = LBFFS_CASE_RUNNING;
    return true;
}

// Admission thread: brings queued cases to step 0 on the set-up stream while the loop thread keeps
// the GPU busy with the resident batch.  First fit over the queue: a case that does not fit the
// arena now waits for a retirement, later smaller cases may pass it.
void run_admitter(lbffs_server* s)
{
    cudaSetDevice(s->d.device);
    long long seen_retired = -1;
    for (;;) {
        std::vector<Request*> cand;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            // wait for a submission or for memory / a slot freed since the last unsuccessful pass
            s->admit_cv.wait(lock, [&] {
                return s->stop || (!s->queue.empty() && !s->free_slots.empty() &&
                                   (seen_retired != s->completed + s->failed || s->admit_poke));
            });
            if (s->stop) return;
            s->admit_poke = false;
            seen_retired = s->completed + s->failed;
            cand.assign(s->queue.begin(), s->queue.end());
        }
        bool any = false;
        for (Request* r : cand) {
            {
                std::lock_guard<std::mutex> lock(s->mu);
                if (s->free_slots.empty() || s->stop) break;
            }
            if (!admit_one(s, r)) continue;  // does not fit now
            any = true;
            std::lock_guard<std::mutex> lock(s->mu);
            s->queue.erase(std::find(s->queue.begin(), s->queue.end(), r));
            if (r->state == LBFFS_CASE_FAILED) {
                s->failed++;
                r->t_done = now_s();
                s->done_cv.notify_all();
            } else {
                s->ready.push_back(r);
                s->cv.notify_all();
            }
        }
        if (any) {
            std::lock_guard<std::mutex> lock(s->mu);
            s->admit_poke = true;  // the queue changed: look again at once
        }
    }
}

cudaError_t build_batch(lbffs_server* s)
{
    for (Group& g : s->groups) g.members.clear();
    for (Request* r : s->resident) {
        const bool les = r->params.les != 0.f;
        Group* g = nullptr;
        for (Group& x : s->groups)
            if (x.storage == r->desc.storage && x.les == les) g = &x;
        if (!g) {
            s->groups.emplace_back();
            g = &s->groups.back();
            g->storage = r->desc.storage;
            g->les = les;
        }
        g->members.push_back(r);
    }
    cudaError_t e = cudaSuccess;
    for (Group& g : s->groups) {
        const int n = (int)g.members.size();
        if (n == 0) {
            g.ntiles = 0;
            g.ntiles_rows = 0;
            g.nspecial = 0;
            g.nhalo = 0;
            continue;
        }
        std::vector<BatchCase> hc(n);
        std::vector<int2> seg_ctas, row_ctas, halo_ctas;
        std::vector<long long> sp(n + 1, 0);
        for (int i = 0; i < n; i++) {
            Request* r = g.members[i];
            r->in_graph = true;
            lbffs_ctx* c = r->ctx;
            for (int p = 0; p < 2; p++) {
                ctx_step_args(c, &r->params, p, p, hc[i].args[p]);
                // the resident cases together exceed L2, whatever one case's size: no policy
                // (evict-first measured 3 % slower on the served sample)
                hc[i].args[p].l2_policy = 0;
                // the batched bulk kernels run no x-face pulls: a case with bulk cells on its x faces
                // keeps the ghost layer
                hc[i].args[p].border_pulls = c->pull_mode == 1 && c->pulls_on && c->n_markers <= 1 ? 1 : 0;
            }
            hc[i].last = hc[i].args[(r->nsteps - 1) & 1];
            hc[i].last.store_all = 1;
            hc[i].nsteps = r->nsteps;
            hc[i].slot = r->slot;
            hc[i].seg_per_row = (c->d.nx + 31) / 32;
            hc[i].dspr = fast_div((uint32_t)hc[i].seg_per_row);
            hc[i].dny = fast_div((uint32_t)c->d.ny);
            // rows that fill most of k_bulk's row tiles run in them (the paths lbffs_step runs);
            // narrow rows in 32-cell segments packed across rows
            hc[i].nxb = (c->d.nx + BULK_BX * BULK_V - 1) / (BULK_BX * BULK_V);
            hc[i].rowtile = LBFFS_BATCH_ROWTILE && 10 * c->d.nx >= 7 * BULK_BX * BULK_V * hc[i].nxb;
            hc[i].tiles = hc[i].rowtile ? hc[i].nxb * c->d.ny * c->d.nz
                                        : (int)(((long long)hc[i].seg_per_row * c->d.ny * c->d.nz +
                                                 BATCH_SEG_PER_TILE - 1) / BATCH_SEG_PER_TILE);
            const int ctas = (hc[i].tiles + BATCH_TILES_PER_CTA - 1) / BATCH_TILES_PER_CTA;
            for (int r = 0; r < ctas; r++) (hc[i].rowtile ? row_ctas : seg_ctas).push_back(make_int2(i, r));
            // a case whose x faces are boundary-kernel faces pulls across its border (no ghost fill)
            if (!hc[i].args[0].border_pulls) {
                const long long hb = halo_blocks(c->pg, 19, 0) + halo_blocks(c->pg, 19, 1) + halo_blocks(c->pg, 19, 2);
                for (long long b = 0; b < hb; b++) halo_ctas.push_back(make_int2(i, (int)b));
            }
            sp[i + 1] = sp[i] + c->n_special;
        }
        size_t cap = g.cap;
        if (n + 1 > (int)g.cap || !g.d_cases) {
            if (g.d_cases) cudaFree(g.d_cases);
            if (g.d_sp) cudaFree(g.d_sp);
            cap = (size_t)(n + 1) * 2;
            if ((e = cudaMalloc(&g.d_cases, sizeof(BatchCase) * cap)) != cudaSuccess) return e;
            if ((e = cudaMalloc(&g.d_sp, sizeof(long long) * cap)) != cudaSuccess) return e;
            g.cap = cap;
        }
        if ((e = cudaMemcpyAsync(g.d_cases, hc.data(), sizeof(BatchCase) * n, cudaMemcpyHostToDevice, s->stream)))
            return e;
        const size_t nctas = seg_ctas.size() + row_ctas.size() + halo_ctas.size();
        if (nctas > g.ctas_cap || !g.d_ctas) {
            if (g.d_ctas) cudaFree(g.d_ctas);
            g.d_ctas = nullptr;
            g.ctas_cap = nctas * 2 + 64;
            if ((e = cudaMalloc(&g.d_ctas, sizeof(int2) * g.ctas_cap)) != cudaSuccess) return e;
        }
        const size_t nseg = seg_ctas.size(), nrow = row_ctas.size();
        seg_ctas.insert(seg_ctas.end(), row_ctas.begin(), row_ctas.end());
        seg_ctas.insert(seg_ctas.end(), halo_ctas.begin(), halo_ctas.end());
        if ((e = cudaMemcpyAsync(g.d_ctas, seg_ctas.data(), sizeof(int2) * nctas, cudaMemcpyHostToDevice, s->stream)))
            return e;
        if ((e = cudaMemcpyAsync(g.d_sp, sp.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice, s->stream)))
            return e;
        g.ntiles = (int)nseg;
        g.ntiles_rows = (int)nrow;
        g.nspecial = sp[n];
        g.nhalo = (long long)halo_ctas.size();
    }
    std::vector<int> slots;
    std::vector<long long> ns;
    for (Request* r : s->resident) {
        slots.push_back(r->slot);
        ns.push_back(r->nsteps);
    }
    s->ntick = (int)slots.size();
    if ((e = grow(&s->d_tick_slots, s->tick_cap, slots.size()))) return e;
    if ((e = grow(&s->d_tick_nsteps, s->tick_cap2, ns.size()))) return e;
    if ((e = cudaMemcpyAsync(s->d_tick_slots, slots.data(), sizeof(int) * slots.size(), cudaMemcpyHostToDevice,
                             s->stream)))
        return e;
    if ((e = cudaMemcpyAsync(s->d_tick_nsteps, ns.data(), sizeof(long long) * ns.size(), cudaMemcpyHostToDevice,
                             s->stream)))
        return e;
    if ((e = cudaStreamSynchronize(s->stream))) return e;

    // capture steps_per_round steps of the whole batch
    cudaGraph_t graph = nullptr;
    if ((e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal))) return e;
    cudaError_t le = cudaSuccess;
    bool any_special = false;
    for (Group& g : s->groups) any_special |= g.nspecial > 0;
    for (int step = 0; step < s->d.steps_per_round && le == cudaSuccess; step++) {
        for (Group& g : s->groups)
            if (le == cudaSuccess && g.nhalo > 0)
                le = batch_halo(g.storage, g.d_cases, g.d_ctas + g.ntiles + g.ntiles_rows, g.nhalo, s->d_done,
                                s->stream);
        // the boundary kernels write other cells than the bulk kernels and read the same source
        // copy: a parallel branch of the graph, joined before the counter tick
        if (le == cudaSuccess && any_special) {
            le = cudaEventRecord(s->fork_ev, s->stream);
            if (le == cudaSuccess) le = cudaStreamWaitEvent(s->branch, s->fork_ev, 0);
            for (Group& g : s->groups)
                if (le == cudaSuccess && g.nspecial > 0)
                    le = batch_special(g.storage, g.nspecial <= LBFFS_SPECIAL_WARP_MAX, g.d_cases, g.d_sp,
                                       (int)g.members.size(), g.nspecial, s->d_done, s->branch);
            if (le == cudaSuccess) le = cudaEventRecord(s->join_ev, s->branch);
        }
        for (Group& g : s->groups) {
            if (le == cudaSuccess && g.ntiles_rows > 0)
                le = batch_bulk(g.storage, g.les, true, g.d_cases, g.d_ctas + g.ntiles, g.ntiles_rows, s->d_done,
                                s->stream);
            if (le == cudaSuccess && g.ntiles > 0)
                le = batch_bulk(g.storage, g.les, false, g.d_cases, g.d_ctas, g.ntiles, s->d_done, s->stream);
        }
        if (le == cudaSuccess && any_special) le = cudaStreamWaitEvent(s->stream, s->join_ev, 0);
        if (le == cudaSuccess) le = batch_tick(s->d_tick_slots, s->d_tick_nsteps, s->ntick, s->d_done, s->stream);
    }
    e = cudaStreamEndCapture(s->stream, &graph);
    if (le != cudaSuccess) e = le;
    if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return e;
    }
    if (s->exec) cudaGraphExecDestroy(s->exec);
    s->exec = nullptr;
    e = cudaGraphInstantiate(&s->exec, graph, 0);
    cudaGraphDestroy(graph);
    s->graph_builds++;
    return e;
}

void retire(lbffs_server* s, Request* r)
{
    lbffs_ctx* c = r->ctx;
    c->stream = s->result_stream;  // no work of this case is pending on the set-up stream
    c->stage = s->stage2;
    const long long parity = r->nsteps & 1;
    c->fcur = c->mcur = (int)parity;
    c->xghost_ok = false;
    const size_t E = (size_t)c->E;
    int err_word = 0;
    cudaMemcpyAsync(&err_word, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    cudaStreamSynchronize(c->stream);
    int rc = LBFFS_OK;
    const int fields[4] = {LBFFS_RHO, LBFFS_U, LBFFS_V, LBFFS_W};
    for (int k = 0; k < 4 && rc == LBFFS_OK; k++) {
        r->res[k].resize(E);
        rc = lbffs_download(c, fields[k], r->res[k].data(), 4 * E);
    }
    if (rc == LBFFS_OK && r->want_f) {
        r->res[4].resize(E * c->Q);
        rc = lbffs_download(c, LBFFS_F, r->res[4].data(), 4 * E * c->Q);
    }
    const double cells = (double)E * (double)r->nsteps;
    if (rc != LBFFS_OK) r->err = c->err;
    else if (err_word) r->err = "non-finite density (divergence)";
    lbffs_destroy(c);
    r->ctx = nullptr;
    std::lock_guard<std::mutex> lock(s->mu);
    s->free_slots.push_back(r->slot);
    r->slot = -1;
    r->t_done = now_s();
    r->bnd[0].clear();
    for (auto& v : r->bnd) std::vector<int>().swap(v);
    std::vector<unsigned char>().swap(r->solid);
    std::vector<unsigned char>().swap(r->nei);
    for (auto* v : {&r->sdf, &r->u0, &r->v0, &r->w0, &r->omega, &r->f}) std::vector<float>().swap(*v);
    if (r->err.empty()) {
        r->state = LBFFS_CASE_DONE;
        s->completed++;
        s->cell_updates += cells;
        s->latency.push_back(r->t_done - r->t_submit);
        s->queue_wait.push_back(r->t_admit - r->t_submit);
        s->t_last = r->t_done;
    } else {
        r->state = LBFFS_CASE_FAILED;
        s->failed++;
    }
    s->done_cv.notify_all();
    s->admit_cv.notify_all();  // memory and a slot came free
}

void run_loop(lbffs_server* s)
{
    cudaSetDevice(s->d.device);
    for (;;) {
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv.wait(lock, [&] {
                return s->stop || !s->ready.empty() || !s->resident.empty() || !s->to_retire.empty();
            });
            if (s->stop) return;
            // admitted cases join the batch at this round boundary
            if (!s->ready.empty()) {
                for (Request* r : s->ready) s->resident.push_back(r);
                s->ready.clear();
                s->rebuild = true;
            }
        }
        bool launched = false;
        if (!s->resident.empty()) {
            if (s->rebuild) {
                const double tb = now_s();
                cudaError_t e = build_batch(s);
                s->build_s += now_s() - tb;
                if (e != cudaSuccess) {
                    std::lock_guard<std::mutex> lock(s->mu);
                    s->err = std::string("batch build: ") + cudaGetErrorString(e);
                    for (Request* r : s->resident) {
                        r->state = LBFFS_CASE_FAILED;
                        r->err = s->err;
                        s->failed++;
                        lbffs_destroy(r->ctx);
                        r->ctx = nullptr;
                        s->free_slots.push_back(r->slot);
                    }
                    s->resident.clear();
                    s->done_cv.notify_all();
                    continue;
                }
                s->rebuild = false;
            }
            cudaEventRecord(s->ev0, s->stream);
            cudaGraphLaunch(s->exec, s->stream);
            cudaEventRecord(s->ev1, s->stream);
            s->resident_sum += (double)s->resident.size();
            cudaMemcpyAsync(s->h_done, s->d_done, sizeof(long long) * s->d.max_cases, cudaMemcpyDeviceToHost,
                            s->stream);
            launched = true;
        }
        // host work overlapped with the round: results of cases that finished earlier, then
        // admission of queued cases (both on the set-up stream)
        std::vector<Request*> done_now;
        {
            std::lock_guard<std::mutex> lock(s->mu);
            done_now.swap(s->to_retire);
        }
        for (Request* r : done_now) retire(s, r);
        if (!launched) continue;
        cudaError_t e = cudaStreamSynchronize(s->stream);
        s->rounds++;
        float round_ms = 0.f;
        if (e == cudaSuccess && cudaEventElapsedTime(&round_ms, s->ev0, s->ev1) == cudaSuccess)
            s->gpu_busy_s += 1e-3 * round_ms;
        if (e != cudaSuccess) {
            std::lock_guard<std::mutex> lock(s->mu);
            s->err = std::string("round: ") + cudaGetErrorString(e);
            s->stop = true;
            for (Request* r : s->resident) {
                r->state = LBFFS_CASE_FAILED;
                r->err = s->err;
            }
            s->done_cv.notify_all();
            return;
        }
        // only cases of this round's graph: a case admitted during the round has a counter the
        // round's read-back may predate
        std::vector<Request*> keep, fin;
        for (Request* r : s->resident) (r->in_graph && s->h_done[r->slot] >= r->nsteps ? fin : keep).push_back(r);
        if (!fin.empty()) {
            s->rebuild = true;  // the next graph no longer references the finished cases
            std::lock_guard<std::mutex> lock(s->mu);
            s->resident.swap(keep);
            for (Request* r : fin) s->to_retire.push_back(r);
        }
    }
}

Request* find(lbffs_server* s, long long id)
{
    auto it = s->all.find(id);
    return it == s->all.end() ? nullptr : it->second.get();
}

double pct(std::vector<double> v, double p)
{
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const double pos = p * (double)(v.size() - 1);
    const size_t i = (size_t)pos;
    const double f = pos - (double)i;
    return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

}  // namespace

namespace lbffs {
__global__ void k_tick(const int* __restrict__ slots, const long long* __restrict__ nsteps, int n,
                       long long* __restrict__ done)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = slots[i];
    if (done[s] < nsteps[i]) done[s] += 1;
}

cudaError_t batch_tick(const int* slots, const long long* nsteps, int n, long long* done, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_tick<<<(n + 127) / 128, 128, 0, st>>>(slots, nsteps, n, done);
    return cudaGetLastError();
}

cudaError_t batch_bulk(int storage, bool les, bool rows, const BatchCase* cases, const int2* cta_run, int nctas,
                       const long long* done, cudaStream_t st)
{
    switch (storage) {
        case ST_FP32: return batch_bulk_s0(les, rows, cases, cta_run, nctas, done, st);
        case ST_FP16S: return batch_bulk_s1(les, rows, cases, cta_run, nctas, done, st);
        case ST_BF16S: return batch_bulk_s2(les, rows, cases, cta_run, nctas, done, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t batch_halo(int storage, const BatchCase* cases, const int2* cta_block, long long nblocks,
                       const long long* done, cudaStream_t st)
{
    switch (storage) {
        case ST_FP32: return batch_halo_s0(cases, cta_block, nblocks, done, st);
        case ST_FP16S: return batch_halo_s1(cases, cta_block, nblocks, done, st);
        case ST_BF16S: return batch_halo_s2(cases, cta_block, nblocks, done, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t batch_special(int storage, bool warp, const BatchCase* cases, const long long* sp_start, int ncases,
                          long long nspecial, const long long* done, cudaStream_t st)
{
    switch (storage) {
        case ST_FP32: return batch_special_s0(warp, cases, sp_start, ncases, nspecial, done, st);
        case ST_FP16S: return batch_special_s1(warp, cases, sp_start, ncases, nspecial, done, st);
        case ST_BF16S: return batch_special_s2(warp, cases, sp_start, ncases, nspecial, done, st);
    }
    return cudaErrorInvalidValue;
}
}  // namespace lbffs

extern "C" int lbffs_server_create(const lbffs_server_desc* desc, lbffs_server** out)
{
    if (!desc || !out) return srv_fail(nullptr, LBFFS_E_ARG, "lbffs_server_create: null argument");
    *out = nullptr;
    if (desc->hbm_budget < ((size_t)1 << 20) || desc->max_cases < 1 || desc->steps_per_round < 1)
        return srv_fail(nullptr, LBFFS_E_ARG, "lbffs_server_create: budget >= 1 MiB, max_cases >= 1, steps >= 1");
    auto s = std::make_unique<lbffs_server>();
    s->d = *desc;
    cudaError_t e = cudaSetDevice(desc->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->setup_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->result_stream, cudaStreamNonBlocking);
    int prio_lo = 0, prio_hi = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s->branch, cudaStreamNonBlocking, prio_hi);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->fork_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->join_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
    if (e == cudaSuccess) e = cudaMalloc(&s->arena_mem, desc->hbm_budget);
    s->stage_elems = (size_t)16 << 20;
    if (e == cudaSuccess) e = cudaMalloc(&s->stage, sizeof(float) * s->stage_elems);
    if (e == cudaSuccess) e = cudaMalloc(&s->stage2, sizeof(float) * s->stage_elems);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_done, sizeof(long long) * desc->max_cases);
    // zeroed on a server stream and waited for (the streams are non-blocking: a legacy-stream
    // memset would not be ordered before their first launches)
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_done, 0, sizeof(long long) * desc->max_cases, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_done, sizeof(long long) * desc->max_cases);
    if (e != cudaSuccess) {
        const std::string m = std::string("lbffs_server_create: ") + cudaGetErrorString(e);
        lbffs_server_destroy(s.release());
        return srv_fail(nullptr, LBFFS_E_CUDA, m);
    }
    s->arena = std::make_unique<Arena>(s->arena_mem, desc->hbm_budget);
    for (int i = desc->max_cases - 1; i >= 0; i--) s->free_slots.push_back(i);
    lbffs_server* p = s.release();
    p->loop = std::thread(run_loop, p);
    p->admitter = std::thread(run_admitter, p);
    *out = p;
    return LBFFS_OK;
}

extern "C" int lbffs_server_destroy(lbffs_server* s)
{
    if (!s) return LBFFS_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    s->admit_cv.notify_all();
    if (s->admitter.joinable()) s->admitter.join();
    if (s->loop.joinable()) s->loop.join();
    cudaSetDevice(s->d.device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->setup_stream) cudaStreamSynchronize(s->setup_stream);
    if (s->result_stream) cudaStreamSynchronize(s->result_stream);
    for (auto& kv : s->all)
        if (kv.second->ctx) lbffs_destroy(kv.second->ctx);
    if (s->exec) cudaGraphExecDestroy(s->exec);
    for (Group& g : s->groups) {
        if (g.d_cases) cudaFree(g.d_cases);
        if (g.d_ctas) cudaFree(g.d_ctas);
        if (g.d_sp) cudaFree(g.d_sp);
    }
    if (s->d_tick_slots) cudaFree(s->d_tick_slots);
    if (s->d_tick_nsteps) cudaFree(s->d_tick_nsteps);
    if (s->d_done) cudaFree(s->d_done);
    if (s->h_done) cudaFreeHost(s->h_done);
    if (s->stage) cudaFree(s->stage);
    if (s->stage2) cudaFree(s->stage2);
    s->arena.reset();
    if (s->arena_mem) cudaFree(s->arena_mem);
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->setup_stream) cudaStreamDestroy(s->setup_stream);
    if (s->result_stream) cudaStreamDestroy(s->result_stream);
    if (s->branch) cudaStreamDestroy(s->branch);
    if (s->fork_ev) cudaEventDestroy(s->fork_ev);
    if (s->join_ev) cudaEventDestroy(s->join_ev);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    delete s;
    return LBFFS_OK;
}

extern "C" int lbffs_server_submit(lbffs_server* s, const lbffs_case* c, long long* id)
{
    if (!s || !c || !id) return srv_fail(s, LBFFS_E_ARG, "lbffs_server_submit: null argument");
    const lbffs_desc& d = c->desc;
    if (d.q != 19 || d.collision != LBFFS_COLL_RR || d.sgs != LBFFS_SGS_SMAGORINSKY)
        return srv_fail(s, LBFFS_E_UNSUPPORTED, "lbffs_server_submit: served cases are D3Q19 RR with Smagorinsky SGS");
    if (d.device != s->d.device) return srv_fail(s, LBFFS_E_ARG, "lbffs_server_submit: case device differs");
    if (d.storage < LBFFS_FP32 || d.storage > LBFFS_BF16S || (d.wall != LBFFS_WALL_BB && d.wall != LBFFS_WALL_IBB) ||
        !(d.cs > 0.f) || d.nx < 1 || d.ny < 1 || d.nz < 1 || d.ny > 65535 || d.nz > 65535 || c->nsteps < 1)
        return srv_fail(s, LBFFS_E_ARG, "lbffs_server_submit: bad case description");
    if (!c->boundary || !c->boundary1 || !c->boundary2 || !c->boundary3 || !c->solid || !c->nei_solid)
        return srv_fail(s, LBFFS_E_ARG, "lbffs_server_submit: boundary and solid arrays are required");
    const size_t E = (size_t)d.nx * d.ny * d.nz;
    if (ctx_footprint(d) > s->d.hbm_budget)
        return srv_fail(s, LBFFS_E_ARG, "lbffs_server_submit: the case can never fit the HBM budget");
    auto r = std::make_unique<Request>();
    r->desc = d;
    r->params = c->params;
    r->nsteps = c->nsteps;
    r->want_f = c->want_f;
    const int* b[4] = {c->boundary, c->boundary1, c->boundary2, c->boundary3};
    for (int k = 0; k < 4; k++) r->bnd[k].assign(b[k], b[k] + E);
    r->solid.assign(c->solid, c->solid + E);
    r->nei.assign(c->nei_solid, c->nei_solid + E);
    auto cp = [&](std::vector<float>& v, const float* p, size_t n) {
        if (p) v.assign(p, p + n);
    };
    cp(r->sdf, c->sdf, E);
    cp(r->u0, c->u0, E);
    cp(r->v0, c->v0, E);
    cp(r->w0, c->w0, E);
    cp(r->omega, c->omega, E);
    cp(r->f, c->f, E * 19);
    {
        std::lock_guard<std::mutex> lock(s->mu);
        r->id = s->next_id++;
        r->t_submit = now_s();
        if (s->t_first < 0) s->t_first = r->t_submit;
        *id = r->id;
        s->queue.push_back(r.get());
        s->all[r->id] = std::move(r);
        s->submitted++;
        s->admit_poke = true;
    }
    s->admit_cv.notify_all();
    return LBFFS_OK;
}

extern "C" int lbffs_server_poll(lbffs_server* s, long long id, int* state)
{
    if (!s || !state) return srv_fail(s, LBFFS_E_ARG, "lbffs_server_poll: null argument");
    std::lock_guard<std::mutex> lock(s->mu);
    Request* r = find(s, id);
    if (!r) return srv_fail(s, LBFFS_E_ARG, "lbffs_server_poll: unknown id");
    *state = r->state;
    return LBFFS_OK;
}

extern "C" int lbffs_server_wait(lbffs_server* s, long long id, double timeout_s)
{
    if (!s) return srv_fail(s, LBFFS_E_ARG, "lbffs_server_wait: null server");
    std::unique_lock<std::mutex> lock(s->mu);
    Request* r = find(s, id);
    if (!r) return srv_fail(s, LBFFS_E_ARG, "lbffs_server_wait: unknown id");
    const bool ok = s->done_cv.wait_for(lock, std::chrono::duration<double>(timeout_s), [&] {
        return r->state == LBFFS_CASE_DONE || r->state == LBFFS_CASE_FAILED || s->stop;
    });
    if (!ok) return LBFFS_E_STATE;
    return r->state == LBFFS_CASE_DONE ? LBFFS_OK : LBFFS_E_STATE;
}

extern "C" int lbffs_server_result(lbffs_server* s, long long id, int field, void* host, size_t bytes)
{
    if (!s || !host) return srv_fail(s, LBFFS_E_ARG, "lbffs_server_result: null argument");
    std::lock_guard<std::mutex> lock(s->mu);
    Request* r = find(s, id);
    if (!r || r->state != LBFFS_CASE_DONE) return srv_fail(s, LBFFS_E_STATE, "lbffs_server_result: case not done");
    int k = field == LBFFS_RHO ? 0 : field == LBFFS_U ? 1 : field == LBFFS_V ? 2 : field == LBFFS_W ? 3
            : field == LBFFS_F ? 4 : -1;
    if (k < 0 || (k == 4 && r->res[4].empty())) return srv_fail(s, LBFFS_E_ARG, "lbffs_server_result: field not kept");
    if (bytes != r->res[k].size() * sizeof(float)) return srv_fail(s, LBFFS_E_ARG, "lbffs_server_result: size mismatch");
    memcpy(host, r->res[k].data(), bytes);
    return LBFFS_OK;
}

extern "C" int lbffs_server_release(lbffs_server* s, long long id)
{
    if (!s) return srv_fail(s, LBFFS_E_ARG, "lbffs_server_release: null server");
    std::lock_guard<std::mutex> lock(s->mu);
    Request* r = find(s, id);
    if (!r) return srv_fail(s, LBFFS_E_ARG, "lbffs_server_release: unknown id");
    if (r->state != LBFFS_CASE_DONE && r->state != LBFFS_CASE_FAILED)
        return srv_fail(s, LBFFS_E_STATE, "lbffs_server_release: case still queued or running");
    s->all.erase(id);
    return LBFFS_OK;
}

extern "C" int lbffs_server_get_stats(lbffs_server* s, lbffs_server_stats* o)
{
    if (!s || !o) return srv_fail(s, LBFFS_E_ARG, "lbffs_server_get_stats: null argument");
    std::lock_guard<std::mutex> lock(s->mu);
    memset(o, 0, sizeof(*o));
    o->submitted = s->submitted;
    o->completed = s->completed;
    o->failed = s->failed;
    o->resident = (long long)s->resident.size();
    o->queued = (long long)s->queue.size();
    o->rounds = s->rounds;
    o->graph_builds = s->graph_builds;
    o->cell_updates = s->cell_updates;
    o->elapsed_s = s->t_first >= 0 && s->completed ? s->t_last - s->t_first : 0.0;
    o->latency_p50_s = pct(s->latency, 0.50);
    o->latency_p99_s = pct(s->latency, 0.99);
    o->latency_max_s = pct(s->latency, 1.0);
    double m = 0;
    for (double v : s->latency) m += v;
    o->latency_mean_s = s->latency.empty() ? 0.0 : m / (double)s->latency.size();
    o->queue_wait_p50_s = pct(s->queue_wait, 0.50);
    o->queue_wait_p99_s = pct(s->queue_wait, 0.99);
    o->hbm_in_use = s->arena ? s->arena->in_use() : 0;
    o->hbm_peak = s->arena ? s->arena->peak() : 0;
    o->hbm_capacity = s->arena ? s->arena->capacity() : 0;
    o->gpu_busy_s = s->gpu_busy_s;
    o->build_s = s->build_s;
    o->mean_resident = s->rounds ? s->resident_sum / (double)s->rounds : 0.0;
    return LBFFS_OK;
}

extern "C" const char* lbffs_server_error(lbffs_server* s, long long id)
{
    if (!s) return "null server";
    std::lock_guard<std::mutex> lock(s->mu);
    if (id < 0) return s->err.c_str();
    Request* r = find(s, id);
    return r ? r->err.c_str() : "unknown id";
}

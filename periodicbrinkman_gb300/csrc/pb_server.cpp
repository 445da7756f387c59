// Continuous-batching request server.
//
// Requests of different sizes are autotuned on submission, assigned to the
// smallest provisioned FFT grid that holds their k-space resolution, and
// queued per grid.  A scheduler thread keeps a fixed set of resident slots
// (capacity plans with their own stream, buffers, pinned staging and CUDA
// graph): whenever a slot is idle it binds the next requests of its grid
// queue that fit its capacity, stages their inputs, and launches the slot's
// graph; slots run concurrently, so requests arriving while others are on the
// GPU are admitted as soon as a slot frees up.  Device memory is fixed at
// creation and bounded by the configured budget (admission by memory
// budget); a request no slot can hold is rejected at submission.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "pb_internal.h"
#include "pbrinkman.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    long long id;
    pb_solve_params p;
    pb::PbTables tab;  // real-space tables, built at submission
    int grid;
    int n_tgt_eff;
    const double *x, *f, *y;
    double* U;
    bool pin_in = false, pin_out = false;  // page-locked client buffers: copied by DMA, no staging
    Clock::time_point t_sub, t_done;
    std::atomic<int> state{0};  // 0 queued, 1 running, 2 done
    int status = PB_OK;
};

struct Slot {
    int grid = 0;
    pb_plan plan = nullptr;
    pb_slot_config cfg{};
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    double *x = nullptr, *f = nullptr, *y = nullptr, *U = nullptr;  // pinned staging
    bool busy = false;
    std::vector<Req*> reqs;
    std::vector<pb_solve_params> params;
    std::vector<pb::PbTables> tabs;
    std::vector<const double*> xs, fs, ys;
    std::vector<double*> Us;
};

std::string g_srv_err;

}  // namespace

struct pb_server_s {
    pb_server_config cfg{};
    std::vector<Slot> slots;
    std::vector<int> grids;
    long long device_bytes = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Req*> inbox;
    std::unordered_map<long long, Req*> reqs;
    std::vector<std::deque<Req*>> queues;  // per grid index
    std::thread worker;
    std::atomic<bool> stop{false};
    std::atomic<long long> next_id{1}, submitted{0}, completed{0}, failed{0}, rejected{0}, batches{0}, kernels{0},
        batched_instances{0};
    int device = 0;
    int npoly = 20;  // far-polynomial terms of every slot
    std::atomic<long long> busy_ns{0};
};

namespace {

bool page_locked(const void* ptr)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

int grid_index(pb_server_s* S, int g)
{
    for (size_t i = 0; i < S->grids.size(); i++)
        if (S->grids[i] >= g) return (int)i;
    return -1;
}

void finish_slot(pb_server_s* S, Slot& sl, int status)
{
    pb::NvtxRange nv("pb_server.finish");
    size_t off = 0;
    // work items beyond the slot's item array: every request of the execution lost pairs
    if (status == PB_OK && (pb::plan_exec_status(sl.plan) & pb::kCapItems)) status = PB_ERR_UNSUPPORTED;
    const int* bad = status == PB_OK ? pb::plan_bad_flags(sl.plan) : nullptr;
    for (size_t k = 0; k < sl.reqs.size(); k++) {
        Req* r = sl.reqs[k];
        size_t nb = 3 * (size_t)r->n_tgt_eff;
        if (status == PB_OK && !r->pin_out) std::memcpy(r->U, sl.U + off, nb * sizeof(double));
        off += nb;
        r->status = (bad && bad[k]) ? PB_ERR_INVALID : status;  // non-finite input, found on the device
        r->t_done = Clock::now();
        r->state.store(2);
        if (r->status == PB_OK)
            S->completed++;
        else
            S->failed++;
    }
    sl.reqs.clear();
    sl.busy = false;
}

bool dispatch(pb_server_s* S, Slot& sl, std::deque<Req*>& q)
{
    if (q.empty()) return false;
    pb::NvtxRange nv("pb_server.dispatch");
    const pb_slot_config& c = sl.cfg;
    // batching window: a short queue waits (up to linger_us after its oldest
    // request arrived) for more requests to share the slot execution
    if (S->cfg.linger_us > 0 && (int)q.size() < c.max_instances &&
        Clock::now() - q.front()->t_sub < std::chrono::microseconds(S->cfg.linger_us))
        return false;
    long long ns = 0, nt = 0, ny = 0;
    sl.reqs.clear();
    sl.params.clear();
    sl.tabs.clear();
    while (!q.empty() && (int)sl.reqs.size() < c.max_instances) {
        Req* r = q.front();
        long long n = r->p.n_src, m = r->n_tgt_eff;
        if (ns + n > c.max_src || nt + m > c.max_tgt) break;
        ns += n;
        nt += m;
        if (r->p.n_tgt > 0) ny += m;
        q.pop_front();
        sl.reqs.push_back(r);
        pb_solve_params p = r->p;
        p.M[0] = p.M[1] = p.M[2] = sl.grid;
        sl.params.push_back(p);
        sl.tabs.push_back(r->tab);
    }
    if (sl.reqs.empty()) return false;
    int rc = pb::plan_bind_prepared(sl.plan, sl.params.data(), sl.tabs.data(), (int)sl.params.size());
    if (rc == PB_ERR_BUDGET && sl.reqs.size() > 1) {
        // cells over capacity: put all back but the first and bind it alone
        for (size_t k = sl.reqs.size(); k-- > 1;) q.push_front(sl.reqs[k]);
        sl.reqs.resize(1);
        sl.params.resize(1);
        sl.tabs.resize(1);
        ns = sl.reqs[0]->p.n_src;
        nt = sl.reqs[0]->n_tgt_eff;
        ny = sl.reqs[0]->p.n_tgt > 0 ? nt : 0;
        rc = pb::plan_bind_prepared(sl.plan, sl.params.data(), sl.tabs.data(), 1);
    }
    if (rc != PB_OK) {
        finish_slot(S, sl, rc);
        return true;
    }
    // page-locked client buffers go to the device directly; others through the slot's staging
    sl.xs.clear();
    sl.fs.clear();
    sl.ys.clear();
    sl.Us.clear();
    size_t xo = 0, yo = 0, uo = 0;
    for (Req* r : sl.reqs) {
        size_t n3 = 3 * (size_t)r->p.n_src, m3 = 3 * (size_t)r->p.n_tgt;
        if (r->pin_in) {
            sl.xs.push_back(r->x);
            sl.fs.push_back(r->f);
            sl.ys.push_back(r->y);
        } else {
            std::memcpy(sl.x + xo, r->x, n3 * sizeof(double));
            std::memcpy(sl.f + xo, r->f, n3 * sizeof(double));
            sl.xs.push_back(sl.x + xo);
            sl.fs.push_back(sl.f + xo);
            xo += n3;
            if (r->p.n_tgt > 0) {
                std::memcpy(sl.y + yo, r->y, m3 * sizeof(double));
                sl.ys.push_back(sl.y + yo);
                yo += m3;
            } else {
                sl.ys.push_back(nullptr);
            }
        }
        sl.Us.push_back(r->pin_out ? r->U : sl.U + uo);
        uo += 3 * (size_t)r->n_tgt_eff;
        r->state.store(1);
    }
    rc = pb::plan_execute_parts(sl.plan, sl.xs.data(), sl.fs.data(), sl.ys.data(), sl.Us.data(), sl.stream);
    if (rc == PB_OK && cudaEventRecord(sl.done, sl.stream) != cudaSuccess) rc = PB_ERR_CUDA;
    if (rc != PB_OK) {
        finish_slot(S, sl, rc);
        return true;
    }
    sl.busy = true;
    S->batches++;
    S->kernels += pb_plan_kernel_count(sl.plan);
    S->batched_instances += (long long)sl.reqs.size();
    return true;
}

void worker_loop(pb_server_s* S)
{
    cudaSetDevice(S->device);
    while (!S->stop.load()) {
        bool did = false;
        for (Slot& sl : S->slots) {
            if (!sl.busy) continue;
            cudaError_t e = cudaEventQuery(sl.done);
            if (e == cudaSuccess) {
                finish_slot(S, sl, PB_OK);
                did = true;
            } else if (e != cudaErrorNotReady) {
                cudaGetLastError();
                finish_slot(S, sl, PB_ERR_CUDA);
                did = true;
            }
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            while (!S->inbox.empty()) {
                Req* r = S->inbox.front();
                S->inbox.pop_front();
                S->queues[r->grid].push_back(r);
            }
        }
        auto t0 = Clock::now();
        for (Slot& sl : S->slots) {
            if (sl.busy) continue;
            int gi = grid_index(S, sl.grid);
            if (gi >= 0 && dispatch(S, sl, S->queues[gi])) did = true;
        }
        if (did) S->busy_ns += std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count();
        if (!did) {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv.wait_for(lk, std::chrono::microseconds(50), [&] { return !S->inbox.empty() || S->stop.load(); });
        }
    }
}

void destroy_slots(pb_server_s* S)
{
    for (Slot& sl : S->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.plan) pb_plan_destroy(sl.plan);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        for (double* p : {sl.x, sl.f, sl.y, sl.U})
            if (p) cudaFreeHost(p);
    }
    S->slots.clear();
}

}  // namespace

extern "C" {

int pb_server_create(const pb_server_config* cfg_in, pb_server* out)
{
    if (!out) return PB_ERR_INVALID;
    *out = nullptr;
    if (pb_device_count() <= 0) return PB_ERR_CUDA;
    pb_server_config cfg = cfg_in ? *cfg_in : pb_server_config{};
    if (cfg.budget_bytes <= 0) cfg.budget_bytes = 150LL << 30;
    if (cfg.max_batch <= 0) cfg.max_batch = 16;
    if (cfg.slots_per_grid <= 0) cfg.slots_per_grid = 2;
    if (cfg.max_src <= 0) cfg.max_src = 1 << 18;
    if (cfg.max_tgt <= 0) cfg.max_tgt = cfg.max_src;
    if (cfg.n_grids <= 0) {
        int dg[] = {8, 16, 32, 64, 128, 256};
        cfg.n_grids = 6;
        for (int i = 0; i < 6; i++) cfg.grids[i] = dg[i];
    }
    if (cfg.n_grids > 8) return PB_ERR_INVALID;
    pb_server_s* S = new pb_server_s();
    S->cfg = cfg;
    cudaGetDevice(&S->device);
    for (int i = 0; i < cfg.n_grids; i++) S->grids.push_back(cfg.grids[i]);
    std::sort(S->grids.begin(), S->grids.end());
    S->queues.resize(S->grids.size());
    long long used = 0;
    for (int g : S->grids) {
        for (int k = 0; k < cfg.slots_per_grid; k++) {
            Slot sl;
            sl.grid = g;
            sl.cfg.M[0] = sl.cfg.M[1] = sl.cfg.M[2] = g;
            // large grids hold fewer instances: keep the grids of one slot near 1/8 of the budget share
            long long gbytes = 3LL * g * g * g * (cfg.precision == PB_PREC_FP64 ? 8 : 4) * 2;
            long long share = cfg.budget_bytes / (long long)(S->grids.size() * cfg.slots_per_grid);
            int B = (int)std::max(1LL, std::min<long long>(cfg.max_batch, share / (2 * gbytes)));
            sl.cfg.max_instances = B;
            sl.cfg.max_src = cfg.max_src;
            sl.cfg.max_tgt = cfg.max_tgt;
            // cells: the autotuner keeps rc >= ~4.6 grid spacings, so an instance has
            // at most (M/2)^3 cells
            sl.cfg.max_cells = (int)std::min<long long>(1 << 21, (long long)B * (g / 2) * (g / 2) * (g / 2));
            sl.cfg.precision = cfg.precision;
            sl.cfg.npoly = S->npoly;
            long long est = pb_slot_estimate_bytes(&sl.cfg);
            if (est < 0 || used + est > cfg.budget_bytes) continue;
            int rc = pb_plan_create_slot(&sl.cfg, &sl.plan);
            if (rc != PB_OK) {
                g_srv_err = pb_last_error();
                S->slots.push_back(sl);
                destroy_slots(S);
                delete S;
                return rc;
            }
            used += est;
            cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
            cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
            size_t xs = 3 * (size_t)cfg.max_src * sizeof(double), ts = 3 * (size_t)cfg.max_tgt * sizeof(double);
            if (cudaMallocHost(&sl.x, xs) != cudaSuccess || cudaMallocHost(&sl.f, xs) != cudaSuccess ||
                cudaMallocHost(&sl.y, ts) != cudaSuccess || cudaMallocHost(&sl.U, ts) != cudaSuccess) {
                S->slots.push_back(sl);
                destroy_slots(S);
                delete S;
                return PB_ERR_NOMEM;
            }
            S->slots.push_back(sl);
        }
    }
    if (S->slots.empty()) {
        delete S;
        return PB_ERR_BUDGET;
    }
    S->device_bytes = used;
    S->worker = std::thread(worker_loop, S);
    *out = S;
    return PB_OK;
}

int pb_server_submit(pb_server S, const pb_solve_params* p, const double* x, const double* f, const double* y,
                     double* U, long long* ticket)
{
    if (!S || !p || !ticket) return PB_ERR_INVALID;
    *ticket = 0;
    if (p->precision != S->cfg.precision) return PB_ERR_INVALID;
    if (p->n_src <= 0 || (p->n_tgt > 0 && !y) || !x || !f || !U) return PB_ERR_INVALID;
    pb::NvtxRange nv("pb_server_submit");
    // autotune and build the real-space tables here, in the caller's thread, so
    // the scheduler only binds.  The instance runs on its slot's grid: when the
    // autotuned grid is not a provisioned one, resolve again for the slot's grid.
    Req* r = new Req();
    pb_instance_info info;
    int rc = pb::prepare_instance(*p, S->npoly, &r->tab, &info);
    if (rc != PB_OK) {
        delete r;
        return rc;
    }
    const int need = std::max(info.M[0], std::max(info.M[1], info.M[2]));
    const int gi = grid_index(S, need);
    if (gi >= 0 && !(info.M[0] == S->grids[gi] && info.M[1] == S->grids[gi] && info.M[2] == S->grids[gi])) {
        pb_solve_params pg = *p;
        pg.M[0] = pg.M[1] = pg.M[2] = S->grids[gi];
        rc = pb::prepare_instance(pg, S->npoly, &r->tab, &info);
        if (rc != PB_OK) {
            delete r;
            return rc;
        }
    }
    int n_tgt_eff = p->n_tgt > 0 ? p->n_tgt : p->n_src;
    const long long cells = (long long)info.ncell[0] * info.ncell[1] * info.ncell[2];
    bool fits = false;
    for (const Slot& sl : S->slots)
        if (gi >= 0 && sl.grid == S->grids[gi] && p->n_src <= sl.cfg.max_src && n_tgt_eff <= sl.cfg.max_tgt &&
            cells <= sl.cfg.max_cells)
            fits = true;
    if (!fits) {
        delete r;
        S->rejected++;
        return PB_ERR_BUDGET;
    }
    r->id = S->next_id++;
    // the resolved splitting, support and grid go with the request, so that
    // binding it reproduces the instance its tables were built for
    r->p = *p;
    r->p.d = info.d;
    r->p.rc = info.rc;
    r->p.P = info.P;
    for (int a = 0; a < 3; a++) r->p.M[a] = info.M[a];
    r->grid = gi;
    r->n_tgt_eff = n_tgt_eff;
    r->x = x;
    r->f = f;
    r->y = y;
    r->U = U;
    r->pin_in = page_locked(x) && page_locked(f) && (p->n_tgt <= 0 || page_locked(y));
    r->pin_out = page_locked(U);
    r->t_sub = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->cfg.queue_capacity > 0 && (long long)S->inbox.size() >= S->cfg.queue_capacity) {
            delete r;
            S->rejected++;
            return PB_ERR_BUSY;
        }
        S->reqs[r->id] = r;
        S->inbox.push_back(r);
    }
    S->submitted++;
    S->cv.notify_one();
    *ticket = r->id;
    return PB_OK;
}

int pb_server_poll(pb_server S, long long ticket, int* state, int* status, double* latency_s)
{
    if (!S) return PB_ERR_INVALID;
    Req* r = nullptr;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->reqs.find(ticket);
        if (it == S->reqs.end()) return PB_ERR_INVALID;
        r = it->second;
    }
    int st = r->state.load();
    if (state) *state = st;
    if (st == 2) {
        if (status) *status = r->status;
        if (latency_s) *latency_s = std::chrono::duration<double>(r->t_done - r->t_sub).count();
    }
    return PB_OK;
}

int pb_server_release(pb_server S, long long ticket)
{
    if (!S) return PB_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return PB_ERR_INVALID;
    if (it->second->state.load() != 2) return PB_ERR_BUSY;
    delete it->second;
    S->reqs.erase(it);
    return PB_OK;
}

int pb_server_wait(pb_server S, long long ticket, double timeout_s, int* status, double* latency_s)
{
    auto t0 = Clock::now();
    while (true) {
        int state = 0;
        int rc = pb_server_poll(S, ticket, &state, status, latency_s);
        if (rc != PB_OK) return rc;
        if (state == 2) return PB_OK;
        if (timeout_s >= 0 && std::chrono::duration<double>(Clock::now() - t0).count() > timeout_s) return PB_ERR_BUSY;
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

int pb_server_drain(pb_server S, double timeout_s)
{
    if (!S) return PB_ERR_INVALID;
    auto t0 = Clock::now();
    while (S->completed.load() + S->failed.load() < S->submitted.load()) {
        if (timeout_s >= 0 && std::chrono::duration<double>(Clock::now() - t0).count() > timeout_s) return PB_ERR_BUSY;
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    return PB_OK;
}

int pb_server_stats(pb_server S, pb_server_counters* out)
{
    if (!S || !out) return PB_ERR_INVALID;
    out->submitted = S->submitted.load();
    out->completed = S->completed.load();
    out->failed = S->failed.load();
    out->rejected = S->rejected.load();
    out->batches = S->batches.load();
    out->mean_batch = out->batches ? (double)S->batched_instances.load() / out->batches : 0.0;
    out->device_bytes = S->device_bytes;
    out->slots = (int)S->slots.size();
    out->kernels = S->kernels.load();
    out->scheduler_busy_s = 1e-9 * (double)S->busy_ns.load();
    return PB_OK;
}

int pb_server_destroy(pb_server S)
{
    if (!S) return PB_OK;
    S->stop.store(true);
    S->cv.notify_all();
    if (S->worker.joinable()) S->worker.join();
    destroy_slots(S);
    for (auto& kv : S->reqs) delete kv.second;
    delete S;
    return PB_OK;
}

}  // extern "C"

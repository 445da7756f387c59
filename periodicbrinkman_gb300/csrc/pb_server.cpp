// Continuous-batching request server.
//
// Requests of different sizes are autotuned on submission, assigned to the
// smallest provisioned FFT grid that holds their k-space resolution, and
// queued per grid.  A scheduler thread keeps a set of slots (capacity plans
// with their own stream, buffers, pinned staging and CUDA graph): whenever a
// slot is idle it binds the next requests of its grid queue that fit its
// capacity, stages their inputs, and launches the slot's graph; slots run
// concurrently, so requests arriving while others are on the GPU are
// admitted as soon as a slot frees up.
//
// Admission by device-memory budget: the resident slots are created with the
// server; the part of the budget they leave is given out as dynamic slots,
// sized for a request that no slot of its grid can hold, or of the resident
// size when a grid's queue backs up while all its slots are busy.  When the
// budget is taken the request waits in its queue; idle dynamic slots are
// released (least recently used first) to make room, and dynamic slots idle
// for dynamic_idle_ms are released anyway.  Only a request that a slot of
// its own could not fit within the whole budget is rejected at submission.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
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
    long long cells = 0;       // real-space cells of the instance on its slot's grid
    bool waited = false;       // counted once in memory_waits
    const double *x, *f, *y;
    double* U;
    bool pin_in = false, pin_out = false;  // page-locked client buffers: copied by DMA, no staging
    Clock::time_point t_sub, t_done;
    std::atomic<int> state{0};  // 0 queued, 1 running, 2 done
    int status = PB_OK;
};

struct Slot {
    int grid = 0;
    bool dynamic = false;       // made from the unused budget; released when idle
    long long bytes = 0;        // device bytes of its plan
    Clock::time_point last_used;
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
    std::vector<std::unique_ptr<Slot>> slots;
    std::vector<int> grids;
    std::atomic<long long> device_bytes{0}, peak_bytes{0}, slots_created{0}, slots_released{0}, memory_waits{0};
    std::atomic<int> nslots{0};
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
    int npoly = 18;  // far-polynomial terms of every slot (longer fits are truncated to it)
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
    // work items beyond the slot's item array: every request of the execution lost pairs;
    // a cell-count scan that gave up: the cell lists of the execution are not valid
    if (status == PB_OK && (pb::plan_exec_status(sl.plan) & pb::kCapItems)) status = PB_ERR_UNSUPPORTED;
    if (status == PB_OK && (pb::plan_exec_status(sl.plan) & pb::kScanStall)) status = PB_ERR_CUDA;
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
    sl.last_used = Clock::now();
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

// Capacity of a slot of grid g holding requests of up to (src, tgt, cells),
// with the batch size of the resident slots (large grids hold fewer instances:
// a slot's grids stay near an eighth of the per-slot budget share).
pb_slot_config slot_config(const pb_server_s* S, int g, long long src, long long tgt, long long cells, int B)
{
    const pb_server_config& cfg = S->cfg;
    pb_slot_config c{};
    c.M[0] = c.M[1] = c.M[2] = g;
    if (B <= 0) {
        long long gbytes = 3LL * g * g * g * (cfg.precision == PB_PREC_FP64 ? 8 : 4) * 2;
        long long share = cfg.budget_bytes / (long long)(S->grids.size() * std::max(1, cfg.slots_per_grid));
        B = (int)std::max(1LL, std::min<long long>(cfg.max_batch, share / (2 * gbytes)));
    }
    c.max_instances = B;
    c.max_src = (int)std::max<long long>(cfg.max_src, src);
    c.max_tgt = (int)std::max<long long>(cfg.max_tgt, tgt);
    // cells: the autotuner keeps rc >= ~4.6 grid spacings, so an instance has at most (M/2)^3 cells
    c.max_cells = (int)std::min<long long>(1 << 21, (long long)B * (g / 2) * (g / 2) * (g / 2));
    c.max_cells = (int)std::max<long long>(c.max_cells, cells);
    c.precision = cfg.precision;
    c.npoly = S->npoly;
    return c;
}

bool holds(const Slot& sl, const Req* r)
{
    return r->p.n_src <= sl.cfg.max_src && r->n_tgt_eff <= sl.cfg.max_tgt && r->cells <= sl.cfg.max_cells;
}

void free_slot(Slot& sl)
{
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.plan) pb_plan_destroy(sl.plan);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    for (double* p : {sl.x, sl.f, sl.y, sl.U})
        if (p) cudaFreeHost(p);
    sl.plan = nullptr;
    sl.done = nullptr;
    sl.stream = nullptr;
    sl.x = sl.f = sl.y = sl.U = nullptr;
}

// Creates a slot with capacity c (device memory accounted by its estimate).
int make_slot(pb_server_s* S, const pb_slot_config& c, bool dynamic, long long est, std::unique_ptr<Slot>& out)
{
    auto sl = std::make_unique<Slot>();
    sl->grid = c.M[0];
    sl->cfg = c;
    sl->dynamic = dynamic;
    sl->bytes = est;
    sl->last_used = Clock::now();
    int rc = pb_plan_create_slot(&c, &sl->plan);
    if (rc != PB_OK) {
        g_srv_err = pb_last_error();
        free_slot(*sl);
        return rc;
    }
    size_t xs = 3 * (size_t)c.max_src * sizeof(double), ts = 3 * (size_t)c.max_tgt * sizeof(double);
    if (cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost(&sl->x, xs) != cudaSuccess || cudaMallocHost(&sl->f, xs) != cudaSuccess ||
        cudaMallocHost(&sl->y, ts) != cudaSuccess || cudaMallocHost(&sl->U, ts) != cudaSuccess) {
        cudaGetLastError();
        free_slot(*sl);
        return PB_ERR_NOMEM;
    }
    long long now = (S->device_bytes += est);
    long long pk = S->peak_bytes.load();
    while (now > pk && !S->peak_bytes.compare_exchange_weak(pk, now)) {
    }
    out = std::move(sl);
    return PB_OK;
}

void release_slot(pb_server_s* S, size_t i)
{
    S->device_bytes -= S->slots[i]->bytes;
    free_slot(*S->slots[i]);
    S->slots.erase(S->slots.begin() + (long)i);
    S->slots_released++;
    S->nslots = (int)S->slots.size();
}

// Releases idle dynamic slots, least recently used first, until `need` bytes
// fit the budget; true when they do.
bool make_room(pb_server_s* S, long long need)
{
    while (S->device_bytes.load() + need > S->cfg.budget_bytes) {
        long best = -1;
        for (size_t i = 0; i < S->slots.size(); i++) {
            const Slot& sl = *S->slots[i];
            if (sl.dynamic && !sl.busy && (best < 0 || sl.last_used < S->slots[(size_t)best]->last_used)) best = (long)i;
        }
        if (best < 0) return false;
        release_slot(S, (size_t)best);
    }
    return true;
}

// The head request of grid gi's queue has no slot to go to: a dynamic slot
// sized for it (or of the resident size, to add concurrency), from the
// unused budget; returns the new slot or null (then the request waits).
Slot* grow(pb_server_s* S, int gi, const Req* head, bool for_capacity)
{
    const int g = S->grids[(size_t)gi];
    int ndyn = 0;
    for (auto& sl : S->slots)
        if (sl->grid == g && sl->dynamic) ndyn++;
    const int max_dyn = S->cfg.max_dynamic_per_grid < 0 ? 0
                        : S->cfg.max_dynamic_per_grid > 0 ? S->cfg.max_dynamic_per_grid
                                                          : std::max(1, S->cfg.slots_per_grid);
    if (!for_capacity && ndyn >= max_dyn) return nullptr;
    // the resident batch size when the budget allows it, else fewer instances
    for (int B = slot_config(S, g, 0, 0, 0, 0).max_instances;; B /= 2) {
        pb_slot_config c = slot_config(S, g, head->p.n_src, head->n_tgt_eff, head->cells, B);
        const long long est = pb_slot_estimate_bytes(&c);
        if (est > 0 && est <= S->cfg.budget_bytes && make_room(S, est)) {
            std::unique_ptr<Slot> sl;
            if (make_slot(S, c, true, est, sl) != PB_OK) return nullptr;
            S->slots_created++;
            S->slots.push_back(std::move(sl));
            S->nslots = (int)S->slots.size();
            return S->slots.back().get();
        }
        if (B <= 1 || !for_capacity) break;
    }
    return nullptr;
}

void worker_loop(pb_server_s* S)
{
    cudaSetDevice(S->device);
    const auto idle_release = std::chrono::milliseconds(S->cfg.dynamic_idle_ms > 0 ? S->cfg.dynamic_idle_ms : 1000);
    while (!S->stop.load()) {
        bool did = false;
        for (auto& slp : S->slots) {
            Slot& sl = *slp;
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
        for (size_t gi = 0; gi < S->grids.size(); gi++) {
            std::deque<Req*>& q = S->queues[gi];
            const int g = S->grids[gi];
            for (size_t k = 0; k < S->slots.size() && !q.empty(); k++) {
                Slot& sl = *S->slots[k];
                if (sl.grid == g && !sl.busy && dispatch(S, sl, q)) did = true;
            }
            if (q.empty()) continue;
            // the head request still waits: no slot of its grid can hold it, or
            // they are all busy while the queue backs up
            Req* head = q.front();
            bool fits = false, all_busy = true;
            for (auto& sl : S->slots)
                if (sl->grid == g) {
                    fits = fits || holds(*sl, head);
                    all_busy = all_busy && sl->busy;
                }
            const bool backlog = all_busy && (int)q.size() >= std::max(2, S->cfg.max_batch);
            if (!fits || backlog) {
                Slot* ns = grow(S, (int)gi, head, !fits);
                if (ns) {
                    if (dispatch(S, *ns, q)) did = true;
                } else if (!fits && !head->waited) {
                    head->waited = true;
                    S->memory_waits++;
                }
            }
        }
        // dynamic slots idle for a while give their memory back
        const auto now = Clock::now();
        for (size_t i = 0; i < S->slots.size();) {
            const Slot& sl = *S->slots[i];
            if (sl.dynamic && !sl.busy && now - sl.last_used > idle_release)
                release_slot(S, i);
            else
                i++;
        }
        if (did) S->busy_ns += std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count();
        if (!did) {
            // While a slot runs, keep polling its completion event (a timed sleep
            // here is rounded up by the OS timer slack, and every request that
            // finishes meanwhile waits out the rest of it); with nothing on the
            // GPU, sleep until a submission arrives.
            bool any_busy = false;
            for (auto& sl : S->slots) any_busy = any_busy || sl->busy;
            if (any_busy) {
                std::this_thread::yield();
            } else {
                std::unique_lock<std::mutex> lk(S->mu);
                S->cv.wait_for(lk, std::chrono::microseconds(50), [&] { return !S->inbox.empty() || S->stop.load(); });
            }
        }
    }
}

void destroy_slots(pb_server_s* S)
{
    for (auto& sl : S->slots) free_slot(*sl);
    S->slots.clear();
    S->device_bytes = 0;
    S->nslots = 0;
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
    if (cfg.max_batch <= 0) cfg.max_batch = 4;
    if (cfg.slots_per_grid <= 0) cfg.slots_per_grid = 4;
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
    for (int g : S->grids) {
        for (int k = 0; k < cfg.slots_per_grid; k++) {
            pb_slot_config c = slot_config(S, g, 0, 0, 0, 0);
            long long est = pb_slot_estimate_bytes(&c);
            if (est < 0 || S->device_bytes.load() + est > cfg.budget_bytes) continue;
            std::unique_ptr<Slot> sl;
            int rc = make_slot(S, c, false, est, sl);
            if (rc != PB_OK) {
                destroy_slots(S);
                delete S;
                return rc;
            }
            S->slots.push_back(std::move(sl));
        }
    }
    S->nslots = (int)S->slots.size();
    if (S->slots.empty()) {
        delete S;
        return PB_ERR_BUDGET;
    }
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
    // admitted when a slot of its own (one instance) would fit the whole budget;
    // whether memory is free now is the scheduler's concern
    bool fits = gi >= 0;
    if (fits) {
        pb_slot_config c = slot_config(S, S->grids[gi], p->n_src, n_tgt_eff, cells, 1);
        const long long est = pb_slot_estimate_bytes(&c);
        fits = est > 0 && est <= S->cfg.budget_bytes;
    }
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
    r->cells = cells;
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
    out->device_bytes = S->device_bytes.load();
    out->slots = S->nslots.load();
    out->peak_device_bytes = S->peak_bytes.load();
    out->slots_created = S->slots_created.load();
    out->slots_released = S->slots_released.load();
    out->memory_waits = S->memory_waits.load();
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

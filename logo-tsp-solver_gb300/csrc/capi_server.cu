// C ABI of the request server (include/logo_gpu.h, "serving").
//
// One scheduler thread owns the device side of small requests
// (n <= LOGO_BATCH_MAX_N):
//   admit   -- FIFO over the pending queue; a request is admitted when a slot
//              is free and the device arena has room for it under the memory
//              budget (first-fit allocator); its coordinates and start tour
//              are copied into the arena, where its tours stay resident;
//   round   -- one serve_round_kernel launch advances every admitted request
//              by a bounded quantum of work (serve.cu);
//   retire  -- finished requests copy their best tour out, free their slot and
//              arena space, and become visible to logo_server_poll.
// Larger requests run on worker threads through the single-instance path
// (logo_ctx, multi-CTA sweeps) under the same memory budget, concurrently
// with the rounds.  No reference counterpart.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/logo_gpu.h"
#include "logo_device.cuh"
#include "batch_internal.h"
#include "logo_internal.h"
#include "serve_internal.h"

using namespace logo;

namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

enum ReqState { kPending = 0, kRunning = 1, kDone = 2 };

struct Req {
    uint64_t id = 0;
    uint32_t n = 0;
    uint64_t seed = 0;
    float margin = 0.f;
    std::vector<logo_xy> xy;
    std::vector<uint32_t> route;  // start tour, then the result
    ReqState state = kPending;
    bool large = false;
    int slot = -1;
    uint64_t arena_off = 0;
    uint64_t mem = 0;
    logo_request_info info{};
    Clock::time_point t_submit, t_admit, t_done;
};

// First-fit allocator over [0, cap) city units with coalescing frees.
class Arena {
public:
    explicit Arena(uint64_t cap = 0) { reset(cap); }
    void reset(uint64_t cap) {
        free_.clear();
        if (cap) free_[0] = cap;
    }
    bool alloc(uint64_t len, uint64_t* off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= len) {
                *off = it->first;
                const uint64_t rest = it->second - len, start = it->first + len;
                free_.erase(it);
                if (rest) free_[start] = rest;
                return true;
            }
        }
        return false;
    }
    void release(uint64_t off, uint64_t len) {
        auto it = free_.emplace(off, len).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }

private:
    std::map<uint64_t, uint64_t> free_;
};

constexpr uint64_t kSmallBytesPerCity = sizeof(float2) + 2 * sizeof(uint32_t);
// device bytes per city of the single-instance path (coordinates, two tour
// buffers of ordered cities and routes, best tour, and the boxed sweep's city
// positions and near-neighbour lists)
constexpr uint64_t kLargeBytesPerCity = 8 + 2 * 16 + 2 * 4 + 16 + 4 + 4 * (1 + kSeedNeighbours);

thread_local std::string g_server_err;

}  // namespace

struct logo_server {
    logo_server_opts opts{};
    int device = 0;
    int sms = 0;
    int occ = 1;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint64_t arena_cap = 0;
    float2* d_coords = nullptr;
    uint32_t* d_route = nullptr;
    uint32_t* d_best = nullptr;
    ServeSlot* d_slots = nullptr;
    ServeSlot* h_slots = nullptr;
    uint32_t* d_units = nullptr;
    uint32_t* h_units = nullptr;
    unsigned int* d_queue = nullptr;
    Arena arena;
    std::vector<int64_t> slot_req;  // request id per slot, -1 if free

    std::mutex mu;
    std::condition_variable cv;       // wakes the scheduler
    std::condition_variable done_cv;  // wakes waiters
    std::deque<uint64_t> pending;
    std::deque<uint64_t> large_ready;  // admitted large requests for the workers
    std::condition_variable large_cv;
    std::unordered_map<uint64_t, Req> reqs;
    uint64_t next_id = 1;
    uint64_t mem_in_use = 0;
    uint32_t running_small = 0, running_large = 0;
    logo_server_stats stats{};
    std::atomic<bool> stop{false};
    std::thread sched;
    std::vector<std::thread> workers;
    std::string err;
};

namespace {

logo_status sfail(logo_server* s, logo_status st, const std::string& m) {
    if (s)
        s->err = m;
    else
        g_server_err = m;
    return st;
}

void finish(logo_server* s, Req& r) {  // with s->mu held
    r.state = kDone;
    r.t_done = Clock::now();
    r.info.queue_ms = ms_since(r.t_submit, r.t_admit);
    r.info.latency_ms = ms_since(r.t_submit, r.t_done);
    s->stats.completed++;
    if (r.info.status != LOGO_OK) s->stats.failed++;
    s->done_cv.notify_all();
}

void run_large(logo_server* s, uint64_t id);

// One of opts.max_large worker threads: solves admitted large requests
// through the single-instance path.
void large_worker(logo_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        uint64_t id;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->large_cv.wait(lk, [&] { return s->stop || !s->large_ready.empty(); });
            if (s->large_ready.empty()) return;  // stopping
            id = s->large_ready.front();
            s->large_ready.pop_front();
        }
        run_large(s, id);
    }
}

void run_large(logo_server* s, uint64_t id) {
    std::vector<logo_xy> xy;
    std::vector<uint32_t> route;
    uint32_t n;
    uint64_t seed;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        Req& r = s->reqs[id];
        xy = r.xy;
        route = r.route;
        n = r.n;
        seed = r.seed;
    }
    logo_ctx* ctx = nullptr;
    logo_stats st{};
    logo_status rc = logo_ctx_create(s->device, xy.data(), n, &ctx);
    if (rc == LOGO_OK)
        rc = logo_ils(ctx, route.data(), s->opts.kicks, seed, s->opts.kick_kind, &st);
    logo_ctx_destroy(ctx);
    std::lock_guard<std::mutex> lk(s->mu);
    Req& r = s->reqs[id];
    r.route = route;
    r.info.start_length = st.start_length;
    r.info.best_length = st.final_length;
    r.info.moves = st.moves;
    r.info.sweeps = st.sweeps;
    r.info.kicks = (uint32_t)st.kicks;
    r.info.accepted = (uint32_t)st.accepted;
    r.info.status = rc;
    s->mem_in_use -= r.mem;
    s->running_large--;
    finish(s, r);
    s->cv.notify_all();
}

// Admits pending requests that fit (FIFO order, skipping over the ones that
// do not fit yet).  Called with s->mu held.
void admit(logo_server* s) {
    for (auto it = s->pending.begin(); it != s->pending.end();) {
        Req& r = s->reqs[*it];
        bool ok = false;
        if (r.large) {
            const uint64_t mem = kLargeBytesPerCity * r.n;
            if (s->running_large < s->opts.max_large && s->mem_in_use + mem <= s->opts.mem_budget) {
                r.mem = mem;
                s->mem_in_use += mem;
                s->running_large++;
                r.state = kRunning;
                r.t_admit = Clock::now();
                s->large_ready.push_back(r.id);
                s->large_cv.notify_one();
                ok = true;
            }
        } else {
            const uint64_t mem = kSmallBytesPerCity * r.n;
            int slot = -1;
            for (size_t k = 0; k < s->slot_req.size(); ++k)
                if (s->slot_req[k] < 0) {
                    slot = (int)k;
                    break;
                }
            uint64_t off = 0;
            if (slot >= 0 && s->mem_in_use + mem <= s->opts.mem_budget &&
                s->arena.alloc(r.n, &off)) {
                r.slot = slot;
                r.arena_off = off;
                r.mem = mem;
                s->mem_in_use += mem;
                s->slot_req[slot] = (int64_t)r.id;
                s->running_small++;
                r.state = kRunning;
                r.t_admit = Clock::now();
                cudaMemcpyAsync(s->d_coords + off, r.xy.data(), sizeof(float2) * r.n,
                                cudaMemcpyHostToDevice, s->stream);
                cudaMemcpyAsync(s->d_route + off, r.route.data(), sizeof(uint32_t) * r.n,
                                cudaMemcpyHostToDevice, s->stream);
                ServeSlot& st = s->h_slots[slot];
                std::memset(&st, 0, sizeof(st));
                st.off = off;
                st.rng = r.seed;
                st.n = r.n;
                st.phase = kServeInit;
                st.kicks_total = s->opts.kicks;
                st.kick_kind = s->opts.kick_kind;
                st.margin = r.margin;
                cudaMemcpyAsync(s->d_slots + slot, &st, sizeof(ServeSlot), cudaMemcpyHostToDevice,
                                s->stream);
                ok = true;
            }
        }
        if (ok) {
            s->stats.admitted++;
            it = s->pending.erase(it);
        } else {
            ++it;
        }
    }
}

void scheduler(logo_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (!s->stop) {
        admit(s);
        if (s->running_small == 0) {
            s->cv.wait_for(lk, std::chrono::milliseconds(2));
            continue;
        }
        // this round's units: running slots, largest first
        std::vector<std::pair<uint32_t, uint32_t>> act;
        uint32_t max_n = 0;
        for (size_t k = 0; k < s->slot_req.size(); ++k)
            if (s->slot_req[k] >= 0) {
                const uint32_t n = s->h_slots[k].n;
                act.emplace_back(n, (uint32_t)k);
                max_n = std::max(max_n, n);
            }
        std::sort(act.begin(), act.end(), [](auto& a, auto& b) { return a.first > b.first; });
        for (size_t k = 0; k < act.size(); ++k) s->h_units[k] = act[k].second;
        const bool large_running = s->running_large > 0;
        lk.unlock();

        ServeArgs A;
        A.coords = s->d_coords;
        A.route = s->d_route;
        A.best = s->d_best;
        A.slots = s->d_slots;
        A.units = s->d_units;
        A.nunits = (uint32_t)act.size();
        A.queue = s->d_queue;
        A.max_n = max_n;
        A.budget_pairs = s->opts.quantum_pairs;
        int occ = 1;
        launch_serve_round(A, 0, nullptr, &occ);
        int full = std::max(1, occ) * s->sms;
        // leave room for the single-instance kernels of large requests
        if (large_running) full = std::max(1, full * 3 / 4);
        const int grid = std::min<int>(full, (int)act.size());
        cudaMemcpyAsync(s->d_units, s->h_units, sizeof(uint32_t) * act.size(),
                        cudaMemcpyHostToDevice, s->stream);
        cudaMemsetAsync(s->d_queue, 0, sizeof(unsigned int), s->stream);
        cudaEventRecord(s->ev0, s->stream);
        cudaError_t e = launch_serve_round(A, grid, s->stream, nullptr);
        cudaEventRecord(s->ev1, s->stream);
        cudaMemcpyAsync(s->h_slots, s->d_slots, sizeof(ServeSlot) * s->slot_req.size(),
                        cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, s->ev0, s->ev1);

        lk.lock();
        s->stats.rounds++;
        s->stats.round_device_ms += ms;
        // retire finished (or failed) requests
        std::vector<uint64_t> done;
        for (size_t k = 0; k < s->slot_req.size(); ++k) {
            if (s->slot_req[k] < 0) continue;
            if (e != cudaSuccess || s->h_slots[k].phase == kServeDone) done.push_back(k);
        }
        for (uint64_t k : done) {
            Req& r = s->reqs[(uint64_t)s->slot_req[k]];
            const ServeSlot& st = s->h_slots[k];
            if (e == cudaSuccess)
                cudaMemcpyAsync(r.route.data(), s->d_best + r.arena_off, sizeof(uint32_t) * r.n,
                                cudaMemcpyDeviceToHost, s->stream);
            r.info.start_length = st.start_len;
            r.info.best_length = st.best_len;
            r.info.moves = st.moves;
            r.info.sweeps = st.sweeps;
            r.info.kicks = st.kicks_done;
            r.info.accepted = st.accepted;
            r.info.status = e != cudaSuccess ? LOGO_ERR_CUDA
                            : (st.status & kErrBadKey) ? LOGO_ERR_DEVICE_FAULT
                            : (st.status & kErrMoveLimit) ? LOGO_ERR_MOVE_LIMIT
                                                          : LOGO_OK;
        }
        if (!done.empty()) cudaStreamSynchronize(s->stream);
        for (uint64_t k : done) {
            Req& r = s->reqs[(uint64_t)s->slot_req[k]];
            s->arena.release(r.arena_off, r.n);
            s->mem_in_use -= r.mem;
            s->slot_req[k] = -1;
            s->running_small--;
            finish(s, r);
        }
        if (e != cudaSuccess) s->err = std::string("round failed: ") + cudaGetErrorString(e);
    }
}

void free_server(logo_server* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    cudaFree(s->d_coords);
    cudaFree(s->d_route);
    cudaFree(s->d_best);
    cudaFree(s->d_slots);
    cudaFree(s->d_units);
    cudaFree(s->d_queue);
    if (s->h_slots) cudaFreeHost(s->h_slots);
    if (s->h_units) cudaFreeHost(s->h_units);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

}  // namespace

extern "C" {

const char* logo_server_last_error(const logo_server* s) {
    return s ? s->err.c_str() : g_server_err.c_str();
}

logo_status logo_server_create(const logo_server_opts* o, logo_server** out) {
    if (!o || !out) return sfail(nullptr, LOGO_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (o->kick_kind != LOGO_KICK_SEGMENT && o->kick_kind != LOGO_KICK_DOUBLE_BRIDGE)
        return sfail(nullptr, LOGO_ERR_INVALID_ARG, "unknown kick kind");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return sfail(nullptr, LOGO_ERR_NO_DEVICE, "no CUDA device");
    if (o->device < 0 || o->device >= ndev)
        return sfail(nullptr, LOGO_ERR_INVALID_ARG, "device index out of range");
    cudaSetDevice(o->device);
    logo_server* s = new logo_server();
    s->opts = *o;
    s->device = o->device;
    if (!s->opts.mem_budget) s->opts.mem_budget = 2ull << 30;
    if (!s->opts.max_large) s->opts.max_large = 2;
    if (!s->opts.quantum_pairs) s->opts.quantum_pairs = 20000000ull;
    if (!s->opts.max_pending) s->opts.max_pending = 1000000;
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, o->device);
    s->sms = prop.multiProcessorCount;
    {
        ServeArgs A{};
        A.max_n = kBatchMaxN;
        launch_serve_round(A, 0, nullptr, &s->occ);
        if (s->occ < 1) s->occ = 1;
    }
    if (!s->opts.max_slots) s->opts.max_slots = (uint32_t)(s->occ * s->sms * 2);
    s->arena_cap = s->opts.mem_budget / kSmallBytesPerCity;
    s->arena.reset(s->arena_cap);
    s->slot_req.assign(s->opts.max_slots, -1);
    auto bail = [&](cudaError_t e, const char* what) {
        g_server_err = std::string(what) + ": " + cudaGetErrorString(e);
        free_server(s);
        return e == cudaErrorMemoryAllocation ? LOGO_ERR_OOM : LOGO_ERR_CUDA;
    };
#define SCK(call)                                      \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) return bail(e_, #call); \
    } while (0)
    SCK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    SCK(cudaEventCreate(&s->ev0));
    SCK(cudaEventCreate(&s->ev1));
    SCK(cudaMalloc(&s->d_coords, sizeof(float2) * s->arena_cap));
    SCK(cudaMalloc(&s->d_route, sizeof(uint32_t) * s->arena_cap));
    SCK(cudaMalloc(&s->d_best, sizeof(uint32_t) * s->arena_cap));
    SCK(cudaMalloc(&s->d_slots, sizeof(ServeSlot) * s->opts.max_slots));
    SCK(cudaMalloc(&s->d_units, sizeof(uint32_t) * s->opts.max_slots));
    SCK(cudaMalloc(&s->d_queue, sizeof(unsigned int)));
    SCK(cudaMallocHost(&s->h_slots, sizeof(ServeSlot) * s->opts.max_slots));
    SCK(cudaMallocHost(&s->h_units, sizeof(uint32_t) * s->opts.max_slots));
#undef SCK
    std::memset(s->h_slots, 0, sizeof(ServeSlot) * s->opts.max_slots);
    for (uint32_t k = 0; k < s->opts.max_large; ++k) s->workers.emplace_back(large_worker, s);
    s->sched = std::thread(scheduler, s);
    *out = s;
    return LOGO_OK;
}

logo_status logo_server_submit(logo_server* s, const logo_xy* coords, uint32_t n,
                               const uint32_t* route, uint64_t seed, uint64_t* id) {
    if (!s || !coords || !route || !id) return LOGO_ERR_INVALID_ARG;
    if (n < 3 || n > LOGO_MAX_CITIES)
        return sfail(s, LOGO_ERR_INVALID_ARG, "n out of range");
    double x0 = coords[0].x, x1 = x0, y0 = coords[0].y, y1 = y0;
    for (uint32_t k = 0; k < n; ++k) {
        const double x = coords[k].x, y = coords[k].y;
        if (!std::isfinite(x) || !std::isfinite(y))
            return sfail(s, LOGO_ERR_INVALID_ARG, "non-finite coordinate");
        x0 = std::min(x0, x); x1 = std::max(x1, x);
        y0 = std::min(y0, y); y1 = std::max(y1, y);
    }
    const double diag = std::sqrt((x1 - x0) * (x1 - x0) + (y1 - y0) * (y1 - y0));
    if (!(diag < LOGO_MAX_DIAGONAL))
        return sfail(s, LOGO_ERR_INVALID_ARG, "coordinate diagonal exceeds LOGO_MAX_DIAGONAL");
    std::vector<uint8_t> seen(n, 0);
    for (uint32_t k = 0; k < n; ++k) {
        if (route[k] >= n || seen[route[k]])
            return sfail(s, LOGO_ERR_INVALID_ARG, "route is not a permutation");
        seen[route[k]] = 1;
    }
    Req r;
    r.n = n;
    r.seed = seed;
    r.margin = filter_margin(diag);
    r.xy.assign(coords, coords + n);
    r.route.assign(route, route + n);
    r.large = n > kBatchMaxN;
    r.info.n = n;
    r.t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->pending.size() >= s->opts.max_pending)
        return sfail(s, LOGO_ERR_BUSY, "pending queue full");
    r.id = s->next_id++;
    *id = r.id;
    s->pending.push_back(r.id);
    s->reqs.emplace(r.id, std::move(r));
    s->stats.submitted++;
    s->cv.notify_all();
    return LOGO_OK;
}

static logo_status take_result(logo_server* s, uint64_t id, uint32_t* route_out,
                               logo_request_info* info) {  // with s->mu held
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return LOGO_ERR_NOT_FOUND;
    Req& r = it->second;
    if (r.state != kDone) return LOGO_ERR_BUSY;
    if (route_out && r.info.status == LOGO_OK)
        std::memcpy(route_out, r.route.data(), sizeof(uint32_t) * r.n);
    if (info) *info = r.info;
    const logo_status st = (logo_status)r.info.status;
    s->reqs.erase(it);
    return st;
}

logo_status logo_server_poll(logo_server* s, uint64_t id, uint32_t* route_out,
                             logo_request_info* info) {
    if (!s) return LOGO_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    return take_result(s, id, route_out, info);
}

logo_status logo_server_wait(logo_server* s, uint64_t id, uint32_t timeout_ms,
                             uint32_t* route_out, logo_request_info* info) {
    if (!s) return LOGO_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    const auto deadline = Clock::now() + std::chrono::milliseconds(timeout_ms);
    for (;;) {
        logo_status st = take_result(s, id, route_out, info);
        if (st != LOGO_ERR_BUSY) return st;
        if (s->done_cv.wait_until(lk, deadline) == std::cv_status::timeout)
            return take_result(s, id, route_out, info);
    }
}

logo_status logo_server_get_stats(logo_server* s, logo_server_stats* out) {
    if (!s || !out) return LOGO_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->pending = s->pending.size();
    out->running_small = s->running_small;
    out->running_large = s->running_large;
    out->mem_in_use = s->mem_in_use;
    out->mem_budget = s->opts.mem_budget;
    return LOGO_OK;
}

logo_status logo_server_destroy(logo_server* s) {
    if (!s) return LOGO_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->large_ready.clear();  // admitted but not started: dropped
    }
    s->cv.notify_all();
    s->large_cv.notify_all();
    if (s->sched.joinable()) s->sched.join();
    for (auto& w : s->workers)
        if (w.joinable()) w.join();
    free_server(s);
    return LOGO_OK;
}

}  // extern "C"

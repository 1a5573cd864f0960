// C ABI of the batched persistent solver and its autotuner
// (include/logo_gpu.h, "batched solving").
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/logo_gpu.h"
#include "batch_internal.h"
#include "logo_device.cuh"
#include "logo_internal.h"

using namespace logo;

namespace {

constexpr int kBuckets = 5;
const uint32_t kBucketHi[kBuckets] = {128, 384, 1024, 2048, kBatchMaxN + 1};

int bucket_of(uint32_t n) {
    for (int b = 0; b < kBuckets; ++b)
        if (n < kBucketHi[b]) return b;
    return kBuckets - 1;
}

const BatchShape kDefaultShape[kBuckets] = {
    {2, 128, 64}, {2, 128, 64}, {4, 256, 64}, {4, 256, 128}, {4, 256, 128}};

thread_local std::string g_batch_err;

}  // namespace

struct logo_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t max_count = 0;
    uint64_t max_cities = 0;
    float2* d_coords = nullptr;
    uint32_t* d_routes = nullptr;
    BatchInstance* d_inst = nullptr;
    uint32_t* d_order = nullptr;
    BatchResult* d_res = nullptr;
    unsigned int* d_queue = nullptr;  // one counter per launch group
    float2* h_coords = nullptr;
    uint32_t* h_routes = nullptr;
    BatchInstance* h_inst = nullptr;
    uint32_t* h_order = nullptr;
    BatchResult* h_res = nullptr;
    SharedBest* d_shared = nullptr;     // multi-start: the group's best (one group)
    uint32_t* d_shared_tours = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    BatchShape table[kBuckets];
    int sms = 0;
    std::string gpu;
    std::string err;
};

namespace {

logo_status bfail(logo_batch* b, logo_status s, const std::string& m) {
    if (b)
        b->err = m;
    else
        g_batch_err = m;
    return s;
}

#define BCK(b, call)                                                                  \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return bfail(b, e_ == cudaErrorMemoryAllocation ? LOGO_ERR_OOM : LOGO_ERR_CUDA, \
                         std::string(#call) + ": " + cudaGetErrorString(e_));          \
    } while (0)

void free_batch(logo_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    cudaFree(b->d_coords);
    cudaFree(b->d_routes);
    cudaFree(b->d_inst);
    cudaFree(b->d_order);
    cudaFree(b->d_res);
    cudaFree(b->d_queue);
    cudaFree(b->d_shared);
    cudaFree(b->d_shared_tours);
    if (b->h_coords) cudaFreeHost(b->h_coords);
    if (b->h_routes) cudaFreeHost(b->h_routes);
    if (b->h_inst) cudaFreeHost(b->h_inst);
    if (b->h_order) cudaFreeHost(b->h_order);
    if (b->h_res) cudaFreeHost(b->h_res);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

bool shape_compiled(const BatchShape& s) {
    BatchShape all[32];
    const int k = batch_shapes(all, 32);
    for (int i = 0; i < k; ++i)
        if (all[i].R == s.R && all[i].NT == s.NT && all[i].TC == s.TC) return true;
    return false;
}

// Validates and packs the instances into the pinned staging buffers (the
// routes only when they are start tours, given = true).
logo_status pack(logo_batch* b, const logo_instance* in, uint32_t count, bool given = true) {
    if (!in && count) return bfail(b, LOGO_ERR_INVALID_ARG, "instances is NULL");
    if (count > b->max_count) return bfail(b, LOGO_ERR_INVALID_ARG, "count exceeds max_count");
    uint64_t off = 0;
    std::vector<uint8_t> seen;
    for (uint32_t k = 0; k < count; ++k) {
        const logo_instance& I = in[k];
        if (!I.coords || !I.route)
            return bfail(b, LOGO_ERR_INVALID_ARG, "instance " + std::to_string(k) + ": NULL array");
        if (I.n < 3 || I.n > kBatchMaxN)
            return bfail(b, LOGO_ERR_INVALID_ARG,
                         "instance " + std::to_string(k) + ": n outside [3, LOGO_BATCH_MAX_N]");
        if (off + I.n > b->max_cities)
            return bfail(b, LOGO_ERR_INVALID_ARG, "total cities exceed max_cities");
        double x0 = I.coords[0].x, x1 = x0, y0 = I.coords[0].y, y1 = y0;
        for (uint32_t c = 0; c < I.n; ++c) {
            const double x = I.coords[c].x, y = I.coords[c].y;
            if (!std::isfinite(x) || !std::isfinite(y))
                return bfail(b, LOGO_ERR_INVALID_ARG,
                             "instance " + std::to_string(k) + ": non-finite coordinate");
            x0 = std::min(x0, x); x1 = std::max(x1, x);
            y0 = std::min(y0, y); y1 = std::max(y1, y);
            b->h_coords[off + c] = make_float2(I.coords[c].x, I.coords[c].y);
        }
        const double diag = std::sqrt((x1 - x0) * (x1 - x0) + (y1 - y0) * (y1 - y0));
        if (!(diag < LOGO_MAX_DIAGONAL))
            return bfail(b, LOGO_ERR_INVALID_ARG,
                         "instance " + std::to_string(k) + ": diagonal exceeds LOGO_MAX_DIAGONAL");
        if (given) {
            seen.assign(I.n, 0);
            for (uint32_t c = 0; c < I.n; ++c) {
                const uint32_t v = I.route[c];
                if (v >= I.n || seen[v])
                    return bfail(b, LOGO_ERR_INVALID_ARG,
                                 "instance " + std::to_string(k) + ": route is not a permutation");
                seen[v] = 1;
                b->h_routes[off + c] = v;
            }
        } else {
            std::memset(b->h_routes + off, 0, sizeof(uint32_t) * I.n);
        }
        BatchInstance d;
        d.off = off;
        d.seed = I.seed;
        d.n = I.n;
        d.margin = filter_margin(diag);
        d.group = kNoGroup;
        d.pad = 0;
        b->h_inst[k] = d;
        off += I.n;
    }
    return LOGO_OK;
}

struct Group {
    BatchShape shape;
    uint32_t first, count, max_n;
};

// Orders instances into launch groups (one per distinct shape), each sorted
// by descending n so the queue hands out the longest work first.
std::vector<Group> plan(logo_batch* b, const logo_instance* in, uint32_t count,
                        const logo_batch_opts& o) {
    const bool fixed = o.shape.rows_per_thread || o.shape.threads_per_cta || o.shape.tile_cols;
    const BatchShape fx{o.shape.rows_per_thread, o.shape.threads_per_cta, o.shape.tile_cols};
    std::vector<uint32_t> ids(count);
    for (uint32_t k = 0; k < count; ++k) ids[k] = k;
    auto shape_of = [&](uint32_t k) { return fixed ? fx : b->table[bucket_of(in[k].n)]; };
    auto key = [](const BatchShape& s) { return s.R * 1000000 + s.NT * 1000 + s.TC; };
    std::stable_sort(ids.begin(), ids.end(), [&](uint32_t a, uint32_t c) {
        const int ka = key(shape_of(a)), kc = key(shape_of(c));
        if (ka != kc) return ka < kc;
        return in[a].n > in[c].n;
    });
    std::vector<Group> g;
    for (uint32_t s = 0; s < count; ++s) {
        const BatchShape sh = shape_of(ids[s]);
        if (g.empty() || key(g.back().shape) != key(sh)) g.push_back(Group{sh, s, 0, 0});
        g.back().count++;
        g.back().max_n = std::max(g.back().max_n, in[ids[s]].n);
        b->h_order[s] = ids[s];
    }
    // the group holding the largest instances goes first
    std::stable_sort(g.begin(), g.end(),
                     [](const Group& a, const Group& c) { return a.max_n > c.max_n; });
    return g;
}

// share: every instance is a replica of one multi-start group (same n) that
// shares its best tour.
logo_status run(logo_batch* b, const logo_instance* in, uint32_t count,
                const logo_batch_opts& o, logo_result* res, double* ms_out,
                bool share = false) {
    BCK(b, cudaSetDevice(b->device));
    if (o.kick_kind != LOGO_KICK_SEGMENT && o.kick_kind != LOGO_KICK_DOUBLE_BRIDGE)
        return bfail(b, LOGO_ERR_INVALID_ARG, "unknown kick kind");
    const bool fixed = o.shape.rows_per_thread || o.shape.threads_per_cta || o.shape.tile_cols;
    if (fixed && !shape_compiled(BatchShape{o.shape.rows_per_thread, o.shape.threads_per_cta,
                                            o.shape.tile_cols}))
        return bfail(b, LOGO_ERR_INVALID_ARG, "shape is not compiled");
    if (o.start != LOGO_START_GIVEN && o.start != LOGO_START_NN && o.start != LOGO_START_MF)
        return bfail(b, LOGO_ERR_INVALID_ARG, "unknown start-tour kind");
    logo_status s = pack(b, in, count, o.start == LOGO_START_GIVEN);
    if (s != LOGO_OK) return s;
    if (count == 0) {
        if (ms_out) *ms_out = 0;
        return LOGO_OK;
    }
    std::vector<Group> groups = plan(b, in, count, o);
    const uint64_t cities = b->h_inst[count - 1].off + b->h_inst[count - 1].n;
    if (share) {
        if (!b->d_shared) BCK(b, cudaMalloc(&b->d_shared, sizeof(SharedBest)));
        if (!b->d_shared_tours)
            BCK(b, cudaMalloc(&b->d_shared_tours, sizeof(uint32_t) * kBatchMaxN));
        const SharedBest init{~0ull, 0u, 0u, 0ull};
        BCK(b, cudaMemcpyAsync(b->d_shared, &init, sizeof(init), cudaMemcpyHostToDevice,
                               b->stream));
        for (uint32_t k = 0; k < count; ++k) b->h_inst[k].group = 0;
    }
    BCK(b, cudaMemcpyAsync(b->d_coords, b->h_coords, sizeof(float2) * cities,
                           cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaMemcpyAsync(b->d_routes, b->h_routes, sizeof(uint32_t) * cities,
                           cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaMemcpyAsync(b->d_inst, b->h_inst, sizeof(BatchInstance) * count,
                           cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaMemcpyAsync(b->d_order, b->h_order, sizeof(uint32_t) * count,
                           cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned int) * 8, b->stream));
    // one CUDA graph per run: every group's persistent launch back to back
    std::vector<int> grids(groups.size());
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        BatchArgs A{};
        A.max_n = groups[gi].max_n;
        int occ = 0;
        BCK(b, launch_batch(A, groups[gi].shape, 0, nullptr, &occ));
        if (occ < 1)
            return bfail(b, LOGO_ERR_INVALID_ARG, "batch shape does not fit on the device");
        uint32_t grid = o.ctas ? o.ctas : (uint32_t)(occ * b->sms);
        grids[gi] = (int)std::min<uint32_t>(grid, groups[gi].count);
    }
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint32_t max_n_all = 0;
    for (uint32_t k = 0; k < count; ++k) max_n_all = std::max(max_n_all, b->h_inst[k].n);
    if (o.start == LOGO_START_MF) BCK(b, prepare_mf_start());
    BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaSuccess;
    // multiple-fragment start tours: built first, then loaded as given tours
    if (o.start == LOGO_START_MF)
        ce = launch_mf_start(b->d_coords, b->d_routes, b->d_inst, b->d_order, count, max_n_all,
                             b->sms, b->stream);
    for (size_t gi = 0; gi < groups.size() && ce == cudaSuccess && gi < 8; ++gi) {
        BatchArgs A;
        A.coords = b->d_coords;
        A.routes = b->d_routes;
        A.inst = b->d_inst;
        A.order = b->d_order + groups[gi].first;
        A.results = b->d_res;
        A.queue = b->d_queue + gi;
        A.count = groups[gi].count;
        A.max_n = groups[gi].max_n;
        A.kicks = o.kicks;
        A.kick_kind = o.kick_kind;
        A.shared = share ? b->d_shared : nullptr;
        A.shared_tours = share ? b->d_shared_tours : nullptr;
        A.start = o.start == LOGO_START_NN ? kStartNN : kStartGiven;
        ce = launch_batch(A, groups[gi].shape, grids[gi], b->stream, nullptr);
    }
    cudaError_t ee = cudaStreamEndCapture(b->stream, &graph);
    if (ce != cudaSuccess || ee != cudaSuccess || groups.size() > 8) {
        if (graph) cudaGraphDestroy(graph);
        return bfail(b, LOGO_ERR_CUDA, std::string("batch capture: ") +
                                           cudaGetErrorString(ce != cudaSuccess ? ce : ee));
    }
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    BCK(b, ce);
    cudaEventRecord(b->ev0, b->stream);
    ce = cudaGraphLaunch(exec, b->stream);
    cudaEventRecord(b->ev1, b->stream);
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(b->h_routes, b->d_routes, sizeof(uint32_t) * cities,
                             cudaMemcpyDeviceToHost, b->stream);
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(b->h_res, b->d_res, sizeof(BatchResult) * count,
                             cudaMemcpyDeviceToHost, b->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(b->stream);
    cudaGraphExecDestroy(exec);
    BCK(b, ce);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    if (ms_out) *ms_out = ms;
    logo_status worst = LOGO_OK;
    for (uint32_t k = 0; k < count; ++k) {
        const BatchInstance& d = b->h_inst[k];
        const BatchResult& r = b->h_res[k];
        logo_status st = LOGO_OK;
        if (r.status & kErrBadKey) st = LOGO_ERR_DEVICE_FAULT;
        else if (r.status & kErrMoveLimit) st = LOGO_ERR_MOVE_LIMIT;
        else if (r.status) st = LOGO_ERR_DEVICE_FAULT;
        if (st == LOGO_OK)
            std::memcpy(in[k].route, b->h_routes + d.off, sizeof(uint32_t) * d.n);
        else
            worst = st;
        if (res) {
            res[k].start_length = r.start_length;
            res[k].best_length = r.best_length;
            res[k].moves = r.moves;
            res[k].sweeps = r.sweeps;
            res[k].kicks = r.kicks;
            res[k].accepted = r.accepted;
            res[k].status = st;
            res[k].pad = 0;
        }
    }
    if (worst != LOGO_OK) return bfail(b, worst, "some instances failed (see results[].status)");
    return LOGO_OK;
}

std::string cache_key(const std::string& gpu, int bucket) {
    return gpu + "|" + std::to_string(bucket);
}

// Cache file: a flat JSON object {"<gpu name>|<bucket>": [R, NT, TC], ...}.
std::map<std::string, BatchShape> read_cache(const char* path) {
    std::map<std::string, BatchShape> m;
    std::ifstream f(path);
    if (!f) return m;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string t = ss.str();
    size_t p = 0;
    while ((p = t.find('"', p)) != std::string::npos) {
        const size_t q = t.find('"', p + 1);
        if (q == std::string::npos) break;
        const std::string k = t.substr(p + 1, q - p - 1);
        const size_t lb = t.find('[', q), rb = t.find(']', q);
        if (lb == std::string::npos || rb == std::string::npos) break;
        BatchShape s{0, 0, 0};
        if (std::sscanf(t.c_str() + lb, "[%d , %d , %d]", &s.R, &s.NT, &s.TC) == 3 ||
            std::sscanf(t.c_str() + lb, "[%d,%d,%d]", &s.R, &s.NT, &s.TC) == 3)
            m[k] = s;
        p = rb + 1;
    }
    return m;
}

void write_cache(const char* path, const std::map<std::string, BatchShape>& m) {
    std::ofstream f(path);
    f << "{\n";
    size_t i = 0;
    for (const auto& kv : m) {
        f << "  \"" << kv.first << "\": [" << kv.second.R << ", " << kv.second.NT << ", "
          << kv.second.TC << "]" << (++i < m.size() ? "," : "") << "\n";
    }
    f << "}\n";
}

}  // namespace

extern "C" {

const char* logo_batch_last_error(const logo_batch* b) {
    return b ? b->err.c_str() : g_batch_err.c_str();
}

logo_status logo_batch_create(int device, uint32_t max_count, uint64_t max_cities,
                              logo_batch** out) {
    if (!out) return bfail(nullptr, LOGO_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (max_count == 0 || max_cities == 0)
        return bfail(nullptr, LOGO_ERR_INVALID_ARG, "empty batch capacity");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return bfail(nullptr, LOGO_ERR_NO_DEVICE, "no CUDA device");
    if (device < 0 || device >= ndev)
        return bfail(nullptr, LOGO_ERR_INVALID_ARG, "device index out of range");
    if (cudaSetDevice(device) != cudaSuccess)
        return bfail(nullptr, LOGO_ERR_CUDA, "cudaSetDevice failed");
    logo_batch* b = new logo_batch();
    b->device = device;
    b->max_count = max_count;
    b->max_cities = max_cities;
    for (int k = 0; k < kBuckets; ++k) b->table[k] = kDefaultShape[k];
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, device);
    b->sms = prop.multiProcessorCount;
    b->gpu = prop.name;
    auto bail = [&](cudaError_t e, const char* what) {
        g_batch_err = std::string(what) + ": " + cudaGetErrorString(e);
        free_batch(b);
        return e == cudaErrorMemoryAllocation ? LOGO_ERR_OOM : LOGO_ERR_CUDA;
    };
#define BCC(call)                                      \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) return bail(e_, #call); \
    } while (0)
    BCC(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    BCC(cudaEventCreate(&b->ev0));
    BCC(cudaEventCreate(&b->ev1));
    BCC(cudaMalloc(&b->d_coords, sizeof(float2) * max_cities));
    BCC(cudaMalloc(&b->d_routes, sizeof(uint32_t) * max_cities));
    BCC(cudaMalloc(&b->d_inst, sizeof(BatchInstance) * max_count));
    BCC(cudaMalloc(&b->d_order, sizeof(uint32_t) * max_count));
    BCC(cudaMalloc(&b->d_res, sizeof(BatchResult) * max_count));
    BCC(cudaMalloc(&b->d_queue, sizeof(unsigned int) * 8));
    BCC(cudaMallocHost(&b->h_coords, sizeof(float2) * max_cities));
    BCC(cudaMallocHost(&b->h_routes, sizeof(uint32_t) * max_cities));
    BCC(cudaMallocHost(&b->h_inst, sizeof(BatchInstance) * max_count));
    BCC(cudaMallocHost(&b->h_order, sizeof(uint32_t) * max_count));
    BCC(cudaMallocHost(&b->h_res, sizeof(BatchResult) * max_count));
#undef BCC
    *out = b;
    return LOGO_OK;
}

logo_status logo_batch_destroy(logo_batch* b) {
    free_batch(b);
    return LOGO_OK;
}

logo_status logo_batch_run(logo_batch* b, const logo_instance* inst, uint32_t count,
                           const logo_batch_opts* opts, logo_result* results,
                           double* device_ms) {
    if (!b || !opts) return LOGO_ERR_INVALID_ARG;
    return run(b, inst, count, *opts, results, device_ms);
}

logo_status logo_batch_solve(const logo_instance* inst, uint32_t count,
                             const logo_batch_opts* opts, logo_result* results,
                             double* device_ms) {
    if (!opts || (!inst && count)) return bfail(nullptr, LOGO_ERR_INVALID_ARG, "NULL argument");
    uint64_t cities = 0;
    for (uint32_t k = 0; k < count; ++k) cities += inst[k].n;
    logo_batch* b = nullptr;
    logo_status s = logo_batch_create(opts->device, std::max(count, 1u),
                                      std::max<uint64_t>(cities, 1), &b);
    if (s != LOGO_OK) return s;
    s = run(b, inst, count, *opts, results, device_ms);
    if (s != LOGO_OK) g_batch_err = b->err;
    free_batch(b);
    return s;
}

logo_status logo_batch_multistart(logo_batch* b, const logo_xy* coords, uint32_t n,
                                  uint32_t* route, uint32_t replicas, uint64_t seed, int share,
                                  const logo_batch_opts* opts, logo_result* results,
                                  uint32_t* best, double* device_ms) {
    if (!b || !opts || !coords || !route) return LOGO_ERR_INVALID_ARG;
    if (replicas == 0 || replicas > b->max_count)
        return bfail(b, LOGO_ERR_INVALID_ARG, "replicas outside [1, max_count]");
    if ((uint64_t)n * replicas > b->max_cities)
        return bfail(b, LOGO_ERR_INVALID_ARG, "n x replicas exceeds max_cities");
    std::vector<uint32_t> tours((size_t)n * replicas);
    std::vector<logo_instance> inst(replicas);
    for (uint32_t k = 0; k < replicas; ++k) {
        std::memcpy(tours.data() + (size_t)k * n, route, sizeof(uint32_t) * n);
        inst[k].coords = coords;
        inst[k].route = tours.data() + (size_t)k * n;
        inst[k].n = n;
        inst[k].seed = seed + k;
    }
    std::vector<logo_result> res(replicas);
    const logo_status s = run(b, inst.data(), replicas, *opts, res.data(), device_ms, share != 0);
    if (results) std::copy(res.begin(), res.end(), results);
    if (s != LOGO_OK) return s;
    uint32_t w = 0;
    for (uint32_t k = 1; k < replicas; ++k)
        if (res[k].best_length < res[w].best_length) w = k;
    std::memcpy(route, tours.data() + (size_t)w * n, sizeof(uint32_t) * n);
    if (best) *best = w;
    return LOGO_OK;
}

logo_status logo_batch_shape_for(const logo_batch* b, uint32_t n, logo_batch_shape* out) {
    if (!b || !out) return LOGO_ERR_INVALID_ARG;
    const BatchShape& s = b->table[bucket_of(n)];
    out->rows_per_thread = s.R;
    out->threads_per_cta = s.NT;
    out->tile_cols = s.TC;
    return LOGO_OK;
}

logo_status logo_batch_autotune(logo_batch* b, const logo_instance* sample, uint32_t count,
                                uint32_t kicks, int kick_kind, const char* cache_path,
                                int reuse) {
    if (!b || (!sample && count)) return LOGO_ERR_INVALID_ARG;
    std::map<std::string, BatchShape> cache;
    if (cache_path) cache = read_cache(cache_path);
    BatchShape shapes[32];
    const int nshapes = batch_shapes(shapes, 32);
    for (int bk = 0; bk < kBuckets; ++bk) {
        const std::string ck = cache_key(b->gpu, bk);
        if (reuse && cache.count(ck) && shape_compiled(cache[ck])) {
            b->table[bk] = cache[ck];
            continue;
        }
        // the sample's instances in this bucket, with private route copies
        std::vector<logo_instance> sub;
        std::vector<std::vector<uint32_t>> routes;
        for (uint32_t k = 0; k < count; ++k)
            if (bucket_of(sample[k].n) == bk) {
                routes.emplace_back(sample[k].route, sample[k].route + sample[k].n);
                sub.push_back(sample[k]);
            }
        if (sub.empty()) continue;
        double best_ms = 1e30;
        BatchShape best = b->table[bk];
        std::vector<uint64_t> ref_len;
        for (int si = 0; si < nshapes; ++si) {
            for (size_t k = 0; k < sub.size(); ++k) {
                std::copy(routes[k].begin(), routes[k].end(), const_cast<uint32_t*>(sub[k].route));
            }
            logo_batch_opts o{};
            o.device = b->device;
            o.kicks = kicks;
            o.kick_kind = kick_kind;
            o.shape = logo_batch_shape{shapes[si].R, shapes[si].NT, shapes[si].TC};
            std::vector<logo_result> res(sub.size());
            double ms = 0;
            logo_status s = run(b, sub.data(), (uint32_t)sub.size(), o, res.data(), &ms);
            if (s == LOGO_ERR_INVALID_ARG) continue;  // shape does not fit this bucket
            if (s != LOGO_OK) return s;
            // every shape must reach the same tours: a free self-check
            std::vector<uint64_t> lens(sub.size());
            for (size_t k = 0; k < sub.size(); ++k) lens[k] = res[k].best_length;
            if (ref_len.empty())
                ref_len = lens;
            else if (lens != ref_len)
                return bfail(b, LOGO_ERR_DEVICE_FAULT, "tile shapes disagree on results");
            if (ms < best_ms) {
                best_ms = ms;
                best = shapes[si];
            }
        }
        for (size_t k = 0; k < sub.size(); ++k)
            std::copy(routes[k].begin(), routes[k].end(), const_cast<uint32_t*>(sub[k].route));
        b->table[bk] = best;
        cache[ck] = best;
    }
    if (cache_path) write_cache(cache_path, cache);
    return LOGO_OK;
}

}  // extern "C"

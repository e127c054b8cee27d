// Serving loop with continuous batching.
//
// Requests above `big_nnz` stored entries take the whole GPU through the persistent
// cooperative solver, one at a time (the "big lane"); all others run as clusters.
//
// A feec_server owns `slots` worker threads. Requests (one SPD solve each: a CSR
// matrix, a right-hand side, a tolerance) wait in a FIFO queue; a free slot takes
// the next request as soon as the device memory budget has room for it, uploads
// the matrix, builds the reference's Rainbow coloring and the multicolor SSOR
// layout, and launches the whole solve as one thread-block cluster on the slot's
// own stream. Requests that arrive while others run are admitted as slots and
// memory free up, and their kernels overlap on the GPU; every request's matrix and
// Krylov vectors stay on the device until it completes. Timing of each request
// (submission, start of its solve, completion) is recorded for latency reports.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "feec_batched.h"
#include "feec_device.cuh"
#include "feec_system.h"

using namespace feec;

namespace feec {
int sell_prepare(feec_system* s, int method);
SellView sell_view(const feec_system* s, int method);
}

namespace {

using clock_type = std::chrono::steady_clock;

// A resident operator: uploaded and prepared once (layouts, coloring, SELL copy), then
// shared by the requests submitted against it. Cluster-solved requests only read its
// layouts; whole-GPU requests run on its system one at a time (the server's big lane).
struct Operator {
    int id = 0;
    feec_system* s = nullptr;
    cudaStream_t home = nullptr;   // the system's creation stream: owns its persistent allocations
    int n = 0;
    long long nnz = 0;
    size_t bytes = 0;       // counted against the budget while the operator is registered
    int users = 0;          // requests queued or running on it (under feec_server::mu)
};

struct Request {
    long long id = 0;
    int n = 0;
    const int* A = nullptr; const int* C = nullptr; const double* V = nullptr;
    std::shared_ptr<Operator> op;   // set: solve against a resident operator (A, C, V unused)
    const double* b = nullptr;
    double* x = nullptr;
    double precision = 1e-10;
    size_t bytes = 0;
    clock_type::time_point t_submit;
};

// The reference's Rainbow coloring (sparse/rainbow.cpp:14-130) depends on the sparsity
// pattern only. A serving process sees the same operators again and again, so colorings
// are kept per pattern, keyed by the row count and a 64-bit hash of the row pointers and
// column indices; a request whose pattern is known skips the greedy coloring.
struct Coloring {
    int nc = 0;
    std::vector<int> F, B, R;
};

unsigned long long pattern_hash(int n, const int* A, const int* C) {
    unsigned long long h = 0x243F6A8885A308D3ull ^ (unsigned long long)n;
    auto mix = [&h](const int* p, size_t count) {
        size_t i = 0;
        for (; i + 2 <= count; i += 2) {
            unsigned long long w;
            std::memcpy(&w, p + i, sizeof(w));
            h = (h ^ w) * 0x9E3779B97F4A7C15ull;
            h ^= h >> 29;
        }
        if (i < count) {
            h = (h ^ (unsigned long long)(unsigned)p[i]) * 0x9E3779B97F4A7C15ull;
            h ^= h >> 29;
        }
    };
    mix(A, (size_t)n + 1);
    mix(C, (size_t)A[n]);
    return h;
}

size_t estimate_bytes(int n, long long nnz) {
    // original CSR + FP32 values, permuted [L|E|U] copy (FP64 + FP32), SELL copy with
    // padding (int + FP32 + FP64), row arrays, solver vectors
    return (size_t)(nnz * (12 + 4 + 16 + 16 * 5 / 4)) + (size_t)n * 200 + (32u << 20);
}

// A request against a resident operator: its own right-hand side, solution and workspace
// (FP64 x, b, residual and five inner vectors).
size_t estimate_rhs_bytes(int n) { return (size_t)n * 80 + (1u << 20); }

}  // namespace

struct feec_server {
    int method = FEEC_METHOD_RAINBOW;
    long long big_nnz = 4000000;       // requests with more stored entries use the whole-GPU solver
    std::mutex big_lane;               // ... one at a time
    int mode = FEEC_MODE_MIXED;
    size_t budget = 0;
    int device = 0;
    std::atomic<size_t> in_use{0};
    std::atomic<size_t> peak{0};
    std::atomic<int> inflight{0};
    std::mutex mu;
    std::condition_variable cv;        // queue / budget / shutdown changes
    std::deque<Request> queue;
    std::vector<feec_request_result> done;
    std::vector<std::thread> workers;
    bool stop = false;
    long long next_id = 1;
    std::mutex color_mu;               // colorings by pattern (see Coloring), oldest dropped first
    std::deque<std::pair<unsigned long long, std::shared_ptr<const Coloring>>> colorings;
    static constexpr size_t kMaxColorings = 64;
    std::map<int, std::shared_ptr<Operator>> ops;   // resident operators (under mu)
    int next_op = 1;
    long long submitted = 0, finished = 0;
    clock_type::time_point t0;
};

namespace {

double ms_since(const feec_server* srv, clock_type::time_point t) {
    return std::chrono::duration<double, std::milli>(t - srv->t0).count();
}

// Uploads a request's (or a resident operator's) matrix and prepares it for the server's
// method: the Rainbow coloring from the cache when the pattern was seen before.
int prepare_system(feec_server* srv, int n, const int* A, const int* C, const double* V, cudaStream_t stream,
                   feec_system** out) {
    feec_system* s = nullptr;
    int st = feec_system_create(&s, n, A, C, V, 1, stream);
    if (st != FEEC_OK) return st;
    struct Guard {
        feec_system*& s;
        bool keep = false;
        ~Guard() { if (!keep) feec_system_destroy(s); }
    } guard{s};
    const bool rainbow = srv->method == FEEC_METHOD_RAINBOW;
    if (rainbow) {
        // the reference's Rainbow ordering (sparse/rainbow.cpp:14-130), from the cache when
        // this pattern was colored before, and the diagonal
        const unsigned long long key = pattern_hash(n, A, C);
        std::shared_ptr<const Coloring> col;
        {
            std::lock_guard<std::mutex> lk(srv->color_mu);
            for (const auto& e : srv->colorings)
                if (e.first == key && (int)e.second->F.size() == n) { col = e.second; break; }
        }
        if (!col) {
            auto c = std::make_shared<Coloring>();
            c->F.resize((size_t)n); c->B.resize((size_t)n + 1); c->R.resize((size_t)n);
            st = feec_rainbow(n, A, C, &c->nc, c->F.data(), c->B.data(), c->R.data());
            if (st != FEEC_OK) return st;
            c->B.resize((size_t)c->nc + 1);
            col = c;
            std::lock_guard<std::mutex> lk(srv->color_mu);
            srv->colorings.emplace_back(key, col);
            if (srv->colorings.size() > feec_server::kMaxColorings) srv->colorings.pop_front();
        }
        std::vector<double> diag((size_t)n, 0.0);
        for (int r = 0; r < n; r++)
            for (int k = A[r]; k < A[r + 1]; k++)
                if (C[k] == r) diag[r] += V[k];
        st = feec_system_set_rainbow(s, diag.data(), 1.0, col->nc, col->F.data(), col->B.data(), col->R.data(), 1);
        if (st != FEEC_OK) return st;
    }
    guard.keep = true;
    *out = s;
    return FEEC_OK;
}

// Solves one request on the prepared system `s` on `stream`; fills `res`.
int solve_on(feec_server* srv, feec_system* s, const Request& rq, cudaStream_t stream, feec_request_result& res) {
    int st = FEEC_OK;
    const bool rainbow = srv->method == FEEC_METHOD_RAINBOW;
    const int is_float = srv->mode == FEEC_MODE_MIXED;
    cudaEvent_t done_ev = nullptr;
    FEEC_TRY(cudaEventCreateWithFlags(&done_ev, cudaEventBlockingSync | cudaEventDisableTiming));
    struct EvGuard { cudaEvent_t e; ~EvGuard() { cudaEventDestroy(e); } } evguard{done_ev};
    if ((long long)s->nnz >= srv->big_nnz) {
        // Large request: the whole GPU for one solve (persistent cooperative kernel). One at a
        // time, so two grid-wide solves never compete for co-residency.
        DevArena io;
        io.stream = stream;
        struct IoGuard { DevArena* m; ~IoGuard() { m->release(); } } ioguard{&io};
        double *b = nullptr, *x = nullptr;
        FEEC_TRY(io.alloc(b, (size_t)rq.n)); FEEC_TRY(io.alloc(x, (size_t)rq.n));
        FEEC_TRY(cudaMemcpyAsync(b, rq.b, sizeof(double) * rq.n, cudaMemcpyHostToDevice, stream));
        FEEC_TRY(cudaMemsetAsync(x, 0, sizeof(double) * rq.n, stream));
        feec_solve_info info;
        // One persistent block per SM (not two): every SM keeps room for a cluster block, so
        // the requests being solved as clusters keep running beside the large solve instead
        // of queueing behind it, and the large solve's cooperative launch finds its blocks a
        // place even while clusters are resident.
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, srv->device);
        feec_system_set_launch(s, sms, 0);
        std::lock_guard<std::mutex> lane(srv->big_lane);
        res.t_start_ms = ms_since(srv, clock_type::now());
        st = feec_system_solve(s, rainbow ? FEEC_METHOD_RAINBOW : FEEC_METHOD_CG, srv->mode, x, b, nullptr,
                               rq.precision, 0, &info, stream);
        FEEC_TRY(cudaMemcpyAsync(rq.x, x, sizeof(double) * rq.n, cudaMemcpyDeviceToHost, stream));
        FEEC_TRY(cudaEventRecord(done_ev, stream));
        FEEC_TRY(cudaEventSynchronize(done_ev));
        res.status = info.status;
        res.iterations = info.iterations;
        res.outer_iterations = info.outer_iterations;
        res.true_relres = info.true_relres;
        res.cluster_blocks = -info.grid_blocks;   // negative: whole-GPU persistent grid
        res.fp64_fallback = info.fp64_fallback;
        res.error_estimate = info.error_estimate;
        return st;
    }
    st = sell_prepare(s, rainbow ? FEEC_METHOD_RAINBOW : FEEC_METHOD_CG);
    if (st != FEEC_OK) return st;
    const size_t n = (size_t)rq.n;
    const size_t tsz = is_float ? sizeof(float) : sizeof(double);
    DevArena mem;
    mem.stream = stream;
    struct MemGuard { DevArena* m; ~MemGuard() { m->release(); } } mguard{&mem};
    double *b = nullptr, *x = nullptr;
    char* w = nullptr;
    SellView* dview = nullptr;
    BatchItem* ditem = nullptr;
    BatchResult* dres = nullptr;
    FEEC_TRY(mem.alloc(b, n)); FEEC_TRY(mem.alloc(x, n));
    BatchItem it{};
    FEEC_TRY(mem.alloc(it.xp, n)); FEEC_TRY(mem.alloc(it.bp, n)); FEEC_TRY(mem.alloc(it.r64, n));
    FEEC_TRY(mem.alloc(w, 5 * n * tsz));
    FEEC_TRY(mem.alloc(dview, 1)); FEEC_TRY(mem.alloc(ditem, 1)); FEEC_TRY(mem.alloc(dres, 1));
    it.r = w; it.d = w + n * tsz; it.m = w + 2 * n * tsz; it.q = w + 3 * n * tsz; it.c = w + 4 * n * tsz;
    it.system = 0; it.nrhs = 1; it.first_result = 0;
    it.b[0] = b; it.x[0] = x;
    const SellView view = sell_view(s, rainbow ? FEEC_METHOD_RAINBOW : FEEC_METHOD_CG);
    FEEC_TRY(cudaMemcpyAsync(b, rq.b, sizeof(double) * n, cudaMemcpyHostToDevice, stream));
    FEEC_TRY(cudaMemsetAsync(x, 0, sizeof(double) * n, stream));
    FEEC_TRY(cudaMemcpyAsync(dview, &view, sizeof(view), cudaMemcpyHostToDevice, stream));
    FEEC_TRY(cudaMemcpyAsync(ditem, &it, sizeof(it), cudaMemcpyHostToDevice, stream));
    FEEC_TRY(cudaMemsetAsync(dres, 0, sizeof(BatchResult), stream));
    BatchArgs a{};
    a.systems = dview; a.items = ditem; a.nitems = 1; a.next_item = nullptr; a.results = dres;
    a.precision = rq.precision;
    a.inner_eta = is_float ? kRestartEta : 1e-30;
    a.err_control = is_float ? 1 : 0;
    a.inner_margin = is_float ? 0.3 : 1.0;
    a.max_iter = rq.n;
    a.max_outer = kMaxReplacements;
    a.stall_check = is_float;
    // cluster size from the work per iteration: about 0.25 M stored entries per block
    const long long nnz = view.nslices > 0 ? s->nnz : 0;
    int blocks = (int)std::min<long long>(16, std::max<long long>(1, nnz / 250000));
    const int maxb = cluster_max_blocks(is_float, rainbow);
    if (blocks > maxb) blocks = maxb;
    // powers of two only
    int p2 = 1;
    while (p2 * 2 <= blocks) p2 *= 2;
    blocks = p2;
    res.t_start_ms = ms_since(srv, clock_type::now());
    FEEC_TRY(launch_cluster(a, 0, is_float, rainbow, blocks, stream));
    BatchResult hr{};
    FEEC_TRY(cudaMemcpyAsync(&hr, dres, sizeof(hr), cudaMemcpyDeviceToHost, stream));
    FEEC_TRY(cudaEventRecord(done_ev, stream));
    FEEC_TRY(cudaEventSynchronize(done_ev));    // blocking wait: slots do not spin on the host
    if (hr.status == kStatusStagnated) {
        // FP32 inner solves stopped gaining digits (an operator too ill-conditioned for FP32):
        // finish in FP64 from the current iterate on the device; the workspace grows to FP64
        // within the bytes the admission estimate counted for this request.
        char* w64 = nullptr;
        FEEC_TRY(mem.alloc(w64, 5 * n * sizeof(double)));
        const size_t d = n * sizeof(double);
        it.r = w64; it.d = w64 + d; it.m = w64 + 2 * d; it.q = w64 + 3 * d; it.c = w64 + 4 * d;
        FEEC_TRY(cudaMemcpyAsync(ditem, &it, sizeof(it), cudaMemcpyHostToDevice, stream));
        FEEC_TRY(cudaMemsetAsync(dres, 0, sizeof(BatchResult), stream));
        a.inner_eta = 1e-30;
        a.err_control = 0;
        a.inner_margin = 1.0;
        a.max_iter = rq.n;
        a.max_outer = kMaxReplacements;
        a.stall_check = 0;
        int b64 = std::min(blocks, cluster_max_blocks(0, rainbow));
        int q2 = 1;
        while (q2 * 2 <= b64) q2 *= 2;
        FEEC_TRY(launch_cluster(a, 0, 0, rainbow, q2, stream));
        BatchResult h2{};
        FEEC_TRY(cudaMemcpyAsync(&h2, dres, sizeof(h2), cudaMemcpyDeviceToHost, stream));
        FEEC_TRY(cudaEventRecord(done_ev, stream));
        FEEC_TRY(cudaEventSynchronize(done_ev));
        h2.iterations += hr.iterations;
        h2.outer += hr.outer;
        h2.fp64_fallback = 1;
        hr = h2;
    }
    FEEC_TRY(cudaMemcpyAsync(rq.x, x, sizeof(double) * n, cudaMemcpyDeviceToHost, stream));
    FEEC_TRY(cudaEventRecord(done_ev, stream));
    FEEC_TRY(cudaEventSynchronize(done_ev));
    res.status = hr.status;
    res.iterations = hr.iterations;
    res.outer_iterations = hr.outer;
    res.true_relres = hr.relres;
    res.cluster_blocks = blocks;
    res.fp64_fallback = hr.fp64_fallback;
    res.error_estimate = hr.err_est;
    return hr.status;
}

// Sets up (unless the request names a resident operator) and solves one request.
int serve_one(feec_server* srv, const Request& rq, cudaStream_t stream, feec_request_result& res) {
    if (rq.op) return solve_on(srv, rq.op->s, rq, stream, res);
    feec_system* s = nullptr;
    const int st = prepare_system(srv, rq.n, rq.A, rq.C, rq.V, stream, &s);
    if (st != FEEC_OK) return st;
    struct Guard { feec_system* s; ~Guard() { feec_system_destroy(s); } } guard{s};
    return solve_on(srv, s, rq, stream, res);
}

void worker_loop(feec_server* srv) {
    cudaSetDevice(srv->device);
    cudaStream_t stream = nullptr;
    if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) return;
    while (true) {
        Request rq;
        {
            std::unique_lock<std::mutex> lk(srv->mu);
            // FIFO admission: the head request waits until the budget has room for it
            srv->cv.wait(lk, [&] {
                return srv->stop || (!srv->queue.empty() && srv->in_use.load() + srv->queue.front().bytes <= srv->budget);
            });
            if (srv->stop && srv->queue.empty()) break;
            if (srv->queue.empty()) continue;
            rq = srv->queue.front();
            srv->queue.pop_front();
            srv->in_use += rq.bytes;
            size_t cur = srv->in_use.load();
            size_t pk = srv->peak.load();
            while (cur > pk && !srv->peak.compare_exchange_weak(pk, cur)) {}
            srv->inflight++;
        }
        srv->cv.notify_all();
        feec_request_result res;
        std::memset(&res, 0, sizeof(res));
        res.id = rq.id;
        res.n = rq.n;
        res.t_submit_ms = ms_since(srv, rq.t_submit);
        const int st = serve_one(srv, rq, stream, res);
        if (st != FEEC_OK && res.status == FEEC_OK) res.status = st;
        res.t_end_ms = ms_since(srv, clock_type::now());
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            srv->in_use -= rq.bytes;
            srv->inflight--;
            srv->finished++;
            if (rq.op) rq.op->users--;
            srv->done.push_back(res);
        }
        srv->cv.notify_all();
    }
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
}

}  // namespace

extern "C" {

int feec_server_create(feec_server** out, size_t hbm_budget_bytes, int slots, int method, int mode) {
    if (!out || hbm_budget_bytes == 0 || slots <= 0 || slots > 256) return FEEC_BADARG;
    if (method != FEEC_METHOD_RAINBOW && method != FEEC_METHOD_CG) return FEEC_BADARG;
    if (mode != FEEC_MODE_MIXED && mode != FEEC_MODE_FP64) return FEEC_BADARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FEEC_NO_DEVICE;
    cudaStream_t lib = nullptr;
    int st = init_device(dev, lib);
    if (st != FEEC_OK) return st;
    feec_server* srv = new (std::nothrow) feec_server();
    if (!srv) return FEEC_OOM;
    srv->method = method;
    srv->mode = mode;
    srv->budget = hbm_budget_bytes;
    srv->device = dev;
    srv->t0 = clock_type::now();
    for (int i = 0; i < slots; i++) srv->workers.emplace_back(worker_loop, srv);
    *out = srv;
    return FEEC_OK;
}

int feec_server_submit(feec_server* srv, int N, const int* A, const int* C, const double* V, const double* b,
                       double* x, double precision, long long* id) {
    if (!srv || N <= 0 || !A || !C || !V || !b || !x || !(precision > 0.0)) return FEEC_BADARG;
    // row pointers must start at 0 and end at a non-negative entry count before the
    // footprint estimate reads A[N] (a negative count would wrap to a huge size)
    if (A[0] != 0 || A[N] < 0) return FEEC_BADARG;
    Request rq;
    rq.n = N; rq.A = A; rq.C = C; rq.V = V; rq.b = b; rq.x = x; rq.precision = precision;
    rq.bytes = estimate_bytes(N, A[N]);
    rq.t_submit = clock_type::now();
    if (rq.bytes > srv->budget) return FEEC_OOM;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->stop) return FEEC_BADARG;
        rq.id = srv->next_id++;
        srv->queue.push_back(rq);
        srv->submitted++;
    }
    srv->cv.notify_all();
    if (id) *id = rq.id;
    return FEEC_OK;
}

int feec_server_add_operator(feec_server* srv, int N, const int* A, const int* C, const double* V, int* op) {
    if (!srv || N <= 0 || !A || !C || !V || !op) return FEEC_BADARG;
    if (A[0] != 0 || A[N] < 0) return FEEC_BADARG;
    auto o = std::make_shared<Operator>();
    o->n = N;
    o->nnz = A[N];
    o->bytes = estimate_bytes(N, A[N]);
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->stop) return FEEC_BADARG;
        // resident bytes are reserved at once: they must fit beside what is running now
        if (srv->in_use.load() + o->bytes > srv->budget) return FEEC_OOM;
        srv->in_use += o->bytes;
        size_t cur = srv->in_use.load(), pk = srv->peak.load();
        while (cur > pk && !srv->peak.compare_exchange_weak(pk, cur)) {}
    }
    auto give_back = [&] {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->in_use -= o->bytes;
        srv->cv.notify_all();
    };
    if (cudaStreamCreateWithFlags(&o->home, cudaStreamNonBlocking) != cudaSuccess) { give_back(); return FEEC_CUDA_ERROR; }
    int st = prepare_system(srv, N, A, C, V, o->home, &o->s);
    // cluster-solved requests share the SELL copy: built here, before any of them reads it
    if (st == FEEC_OK && (long long)o->nnz < srv->big_nnz)
        st = sell_prepare(o->s, srv->method == FEEC_METHOD_RAINBOW ? FEEC_METHOD_RAINBOW : FEEC_METHOD_CG);
    cudaStreamSynchronize(o->home);
    if (st != FEEC_OK) {
        if (o->s) feec_system_destroy(o->s);
        cudaStreamDestroy(o->home);
        give_back();
        return st;
    }
    std::lock_guard<std::mutex> lk(srv->mu);
    o->id = srv->next_op++;
    srv->ops[o->id] = o;
    *op = o->id;
    return FEEC_OK;
}

int feec_server_submit_rhs(feec_server* srv, int op, const double* b, double* x, double precision, long long* id) {
    if (!srv || !b || !x || !(precision > 0.0)) return FEEC_BADARG;
    Request rq;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->stop) return FEEC_BADARG;
        auto it = srv->ops.find(op);
        if (it == srv->ops.end()) return FEEC_BADARG;
        rq.op = it->second;
        rq.n = rq.op->n;
        rq.b = b; rq.x = x; rq.precision = precision;
        rq.bytes = estimate_rhs_bytes(rq.n);
        rq.t_submit = clock_type::now();
        if (rq.bytes > srv->budget) return FEEC_OOM;
        rq.op->users++;
        rq.id = srv->next_id++;
        srv->queue.push_back(rq);
        srv->submitted++;
    }
    srv->cv.notify_all();
    if (id) *id = rq.id;
    return FEEC_OK;
}

int feec_server_remove_operator(feec_server* srv, int op) {
    if (!srv) return FEEC_BADARG;
    std::shared_ptr<Operator> o;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        auto it = srv->ops.find(op);
        if (it == srv->ops.end() || it->second->users > 0) return FEEC_BADARG;
        o = it->second;
        srv->ops.erase(it);
    }
    feec_system_destroy(o->s);
    o->s = nullptr;
    cudaStreamDestroy(o->home);
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->in_use -= o->bytes;
    }
    srv->cv.notify_all();
    return FEEC_OK;
}

int feec_server_poll(feec_server* srv, feec_request_result* out, int max_out, int* nout) {
    if (!srv || !nout || (max_out > 0 && !out)) return FEEC_BADARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    const int k = std::min<int>(max_out, (int)srv->done.size());
    for (int i = 0; i < k; i++) out[i] = srv->done[i];
    srv->done.erase(srv->done.begin(), srv->done.begin() + k);
    *nout = k;
    return FEEC_OK;
}

int feec_server_wait(feec_server* srv, double timeout_s) {
    if (!srv) return FEEC_BADARG;
    std::unique_lock<std::mutex> lk(srv->mu);
    const bool ok = srv->cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                     [&] { return srv->finished == srv->submitted; });
    return ok ? FEEC_OK : FEEC_TIMEOUT;
}

int feec_server_stats(feec_server* srv, size_t* bytes_in_use, size_t* peak_bytes, int* inflight, long long* queued) {
    if (!srv) return FEEC_BADARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    if (bytes_in_use) *bytes_in_use = srv->in_use.load();
    if (peak_bytes) *peak_bytes = srv->peak.load();
    if (inflight) *inflight = srv->inflight.load();
    if (queued) *queued = (long long)srv->queue.size();
    return FEEC_OK;
}

int feec_server_destroy(feec_server* srv) {
    if (!srv) return FEEC_OK;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
    }
    srv->cv.notify_all();
    for (auto& t : srv->workers) t.join();
    for (auto& e : srv->ops) {
        feec_system_destroy(e.second->s);
        cudaStreamDestroy(e.second->home);
    }
    srv->ops.clear();
    delete srv;
    return FEEC_OK;
}

}  // extern "C"

// Host side of the batched engine: SELL-32 preparation of a system and the two
// batched entry points of the C ABI (many right-hand sides of one system, or
// many systems with one right-hand side each).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "feec_batched.h"
#include "feec_device.cuh"
#include "feec_system.h"

using namespace feec;

namespace feec {
int sell_prepare(feec_system* s, int method);
SellView sell_view(const feec_system* s, int method);
}

namespace feec {


// Builds (once per system and ordering) the SELL-32 layout: slices of 32 rows that
// never cross a color, blocks [L | E | U] per slice (natural order: one block).
int sell_prepare(feec_system* s, int method) {
    if (method != FEEC_METHOD_RAINBOW && method != FEEC_METHOD_CG) return FEEC_BADARG;
    const bool rb = method == FEEC_METHOD_RAINBOW;
    SellData& D = s->sell[rb ? 1 : 0];
    if (D.ready) return FEEC_OK;
    if (rb && s->prepared != FEEC_METHOD_RAINBOW) return FEEC_BADARG;
    HomeStreamScope home(s);
    D.mem.release();
    D.mem.stream = s->stream;
    cudaStream_t st = s->stream;
    const int n = s->n;
    std::vector<int> ranges;
    if (rb) {
        ranges.resize((size_t)s->nf + 1);
        FEEC_TRY(cudaMemcpyAsync(ranges.data(), s->fptr, sizeof(int) * ranges.size(), cudaMemcpyDeviceToHost, st));
        FEEC_TRY(cudaStreamSynchronize(st));
    } else {
        ranges = {0, n};
    }
    const int ncolors = (int)ranges.size() - 1;
    std::vector<int> row0, nrow, cslice(1, 0);
    for (int c = 0; c < ncolors; c++) {
        for (int r = ranges[c]; r < ranges[c + 1]; r += 32) {
            row0.push_back(r);
            nrow.push_back(std::min(32, ranges[c + 1] - r));
        }
        cslice.push_back((int)row0.size());
    }
    const int ns = (int)row0.size();
    DevArena& M = D.mem;
    FEEC_TRY(M.alloc(D.slice_row0, ns)); FEEC_TRY(M.alloc(D.slice_nrow, ns)); FEEC_TRY(M.alloc(D.slice_len, ns));
    FEEC_TRY(M.alloc(D.slice_off, ns)); FEEC_TRY(M.alloc(D.color_slice, cslice.size()));
    FEEC_TRY(cudaMemcpyAsync(D.slice_row0, row0.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, st));
    FEEC_TRY(cudaMemcpyAsync(D.slice_nrow, nrow.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, st));
    FEEC_TRY(cudaMemcpyAsync(D.color_slice, cslice.data(), sizeof(int) * cslice.size(), cudaMemcpyHostToDevice, st));
    const int* rp = rb ? s->rp : s->A;
    const int* cin = rb ? s->ci : s->C;
    const double* vin = rb ? s->val : s->V;
    FEEC_TRY(launch_sell_lengths(ns, D.slice_row0, D.slice_nrow, rp, rb ? s->lsplit : nullptr,
                                 rb ? s->usplit : nullptr, D.slice_len, st));
    std::vector<int4> len((size_t)ns);
    FEEC_TRY(cudaMemcpyAsync(len.data(), D.slice_len, sizeof(int4) * ns, cudaMemcpyDeviceToHost, st));
    FEEC_TRY(cudaStreamSynchronize(st));
    std::vector<long long> off((size_t)ns);
    long long total = 0;
    for (int i = 0; i < ns; i++) {
        off[i] = total;
        total += 32ll * (len[i].x + len[i].y + len[i].z);
    }
    FEEC_TRY(cudaMemcpyAsync(D.slice_off, off.data(), sizeof(long long) * ns, cudaMemcpyHostToDevice, st));
    FEEC_TRY(M.alloc(D.ci, (size_t)total)); FEEC_TRY(M.alloc(D.val32, (size_t)total));
    FEEC_TRY(M.alloc(D.val64, (size_t)total));
    FEEC_TRY(launch_sell_fill(ns, D.slice_row0, D.slice_nrow, D.slice_len, D.slice_off, rp, rb ? s->lsplit : nullptr,
                              rb ? s->usplit : nullptr, cin, vin, D.ci, D.val32, D.val64, st));
    if (!rb) {
        std::vector<int> id((size_t)n);
        std::iota(id.begin(), id.end(), 0);
        FEEC_TRY(M.alloc(D.ident, n));
        FEEC_TRY(cudaMemcpyAsync(D.ident, id.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
    }
    FEEC_TRY(cudaStreamSynchronize(st));
    D.nslices = ns;
    D.ncolors = ncolors;
    D.entries = total;
    D.ready = true;
    return FEEC_OK;
}

SellView sell_view(const feec_system* s, int method) {
    const bool rb = method == FEEC_METHOD_RAINBOW;
    const SellData& D = s->sell[rb ? 1 : 0];
    SellView v{};
    v.n = s->n; v.nslices = D.nslices; v.ncolors = D.ncolors;
    v.perm = rb ? s->perm : D.ident;
    v.slice_row0 = D.slice_row0; v.slice_nrow = D.slice_nrow; v.slice_len = D.slice_len; v.slice_off = D.slice_off;
    v.color_slice = D.color_slice; v.ci = D.ci; v.val32 = D.val32; v.val64 = D.val64;
    v.wd32 = rb ? s->wd32 : nullptr; v.sd32 = rb ? s->sd32 : nullptr;
    v.wd64 = rb ? s->wd : nullptr; v.sd64 = rb ? s->sd : nullptr;
    return v;
}

}  // namespace feec

namespace {

struct Job {
    int system;
    int nrhs;
    int first;
    const double* b[kBatchMaxK];
    double* x[kBatchMaxK];
};

// One launch of the batched kernel over `jobs`; the per-column results come back in `res`.
// team_blocks >= 2: clusters of that many blocks are the teams (threads is then the cluster
// kernel's fixed block size); teams = 0 fills the GPU with resident teams.
int run_batch_results(cudaStream_t st, const std::vector<feec_system*>& systems, std::vector<Job>& jobs, int method,
                      int mode, int K, double precision, int max_iter, int nresults, int teams, int threads,
                      int team_blocks, int max_outer, bool stall_check, std::vector<BatchResult>& res,
                      float* elapsed_ms) {
    const int is_float = mode == FEEC_MODE_MIXED ? 1 : 0;
    const size_t tsz = is_float ? sizeof(float) : sizeof(double);
    // largest systems first, so the tail of the batch is short
    std::stable_sort(jobs.begin(), jobs.end(),
                     [&](const Job& a, const Job& b) { return systems[a.system]->n > systems[b.system]->n; });
    DevArena tmp;
    tmp.stream = st;
    std::vector<SellView> views;
    for (auto* s : systems) views.push_back(sell_view(s, method));
    SellView* dviews = nullptr;
    BatchItem* ditems = nullptr;
    BatchResult* dres = nullptr;
    int* dnext = nullptr;
    FEEC_TRY(tmp.alloc(dviews, views.size()));
    FEEC_TRY(tmp.alloc(ditems, jobs.size()));
    FEEC_TRY(tmp.alloc(dres, (size_t)nresults));
    FEEC_TRY(tmp.alloc(dnext, 1));
    std::vector<BatchItem> items(jobs.size());
    for (size_t i = 0; i < jobs.size(); i++) {
        const Job& jb = jobs[i];
        const size_t len = (size_t)systems[jb.system]->n * K;
        BatchItem& it = items[i];
        std::memset(&it, 0, sizeof(it));
        it.system = jb.system; it.nrhs = jb.nrhs; it.first_result = jb.first;
        for (int j = 0; j < kBatchMaxK; j++) { it.b[j] = jb.b[j]; it.x[j] = jb.x[j]; }
        FEEC_TRY(tmp.alloc(it.xp, len)); FEEC_TRY(tmp.alloc(it.bp, len)); FEEC_TRY(tmp.alloc(it.r64, len));
        char* w = nullptr;
        FEEC_TRY(tmp.alloc(w, 5 * len * tsz));
        it.r = w; it.d = w + len * tsz; it.m = w + 2 * len * tsz; it.q = w + 3 * len * tsz; it.c = w + 4 * len * tsz;
    }
    FEEC_TRY(cudaMemcpyAsync(dviews, views.data(), sizeof(SellView) * views.size(), cudaMemcpyHostToDevice, st));
    FEEC_TRY(cudaMemcpyAsync(ditems, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice, st));
    FEEC_TRY(cudaMemsetAsync(dnext, 0, sizeof(int), st));
    FEEC_TRY(cudaMemsetAsync(dres, 0, sizeof(BatchResult) * nresults, st));
    BatchArgs a{};
    a.systems = dviews; a.items = ditems; a.nitems = (int)items.size(); a.next_item = dnext; a.results = dres;
    a.precision = precision;
    // segment factor (FP32: a fresh inner solve asks for a fall of kRestartEta or what the
    // target still needs; FP64: only the target); the autotuner's trials (max_outer > 0) run
    // a fixed iteration count in one segment
    a.inner_eta = (is_float && max_outer <= 0) ? kRestartEta : 1e-30;
    a.err_control = (is_float && max_outer <= 0) ? 1 : 0;
    a.inner_margin = is_float ? 0.3 : 1.0;   // FP64 recursion tracks the true residual closely
    a.max_iter = max_iter;
    a.max_outer = max_outer > 0 ? max_outer : kMaxReplacements;
    a.stall_check = (is_float && stall_check) ? 1 : 0;
    cudaEvent_t e0, e1;
    FEEC_TRY(cudaEventCreate(&e0));
    FEEC_TRY(cudaEventCreate(&e1));
    FEEC_TRY(cudaEventRecord(e0, st));
    if (team_blocks >= 2)
        FEEC_TRY(launch_batched_clusters(a, is_float, K, method == FEEC_METHOD_RAINBOW, team_blocks, teams, st));
    else
        FEEC_TRY(launch_batched(a, is_float, K, method == FEEC_METHOD_RAINBOW, threads, teams, st));
    FEEC_TRY(cudaEventRecord(e1, st));
    res.assign((size_t)nresults, BatchResult{});
    FEEC_TRY(cudaMemcpyAsync(res.data(), dres, sizeof(BatchResult) * nresults, cudaMemcpyDeviceToHost, st));
    FEEC_TRY(cudaStreamSynchronize(st));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    tmp.release();
    FEEC_TRY(cudaStreamSynchronize(st));
    if (elapsed_ms) *elapsed_ms = ms;
    return FEEC_OK;
}

// Columns that the stall check stopped (an operator too ill-conditioned for FP32 inner
// solves) continue from their current iterate — already written back to the caller's
// x — in the FP64 batched solver, one column per team, with a fresh budget of max_iter
// iterations; their results are merged.
int rescue_stagnated(cudaStream_t st, const std::vector<feec_system*>& systems, const std::vector<Job>& jobs,
                     int method, double precision, int max_iter, std::vector<BatchResult>& res, float* extra_ms) {
    std::vector<Job> again;
    std::vector<int> slot;
    for (const Job& jb : jobs)
        for (int j = 0; j < jb.nrhs; j++) {
            const int r = jb.first + j;
            if (res[r].status != kStatusStagnated) continue;
            Job nj{};
            nj.system = jb.system; nj.nrhs = 1; nj.first = (int)again.size();
            nj.b[0] = jb.b[j]; nj.x[0] = jb.x[j];
            again.push_back(nj);
            slot.push_back(r);
        }
    if (again.empty()) return FEEC_OK;
    std::vector<BatchResult> r2;
    float ms = 0.0f;
    const int st2 = run_batch_results(st, systems, again, method, FEEC_MODE_FP64, 1, precision, max_iter,
                                      (int)again.size(), 0, 256, 1, 0, false, r2, &ms);
    if (st2 != FEEC_OK) return st2;
    for (size_t k = 0; k < slot.size(); k++) {
        BatchResult& d = res[slot[k]];
        d.status = r2[k].status;
        d.iterations += r2[k].iterations;
        d.outer += r2[k].outer;
        d.relres = r2[k].relres;
        d.err_est = r2[k].err_est;
        d.fp64_fallback = 1;
    }
    if (extra_ms) *extra_ms += ms;
    return FEEC_OK;
}

void fill_infos(const std::vector<BatchResult>& res, double precision, float ms, int grid, feec_solve_info* infos,
                int& worst, int inner_fp64 = 0) {
    worst = FEEC_OK;
    for (size_t i = 0; i < res.size(); i++) {
        if (res[i].status != FEEC_OK && worst == FEEC_OK) worst = res[i].status;
        if (infos) {
            feec_solve_info& f = infos[i];
            std::memset(&f, 0, sizeof(f));
            f.status = res[i].status;
            f.iterations = res[i].iterations;
            f.outer_iterations = res[i].outer;
            f.true_relres = res[i].relres;
            f.tolerance = precision;
            f.final_norm = res[i].relres;
            f.device_ms = ms;
            f.lanes_per_row = 1;
            f.grid_blocks = grid;
            f.fp64_fallback = res[i].fp64_fallback;
            f.inner_fp64 = inner_fp64;
            f.error_estimate = res[i].err_est;
        }
    }
}

int run_batch(cudaStream_t st, const std::vector<feec_system*>& systems, std::vector<Job>& jobs, int method, int mode,
              int K, double precision, int max_iter, int nresults, feec_solve_info* infos, int teams, int threads,
              int team_blocks = 1, int max_outer = 0, float* elapsed_ms = nullptr, long long* iter_sum = nullptr) {
    const int is_float = mode == FEEC_MODE_MIXED ? 1 : 0;
    std::vector<BatchResult> res;
    float ms = 0.0f;
    const bool rescue = is_float && max_outer == 0;   // the autotuner's trials run a fixed iteration count
    int st2 = run_batch_results(st, systems, jobs, method, mode, K, precision, max_iter, nresults, teams, threads,
                                team_blocks, max_outer, rescue, res, &ms);
    if (st2 != FEEC_OK) return st2;
    if (rescue) {
        st2 = rescue_stagnated(st, systems, jobs, method, precision, max_iter, res, &ms);
        if (st2 != FEEC_OK) return st2;
    }
    if (elapsed_ms) *elapsed_ms = ms;
    if (iter_sum) {
        long long t = 0;
        for (int i = 0; i < nresults; i++) t += res[i].iterations;
        *iter_sum = t;
    }
    const int rb = method == FEEC_METHOD_RAINBOW;
    int grid = 0;
    if (team_blocks >= 2) {
        const int nc = teams > 0 ? teams : cluster_batched_resident(is_float, K, rb, team_blocks);
        grid = std::min<int>(nc, (int)jobs.size()) * team_blocks;
    } else {
        grid = teams > 0 ? teams : std::min<int>(batched_resident_teams(is_float, K, rb, threads), (int)jobs.size());
    }
    int worst = FEEC_OK;
    fill_infos(res, precision, ms, grid, infos, worst);
    return worst;
}

struct TunedConfig {
    bool valid = false;
    int K = 0, threads = 0;
    double rhs_iters_per_s = 0.0;
};

int jobs_for(feec_system* s, int nrhs, int K, double* X, const double* Bm, std::vector<Job>& jobs) {
    const size_t n = (size_t)s->n;
    jobs.clear();
    for (int j0 = 0; j0 < nrhs; j0 += K) {
        Job jb{};
        jb.system = 0; jb.first = j0; jb.nrhs = std::min(K, nrhs - j0);
        for (int j = 0; j < jb.nrhs; j++) { jb.b[j] = Bm + (j0 + j) * n; jb.x[j] = X + (j0 + j) * n; }
        jobs.push_back(jb);
    }
    return FEEC_OK;
}

int pick_k(int mode, int rhs_per_team) {
    const int kmax = batched_max_k(mode == FEEC_MODE_MIXED);
    int K = rhs_per_team > 0 ? rhs_per_team : kmax;
    if (K > kmax) K = kmax;
    if (K != 1 && K != 2 && K != 4 && K != 8) K = K >= 8 ? 8 : (K >= 4 ? 4 : (K >= 2 ? 2 : 1));
    if (K > kmax) K = kmax;
    return K;
}

}  // namespace

extern "C" {

int feec_system_solve_batch(feec_system* s, int method, int mode, int nrhs, double* X, const double* Bm,
                            double precision, int max_iter, int rhs_per_team, feec_solve_info* infos, void* stream) {
    if (!s || nrhs <= 0 || !X || !Bm || !(precision > 0.0)) return FEEC_BADARG;
    if (method != FEEC_METHOD_CG && method != FEEC_METHOD_RAINBOW) return FEEC_BADARG;
    if (mode != FEEC_MODE_MIXED && mode != FEEC_MODE_FP64) return FEEC_BADARG;
    cudaStream_t keep = s->stream;
    if (stream) { s->stream = (cudaStream_t)stream; }
    int st = sell_prepare(s, method);
    if (st == FEEC_OK) {
        int K = pick_k(mode, rhs_per_team);
        int threads = 256, blocks = 1;
        if (rhs_per_team == 0 && s->tuned_k[method][mode] > 0) {
            K = s->tuned_k[method][mode];
            threads = s->tuned_threads[method][mode];
            blocks = std::max(1, s->tuned_blocks[method][mode]);
        }
        std::vector<feec_system*> systems{s};
        std::vector<Job> jobs;
        jobs_for(s, nrhs, K, X, Bm, jobs);
        st = run_batch(s->stream, systems, jobs, method, mode, K, precision, max_iter > 0 ? max_iter : s->n, nrhs,
                       infos, blocks >= 2 ? 0 : s->user_blocks, threads, blocks);
    }
    s->stream = keep;
    return st;
}

int feec_system_set_batch_config(feec_system* s, int method, int mode, int rhs_per_team, int team_threads,
                                 int team_blocks) {
    if (!s || (method != FEEC_METHOD_CG && method != FEEC_METHOD_RAINBOW) ||
        (mode != FEEC_MODE_MIXED && mode != FEEC_MODE_FP64))
        return FEEC_BADARG;
    const int is_float = mode == FEEC_MODE_MIXED;
    if (rhs_per_team == 0) {   // forget the configuration: automatic choice again
        s->tuned_k[method][mode] = 0; s->tuned_threads[method][mode] = 0; s->tuned_blocks[method][mode] = 0;
        s->tuned_rate[method][mode] = 0.0;
        return FEEC_OK;
    }
    if (pick_k(mode, rhs_per_team) != rhs_per_team) return FEEC_BADARG;
    if (team_blocks < 1 || team_blocks > 16 || (team_blocks & (team_blocks - 1)) != 0) return FEEC_BADARG;
    if (team_blocks == 1 && batched_team_threads(is_float, team_threads) != team_threads) return FEEC_BADARG;
    if (team_blocks == 1 && team_threads == 1024 && rhs_per_team > 2) return FEEC_BADARG;
    if (team_blocks == 1 && rhs_per_team == 8 && team_threads != 256 && team_threads != 512) return FEEC_BADARG;
    if (team_blocks >= 2) {
        if (cluster_batched_resident(is_float, rhs_per_team, method == FEEC_METHOD_RAINBOW, team_blocks) <= 0)
            return FEEC_BADARG;
        team_threads = cluster_batched_threads();
    }
    s->tuned_k[method][mode] = rhs_per_team;
    s->tuned_threads[method][mode] = team_threads;
    s->tuned_blocks[method][mode] = team_blocks;
    s->tuned_rate[method][mode] = 0.0;
    return FEEC_OK;
}

// Autotuner of the batched engine: for every candidate (right-hand sides per team; team
// size 128..1024 threads for a one-block team, or 2..16 blocks for a cluster team when
// the batch has fewer work items than the GPU holds block teams) it runs a short trial
// on the system itself — the batch's columns (without a size hint, one work item per
// resident team), a fixed number of inner iterations — and rates it in
// column-iterations per second. The three best are trialled again at two lengths, and
// the difference rates the iterations alone (a solve's set-up favours wide teams in a
// short trial). The winner is cached for this system and used by
// feec_system_solve_batch when rhs_per_team is 0.
int feec_system_tune_batch(feec_system* s, int method, int mode, int nrhs_hint, int* rhs_per_team, int* team_threads,
                           int* team_blocks, double* rhs_iters_per_s) {
    if (!s || (method != FEEC_METHOD_CG && method != FEEC_METHOD_RAINBOW) ||
        (mode != FEEC_MODE_MIXED && mode != FEEC_MODE_FP64))
        return FEEC_BADARG;
    int st = sell_prepare(s, method);
    if (st != FEEC_OK) return st;
    const int is_float = mode == FEEC_MODE_MIXED;
    const int rb = method == FEEC_METHOD_RAINBOW;
    struct Candidate { int K, threads, blocks, resident; };
    std::vector<Candidate> cands;
    const int Ks[4] = {1, 2, 4, 8};
    const int Ts[4] = {128, 256, 512, 1024};
    const int Cs[4] = {2, 4, 8, 16};
    for (int K : Ks) {
        if (K > batched_max_k(is_float)) continue;
        for (int T : Ts) {
            if (batched_team_threads(is_float, T) != T) continue;
            if (T == 1024 && K > 2) continue;
            if (K == 8 && T != 256 && T != 512) continue;
            cands.push_back({K, T, 1, batched_resident_teams(is_float, K, rb, T)});
        }
        const int items = nrhs_hint > 0 ? (nrhs_hint + K - 1) / K : 0;
        if (items > 0 && items < batched_resident_teams(is_float, K, rb, cluster_batched_threads()))
            for (int C : Cs) {
                const int res = cluster_batched_resident(is_float, K, rb, C);
                if (res > 0) cands.push_back({K, cluster_batched_threads(), C, res});
            }
    }
    const size_t n = (size_t)s->n;
    // A rough right-hand side (U[-1, 1) from a fixed-seed LCG): a smooth one such as all
    // ones converges within a few iterations and would time set-up instead of iterations.
    std::vector<double> rhs(n);
    {
        unsigned long long g = 0x9E3779B97F4A7C15ull;
        for (size_t i = 0; i < n; i++) {
            g = g * 6364136223846793005ull + 1442695040888963407ull;
            rhs[i] = (double)(g >> 11) * (2.0 / 9007199254740992.0) - 1.0;
        }
    }
    // One trial: `iters` inner iterations of every column; time and column-iterations done.
    auto trial = [&](const Candidate& c, int iters, float& ms, long long& its) -> int {
        const int K = c.K;
        // the whole batch when its size is known (a batch with more work items than resident
        // teams runs in waves, and the trial must see them), else one item per resident team
        const int cols = nrhs_hint > 0 ? ((nrhs_hint + K - 1) / K) * K : c.resident * K;
        DevArena tmp; tmp.stream = s->stream;
        double *B = nullptr, *X = nullptr;
        FEEC_TRY(tmp.alloc(B, n * cols)); FEEC_TRY(tmp.alloc(X, n * cols));
        FEEC_TRY(cudaMemcpyAsync(B, rhs.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s->stream));
        for (int done = 1; done < cols;) {   // replicate on the device, doubling the filled columns
            const int m = std::min(done, cols - done);
            FEEC_TRY(cudaMemcpyAsync(B + done * n, B, sizeof(double) * n * m, cudaMemcpyDeviceToDevice, s->stream));
            done += m;
        }
        FEEC_TRY(cudaMemsetAsync(X, 0, sizeof(double) * n * cols, s->stream));
        std::vector<feec_system*> systems{s};
        std::vector<Job> jobs;
        jobs_for(s, cols, K, X, B, jobs);
        ms = 0.0f; its = 0;
        const int e = run_batch(s->stream, systems, jobs, method, mode, K, 1e-300, iters, cols, nullptr, 0, c.threads,
                                c.blocks, 1, &ms, &its);
        tmp.release();
        cudaStreamSynchronize(s->stream);
        return (e == FEEC_OK || e == FEEC_MAXITER) ? FEEC_OK : e;
    };
    // Screening: a short trial per candidate (its rate includes the set-up of a solve).
    std::vector<std::pair<double, size_t>> screened;
    for (size_t ci = 0; ci < cands.size(); ci++) {
        float ms; long long its;
        st = trial(cands[ci], 12, ms, its);
        if (st != FEEC_OK) return st;
        screened.push_back({ms > 0.0f ? (double)its / (ms * 1e-3) : 0.0, ci});
    }
    std::sort(screened.begin(), screened.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    // Final: the best three by screening, rated on the difference of a long and a short trial,
    // so the rate is that of the iterations alone, without the set-up of a solve.
    TunedConfig best;
    int best_blocks = 1;
    for (size_t r = 0; r < screened.size() && r < 3; r++) {
        const Candidate& c = cands[screened[r].second];
        float ms1, ms2; long long its1, its2;
        st = trial(c, 6, ms1, its1);
        if (st != FEEC_OK) return st;
        st = trial(c, 30, ms2, its2);
        if (st != FEEC_OK) return st;
        const double rate = (ms2 > ms1 && its2 > its1) ? (double)(its2 - its1) / ((ms2 - ms1) * 1e-3) : screened[r].first;
        if (rate > best.rhs_iters_per_s) {
            best.valid = true; best.K = c.K; best.threads = c.threads; best.rhs_iters_per_s = rate;
            best_blocks = c.blocks;
        }
    }
    if (!best.valid) return FEEC_CUDA_ERROR;
    s->tuned_k[method][mode] = best.K;
    s->tuned_threads[method][mode] = best.threads;
    s->tuned_blocks[method][mode] = best_blocks;
    s->tuned_rate[method][mode] = best.rhs_iters_per_s;
    if (rhs_per_team) *rhs_per_team = best.K;
    if (team_threads) *team_threads = best.threads;
    if (team_blocks) *team_blocks = best_blocks;
    if (rhs_iters_per_s) *rhs_iters_per_s = best.rhs_iters_per_s;
    return FEEC_OK;
}

int feec_solve_many(int nsys, feec_system* const* systems, int method, int mode, double* const* x,
                    const double* const* b, double precision, int max_iter, feec_solve_info* infos, void* stream) {
    if (nsys <= 0 || !systems || !x || !b || !(precision > 0.0)) return FEEC_BADARG;
    if (method != FEEC_METHOD_CG && method != FEEC_METHOD_RAINBOW) return FEEC_BADARG;
    if (mode != FEEC_MODE_MIXED && mode != FEEC_MODE_FP64) return FEEC_BADARG;
    cudaStream_t st = stream ? (cudaStream_t)stream : systems[0]->stream;
    std::vector<feec_system*> sys(systems, systems + nsys);
    int maxn = 0;
    for (int i = 0; i < nsys; i++) {
        if (!sys[i] || !x[i] || !b[i]) return FEEC_BADARG;
        cudaStream_t keep = sys[i]->stream;
        sys[i]->stream = st;
        const int e = sell_prepare(sys[i], method);
        sys[i]->stream = keep;
        if (e != FEEC_OK) return e;
        maxn = std::max(maxn, sys[i]->n);
    }
    std::vector<Job> jobs((size_t)nsys);
    for (int i = 0; i < nsys; i++) {
        Job& jb = jobs[i];
        std::memset(&jb, 0, sizeof(jb));
        jb.system = i; jb.nrhs = 1; jb.first = i; jb.b[0] = b[i]; jb.x[0] = x[i];
    }
    return run_batch(st, sys, jobs, method, mode, 1, precision, max_iter > 0 ? max_iter : maxn, nsys, infos, 0, 256);
}

// ---------------------------------------------------------------------------
// Reusable batch: the systems, their right-hand-side / solution buffers, the work
// table and all workspace are set up once; the launch sequence (queue reset,
// result reset, batched kernel) is captured in a CUDA graph and replayed by
// feec_batch_run, so a repeated batch costs one graph launch.
// ---------------------------------------------------------------------------
struct feec_batch {
    cudaStream_t stream = nullptr;        // own stream: the graph is captured on and replayed on it
    cudaStream_t user_stream = nullptr;   // the caller's stream (may be the legacy default stream)
    cudaEvent_t ev_in = nullptr;
    bool own_stream = false;
    DevArena mem;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    BatchResult* dres = nullptr;
    BatchResult* hres = nullptr;          // pinned: the result copy of a launch is asynchronous
    bool pending = false;                 // launched and not yet finished
    int nresults = 0;
    double precision = 0.0;
    int teams = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    // for the FP64 finish of stagnated systems (mixed precision only)
    int method = 0, mode = 0, max_iter = 0;
    int inner_fp64 = 0;                   // mixed: the FP64 graph measured faster at creation
    std::vector<feec_system*> systems;
    std::vector<Job> jobs;
};

int feec_batch_create(feec_batch** out, int nsys, feec_system* const* systems, int method, int mode, double* const* x,
                      const double* const* b, double precision, int max_iter, int team_threads, void* stream) {
    if (!out || nsys <= 0 || !systems || !x || !b || !(precision > 0.0)) return FEEC_BADARG;
    if (method != FEEC_METHOD_CG && method != FEEC_METHOD_RAINBOW) return FEEC_BADARG;
    if (mode != FEEC_MODE_MIXED && mode != FEEC_MODE_FP64) return FEEC_BADARG;
    *out = nullptr;
    feec_batch* bt = new (std::nothrow) feec_batch();
    if (!bt) return FEEC_OOM;
    struct Cleanup {                      // a failed create releases whatever it made
        feec_batch*& p;
        bool keep = false;
        ~Cleanup() {
            if (!keep && p) {
                feec_batch_destroy(p);
                p = nullptr;
            }
        }
    } cleanup{bt};
    // The legacy default stream cannot be captured: the batch owns a non-blocking
    // stream and orders it after the caller's stream with an event on every run.
    bt->user_stream = (cudaStream_t)stream;
    FEEC_TRY(cudaStreamSynchronize(bt->user_stream));
    FEEC_TRY(cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking));
    bt->own_stream = true;
    FEEC_TRY(cudaEventCreateWithFlags(&bt->ev_in, cudaEventDisableTiming));
    bt->mem.stream = bt->stream;
    bt->precision = precision;
    int maxn = 0;
    std::vector<feec_system*> sys(systems, systems + nsys);
    for (int i = 0; i < nsys; i++) {
        if (!sys[i] || !x[i] || !b[i]) return FEEC_BADARG;
        cudaStream_t keep = sys[i]->stream;
        sys[i]->stream = bt->stream;
        const int e = sell_prepare(sys[i], method);
        sys[i]->stream = keep;
        if (e != FEEC_OK) return e;
        maxn = std::max(maxn, sys[i]->n);
    }
    const int is_float = mode == FEEC_MODE_MIXED;
    // FP64-sized workspace in both modes: a mixed batch also captures and times the FP64
    // iteration (below)
    const size_t tsz = sizeof(double);
    // largest systems first
    std::vector<int> order((size_t)nsys);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return sys[a]->n > sys[c]->n; });
    std::vector<SellView> views;
    for (auto* sp : sys) views.push_back(sell_view(sp, method));
    SellView* dviews = nullptr;
    BatchItem* ditems = nullptr;
    int* dnext = nullptr;
    DevArena& M = bt->mem;
    FEEC_TRY(M.alloc(dviews, views.size()));
    FEEC_TRY(M.alloc(ditems, (size_t)nsys));
    FEEC_TRY(M.alloc(bt->dres, (size_t)nsys));
    FEEC_TRY(M.alloc(dnext, 1));
    std::vector<BatchItem> items((size_t)nsys);
    for (int k = 0; k < nsys; k++) {
        const int i = order[k];
        const size_t len = (size_t)sys[i]->n;
        BatchItem& it = items[k];
        std::memset(&it, 0, sizeof(it));
        it.system = i; it.nrhs = 1; it.first_result = i;
        it.b[0] = b[i]; it.x[0] = x[i];
        FEEC_TRY(M.alloc(it.xp, len)); FEEC_TRY(M.alloc(it.bp, len)); FEEC_TRY(M.alloc(it.r64, len));
        char* w = nullptr;
        FEEC_TRY(M.alloc(w, 5 * len * tsz));
        it.r = w; it.d = w + len * tsz; it.m = w + 2 * len * tsz; it.q = w + 3 * len * tsz; it.c = w + 4 * len * tsz;
    }
    FEEC_TRY(cudaMemcpyAsync(dviews, views.data(), sizeof(SellView) * views.size(), cudaMemcpyHostToDevice, bt->stream));
    FEEC_TRY(cudaMemcpyAsync(ditems, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice, bt->stream));
    FEEC_TRY(cudaStreamSynchronize(bt->stream));
    BatchArgs a{};
    a.systems = dviews; a.items = ditems; a.nitems = nsys; a.next_item = dnext; a.results = bt->dres;
    a.precision = precision;
    a.inner_eta = is_float ? kRestartEta : 1e-30;
    a.err_control = is_float ? 1 : 0;
    a.inner_margin = is_float ? 0.3 : 1.0;
    a.max_iter = max_iter > 0 ? max_iter : maxn;
    a.max_outer = kMaxReplacements;
    a.stall_check = is_float;
    bt->method = method; bt->mode = mode; bt->max_iter = a.max_iter;
    bt->systems = sys;
    for (int i = 0; i < nsys; i++) {
        Job jb{};
        jb.system = i; jb.nrhs = 1; jb.first = i; jb.b[0] = b[i]; jb.x[0] = x[i];
        bt->jobs.push_back(jb);
    }
    const int threads = team_threads > 0 ? team_threads : 256;
    const bool rainbow = method == FEEC_METHOD_RAINBOW;
    bt->teams = std::min(nsys, batched_resident_teams(is_float, 1, rainbow, threads));
    const int teams64 = std::min(nsys, batched_resident_teams(0, 1, rainbow, threads));
    // capture a launch sequence (batched_resident_teams above already set the kernels'
    // attributes, so nothing but stream work happens while capturing)
    auto capture = [&](const BatchArgs& args, int f, int teams, cudaGraph_t& g, cudaGraphExec_t& ex) -> int {
        FEEC_TRY(cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeRelaxed));
        cudaMemsetAsync(dnext, 0, sizeof(int), bt->stream);
        cudaMemsetAsync(bt->dres, 0, sizeof(BatchResult) * nsys, bt->stream);
        const cudaError_t le = launch_batched(args, f, 1, rainbow, threads, teams, bt->stream);
        const cudaError_t ce = cudaStreamEndCapture(bt->stream, &g);
        if (le != cudaSuccess) return cuda_status(le);
        if (ce != cudaSuccess) return cuda_status(ce);
        FEEC_TRY(cudaGraphInstantiate(&ex, g, 0));
        return FEEC_OK;
    };
    int st = capture(a, is_float, bt->teams, bt->graph, bt->exec);
    if (st != FEEC_OK) return st;
    FEEC_TRY(cudaEventCreate(&bt->e0));
    FEEC_TRY(cudaEventCreate(&bt->e1));
    FEEC_TRY(cudaMallocHost(&bt->hres, sizeof(BatchResult) * (size_t)nsys));
    bt->nresults = nsys;
    if (is_float) {
        // FP32 storage pays where the batch is bound by memory traffic; for batches of small
        // systems the FP32 segments' extra iterations can cost more than it saves (512 2D
        // systems of 81 to 66,049 unknowns: 580 solves/s mixed against 706 in FP64). The
        // batch is replayed once each way from the same initial guess (the FP32 run
        // including the FP64 finish of stagnated systems), x is put back, and the faster
        // graph is kept; results report it in inner_fp64.
        BatchArgs a64 = a;
        a64.inner_eta = 1e-30;
        a64.err_control = 0;
        a64.inner_margin = 1.0;
        a64.stall_check = 0;
        cudaGraph_t g64 = nullptr;
        cudaGraphExec_t ex64 = nullptr;
        struct GraphGuard {
            cudaGraph_t& g; cudaGraphExec_t& ex;
            ~GraphGuard() { if (ex) cudaGraphExecDestroy(ex); if (g) cudaGraphDestroy(g); }
        } gguard{g64, ex64};
        st = capture(a64, 0, teams64, g64, ex64);
        if (st != FEEC_OK) return st;
        std::vector<size_t> off((size_t)nsys + 1, 0);
        for (int i = 0; i < nsys; i++) off[i + 1] = off[i] + (size_t)sys[i]->n;
        double* xsave = nullptr;
        FEEC_TRY(M.alloc(xsave, off[nsys]));
        for (int i = 0; i < nsys; i++)
            FEEC_TRY(cudaMemcpyAsync(xsave + off[i], x[i], sizeof(double) * sys[i]->n, cudaMemcpyDeviceToDevice,
                                     bt->stream));
        auto restore = [&]() -> int {
            for (int i = 0; i < nsys; i++)
                FEEC_TRY(cudaMemcpyAsync(x[i], xsave + off[i], sizeof(double) * sys[i]->n, cudaMemcpyDeviceToDevice,
                                         bt->stream));
            return FEEC_OK;
        };
        auto trial = [&](cudaGraphExec_t ex, bool f32, float& ms) -> int {
            FEEC_TRY(cudaEventRecord(bt->e0, bt->stream));
            FEEC_TRY(cudaGraphLaunch(ex, bt->stream));
            note_launch();
            FEEC_TRY(cudaEventRecord(bt->e1, bt->stream));
            FEEC_TRY(cudaMemcpyAsync(bt->hres, bt->dres, sizeof(BatchResult) * nsys, cudaMemcpyDeviceToHost,
                                     bt->stream));
            FEEC_TRY(cudaStreamSynchronize(bt->stream));
            FEEC_TRY(cudaEventElapsedTime(&ms, bt->e0, bt->e1));
            if (f32) {
                std::vector<BatchResult> res(bt->hres, bt->hres + nsys);
                const int e = rescue_stagnated(bt->stream, bt->systems, bt->jobs, method, precision, a.max_iter,
                                               res, &ms);
                if (e != FEEC_OK) return e;
            }
            return FEEC_OK;
        };
        float t32 = 0.0f, t64 = 0.0f;
        if ((st = trial(bt->exec, true, t32)) != FEEC_OK) return st;
        if ((st = restore()) != FEEC_OK) return st;
        if ((st = trial(ex64, false, t64)) != FEEC_OK) return st;
        if ((st = restore()) != FEEC_OK) return st;
        FEEC_TRY(cudaStreamSynchronize(bt->stream));
        if (t64 < t32) {
            std::swap(bt->graph, g64);
            std::swap(bt->exec, ex64);   // the guard destroys the FP32 graph
            bt->teams = teams64;
            bt->inner_fp64 = 1;
        }
    }
    cleanup.keep = true;
    *out = bt;
    return FEEC_OK;
}

int feec_batch_launch(feec_batch* bt) {
    if (!bt || bt->pending) return FEEC_BADARG;
    FEEC_TRY(cudaEventRecord(bt->ev_in, bt->user_stream));     // inputs written on the caller's stream
    FEEC_TRY(cudaStreamWaitEvent(bt->stream, bt->ev_in, 0));
    FEEC_TRY(cudaEventRecord(bt->e0, bt->stream));
    FEEC_TRY(cudaGraphLaunch(bt->exec, bt->stream));
    note_launch();
    cudaError_t e = cudaEventRecord(bt->e1, bt->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(bt->hres, bt->dres, sizeof(BatchResult) * bt->nresults, cudaMemcpyDeviceToHost,
                            bt->stream);
    if (e != cudaSuccess) {                                      // the replay is in flight: let it end
        cudaStreamSynchronize(bt->stream);
        return cuda_status(e);
    }
    bt->pending = true;
    return FEEC_OK;
}

int feec_batch_finish(feec_batch* bt, feec_solve_info* infos, double* device_ms) {
    if (!bt || !bt->pending) return FEEC_BADARG;
    bt->pending = false;
    FEEC_TRY(cudaStreamSynchronize(bt->stream));
    std::vector<BatchResult> res(bt->hres, bt->hres + bt->nresults);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, bt->e0, bt->e1);
    if (bt->mode == FEEC_MODE_MIXED && !bt->inner_fp64) {
        const int st = rescue_stagnated(bt->stream, bt->systems, bt->jobs, bt->method, bt->precision, bt->max_iter,
                                        res, &ms);
        if (st != FEEC_OK) return st;
    }
    if (device_ms) *device_ms = ms;
    int worst = FEEC_OK;
    fill_infos(res, bt->precision, ms, bt->teams, infos, worst, bt->inner_fp64);
    return worst;
}

int feec_batch_run(feec_batch* bt, feec_solve_info* infos, double* device_ms) {
    const int st = feec_batch_launch(bt);
    if (st != FEEC_OK) return st;
    return feec_batch_finish(bt, infos, device_ms);
}

int feec_batch_destroy(feec_batch* bt) {
    if (!bt) return FEEC_OK;
    cudaStreamSynchronize(bt->stream);
    if (bt->exec) cudaGraphExecDestroy(bt->exec);
    if (bt->graph) cudaGraphDestroy(bt->graph);
    if (bt->e0) cudaEventDestroy(bt->e0);
    if (bt->e1) cudaEventDestroy(bt->e1);
    bt->mem.release();
    cudaStreamSynchronize(bt->stream);
    if (bt->ev_in) cudaEventDestroy(bt->ev_in);
    if (bt->own_stream) cudaStreamDestroy(bt->stream);
    if (bt->hres) cudaFreeHost(bt->hres);
    delete bt;
    return FEEC_OK;
}

}  // extern "C"

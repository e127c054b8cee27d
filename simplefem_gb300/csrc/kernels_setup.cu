// Non-persistent kernels: CSR SpMV (MatrixCSR::apply), FP64 residuals and
// norms for the defect-correction loop, diagonal extraction, and the integer
// layout work that turns a CSR matrix plus an ordering into the row-permuted
// [L | E | U] split layout that the SSOR / multicolor SSOR sweeps stream.
#include <cstdint>

#include "feec_batched.h"
#include "feec_device.cuh"
#include "feec_internal.h"

namespace feec {

namespace {

constexpr int kBlock = 256;

template <int LANES>
__global__ void __launch_bounds__(kBlock) spmv_f64_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                                                          const double* __restrict__ v, const double* __restrict__ x,
                                                          double* __restrict__ y, double scaling) {
    const int lane = threadIdx.x & (LANES - 1);
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) / LANES;
    const bool act = row < n;
    const int lo = act ? __ldg(&rp[row]) : 0, hi = act ? __ldg(&rp[row + 1]) : 0;
    double s = 0.0;
    for (int j = lo + lane; j < hi; j += LANES) s = fma(__ldg(&v[j]), __ldg(&x[__ldg(&ci[j])]), s);
    #pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off, LANES);
    if (act && lane == 0) y[row] = scaling * s;
}

// r = b - A x and per-block partial sums of r^2 (for ||r||); partial_sq may be null.
template <int LANES>
__global__ void __launch_bounds__(kBlock) residual_f64_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                                                              const double* __restrict__ v, const double* __restrict__ b,
                                                              const double* __restrict__ x, double* __restrict__ r,
                                                              double* __restrict__ partial_sq) {
    const int lane = threadIdx.x & (LANES - 1);
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) / LANES;
    const bool act = row < n;
    const int lo = act ? __ldg(&rp[row]) : 0, hi = act ? __ldg(&rp[row + 1]) : 0;
    double s = 0.0;
    for (int j = lo + lane; j < hi; j += LANES) s = fma(__ldg(&v[j]), __ldg(&x[__ldg(&ci[j])]), s);
    #pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off, LANES);
    double sq = 0.0;
    if (act && lane == 0) {
        const double ri = __ldg(&b[row]) - s;
        r[row] = ri;
        sq = ri * ri;
    }
    if (partial_sq) {
        double vv[1] = {sq};
        block_reduce<double, 1>(vv);
        if (threadIdx.x == 0) partial_sq[blockIdx.x] = vv[0];
    }
}

// Deterministic single-block sum of squares (or sum, if `square` is false).
__global__ void __launch_bounds__(1024) sum_kernel(int n, const double* __restrict__ v, double* out, int square) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double t = v[i];
        s += square ? t * t : t;
    }
    double vv[1] = {s};
    block_reduce<double, 1>(vv);
    if (threadIdx.x == 0) *out = vv[0];
}

__global__ void diagonal_kernel(int n, const int* __restrict__ A, const int* __restrict__ C, const double* __restrict__ V,
                                double* __restrict__ d) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double s = 0.0;
    for (int i = A[r]; i < A[r + 1]; i++)
        if (C[i] == r) s += V[i];
    d[r] = s;
}

// Structural check of a square CSR matrix: A[0] == 0, A non-decreasing, A[n] == nnz,
// 0 <= C < n. Any violation sets *bad (nothing is indexed through unchecked values).
__global__ void validate_csr_kernel(int n, int ncols, int nnz, const int* __restrict__ A, const int* __restrict__ C,
                                    int* bad) {
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = tid; i < n; i += stride) {
        const int a0 = A[i], a1 = A[i + 1];
        if (a1 < a0 || a0 < 0 || a1 > nnz) atomicExch(bad, 1);
    }
    if (tid == 0 && (A[0] != 0 || A[n] != nnz)) atomicExch(bad, 1);
    for (long long j = tid; j < nnz; j += stride) {
        const int c = C[j];
        if (c < 0 || c >= ncols) atomicExch(bad, 1);
    }
}

__global__ void row_lengths_kernel(int n, const int* __restrict__ A, const int* __restrict__ perm, int* __restrict__ len) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int o = perm ? perm[i] : i;
    len[i] = A[o + 1] - A[o];
}

__global__ void inverse_perm_kernel(int n, const int* __restrict__ perm, int* __restrict__ iperm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) iperm[perm[i]] = i;
}

// Row i of the new layout is old row perm[i]; entries are reordered into
// [key(col) < key(row) | == | >] keeping their original relative order, and
// columns are renumbered through iperm. key == null means key(j) = j.
__global__ void permute_split_kernel(int n, const int* __restrict__ A, const int* __restrict__ C,
                                     const double* __restrict__ V, const int* __restrict__ perm,
                                     const int* __restrict__ iperm, const int* __restrict__ key,
                                     const int* __restrict__ new_rp, int* __restrict__ out_ci,
                                     double* __restrict__ out_v, float* __restrict__ out_v32,
                                     int* __restrict__ lsplit, int* __restrict__ usplit) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int o = perm ? perm[i] : i;
    const int ko = key ? key[o] : o;
    int w = new_rp[i];
    for (int pass = 0; pass < 3; pass++) {
        if (pass == 1) lsplit[i] = w;
        if (pass == 2) usplit[i] = w;
        for (int j = A[o]; j < A[o + 1]; j++) {
            const int c = C[j];
            const int kc = key ? key[c] : c;
            const int cls = kc < ko ? 0 : (kc == ko ? 1 : 2);
            if (cls != pass) continue;
            out_ci[w] = iperm ? iperm[c] : c;
            const double val = V[j];
            if (out_v) out_v[w] = val;
            if (out_v32) out_v32[w] = (float)val;
            w++;
        }
    }
}

__global__ void gather_f64_kernel(int n, const int* __restrict__ perm, const double* __restrict__ src, double* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[perm ? perm[i] : i];
}

__global__ void scatter_f64_kernel(int n, const int* __restrict__ perm, const double* __restrict__ src, double* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[perm ? perm[i] : i] = src[i];
}

__global__ void gather_to_f32_kernel(int n, const int* __restrict__ perm, const double* __restrict__ src, float* __restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (float)src[perm ? perm[i] : i];
}

__global__ void cast_kernel(size_t n, const double* __restrict__ src, float* __restrict__ dst) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

// Sweep factors of the SSOR sweeps: wd = omega / D and sd = D (2 - omega) / omega
// (wd = 0 marks the rows with D == 0 that the reference skips).
__global__ void sweep_factors_kernel(int n, const double* __restrict__ diag, double omega, double* __restrict__ wd,
                                     double* __restrict__ sd, float* __restrict__ wd32, float* __restrict__ sd32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double D = diag[i];
    const double w = (D == 0.0) ? 0.0 : omega / D;
    const double t = D * ((2.0 - omega) / omega);
    wd[i] = w; sd[i] = t;
    wd32[i] = (D == 0.0) ? 0.0f : (float)(omega / D);
    sd32[i] = (float)t;
}

// r32[i] = r[i] * (*inv_norm)   (scaled residual handed to the FP32 inner solve)
__global__ void scaled_cast_kernel(int n, const double* __restrict__ r, const double* __restrict__ inv_norm,
                                   float* __restrict__ r32) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r32[i] = (float)(r[i] * (*inv_norm));
}

// x[perm[i]] += (*norm) * c32[i]    (FP64 solution update of the defect correction)
__global__ void update_x_kernel(int n, const int* __restrict__ perm, const float* __restrict__ c32,
                                const double* __restrict__ norm, double* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[perm ? perm[i] : i] += (*norm) * (double)c32[i];
}

// The same update, plus per-block partial sums of the squared correction and of the
// squared new iterate (partials[blk] and partials[gridDim.x + blk]): the defect
// correction's error estimate compares the size of each correction with the solution.
__global__ void update_x_norms_kernel(int n, const float* __restrict__ c32, const double* __restrict__ norm,
                                      double* __restrict__ x, double* __restrict__ partials) {
    const double s = *norm;
    double cc = 0.0, xx = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double c = s * (double)c32[i];
        const double xn = x[i] + c;
        x[i] = xn;
        cc += c * c;
        xx += xn * xn;
    }
    double v[2] = {cc, xx};
    block_reduce<double, 2>(v);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = v[0];
        partials[gridDim.x + blockIdx.x] = v[1];
    }
}

// SELL-32 block lengths of each slice: the longest L, E and U part over its rows.
// lsplit == null: the whole row is one block (U), for the unpreconditioned CG.
__global__ void sell_lengths_kernel(int nslices, const int* __restrict__ row0, const int* __restrict__ nrow,
                                    const int* __restrict__ rp, const int* __restrict__ lsplit,
                                    const int* __restrict__ usplit, int4* __restrict__ len) {
    const int sl = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (sl >= nslices) return;
    int l = 0, e = 0, u = 0;
    if (lane < nrow[sl]) {
        const int i = row0[sl] + lane;
        const int a = rp[i], b = rp[i + 1];
        if (lsplit) { l = lsplit[i] - a; e = usplit[i] - lsplit[i]; u = b - usplit[i]; }
        else { u = b - a; }
    }
    #pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        l = max(l, __shfl_xor_sync(0xffffffffu, l, off));
        e = max(e, __shfl_xor_sync(0xffffffffu, e, off));
        u = max(u, __shfl_xor_sync(0xffffffffu, u, off));
    }
    if (lane == 0) len[sl] = make_int4(l, e, u, 0);
}

// Column-major fill of each slice; padding entries get value 0 and the column of
// the slice's first row, so every gathered index stays valid.
__global__ void sell_fill_kernel(int nslices, const int* __restrict__ row0, const int* __restrict__ nrow,
                                 const int4* __restrict__ len, const long long* __restrict__ off,
                                 const int* __restrict__ rp, const int* __restrict__ lsplit,
                                 const int* __restrict__ usplit, const int* __restrict__ ci_in,
                                 const double* __restrict__ val_in, int* __restrict__ ci, float* __restrict__ val32,
                                 double* __restrict__ val64) {
    const int sl = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (sl >= nslices) return;
    const int4 L = len[sl];
    const long long base = off[sl];
    const int r0 = row0[sl];
    const bool act = lane < nrow[sl];
    const int i = r0 + lane;
    int seg_lo[3] = {0, 0, 0}, seg_hi[3] = {0, 0, 0};
    if (act) {
        const int a = rp[i], b = rp[i + 1];
        if (lsplit) {
            seg_lo[0] = a; seg_hi[0] = lsplit[i];
            seg_lo[1] = lsplit[i]; seg_hi[1] = usplit[i];
            seg_lo[2] = usplit[i]; seg_hi[2] = b;
        } else {
            seg_lo[2] = a; seg_hi[2] = b;
        }
    }
    const int blen[3] = {L.x, L.y, L.z};
    long long o = base;
    for (int blk = 0; blk < 3; blk++) {
        for (int k = 0; k < blen[blk]; k++) {
            const int j = seg_lo[blk] + k;
            const bool real = act && j < seg_hi[blk];
            const long long dst = o + (long long)k * 32 + lane;
            ci[dst] = real ? ci_in[j] : r0;
            const double v = real ? val_in[j] : 0.0;
            if (val64) val64[dst] = v;
            if (val32) val32[dst] = (float)v;
        }
        o += (long long)blen[blk] * 32;
    }
}

// SELL-32 SpMV, one thread per row. The matrix is streamed once (evict-first loads,
// so it does not push x out of L2); a chunk of column indices and values is loaded
// before its gathers so every warp keeps several requests in flight.
template <typename T>
__global__ void __launch_bounds__(256) sell_spmv_kernel(SellView v, const T* __restrict__ x, T* __restrict__ y, T scaling) {
    const T* __restrict__ val = sizeof(T) == 4 ? (const T*)v.val32 : (const T*)v.val64;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int sl = gw; sl < v.nslices; sl += nw) {
        const int row0 = __ldg(&v.slice_row0[sl]);
        const int nrow = __ldg(&v.slice_nrow[sl]);
        const int4 len = __ldg(&v.slice_len[sl]);
        const long long off = __ldg(&v.slice_off[sl]);
        const int L = len.x + len.y + len.z;
        T s = T(0);
        constexpr int CH = 8;
        // software-pipelined: the next chunk's indices and values are requested together
        // with the current chunk's gathers, so a chunk costs one memory round trip
        int c[CH]; T a[CH];
        #pragma unroll
        for (int u = 0; u < CH; u++) {
            const bool ok = u < L;
            const long long p = off + (long long)u * 32 + lane;
            c[u] = ok ? __ldcs(&v.ci[p]) : 0;
            a[u] = ok ? __ldcs(&val[p]) : T(0);
        }
        for (int k0 = 0; k0 < L; k0 += CH) {
            T xv[CH];
            #pragma unroll
            for (int u = 0; u < CH; u++) xv[u] = __ldg(&x[c[u]]);
            int cn[CH]; T an[CH];
            #pragma unroll
            for (int u = 0; u < CH; u++) {
                const bool ok = k0 + CH + u < L;
                const long long p = off + (long long)(k0 + CH + u) * 32 + lane;
                cn[u] = ok ? __ldcs(&v.ci[p]) : 0;
                an[u] = ok ? __ldcs(&val[p]) : T(0);
            }
            #pragma unroll
            for (int u = 0; u < CH; u++) s = fma(a[u], xv[u], s);
            #pragma unroll
            for (int u = 0; u < CH; u++) { c[u] = cn[u]; a[u] = an[u]; }
        }
        // FP64 issues at 2 lanes/clk/SM on this part: skip the multiply when scaling == 1
        if (lane < nrow) y[row0 + lane] = scaling == T(1) ? s : scaling * s;
    }
}

// ---- exclusive scan of int32 (three-phase, 4096 elements per block) ----
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
    __shared__ int s_warp[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
    #pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < (blockDim.x >> 5) ? s_warp[lane] : 0;
        #pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    const int warp_prefix = warp > 0 ? s_warp[warp - 1] : 0;
    if (total) *total = s_warp[(blockDim.x >> 5) - 1];
    const int res = warp_prefix + x - v;
    __syncthreads();
    return res;
}

__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(int n, const int* __restrict__ in, int* __restrict__ out,
                                                                 int* __restrict__ tile_sums) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int local = 0;
    #pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        local += v[k];
    }
    int total = 0;
    int pre = block_exclusive_scan(local, &total);
    #pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) out[base + k] = pre;
        pre += v[k];
    }
    if (threadIdx.x == 0 && tile_sums) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) scan_add_kernel(int n, int* __restrict__ out, const int* __restrict__ tile_prefix) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    const int add = tile_prefix[blockIdx.x];
    #pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) out[base + k] += add;
}

inline int grid_for(long long n, int block) { return (int)((n + block - 1) / block); }

template <typename K, typename... Args>
cudaError_t launch(K kernel, int grid, int block, cudaStream_t s, Args... args) {
    if (grid <= 0) return cudaSuccess;
    note_launch();
    kernel<<<grid, block, 0, s>>>(args...);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_spmv_f64(int n, const int* rp, const int* ci, const double* v, const double* x, double* y,
                            double scaling, int lanes, cudaStream_t s) {
    const int grid = grid_for((long long)n * lanes, kBlock);
    switch (lanes) {
        case 1: return launch(spmv_f64_kernel<1>, grid, kBlock, s, n, rp, ci, v, x, y, scaling);
        case 2: return launch(spmv_f64_kernel<2>, grid, kBlock, s, n, rp, ci, v, x, y, scaling);
        case 4: return launch(spmv_f64_kernel<4>, grid, kBlock, s, n, rp, ci, v, x, y, scaling);
        case 8: return launch(spmv_f64_kernel<8>, grid, kBlock, s, n, rp, ci, v, x, y, scaling);
        case 16: return launch(spmv_f64_kernel<16>, grid, kBlock, s, n, rp, ci, v, x, y, scaling);
        default: return launch(spmv_f64_kernel<32>, grid_for((long long)n * 32, kBlock), kBlock, s, n, rp, ci, v, x, y, scaling);
    }
}

cudaError_t launch_residual_f64(int n, const int* rp, const int* ci, const double* v, const double* b, const double* x,
                                double* r, double* partial_sq, int lanes, cudaStream_t s) {
    const int grid = grid_for((long long)n * lanes, kBlock);
    switch (lanes) {
        case 1: return launch(residual_f64_kernel<1>, grid, kBlock, s, n, rp, ci, v, b, x, r, partial_sq);
        case 2: return launch(residual_f64_kernel<2>, grid, kBlock, s, n, rp, ci, v, b, x, r, partial_sq);
        case 4: return launch(residual_f64_kernel<4>, grid, kBlock, s, n, rp, ci, v, b, x, r, partial_sq);
        case 8: return launch(residual_f64_kernel<8>, grid, kBlock, s, n, rp, ci, v, b, x, r, partial_sq);
        case 16: return launch(residual_f64_kernel<16>, grid, kBlock, s, n, rp, ci, v, b, x, r, partial_sq);
        default: return launch(residual_f64_kernel<32>, grid_for((long long)n * 32, kBlock), kBlock, s, n, rp, ci, v, b, x, r, partial_sq);
    }
}

int residual_blocks(int n, int lanes) { return grid_for((long long)n * lanes, kBlock); }

cudaError_t launch_sum_sq_f64(int n, const double* v, double* out, cudaStream_t s) {
    return launch(sum_kernel, 1, 1024, s, n, v, out, 1);
}

cudaError_t launch_sum_f64(int n, const double* v, double* out, cudaStream_t s) {
    return launch(sum_kernel, 1, 1024, s, n, v, out, 0);
}

cudaError_t launch_diagonal_f64(int n, const int* A, const int* C, const double* V, double* d, cudaStream_t s) {
    return launch(diagonal_kernel, grid_for(n, kBlock), kBlock, s, n, A, C, V, d);
}

cudaError_t launch_validate_csr_cols(int n, int ncols, int nnz, const int* A, const int* C, int* bad, cudaStream_t s) {
    long long work = (long long)n > (long long)nnz ? n : nnz;
    int grid = grid_for(work, kBlock);
    if (grid > 8192) grid = 8192;
    if (grid < 1) grid = 1;
    return launch(validate_csr_kernel, grid, kBlock, s, n, ncols, nnz, A, C, bad);
}

cudaError_t launch_validate_csr(int n, int nnz, const int* A, const int* C, int* bad, cudaStream_t s) {
    return launch_validate_csr_cols(n, n, nnz, A, C, bad, s);
}

cudaError_t launch_row_lengths(int n, const int* A, const int* perm, int* len, cudaStream_t s) {
    return launch(row_lengths_kernel, grid_for(n, kBlock), kBlock, s, n, A, perm, len);
}

cudaError_t launch_inverse_perm(int n, const int* perm, int* iperm, cudaStream_t s) {
    return launch(inverse_perm_kernel, grid_for(n, kBlock), kBlock, s, n, perm, iperm);
}

cudaError_t launch_permute_split(int n, const int* A, const int* C, const double* V, const int* perm, const int* iperm,
                                 const int* key, const int* new_rp, int* out_ci, double* out_v, float* out_v32,
                                 int* lsplit, int* usplit, cudaStream_t s) {
    return launch(permute_split_kernel, grid_for(n, 128), 128, s, n, A, C, V, perm, iperm, key, new_rp, out_ci, out_v,
                  out_v32, lsplit, usplit);
}

cudaError_t launch_gather_f64(int n, const int* perm, const double* src, double* dst, cudaStream_t s) {
    return launch(gather_f64_kernel, grid_for(n, kBlock), kBlock, s, n, perm, src, dst);
}

cudaError_t launch_scatter_f64(int n, const int* perm, const double* src, double* dst, cudaStream_t s) {
    return launch(scatter_f64_kernel, grid_for(n, kBlock), kBlock, s, n, perm, src, dst);
}

cudaError_t launch_gather_to_f32(int n, const int* perm, const double* src, float* dst, cudaStream_t s) {
    return launch(gather_to_f32_kernel, grid_for(n, kBlock), kBlock, s, n, perm, src, dst);
}

cudaError_t launch_cast_f64_f32(size_t n, const double* src, float* dst, cudaStream_t s) {
    int grid = (int)((n + kBlock - 1) / kBlock);
    if (grid > 4096) grid = 4096;
    return launch(cast_kernel, grid, kBlock, s, n, src, dst);
}

cudaError_t launch_sweep_factors(int n, const double* diag, double omega, double* wd, double* sd, float* wd32,
                                 float* sd32, cudaStream_t s) {
    return launch(sweep_factors_kernel, grid_for(n, kBlock), kBlock, s, n, diag, omega, wd, sd, wd32, sd32);
}

cudaError_t launch_scaled_cast(int n, const double* r, const double* inv_norm_dev, float* r32, cudaStream_t s) {
    return launch(scaled_cast_kernel, grid_for(n, kBlock), kBlock, s, n, r, inv_norm_dev, r32);
}

int update_norm_blocks(int n) {
    const int g = grid_for(n, kBlock);
    return g < 1024 ? (g < 1 ? 1 : g) : 1024;
}

cudaError_t launch_update_x_norms(int n, const float* c32, const double* norm_dev, double* x, double* partials,
                                  double* out2, cudaStream_t s) {
    const int g = update_norm_blocks(n);
    cudaError_t e = launch(update_x_norms_kernel, g, kBlock, s, n, c32, norm_dev, x, partials);
    if (e == cudaSuccess) e = launch(sum_kernel, 1, 1024, s, g, partials, out2, 0);
    if (e == cudaSuccess) e = launch(sum_kernel, 1, 1024, s, g, partials + g, out2 + 1, 0);
    return e;
}

cudaError_t launch_update_x(int n, const int* perm, const float* c32, const double* norm_dev, double* x, cudaStream_t s) {
    return launch(update_x_kernel, grid_for(n, kBlock), kBlock, s, n, perm, c32, norm_dev, x);
}

cudaError_t launch_sell_spmv(const SellView& v, int is_float, const void* x, void* y, double scaling, cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = grid_for((long long)v.nslices * 32, 256);
    if (grid > sms * 8) grid = sms * 8;
    if (is_float)
        return launch(sell_spmv_kernel<float>, grid, 256, s, v, (const float*)x, (float*)y, (float)scaling);
    return launch(sell_spmv_kernel<double>, grid, 256, s, v, (const double*)x, (double*)y, scaling);
}

cudaError_t launch_sell_lengths(int nslices, const int* slice_row0, const int* slice_nrow, const int* rp,
                                const int* lsplit, const int* usplit, int4* slice_len, cudaStream_t s) {
    return launch(sell_lengths_kernel, grid_for((long long)nslices * 32, kBlock), kBlock, s, nslices, slice_row0,
                  slice_nrow, rp, lsplit, usplit, slice_len);
}

cudaError_t launch_sell_fill(int nslices, const int* slice_row0, const int* slice_nrow, const int4* slice_len,
                             const long long* slice_off, const int* rp, const int* lsplit, const int* usplit,
                             const int* ci_in, const double* val_in, int* ci, float* val32, double* val64,
                             cudaStream_t s) {
    return launch(sell_fill_kernel, grid_for((long long)nslices * 32, kBlock), kBlock, s, nslices, slice_row0,
                  slice_nrow, slice_len, slice_off, rp, lsplit, usplit, ci_in, val_in, ci, val32, val64);
}

size_t scan_scratch_ints(int n) {
    const long long tiles = ((long long)n + kScanTile - 1) / kScanTile;
    if (tiles <= 1) return 1;
    return (size_t)(2 * tiles) + scan_scratch_ints((int)tiles);
}

// Exclusive scan of n ints; out may alias nothing in `in`. scratch holds scan_scratch_ints(n) ints.
cudaError_t launch_exclusive_scan(int n, const int* in, int* out, int* scratch, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int tiles = grid_for(n, kScanTile);
    cudaError_t e = launch(scan_tiles_kernel, tiles, kScanThreads, s, n, in, out, tiles > 1 ? scratch : (int*)nullptr);
    if (e != cudaSuccess || tiles == 1) return e;
    int* sums = scratch;
    int* prefix = scratch + tiles;
    e = launch_exclusive_scan(tiles, sums, prefix, scratch + 2 * (size_t)tiles, s);
    if (e != cudaSuccess) return e;
    return launch(scan_add_kernel, tiles, kScanThreads, s, n, out, (const int*)prefix);
}

}  // namespace feec

// CSR algebra on the device — the step before the solver path in FEEC++ (assembly of
// stiffness and mass matrices as products and sums of FEEC operators):
//
//   feec_csr_add        MatrixCSRAddition            (sparse/matcsr.cpp:707-765)
//   feec_csr_multiply   MatrixCSRMultiplication      (sparse/matcsr.cpp:767-849)
//   feec_csr_transpose  MatrixCSR::getTranspose      (sparse/matcsr.cpp:291-350)
//   feec_coo_to_csr     MatrixCSR(const SparseMatrix&) (sparse/matcsr.cpp:43-89,
//                       with SparseMatrix::sortandcompressentries, sparsematrix.cpp:405-458)
//
// The reference builds every result by laying the entries of each row out in a fixed
// order and then compressing rows with sort_and_compress_csrdata_reduced
// (sparse/matcsr.cpp:585-688): an exchange sort that merges equal columns into the
// first (zeroing the later one), then the nonzeros kept in order. Which entries meet in
// which order decides the rounding of merged sums, so the device lays entries out in
// the same order and runs the same per-row exchange sort (one warp per row, its passes
// pipelined across the lanes); its results are bit-identical to the reference's. (The reference's final zero bubble pass
// is a stable partition of nonzeros before zeros; the device does that partition
// directly.) The expansions, counts and prefix sums around it are parallel.
//
// COO -> CSR: the reference sorts entries with std::sort, which leaves entries of equal
// (row, column) in an unspecified order; here equal positions are summed in input
// order (an ordering the device makes deterministic), so sums of duplicates may differ
// from the reference's in rounding while the structure is identical.
//
// Entry points take host pointers, like feec_csr_apply; inputs are checked on the host
// (row pointers monotone from 0, columns in range) before any kernel indexes through them.
#include <algorithm>
#include <climits>
#include <vector>

#include "feec_device.cuh"
#include "feec_internal.h"
#include "feec_system.h"

namespace feec {
namespace {

constexpr int kAlgBlock = 256;

int grid_of(long long n) { return (int)std::max<long long>(1, (n + kAlgBlock - 1) / kAlgBlock); }

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarpsPerBlock = 4;
constexpr int kWarpBlock = kWarpsPerBlock * 32;
constexpr int kRowCap = 1024;   // (column, slot) entries of one row staged in shared memory per warp (8 KB)

int warp_grid(long long rows) { return (int)std::max<long long>(1, (rows + kWarpsPerBlock - 1) / kWarpsPerBlock); }

// The sort carries, for each entry, its column and a slot: the position of its value in a
// value array that stays in place. Bit 31 of the slot marks a value known to be zero
// (initially zero, or emptied by a merge). A merge with a zero operand moves slots
// instead of values (x + 0 and 0 + x are x, up to the sign of a zero sum, and zeros are
// dropped afterwards), so the pipeline is 32-bit integer work; only a merge of two
// nonzeros adds, out of line and in the value array. A sum that cancels to zero keeps its
// slot unflagged: adding into it later gives exactly the other operand, as the serial
// sort does.
constexpr int kZeroSlot = (int)0x80000000u;

// v[r] += v[x] where `add` is set. Kept out of line: compiled inline, the add is
// if-converted and then occupies the FP64 pipe on every step of the sort.
__device__ __noinline__ void slot_add(bool add, double* v, int r, int x) {
    if (add) v[r] = v[r] + v[x];
}

// The reference's per-row exchange sort (sparse/matcsr.cpp:601-622) on the entries
// cs[0, L) = (column, slot), values v[slot], run by one warp as a systolic pipeline. Pass p
// of the reference keeps a running minimum (column, value) in a register, scans positions
// p+1.., merges equal columns into it (zeroing the merged entry) and swaps smaller ones in;
// at its end the register is stored at position p. Lane k runs pass i+k of a sweep of 32
// passes, one step behind lane k-1: it receives each entry after lane k-1 has processed it
// and hands it on. Every pass therefore sees every position in exactly the state the serial
// sort gives it, and every sum is formed in the serial order, at about L*L/64 warp steps
// instead of L*L/2 serial ones. The stream enters at lane 0 (a broadcast load one entry
// ahead) and leaves at lane 31; columns are >= 0, -1 marks no entry.
__device__ void warp_exchange_sort(int2* cs, double* v, int L, int lane) {
    for (int i = 0; i < L; i += 32) {
        int rc = 0, rs = 0;                   // register of pass i + lane
        int pc = -1, ps = 0;                  // entry this lane hands on (-1: none)
        int2 nx = cs[i];                      // next entry of the stream (all lanes)
        const int steps = (L - i) + 31;
        for (int s = 0; s < steps; s++) {
            int xc = __shfl_up_sync(kFull, pc, 1);
            int xs = __shfl_up_sync(kFull, ps, 1);
            if (lane == 0) { xc = nx.x; xs = nx.y; }
            const int q1 = i + s + 1;
            if (q1 < L) nx = cs[q1]; else nx.x = -1;
            const bool valid = xc >= 0;
            const bool reg = valid && s == 2 * lane;          // position i + lane: the register
            const bool proc = valid && !reg;
            const bool eq = proc && xc == rc;
            const bool lt = proc && xc < rc;
            const bool rz = rs < 0, xz = xs < 0;
            const bool add = eq && !rz && !xz;
            if (__any_sync(kFull, add)) slot_add(add, v, rs, xs);   // rare: a real call
            if (eq) {
                if (rz) { const int t = rs; rs = xs; xs = t; }  // the register takes the value
                else if (!xz) xs |= kZeroSlot;                  // the merged entry is now zero
            }
            const int oc = lt ? rc : xc;
            const int os = lt ? rs : xs;
            if (lt || reg) { rc = xc; rs = xs; }
            pc = proc ? oc : -1;
            ps = os;
            if (lane == 31) {
                if (pc >= 0) cs[i + s - 31] = make_int2(pc, ps);
                pc = -1;
            }
        }
        if (i + lane < L) cs[i + lane] = make_int2(rc, rs);
        __syncwarp();
    }
}

// The nonzero entries of the sorted row, in order, written to (dc, dv); returns their
// count. This is the reference's zero bubble pass (:624-649), a stable partition.
__device__ int warp_keep_nonzeros(const int2* cs, const double* v, int L, int* __restrict__ dc,
                                  double* __restrict__ dv, int lane) {
    int k = 0;
    for (int base = 0; base < L; base += 32) {
        const int q = base + lane;
        int2 e = make_int2(0, kZeroSlot);
        if (q < L) e = cs[q];
        double val = 0.0;
        if (e.y >= 0) val = v[e.y];
        const bool keep = e.y >= 0 && ((__double_as_longlong(val) << 1) != 0);
        const unsigned m = __ballot_sync(kFull, keep);
        if (keep) { const int d = k + __popc(m & ((1u << lane) - 1u)); dc[d] = e.x; dv[d] = val; }
        k += __popc(m);
    }
    return k;
}

// One warp per row: the row's entries get slots (zero values flagged), are sorted and
// merged (the (column, slot) stream in shared memory when the row fits, else in the global
// scratch `cs`; the values stay in V, where only merges of two nonzeros and the final pass
// touch them), and the nonzeros are written to (Co, Vo) from the row's start; cnt[r] =
// their count.
__global__ void __launch_bounds__(kWarpBlock)
compress_rows_kernel(int rows, const int* __restrict__ A, const int* __restrict__ C, double* V, int2* cs,
                     int* __restrict__ Co, double* __restrict__ Vo, int* __restrict__ cnt) {
    __shared__ int2 scs[kWarpsPerBlock][kRowCap];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int r = blockIdx.x * kWarpsPerBlock + w;
    if (r >= rows) return;
    const int lo = A[r], L = A[r + 1] - lo;
    int2* rcs = L <= kRowCap ? scs[w] : cs + lo;
    double* rv = V + lo;
    for (int q = lane; q < L; q += 32) {
        const int zero = ((__double_as_longlong(rv[q]) << 1) == 0) ? kZeroSlot : 0;
        rcs[q] = make_int2(C[lo + q], q | zero);
    }
    __syncwarp();
    warp_exchange_sort(rcs, rv, L, lane);
    const int k = warp_keep_nonzeros(rcs, rv, L, Co + lo, Vo + lo, lane);
    if (lane == 0) cnt[r] = k;
}

// Compaction, one warp per row: the first cnt[r] entries of row r move to the
// exclusive prefix offset off[r].
__global__ void compact_rows_kernel(int rows, const int* __restrict__ A, const int* __restrict__ cnt,
                                    const int* __restrict__ off, const int* __restrict__ C, const double* __restrict__ V,
                                    int* __restrict__ Co, double* __restrict__ Vo, int* __restrict__ Ao) {
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (r >= rows) return;
    const int src = A[r], dst = off[r], k = cnt[r];
    for (int t = lane; t < k; t += 32) { Co[dst + t] = C[src + t]; Vo[dst + t] = V[src + t]; }
    if (lane == 0) {
        Ao[r] = dst;
        if (r == rows - 1) Ao[rows] = dst + k;
    }
}

// s1 * row r of the first matrix, then s2 * row r of the second (:736-752), one warp per row.
__global__ void add_layout_kernel(int rows, const int* __restrict__ A1, const int* __restrict__ C1,
                                  const double* __restrict__ V1, const int* __restrict__ A2, const int* __restrict__ C2,
                                  const double* __restrict__ V2, double s1, double s2, const int* __restrict__ A,
                                  int* __restrict__ C, double* __restrict__ V) {
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (r >= rows) return;
    const int k = A[r], lo1 = A1[r], n1 = A1[r + 1] - lo1, lo2 = A2[r], n2 = A2[r + 1] - lo2;
    for (int t = lane; t < n1; t += 32) { C[k + t] = C1[lo1 + t]; V[k + t] = s1 * V1[lo1 + t]; }
    for (int t = lane; t < n2; t += 32) { C[k + n1 + t] = C2[lo2 + t]; V[k + n1 + t] = s2 * V2[lo2 + t]; }
}

__global__ void add_lengths_kernel(int rows, const int* __restrict__ A1, const int* __restrict__ A2, int* __restrict__ len) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < rows) len[r] = (A1[r + 1] - A1[r]) + (A2[r + 1] - A2[r]);
}

__global__ void mul_lengths_kernel(int rows, const int* __restrict__ A1, const int* __restrict__ C1,
                                   const int* __restrict__ A2, long long* __restrict__ len) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    long long n = 0;
    for (int c1 = A1[r]; c1 < A1[r + 1]; c1++) n += A2[C1[c1] + 1] - A2[C1[c1]];
    len[r] = n;
}

// Products of row r in the reference's order (:819-832), one warp per row: the row of
// the second matrix that each entry of row r selects is copied scaled, lanes in parallel.
__global__ void mul_layout_kernel(int rows, const int* __restrict__ A1, const int* __restrict__ C1,
                                  const double* __restrict__ V1, const int* __restrict__ A2, const int* __restrict__ C2,
                                  const double* __restrict__ V2, const int* __restrict__ A, int* __restrict__ C,
                                  double* __restrict__ V) {
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (r >= rows) return;
    int k = A[r];
    for (int c1 = A1[r]; c1 < A1[r + 1]; c1++) {
        const int m = C1[c1];
        const double v1 = V1[c1];
        const int lo2 = A2[m], n2 = A2[m + 1] - lo2;
        for (int t = lane; t < n2; t += 32) { C[k + t] = C2[lo2 + t]; V[k + t] = v1 * V2[lo2 + t]; }
        k += n2;
    }
}

__global__ void count_keys_kernel(long long n, const int* __restrict__ key, const unsigned char* __restrict__ keep,
                                  int* __restrict__ cnt) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n && (!keep || keep[i])) atomicAdd(&cnt[key[i]], 1);
}

// Scatter of entry indices into buckets (order inside a bucket is arbitrary; the bucket
// is sorted by entry index afterwards, which makes the result deterministic).
__global__ void bucket_kernel(long long n, const int* __restrict__ key, const unsigned char* __restrict__ keep,
                              const int* __restrict__ start, int* __restrict__ fill, long long* __restrict__ idx) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n || (keep && !keep[i])) return;
    const int b = key[i];
    const int pos = atomicAdd(&fill[b], 1);
    idx[start[b] + pos] = i;
}

// Sort the entry indices of each bucket: ascending (COO rows: input order), or descending
// (transpose columns: the reference fills a column from its end in row order, :319-338).
__global__ void sort_bucket_kernel(int nb, const int* __restrict__ start, long long* idx, int descending) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int lo = start[b], hi = start[b + 1];
    for (int i = lo + 1; i < hi; i++) {
        const long long v = idx[i];
        int j = i - 1;
        while (j >= lo && (descending ? idx[j] < v : idx[j] > v)) { idx[j + 1] = idx[j]; j--; }
        idx[j + 1] = v;
    }
}

// Transpose, one warp per column: entry i of the CSR (row row_of[i]) goes to its
// column's bucket position.
__global__ void transpose_fill_kernel(int ncols, const int* __restrict__ B, const long long* __restrict__ idx,
                                      const int* __restrict__ row_of, const double* __restrict__ V, int* __restrict__ D,
                                      double* __restrict__ W) {
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (c >= ncols) return;
    for (int k = B[c] + lane; k < B[c + 1]; k += 32) { const long long i = idx[k]; D[k] = row_of[i]; W[k] = V[i]; }
}

__global__ void row_of_kernel(int rows, const int* __restrict__ A, int* __restrict__ row_of) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    for (int i = A[r]; i < A[r + 1]; i++) row_of[i] = r;
}

__global__ void nonzero_kernel(long long n, const double* __restrict__ v, unsigned char* __restrict__ keep) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) keep[i] = v[i] != 0.0;
}

// COO row: entries (in input order) sorted by column (stable), equal columns summed in
// that order (sparsematrix.cpp:430-452), written to C/V from the bucket start.
__global__ void coo_row_kernel(int rows, const int* __restrict__ start, long long* idx, const int* __restrict__ col,
                               const double* __restrict__ val, int* __restrict__ C, double* __restrict__ V,
                               int* __restrict__ cnt) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const int lo = start[r], hi = start[r + 1];
    for (int i = lo + 1; i < hi; i++) {           // stable insertion sort by column
        const long long v = idx[i];
        const int cv = col[v];
        int j = i - 1;
        while (j >= lo && col[idx[j]] > cv) { idx[j + 1] = idx[j]; j--; }
        idx[j + 1] = v;
    }
    int k = lo;
    for (int i = lo; i < hi; i++) {
        const long long e = idx[i];
        if (k > lo && C[k - 1] == col[e]) V[k - 1] += val[e];
        else { C[k] = col[e]; V[k] = val[e]; k++; }
    }
    cnt[r] = k - lo;
}

__global__ void ll_to_int_kernel(int n, const long long* __restrict__ in, int* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (int)in[i];
}

// ---- SparseMatrixMultiplication (sparse/sparsematrix.cpp:609-722) ----------------------
// Per left row i, the products L(i,k) R(k,j) for k ascending (the left CSR row is sorted
// by k) are accumulated into a hash table keyed by j: within one k the columns j are
// distinct, so the lanes of a warp add one right row in parallel without meeting, and
// every entry receives its products in k order, the order in which the reference's
// stable emission (k, then i, then j) lists them. Zero products are skipped (the
// reference drops them before merging); the first product of an entry is stored, the
// later ones added, as the reference's compression does.

constexpr int kHashWarps = 2;
constexpr int kHashSlots = 2048;                 // shared table per warp: 24 KB
constexpr int kHashMaxKeys = kHashSlots * 3 / 4;

__device__ __forceinline__ unsigned col_hash(int j) { return (unsigned)j * 2654435761u; }

__device__ __forceinline__ int next_pow2_at_least(long long x, int lo) {
    int h = lo;
    while (h < x && h < (1 << 30)) h <<= 1;
    return h;
}

// Accumulates row i into (keys, vals)[0, H) (keys preset to -1). Returns the number of
// distinct columns, or -1 once more than max_keys would be held (the caller retries the
// row with a larger table).
__device__ int product_row_accumulate(int i, const int* __restrict__ LA, const int* __restrict__ LC,
                                      const double* __restrict__ LV, const int* __restrict__ RA,
                                      const int* __restrict__ RC, const double* __restrict__ RV, int* keys,
                                      double* vals, int H, int max_keys, int lane) {
    int distinct = 0;
    for (int a = LA[i]; a < LA[i + 1]; a++) {
        const int k = LC[a];
        const double lv = LV[a];
        const int lo = RA[k], len = RA[k + 1] - lo;
        for (int base = 0; base < len; base += 32) {
            const int t = base + lane;
            bool created = false, placed = true;
            if (t < len) {
                const int j = RC[lo + t];
                const double prod = lv * RV[lo + t];
                if (prod != 0.0) {
                    unsigned h = col_hash(j) & (unsigned)(H - 1);
                    placed = false;
                    for (int probe = 0; probe < H; probe++) {
                        const int cur = *((volatile int*)&keys[h]);
                        if (cur == j) { placed = true; break; }
                        if (cur == -1) {
                            const int prev = atomicCAS(&keys[h], -1, j);
                            if (prev == -1) { created = true; placed = true; break; }
                            if (prev == j) { placed = true; break; }
                        }
                        h = (h + 1) & (unsigned)(H - 1);
                    }
                    if (created) vals[h] = prod;
                    else if (placed) vals[h] = vals[h] + prod;
                }
            }
            distinct += __popc(__ballot_sync(kFull, created));
            const bool lost = __any_sync(kFull, !placed);
            __syncwarp();
            if (lost || distinct > max_keys) return -1;
        }
    }
    return distinct;
}

// The table's d entries moved to its front (in place), then written to (oc, ov) sorted
// by column (rank = number of smaller columns).
__device__ void table_to_sorted_row(int* keys, double* vals, int H, int* __restrict__ oc, double* __restrict__ ov,
                                    int lane) {
    int d = 0;
    for (int base = 0; base < H; base += 32) {
        const int key = keys[base + lane];
        const double val = vals[base + lane];
        const bool occ = key >= 0;
        const unsigned m = __ballot_sync(kFull, occ);
        __syncwarp();
        if (occ) { const int at = d + __popc(m & ((1u << lane) - 1u)); keys[at] = key; vals[at] = val; }
        d += __popc(m);
        __syncwarp();
    }
    for (int base = 0; base < d; base += 32) {
        const int e = base + lane;
        const int ke = e < d ? keys[e] : 0;
        int rank = 0;
        for (int f = 0; f < d; f++) rank += keys[f] < ke;
        if (e < d) { oc[rank] = ke; ov[rank] = vals[e]; }
    }
    __syncwarp();
}

// E[i] = min(products of row i, columns): room for row i's distinct columns.
__global__ void product_room_kernel(int rows, int cols, const long long* __restrict__ P, int* __restrict__ E,
                                    unsigned long long* __restrict__ total) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    const int e = (int)(P[i] < cols ? P[i] : cols);
    E[i] = e;
    atomicAdd(total, (unsigned long long)e);
}

// One warp per left row, table in shared memory; rows that overflow it are flagged.
__global__ void __launch_bounds__(kHashWarps * 32)
coo_product_rows_kernel(int rows, const int* __restrict__ LA, const int* __restrict__ LC, const double* __restrict__ LV,
                        const int* __restrict__ RA, const int* __restrict__ RC, const double* __restrict__ RV,
                        const int* __restrict__ E, const int* __restrict__ SD, int* __restrict__ RCo,
                        double* __restrict__ RVo, int* __restrict__ cnt, int* __restrict__ big) {
    __shared__ int skeys[kHashWarps][kHashSlots];
    __shared__ double svals[kHashWarps][kHashSlots];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i = blockIdx.x * kHashWarps + w;
    if (i >= rows) return;
    const int H = next_pow2_at_least(2LL * E[i], 32) < kHashSlots ? next_pow2_at_least(2LL * E[i], 32) : kHashSlots;
    for (int q = lane; q < H; q += 32) skeys[w][q] = -1;
    __syncwarp();
    const int d = product_row_accumulate(i, LA, LC, LV, RA, RC, RV, skeys[w], svals[w], H,
                                         H == kHashSlots ? kHashMaxKeys : H, lane);
    if (d < 0) {
        if (lane == 0) { big[i] = 1; cnt[i] = 0; }
        return;
    }
    table_to_sorted_row(skeys[w], svals[w], H, RCo + SD[i], RVo + SD[i], lane);
    if (lane == 0) { big[i] = 0; cnt[i] = d; }
}

// Table sizes in global memory for the flagged rows (0 for the others).
__global__ void big_table_size_kernel(int rows, const int* __restrict__ E, const int* __restrict__ big,
                                      int* __restrict__ G, unsigned long long* __restrict__ total) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    const int g = big[i] ? next_pow2_at_least(2LL * E[i], 32) : 0;
    G[i] = g;
    if (g) atomicAdd(total, (unsigned long long)g);
}

// The flagged rows again, each with a global table of at least twice its room.
__global__ void coo_product_big_rows_kernel(int rows, const int* __restrict__ LA, const int* __restrict__ LC,
                                            const double* __restrict__ LV, const int* __restrict__ RA,
                                            const int* __restrict__ RC, const double* __restrict__ RV,
                                            const int* __restrict__ big, const int* __restrict__ GO,
                                            int* __restrict__ gkeys, double* __restrict__ gvals,
                                            const int* __restrict__ SD, int* __restrict__ RCo,
                                            double* __restrict__ RVo, int* __restrict__ cnt, int* __restrict__ err) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (i >= rows || !big[i]) return;
    const int H = GO[i + 1] - GO[i];
    int* keys = gkeys + GO[i];
    double* vals = gvals + GO[i];
    for (int q = lane; q < H; q += 32) keys[q] = -1;
    __syncwarp();
    const int d = product_row_accumulate(i, LA, LC, LV, RA, RC, RV, keys, vals, H, H, lane);
    if (d < 0) {                     // cannot happen: H >= 2 * (room of the row)
        if (lane == 0) { atomicExch(err, 1); cnt[i] = 0; }
        return;
    }
    table_to_sorted_row(keys, vals, H, RCo + SD[i], RVo + SD[i], lane);
    if (lane == 0) cnt[i] = d;
}

// Host-side checks of a CSR given by host pointers.
bool csr_ok(int rows, int cols, const int* A, const int* C) {
    if (rows < 0 || cols < 0 || !A || A[0] != 0) return false;
    for (int r = 0; r < rows; r++) if (A[r + 1] < A[r]) return false;
    const int nnz = A[rows];
    if (nnz > 0 && !C) return false;
    for (int i = 0; i < nnz; i++) if (C[i] < 0 || C[i] >= cols) return false;
    return true;
}

// Compress the rows laid out at (dA, dC, dV), compact them into (oA, oC, oV) on the device.
int compress_and_compact(DevArena& m, cudaStream_t s, int rows, int* dA, int* dC, double* dV, int*& oA, int*& oC,
                         double*& oV, int& nnz_out) {
    int *cnt = nullptr, *off = nullptr, *scr = nullptr, *Co = nullptr, total = 0;
    int2* cs = nullptr;
    double* Vo = nullptr;
    FEEC_TRY(cudaMemcpyAsync(&total, dA + rows, sizeof(int), cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaStreamSynchronize(s));
    FEEC_TRY(m.alloc(cnt, (size_t)rows + 1)); FEEC_TRY(m.alloc(off, (size_t)rows + 1));
    FEEC_TRY(m.alloc(scr, scan_scratch_ints(rows + 1)));
    FEEC_TRY(m.alloc(cs, (size_t)std::max(total, 1))); FEEC_TRY(m.alloc(Co, (size_t)std::max(total, 1)));
    FEEC_TRY(m.alloc(Vo, (size_t)std::max(total, 1)));
    FEEC_TRY(cudaMemsetAsync(cnt + rows, 0, sizeof(int), s));
    note_launch();
    compress_rows_kernel<<<warp_grid(rows), kWarpBlock, 0, s>>>(rows, dA, dC, dV, cs, Co, Vo, cnt);
    FEEC_TRY(cudaGetLastError());
    FEEC_TRY(launch_exclusive_scan(rows + 1, cnt, off, scr, s));
    FEEC_TRY(cudaMemcpyAsync(&nnz_out, off + rows, sizeof(int), cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaStreamSynchronize(s));
    FEEC_TRY(m.alloc(oA, (size_t)rows + 1)); FEEC_TRY(m.alloc(oC, (size_t)std::max(nnz_out, 1)));
    FEEC_TRY(m.alloc(oV, (size_t)std::max(nnz_out, 1)));
    if (rows == 0) FEEC_TRY(cudaMemsetAsync(oA, 0, sizeof(int), s));
    note_launch();
    compact_rows_kernel<<<warp_grid(rows), kWarpBlock, 0, s>>>(rows, dA, cnt, off, Co, Vo, oC, oV, oA);
    FEEC_TRY(cudaGetLastError());
    return FEEC_OK;
}

int download(cudaStream_t s, int rows, int nnz, const int* oA, const int* oC, const double* oV, int* A, int* C,
             double* V) {
    FEEC_TRY(cudaMemcpyAsync(A, oA, sizeof(int) * ((size_t)rows + 1), cudaMemcpyDeviceToHost, s));
    if (nnz > 0) {
        FEEC_TRY(cudaMemcpyAsync(C, oC, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToHost, s));
        FEEC_TRY(cudaMemcpyAsync(V, oV, sizeof(double) * (size_t)nnz, cudaMemcpyDeviceToHost, s));
    }
    FEEC_TRY(cudaStreamSynchronize(s));
    return FEEC_OK;
}

template <typename T>
int upload(DevArena& m, cudaStream_t s, T*& d, const T* h, size_t n) {
    FEEC_TRY(m.alloc(d, std::max<size_t>(n, 1)));
    if (n) FEEC_TRY(cudaMemcpyAsync(d, h, sizeof(T) * n, cudaMemcpyHostToDevice, s));
    return FEEC_OK;
}

// COO entries on the device (indices already checked) to a row-sorted CSR with equal
// positions summed in input order and zero values dropped first.
int coo_to_csr_dev(DevArena& m, cudaStream_t s, int rows, long long count, const int* dr, const int* dc,
                   const double* dv, int*& oA, int*& oC, double*& oV, int& n) {
    unsigned char* keep; int *cnt, *start, *fill, *scr, *dC, *rc; long long* idx; double* dV;
    FEEC_TRY(m.alloc(keep, (size_t)std::max<long long>(count, 1)));
    FEEC_TRY(m.alloc(cnt, (size_t)rows + 1)); FEEC_TRY(m.alloc(start, (size_t)rows + 1));
    FEEC_TRY(m.alloc(fill, (size_t)rows + 1)); FEEC_TRY(m.alloc(scr, scan_scratch_ints(rows + 1)));
    FEEC_TRY(m.alloc(idx, (size_t)std::max<long long>(count, 1)));
    FEEC_TRY(m.alloc(dC, (size_t)std::max<long long>(count, 1))); FEEC_TRY(m.alloc(dV, (size_t)std::max<long long>(count, 1)));
    FEEC_TRY(m.alloc(rc, (size_t)rows + 1));
    FEEC_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * ((size_t)rows + 1), s));
    FEEC_TRY(cudaMemsetAsync(fill, 0, sizeof(int) * ((size_t)rows + 1), s));
    FEEC_TRY(cudaMemsetAsync(rc, 0, sizeof(int) * ((size_t)rows + 1), s));
    note_launch();
    nonzero_kernel<<<grid_of(count), kAlgBlock, 0, s>>>(count, dv, keep);          // zeros dropped (:411-420)
    note_launch();
    count_keys_kernel<<<grid_of(count), kAlgBlock, 0, s>>>(count, dr, keep, cnt);
    FEEC_TRY(cudaGetLastError());
    FEEC_TRY(launch_exclusive_scan(rows + 1, cnt, start, scr, s));
    note_launch();
    bucket_kernel<<<grid_of(count), kAlgBlock, 0, s>>>(count, dr, keep, start, fill, idx);
    note_launch();
    sort_bucket_kernel<<<grid_of(rows), kAlgBlock, 0, s>>>(rows, start, idx, 0);
    note_launch();
    coo_row_kernel<<<grid_of(rows), kAlgBlock, 0, s>>>(rows, start, idx, dc, dv, dC, dV, rc);
    FEEC_TRY(cudaGetLastError());
    // rows now hold their merged entries from start[r]; compact them
    int* off;
    FEEC_TRY(m.alloc(off, (size_t)rows + 1));
    FEEC_TRY(launch_exclusive_scan(rows + 1, rc, off, scr, s));
    FEEC_TRY(cudaMemcpyAsync(&n, off + rows, sizeof(int), cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaStreamSynchronize(s));
    FEEC_TRY(m.alloc(oA, (size_t)rows + 1)); FEEC_TRY(m.alloc(oC, (size_t)std::max(n, 1)));
    FEEC_TRY(m.alloc(oV, (size_t)std::max(n, 1)));
    if (rows == 0) FEEC_TRY(cudaMemsetAsync(oA, 0, sizeof(int), s));
    note_launch();
    compact_rows_kernel<<<warp_grid(rows), kWarpBlock, 0, s>>>(rows, start, rc, off, dC, dV, oC, oV, oA);
    FEEC_TRY(cudaGetLastError());
    return FEEC_OK;
}

struct Scope {   // device arena released and the stream drained on every return path
    DevArena m;
    cudaStream_t s;
    ~Scope() { m.release(); cudaStreamSynchronize(s); }
};

}  // namespace
}  // namespace feec

using namespace feec;

extern "C" {

int feec_csr_add(int rows, int cols, const int* A1, const int* C1, const double* V1, const int* A2, const int* C2,
                 const double* V2, double s1, double s2, int* A, int* C, double* V, int* nnz) {
    if (!csr_ok(rows, cols, A1, C1) || !csr_ok(rows, cols, A2, C2) || !A || !nnz) return FEEC_BADARG;
    const long long cap = (long long)A1[rows] + A2[rows];
    if (cap > INT_MAX || (cap > 0 && (!C || !V || (A1[rows] > 0 && !V1) || (A2[rows] > 0 && !V2)))) return FEEC_BADARG;
    int dev = 0; cudaStream_t s = nullptr;
    int st = init_device(dev, s);
    if (st != FEEC_OK) return st;
    Scope sc{DevArena{}, s}; sc.m.stream = s;
    int *dA1, *dC1, *dA2, *dC2; double *dV1, *dV2;
    if ((st = upload(sc.m, s, dA1, A1, (size_t)rows + 1)) || (st = upload(sc.m, s, dC1, C1, (size_t)A1[rows])) ||
        (st = upload(sc.m, s, dV1, V1, (size_t)A1[rows])) || (st = upload(sc.m, s, dA2, A2, (size_t)rows + 1)) ||
        (st = upload(sc.m, s, dC2, C2, (size_t)A2[rows])) || (st = upload(sc.m, s, dV2, V2, (size_t)A2[rows])))
        return st;
    int *len, *dA, *dC, *scr; double* dV;
    FEEC_TRY(sc.m.alloc(len, (size_t)rows + 1)); FEEC_TRY(sc.m.alloc(dA, (size_t)rows + 1));
    FEEC_TRY(sc.m.alloc(scr, scan_scratch_ints(rows + 1)));
    FEEC_TRY(sc.m.alloc(dC, (size_t)std::max<long long>(cap, 1))); FEEC_TRY(sc.m.alloc(dV, (size_t)std::max<long long>(cap, 1)));
    FEEC_TRY(cudaMemsetAsync(len + rows, 0, sizeof(int), s));
    note_launch();
    add_lengths_kernel<<<grid_of(rows), kAlgBlock, 0, s>>>(rows, dA1, dA2, len);
    FEEC_TRY(cudaGetLastError());
    FEEC_TRY(launch_exclusive_scan(rows + 1, len, dA, scr, s));
    note_launch();
    add_layout_kernel<<<warp_grid(rows), kWarpBlock, 0, s>>>(rows, dA1, dC1, dV1, dA2, dC2, dV2, s1, s2, dA, dC, dV);
    FEEC_TRY(cudaGetLastError());
    int *oA, *oC; double* oV; int n = 0;
    if ((st = compress_and_compact(sc.m, s, rows, dA, dC, dV, oA, oC, oV, n)) != FEEC_OK) return st;
    if ((st = download(s, rows, n, oA, oC, oV, A, C, V)) != FEEC_OK) return st;
    *nnz = n;
    return FEEC_OK;
}

int feec_csr_multiply_size(int rows, int inner, const int* A1, const int* C1, const int* A2, long long* size) {
    if (!csr_ok(rows, inner, A1, C1) || !A2 || !size) return FEEC_BADARG;
    for (int r = 0; r < inner; r++) if (A2[r + 1] < A2[r] || A2[0] != 0) return FEEC_BADARG;
    long long total = 0;
    for (int r = 0; r < rows; r++)
        for (int c1 = A1[r]; c1 < A1[r + 1]; c1++) total += A2[C1[c1] + 1] - A2[C1[c1]];
    *size = total;
    return FEEC_OK;
}

int feec_csr_multiply(int rows, int inner, int cols, const int* A1, const int* C1, const double* V1, const int* A2,
                      const int* C2, const double* V2, int* A, int* C, double* V, int* nnz) {
    if (!csr_ok(rows, inner, A1, C1) || !csr_ok(inner, cols, A2, C2) || !A || !nnz) return FEEC_BADARG;
    if ((A1[rows] > 0 && !V1) || (A2[inner] > 0 && !V2)) return FEEC_BADARG;
    long long cap = 0;
    int st = feec_csr_multiply_size(rows, inner, A1, C1, A2, &cap);
    if (st != FEEC_OK) return st;
    if (cap > INT_MAX || (cap > 0 && (!C || !V))) return FEEC_BADARG;
    int dev = 0; cudaStream_t s = nullptr;
    if ((st = init_device(dev, s)) != FEEC_OK) return st;
    Scope sc{DevArena{}, s}; sc.m.stream = s;
    int *dA1, *dC1, *dA2, *dC2; double *dV1, *dV2;
    if ((st = upload(sc.m, s, dA1, A1, (size_t)rows + 1)) || (st = upload(sc.m, s, dC1, C1, (size_t)A1[rows])) ||
        (st = upload(sc.m, s, dV1, V1, (size_t)A1[rows])) || (st = upload(sc.m, s, dA2, A2, (size_t)inner + 1)) ||
        (st = upload(sc.m, s, dC2, C2, (size_t)A2[inner])) || (st = upload(sc.m, s, dV2, V2, (size_t)A2[inner])))
        return st;
    long long* len64; int *len, *dA, *dC, *scr; double* dV;
    FEEC_TRY(sc.m.alloc(len64, (size_t)rows + 1)); FEEC_TRY(sc.m.alloc(len, (size_t)rows + 1));
    FEEC_TRY(sc.m.alloc(dA, (size_t)rows + 1)); FEEC_TRY(sc.m.alloc(scr, scan_scratch_ints(rows + 1)));
    FEEC_TRY(sc.m.alloc(dC, (size_t)std::max<long long>(cap, 1))); FEEC_TRY(sc.m.alloc(dV, (size_t)std::max<long long>(cap, 1)));
    FEEC_TRY(cudaMemsetAsync(len + rows, 0, sizeof(int), s));
    note_launch();
    mul_lengths_kernel<<<grid_of(rows), kAlgBlock, 0, s>>>(rows, dA1, dC1, dA2, len64);
    note_launch();
    ll_to_int_kernel<<<grid_of(rows), kAlgBlock, 0, s>>>(rows, len64, len);   // cap <= INT_MAX: every row fits
    FEEC_TRY(cudaGetLastError());
    FEEC_TRY(launch_exclusive_scan(rows + 1, len, dA, scr, s));
    note_launch();
    mul_layout_kernel<<<warp_grid(rows), kWarpBlock, 0, s>>>(rows, dA1, dC1, dV1, dA2, dC2, dV2, dA, dC, dV);
    FEEC_TRY(cudaGetLastError());
    int *oA, *oC; double* oV; int n = 0;
    if ((st = compress_and_compact(sc.m, s, rows, dA, dC, dV, oA, oC, oV, n)) != FEEC_OK) return st;
    if ((st = download(s, rows, n, oA, oC, oV, A, C, V)) != FEEC_OK) return st;
    *nnz = n;
    return FEEC_OK;
}

int feec_csr_transpose(int rows, int cols, const int* A, const int* C, const double* V, int* B, int* D, double* W,
                       int* nnz) {
    if (!csr_ok(rows, cols, A, C) || !B || !nnz) return FEEC_BADARG;
    const int m = A[rows];
    if (m > 0 && (!V || !D || !W)) return FEEC_BADARG;
    int dev = 0; cudaStream_t s = nullptr;
    int st = init_device(dev, s);
    if (st != FEEC_OK) return st;
    Scope sc{DevArena{}, s}; sc.m.stream = s;
    int *dA, *dC; double* dV;
    if ((st = upload(sc.m, s, dA, A, (size_t)rows + 1)) || (st = upload(sc.m, s, dC, C, (size_t)m)) ||
        (st = upload(sc.m, s, dV, V, (size_t)m)))
        return st;
    int *cnt, *dB, *fill, *row_of, *scr, *dD; long long* idx; double* dW;
    FEEC_TRY(sc.m.alloc(cnt, (size_t)cols + 1)); FEEC_TRY(sc.m.alloc(dB, (size_t)cols + 1));
    FEEC_TRY(sc.m.alloc(fill, (size_t)cols + 1)); FEEC_TRY(sc.m.alloc(scr, scan_scratch_ints(cols + 1)));
    FEEC_TRY(sc.m.alloc(row_of, (size_t)std::max(m, 1))); FEEC_TRY(sc.m.alloc(idx, (size_t)std::max(m, 1)));
    FEEC_TRY(sc.m.alloc(dD, (size_t)std::max(m, 1))); FEEC_TRY(sc.m.alloc(dW, (size_t)std::max(m, 1)));
    FEEC_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * ((size_t)cols + 1), s));
    FEEC_TRY(cudaMemsetAsync(fill, 0, sizeof(int) * ((size_t)cols + 1), s));
    note_launch();
    count_keys_kernel<<<grid_of(m), kAlgBlock, 0, s>>>(m, dC, nullptr, cnt);
    FEEC_TRY(cudaGetLastError());
    FEEC_TRY(launch_exclusive_scan(cols + 1, cnt, dB, scr, s));
    note_launch();
    row_of_kernel<<<grid_of(rows), kAlgBlock, 0, s>>>(rows, dA, row_of);
    note_launch();
    bucket_kernel<<<grid_of(m), kAlgBlock, 0, s>>>(m, dC, nullptr, dB, fill, idx);
    note_launch();
    sort_bucket_kernel<<<grid_of(cols), kAlgBlock, 0, s>>>(cols, dB, idx, 1);
    note_launch();
    transpose_fill_kernel<<<warp_grid(cols), kWarpBlock, 0, s>>>(cols, dB, idx, row_of, dV, dD, dW);
    FEEC_TRY(cudaGetLastError());
    int *oA, *oC; double* oV; int n = 0;
    if ((st = compress_and_compact(sc.m, s, cols, dB, dD, dW, oA, oC, oV, n)) != FEEC_OK) return st;
    if ((st = download(s, cols, n, oA, oC, oV, B, D, W)) != FEEC_OK) return st;
    *nnz = n;
    return FEEC_OK;
}

int feec_coo_to_csr(int rows, int cols, long long count, const int* r, const int* c, const double* v, int* A, int* C,
                    double* V, int* nnz) {
    if (rows < 0 || cols < 0 || count < 0 || count > INT_MAX || !A || !nnz) return FEEC_BADARG;
    if (count > 0 && (!r || !c || !v || !C || !V)) return FEEC_BADARG;
    for (long long i = 0; i < count; i++)
        if (r[i] < 0 || r[i] >= rows || c[i] < 0 || c[i] >= cols) return FEEC_BADARG;
    int dev = 0; cudaStream_t s = nullptr;
    int st = init_device(dev, s);
    if (st != FEEC_OK) return st;
    Scope sc{DevArena{}, s}; sc.m.stream = s;
    int *dr, *dc; double* dv;
    if ((st = upload(sc.m, s, dr, r, (size_t)count)) || (st = upload(sc.m, s, dc, c, (size_t)count)) ||
        (st = upload(sc.m, s, dv, v, (size_t)count)))
        return st;
    int *oA, *oC; double* oV; int n = 0;
    if ((st = coo_to_csr_dev(sc.m, s, rows, count, dr, dc, dv, oA, oC, oV, n)) != FEEC_OK) return st;
    if ((st = download(s, rows, n, oA, oC, oV, A, C, V)) != FEEC_OK) return st;
    *nnz = n;
    return FEEC_OK;
}

int feec_coo_multiply_size(int inner, long long ln, const int* lc, long long rn, const int* rr, long long* size) {
    if (inner < 0 || ln < 0 || rn < 0 || !size || (ln > 0 && !lc) || (rn > 0 && !rr)) return FEEC_BADARG;
    std::vector<long long> a((size_t)inner + 1, 0), b((size_t)inner + 1, 0);
    for (long long i = 0; i < ln; i++) { if (lc[i] < 0 || lc[i] >= inner) return FEEC_BADARG; a[lc[i]]++; }
    for (long long i = 0; i < rn; i++) { if (rr[i] < 0 || rr[i] >= inner) return FEEC_BADARG; b[rr[i]]++; }
    long long total = 0;
    for (int k = 0; k < inner; k++) total += a[k] * b[k];
    *size = total;
    return FEEC_OK;
}

int feec_coo_multiply(int lrows, int inner, int rcols, long long ln, const int* lr, const int* lc, const double* lv,
                      long long rn, const int* rr, const int* rc, const double* rv, int* out_r, int* out_c,
                      double* out_v, long long* count) {
    if (lrows < 0 || inner < 0 || rcols < 0 || ln < 0 || rn < 0 || ln > INT_MAX || rn > INT_MAX || !count)
        return FEEC_BADARG;
    if ((ln > 0 && (!lr || !lc || !lv)) || (rn > 0 && (!rr || !rc || !rv))) return FEEC_BADARG;
    for (long long i = 0; i < ln; i++)
        if (lr[i] < 0 || lr[i] >= lrows || lc[i] < 0 || lc[i] >= inner) return FEEC_BADARG;
    for (long long i = 0; i < rn; i++)
        if (rr[i] < 0 || rr[i] >= inner || rc[i] < 0 || rc[i] >= rcols) return FEEC_BADARG;
    int dev = 0; cudaStream_t s = nullptr;
    int st = init_device(dev, s);
    if (st != FEEC_OK) return st;
    Scope sc{DevArena{}, s}; sc.m.stream = s;
    int *dlr, *dlc, *drr, *drc; double *dlv, *drv;
    if ((st = upload(sc.m, s, dlr, lr, (size_t)ln)) || (st = upload(sc.m, s, dlc, lc, (size_t)ln)) ||
        (st = upload(sc.m, s, dlv, lv, (size_t)ln)) || (st = upload(sc.m, s, drr, rr, (size_t)rn)) ||
        (st = upload(sc.m, s, drc, rc, (size_t)rn)) || (st = upload(sc.m, s, drv, rv, (size_t)rn)))
        return st;
    // both operands compressed (zeros dropped, equal positions summed in input order), as CSR
    int *LA, *LC, *RA, *RC; double *LV, *RV; int lnnz = 0, rnnz = 0;
    if ((st = coo_to_csr_dev(sc.m, s, lrows, ln, dlr, dlc, dlv, LA, LC, LV, lnnz)) != FEEC_OK) return st;
    if ((st = coo_to_csr_dev(sc.m, s, inner, rn, drr, drc, drv, RA, RC, RV, rnnz)) != FEEC_OK) return st;
    // room per row and the offsets of the rows' sorted entries
    long long* P; int *E, *SD, *scr, *cnt, *big; unsigned long long* tot;
    FEEC_TRY(sc.m.alloc(P, (size_t)lrows + 1)); FEEC_TRY(sc.m.alloc(E, (size_t)lrows + 1));
    FEEC_TRY(sc.m.alloc(SD, (size_t)lrows + 1)); FEEC_TRY(sc.m.alloc(scr, scan_scratch_ints(lrows + 1)));
    FEEC_TRY(sc.m.alloc(cnt, (size_t)lrows + 1)); FEEC_TRY(sc.m.alloc(big, (size_t)lrows + 1));
    FEEC_TRY(sc.m.alloc(tot, 2));
    FEEC_TRY(cudaMemsetAsync(tot, 0, 2 * sizeof(unsigned long long), s));
    FEEC_TRY(cudaMemsetAsync(E + lrows, 0, sizeof(int), s));
    FEEC_TRY(cudaMemsetAsync(cnt + lrows, 0, sizeof(int), s));
    FEEC_TRY(cudaMemsetAsync(big + lrows, 0, sizeof(int), s));
    note_launch();
    mul_lengths_kernel<<<grid_of(lrows), kAlgBlock, 0, s>>>(lrows, LA, LC, RA, P);
    note_launch();
    product_room_kernel<<<grid_of(lrows), kAlgBlock, 0, s>>>(lrows, rcols, P, E, tot);
    FEEC_TRY(cudaGetLastError());
    unsigned long long room = 0;
    FEEC_TRY(cudaMemcpyAsync(&room, tot, sizeof(room), cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaStreamSynchronize(s));
    if (room > (unsigned long long)INT_MAX) return FEEC_BADARG;      // int offsets, as MatrixCSR's
    FEEC_TRY(launch_exclusive_scan(lrows + 1, E, SD, scr, s));
    int* RCo; double* RVo;
    FEEC_TRY(sc.m.alloc(RCo, (size_t)std::max<unsigned long long>(room, 1)));
    FEEC_TRY(sc.m.alloc(RVo, (size_t)std::max<unsigned long long>(room, 1)));
    note_launch();
    coo_product_rows_kernel<<<(int)std::max<long long>(1, (lrows + kHashWarps - 1) / kHashWarps), kHashWarps * 32, 0, s>>>(
        lrows, LA, LC, LV, RA, RC, RV, E, SD, RCo, RVo, cnt, big);
    FEEC_TRY(cudaGetLastError());
    // rows whose distinct columns overflow the shared table: again, with global tables
    int *G, *GO, *err;
    FEEC_TRY(sc.m.alloc(G, (size_t)lrows + 1)); FEEC_TRY(sc.m.alloc(GO, (size_t)lrows + 1)); FEEC_TRY(sc.m.alloc(err, 1));
    FEEC_TRY(cudaMemsetAsync(G + lrows, 0, sizeof(int), s));
    FEEC_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
    note_launch();
    big_table_size_kernel<<<grid_of(lrows), kAlgBlock, 0, s>>>(lrows, E, big, G, tot + 1);
    FEEC_TRY(cudaGetLastError());
    unsigned long long gsize = 0;
    FEEC_TRY(cudaMemcpyAsync(&gsize, tot + 1, sizeof(gsize), cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaStreamSynchronize(s));
    if (gsize > 0) {
        if (gsize > (unsigned long long)INT_MAX) return FEEC_OOM;
        FEEC_TRY(launch_exclusive_scan(lrows + 1, G, GO, scr, s));
        int* gkeys; double* gvals;
        FEEC_TRY(sc.m.alloc(gkeys, (size_t)gsize)); FEEC_TRY(sc.m.alloc(gvals, (size_t)gsize));
        note_launch();
        coo_product_big_rows_kernel<<<warp_grid(lrows), kWarpBlock, 0, s>>>(lrows, LA, LC, LV, RA, RC, RV, big, GO,
                                                                          gkeys, gvals, SD, RCo, RVo, cnt, err);
        FEEC_TRY(cudaGetLastError());
        int herr = 0;
        FEEC_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
        FEEC_TRY(cudaStreamSynchronize(s));
        if (herr) return FEEC_CUDA_ERROR;
    }
    // compaction to the final row-sorted entries, then their rows
    int *off, *oA, *oC, *orow; double* oV; int n = 0;
    FEEC_TRY(sc.m.alloc(off, (size_t)lrows + 1));
    FEEC_TRY(launch_exclusive_scan(lrows + 1, cnt, off, scr, s));
    FEEC_TRY(cudaMemcpyAsync(&n, off + lrows, sizeof(int), cudaMemcpyDeviceToHost, s));
    FEEC_TRY(cudaStreamSynchronize(s));
    if (n > 0 && (!out_r || !out_c || !out_v)) return FEEC_BADARG;
    FEEC_TRY(sc.m.alloc(oA, (size_t)lrows + 1)); FEEC_TRY(sc.m.alloc(oC, (size_t)std::max(n, 1)));
    FEEC_TRY(sc.m.alloc(oV, (size_t)std::max(n, 1))); FEEC_TRY(sc.m.alloc(orow, (size_t)std::max(n, 1)));
    if (lrows == 0) FEEC_TRY(cudaMemsetAsync(oA, 0, sizeof(int), s));
    note_launch();
    compact_rows_kernel<<<warp_grid(lrows), kWarpBlock, 0, s>>>(lrows, SD, cnt, off, RCo, RVo, oC, oV, oA);
    note_launch();
    row_of_kernel<<<grid_of(lrows), kAlgBlock, 0, s>>>(lrows, oA, orow);
    FEEC_TRY(cudaGetLastError());
    if (n > 0) {
        FEEC_TRY(cudaMemcpyAsync(out_r, orow, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, s));
        FEEC_TRY(cudaMemcpyAsync(out_c, oC, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, s));
        FEEC_TRY(cudaMemcpyAsync(out_v, oV, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, s));
    }
    FEEC_TRY(cudaStreamSynchronize(s));
    *count = n;
    return FEEC_OK;
}

}  // extern "C"

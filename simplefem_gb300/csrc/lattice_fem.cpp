// Synthetic SPD workloads for the CSR Krylov path: Lagrange P_r stiffness plus
// (coefficient) mass on the uniformly refined unit square / unit cube.
//
// The reference builds these matrices through its FEEC route
// (tests/solverfem/csrsolver_stiff.cpp:209-243): mesh UnitSquare2D_simple
// (mesh/examples2D.hpp:194-210) or UnitCube3D (mesh/examples3D.hpp:14-37),
// refined by mesh/mesh.simplicial2D.cpp:2196-2205 resp.
// mesh/mesh.simplicial3D.ur.cxx:17-134, then K = (D I)^T M1 (D I) and
// M = I^T M0 I in the Bernstein (Sullivan) basis lambda^alpha, |alpha| = r
// (fem/global.inclsullivan.cpp:20). Both refinements keep every simplex a
// Kuhn simplex (the 3D split uses the 02-13 diagonal of the inner octahedron),
// so the refined mesh is the Kuhn triangulation of the 2^L grid and the
// degrees of freedom of P_r sit on the lattice with spacing h/r. This file
// assembles the same operator directly on that lattice, numbered
// lexicographically (x fastest), row by row, without a COO detour:
//   mass_ab  = |T| d! (a+b)! / (2r+d)!
//   stiff_ab = sum_ij a_i b_j (grad l_i . grad l_j) |T| d! (a+b-e_i-e_j)! / (2r-2+d)!
// A numbering-independent comparison against the reference's own matrices
// lives in the tests (same entries up to the permutation of unknowns).
//
// Host-only C++ (OpenMP), built into libfeec_workload.so.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct Element {
    int d = 0, r = 0, nloc = 0;
    std::vector<int> alpha;        // nloc x (d+1) multi-indices
    std::vector<double> mass;      // nloc x nloc, reference scaling (times h^d)
    std::vector<double> stiff;     // nloc x nloc, reference scaling (times h^(d-2))
};

double factorial(int k) { double f = 1.0; for (int i = 2; i <= k; i++) f *= i; return f; }

Element make_element(int d, int r) {
    Element e; e.d = d; e.r = r;
    // multi-indices of degree r over d+1 barycentric coordinates, lexicographic
    for (int i0 = 0; i0 <= r; i0++)
        for (int i1 = 0; i1 <= r - i0; i1++) {
            if (d == 2) { int i2 = r - i0 - i1; e.alpha.insert(e.alpha.end(), {i0, i1, i2}); continue; }
            for (int i2 = 0; i2 <= r - i0 - i1; i2++) { int i3 = r - i0 - i1 - i2; e.alpha.insert(e.alpha.end(), {i0, i1, i2, i3}); }
        }
    e.nloc = (int)e.alpha.size() / (d + 1);
    // Gram matrix of barycentric gradients of the path-ordered Kuhn simplex, times h^2
    std::vector<double> G((d + 1) * (d + 1), 0.0);
    for (int i = 0; i <= d; i++) {
        G[i * (d + 1) + i] = (i == 0 || i == d) ? 1.0 : 2.0;
        if (i + 1 <= d) { G[i * (d + 1) + i + 1] = -1.0; G[(i + 1) * (d + 1) + i] = -1.0; }
    }
    const double vol = 1.0 / factorial(d);  // |T| / h^d
    e.mass.assign(e.nloc * e.nloc, 0.0);
    e.stiff.assign(e.nloc * e.nloc, 0.0);
    for (int p = 0; p < e.nloc; p++)
        for (int q = 0; q < e.nloc; q++) {
            const int* A = &e.alpha[p * (d + 1)];
            const int* B = &e.alpha[q * (d + 1)];
            double fm = 1.0;
            for (int i = 0; i <= d; i++) fm *= factorial(A[i] + B[i]);
            e.mass[p * e.nloc + q] = vol * factorial(d) * fm / factorial(2 * r + d);
            double s = 0.0;
            for (int i = 0; i <= d; i++)
                for (int j = 0; j <= d; j++) {
                    if (A[i] == 0 || B[j] == 0 || G[i * (d + 1) + j] == 0.0) continue;
                    int g[4];
                    bool ok = true;
                    for (int k = 0; k <= d; k++) { g[k] = A[k] + B[k] - (k == i) - (k == j); if (g[k] < 0) ok = false; }
                    if (!ok) continue;
                    double f = 1.0;
                    for (int k = 0; k <= d; k++) f *= factorial(g[k]);
                    s += A[i] * B[j] * G[i * (d + 1) + j] * vol * factorial(d) * f / factorial(2 * r - 2 + d);
                }
            e.stiff[p * e.nloc + q] = s;
        }
    return e;
}

uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double unit_double(uint64_t& s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

// Per-cell coefficient: a hash of the cell's vertex-coordinate sum in units of h,
// so that the field does not depend on how cells are numbered.
double cell_coefficient(uint64_t seed, int64_t sx, int64_t sy, int64_t sz) {
    uint64_t s = seed ^ ((uint64_t)sx * 0x9E3779B97F4A7C15ull) ^ ((uint64_t)sy * 0xC2B2AE3D27D4EB4Full) ^ ((uint64_t)sz * 0x165667B19E3779F9ull);
    return std::pow(10.0, 2.0 * unit_double(s) - 1.0);
}

struct Lattice {
    int d, r, L;
    int64_t n, m, N;  // cells per axis, lattice points per axis, unknowns
    uint64_t seed;
    Element el;
    std::vector<int> alpha_index;  // (r+1)^(d+1) -> local index, -1 if |alpha| != r
};

bool make_lattice(int d, int r, int L, uint64_t seed, Lattice& lat) {
    if ((d != 2 && d != 3) || r < 1 || r > 4 || L < 0 || L > 12) return false;
    lat.d = d; lat.r = r; lat.L = L; lat.seed = seed;
    lat.n = (int64_t)1 << L;
    lat.m = r * lat.n + 1;
    lat.N = 1; for (int i = 0; i < d; i++) lat.N *= lat.m;
    if (lat.N > (int64_t)1 << 30) return false;
    lat.el = make_element(d, r);
    int64_t cube = 1; for (int i = 0; i <= d; i++) cube *= (r + 1);
    lat.alpha_index.assign(cube, -1);
    for (int p = 0; p < lat.el.nloc; p++) {
        int64_t key = 0;
        for (int i = d; i >= 0; i--) key = key * (r + 1) + lat.el.alpha[p * (d + 1) + i];
        lat.alpha_index[key] = p;
    }
    return true;
}

// Assemble row `row` into the (2r+1)^d window; returns the number of entries and,
// if cols/vals are given, writes them in ascending column order.
int assemble_row(const Lattice& lat, int64_t row, std::vector<double>& win, std::vector<unsigned char>& used,
                 int32_t* cols, double* vals) {
    const int d = lat.d, r = lat.r;
    const int64_t m = lat.m, n = lat.n;
    const int W = 2 * r + 1;
    const int wsize = (d == 2) ? W * W : W * W * W;
    std::fill(win.begin(), win.begin() + wsize, 0.0);
    std::fill(used.begin(), used.begin() + wsize, 0);
    int64_t p[3] = {row % m, (row / m) % m, d == 3 ? row / (m * m) : 0};
    const double h = 1.0 / (double)n;
    const double hm = (d == 2) ? h * h : h * h * h;       // mass scaling h^d
    const double hs = (d == 2) ? 1.0 : h;                 // stiffness scaling h^(d-2)
    // candidate cells per axis
    int64_t cand[3][2]; int ncand[3];
    for (int a = 0; a < 3; a++) {
        if (a >= d) { cand[a][0] = 0; ncand[a] = 1; continue; }
        ncand[a] = 0;
        if (p[a] % r == 0) {
            int64_t c0 = p[a] / r - 1, c1 = p[a] / r;
            if (c0 >= 0) cand[a][ncand[a]++] = c0;
            if (c1 < n) cand[a][ncand[a]++] = c1;
        } else {
            cand[a][ncand[a]++] = p[a] / r;
        }
    }
    static const int perm2[2][2] = {{0, 1}, {1, 0}};
    static const int perm3[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    const int nperm = (d == 2) ? 2 : 6;
    const Element& el = lat.el;
    for (int iz = 0; iz < ncand[2]; iz++)
    for (int iy = 0; iy < ncand[1]; iy++)
    for (int ix = 0; ix < ncand[0]; ix++) {
        const int64_t c[3] = {cand[0][ix], cand[1][iy], cand[2][iz]};
        int64_t t[3];
        for (int a = 0; a < 3; a++) t[a] = (a < d) ? p[a] - r * c[a] : 0;
        for (int ip = 0; ip < nperm; ip++) {
            const int* pi = (d == 2) ? perm2[ip] : perm3[ip];
            bool inside = true;
            for (int k = 0; k + 1 < d; k++) if (t[pi[k]] < t[pi[k + 1]]) inside = false;
            if (!inside) continue;
            // barycentric multi-index of the row point in this simplex
            int al[4];
            al[0] = (int)(r - t[pi[0]]);
            for (int k = 1; k < d; k++) al[k] = (int)(t[pi[k - 1]] - t[pi[k]]);
            al[d] = (int)t[pi[d - 1]];
            int64_t key = 0;
            for (int i = d; i >= 0; i--) key = key * (r + 1) + al[i];
            const int a = lat.alpha_index[key];
            // coefficient: vertex-coordinate sum of the simplex, in units of h
            double coef = 1.0;
            if (lat.seed != 0) {
                int64_t S[3] = {0, 0, 0};
                int64_t v[3] = {c[0], c[1], c[2]};
                for (int a2 = 0; a2 < d; a2++) S[a2] += v[a2];
                for (int k = 0; k < d; k++) { v[pi[k]] += 1; for (int a2 = 0; a2 < d; a2++) S[a2] += v[a2]; }
                coef = cell_coefficient(lat.seed, S[0], S[1], S[2]);
            }
            for (int b = 0; b < el.nloc; b++) {
                const int* be = &el.alpha[b * (d + 1)];
                int64_t off[3] = {0, 0, 0};
                int suffix = 0;
                for (int k = d; k >= 1; k--) { suffix += be[k]; off[pi[k - 1]] = suffix; }
                int64_t q[3];
                for (int a2 = 0; a2 < 3; a2++) q[a2] = (a2 < d) ? r * c[a2] + off[a2] : 0;
                int w = 0;
                for (int a2 = d - 1; a2 >= 0; a2--) w = w * W + (int)(q[a2] - p[a2] + r);
                win[w] += coef * hm * el.mass[a * el.nloc + b] + hs * el.stiff[a * el.nloc + b];
                used[w] = 1;
            }
        }
    }
    int cnt = 0;
    for (int w = 0; w < wsize; w++) {
        if (!used[w]) continue;
        if (cols) {
            int o[3] = {w % W - r, (w / W) % W - r, d == 3 ? w / (W * W) - r : 0};
            cols[cnt] = (int32_t)(row + o[0] + m * (o[1] + m * o[2]));
            vals[cnt] = win[w];
        }
        cnt++;
    }
    return cnt;
}

}  // namespace

extern "C" {

// Number of unknowns and stored entries of the lattice operator (dim 2|3, degree r, level L).
int feec_lattice_size(int dim, int r, int L, int64_t* n_rows, int64_t* nnz) {
    Lattice lat;
    if (!make_lattice(dim, r, L, 0, lat)) return 5;
    const int W = 2 * r + 1;
    const int wsize = (dim == 2) ? W * W : W * W * W;
    int64_t total = 0;
    #pragma omp parallel reduction(+:total)
    {
        std::vector<double> win(wsize); std::vector<unsigned char> used(wsize);
        #pragma omp for schedule(static)
        for (int64_t i = 0; i < lat.N; i++) total += assemble_row(lat, i, win, used, nullptr, nullptr);
    }
    *n_rows = lat.N; *nnz = total;
    return 0;
}

// Fills A[N+1], C[nnz], V[nnz] (caller-allocated, sizes from feec_lattice_size).
// coef_seed == 0: unit mass; otherwise the mass is weighted cell by cell by a
// log-uniform [0.1, 10] factor hashed from the cell position.
int feec_lattice_assemble(int dim, int r, int L, uint64_t coef_seed, int32_t* A, int32_t* C, double* V) {
    Lattice lat;
    if (!make_lattice(dim, r, L, coef_seed, lat)) return 5;
    const int W = 2 * r + 1;
    const int wsize = (dim == 2) ? W * W : W * W * W;
    std::vector<int32_t> len(lat.N);
    #pragma omp parallel
    {
        std::vector<double> win(wsize); std::vector<unsigned char> used(wsize);
        #pragma omp for schedule(static)
        for (int64_t i = 0; i < lat.N; i++) len[i] = assemble_row(lat, i, win, used, nullptr, nullptr);
    }
    A[0] = 0;
    for (int64_t i = 0; i < lat.N; i++) A[i + 1] = A[i] + len[i];
    #pragma omp parallel
    {
        std::vector<double> win(wsize); std::vector<unsigned char> used(wsize);
        #pragma omp for schedule(static)
        for (int64_t i = 0; i < lat.N; i++) assemble_row(lat, i, win, used, C + A[i], V + A[i]);
    }
    return 0;
}

// Positions of the unknowns (N x dim doubles), lexicographic lattice order.
int feec_lattice_positions(int dim, int r, int L, double* pos) {
    Lattice lat;
    if (!make_lattice(dim, r, L, 0, lat)) return 5;
    const double s = 1.0 / (double)(lat.m - 1);
    for (int64_t i = 0; i < lat.N; i++) {
        int64_t p[3] = {i % lat.m, (i / lat.m) % lat.m, i / (lat.m * lat.m)};
        for (int a = 0; a < dim; a++) pos[i * dim + a] = (double)p[a] * s;
    }
    return 0;
}

// out[i] = lo + (hi - lo) * u_i with u_i the i-th SplitMix64 draw from `seed`.
void feec_uniform_vector(uint64_t seed, int64_t n, double lo, double hi, double* out) {
    #pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        uint64_t s = seed + (uint64_t)i * 0x9E3779B97F4A7C15ull;
        out[i] = lo + (hi - lo) * unit_double(s);
    }
}

}  // extern "C"

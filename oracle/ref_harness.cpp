// Test infrastructure, not product code.
//
// Drives the unmodified FEEC++ reference (linked from its own object files,
// built by oracle/Makefile.ref) so that the tests can pin the oracle and the
// GPU path against the reference's own outputs. Only tests/golden/make_golden.py
// runs this binary, and only where the reference sources are present.
//
// Commands (all files little-endian, formats documented in tests/golden/README):
//   assemble <dim> <r> <L> <coef_seed> <out.csr>
//       Mesh UnitSquare2D_simple (mesh/examples2D.hpp:194-210) or UnitCube3D
//       (mesh/examples3D.hpp:14-37), uniformly refined L times; Lagrange P_r
//       stiffness + mass assembled through the FEEC route that
//       tests/solverfem/csrsolver_stiff.cpp:209-243 uses. coef_seed != 0 scales
//       the broken scalar mass cell by cell with a log-uniform [0.1,10] factor
//       hashed from the cell position (cell_coefficient below).
//       Writes the CSR plus the position of every global degree of freedom.
//   solve <cg|diag|ssor|rainbow|eisenstat|eisenstat_rainbow|cr|cr_textbook|minres|chebyshev>
//         <in.csr> <in.vec b> <in.vec x0> <precision> <omega> <out.sol>
//       Calls ConjugateGradientSolverCSR{,_DiagonalPreconditioner (precon = 1/diagonal),_SSOR,_Rainbow,
//       _SSOR_Eisenstat,_Eisenstat_Rainbow}, ConjugateResidualSolverCSR{,_textbook}, MINRESCSR or
//       ChebyshevIteration_DiagonalPreconditioner (precon = 1/diagonal, omega = "lower:upper")
//       (solver/sparsesolver.hpp)
//       with print_modulo = -3; writes K, x, residual, solve seconds.
//   rainbow <in.csr> <out.rb>        Rainbow(A) (sparse/rainbow.cpp:14-130)
//   apply <in.csr> <in.vec> <scaling> <out.vec>   MatrixCSR::apply (sparse/matcsr.cpp:216-244)
//   diag <in.csr> <out.vec>          MatrixCSR::getDiagonal (sparse/matcsr.cpp:266-286)
//   csradd <a.csr> <b.csr> <s1> <s2> <out.csr>   MatrixCSRAddition (sparse/matcsr.cpp:707-765)
//   csrmul <a.csr> <b.csr> <out.csr>             MatrixCSRMultiplication (sparse/matcsr.cpp:767-849)
//   csrtrans <a.csr> <out.csr>                   MatrixCSR::getTranspose (sparse/matcsr.cpp:291-350)
//   coo2csr <in.coo> <out.csr>                   MatrixCSR(SparseMatrix) (sparse/matcsr.cpp:43-89)
//   coomul <a.coo> <b.coo> <out.coo>             SparseMatrixMultiplication (sparse/sparsematrix.cpp:609-722)
//   hhs <A.csr> <B.csr> <Bt.csr> <C.csr> <PA.csr|-> <PC.csr|-> <bA.vec> <bC.vec> <precision> <inner_precision> <out>
//       HodgeHerzogSoodhalterMethod (solver/systemsparsesolver.hpp:74-95) from x = 0, print_modulo -3;
//       writes int64 {dim_A, dim_C, K} then x_A and x_C
//   hodge <diagonal|ssor|textbook|plain> <A.csr> <B.csr> <Bt.csr> <C.csr> <b.vec> <precision> <inner_precision> <out.sol>
//       HodgeConjugateResidualSolverCSR{_diagonal,_SSOR,_textbook,} (solver/systemsparsesolver.hpp:10-72)
//       from x0 = 0 with print_modulo = -3 and inner print_modulo = -3

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "base/include.hpp"
#include "sparse/sparsematrix.hpp"
#include "sparse/matcsr.hpp"
#include "sparse/rainbow.hpp"
#include "mesh/mesh.simplicial2D.hpp"
#include "mesh/mesh.simplicial3D.hpp"
#include "mesh/examples2D.hpp"
#include "mesh/examples3D.hpp"
#include "solver/sparsesolver.hpp"
#include "solver/systemsparsesolver.hpp"
#include "fem/global.inclsullivan.hpp"
#include "fem/global.massmatrix.hpp"
#include "fem/global.diffmatrix.hpp"
#include "combinatorics/generatemultiindices.hpp"

static void die(const char* m) { std::fprintf(stderr, "ref_harness: %s\n", m); std::exit(2); }

struct Csr { int64_t n = 0, ncols = 0, nnz = 0, pdim = 0; std::vector<int> A, C; std::vector<double> V, pos; };

static void write_csr(const char* path, const Csr& m) {
    FILE* f = std::fopen(path, "wb"); if (!f) die("cannot write csr");
    const char magic[8] = {'F','E','E','C','C','S','R','1'};
    std::fwrite(magic, 1, 8, f);
    int64_t hdr[4] = {m.n, m.ncols, m.nnz, m.pdim};
    std::fwrite(hdr, 8, 4, f);
    std::fwrite(m.A.data(), 4, m.n + 1, f);
    std::fwrite(m.C.data(), 4, m.nnz, f);
    std::fwrite(m.V.data(), 8, m.nnz, f);
    if (m.pdim) std::fwrite(m.pos.data(), 8, m.n * m.pdim, f);
    std::fclose(f);
}

static Csr read_csr(const char* path) {
    FILE* f = std::fopen(path, "rb"); if (!f) die("cannot read csr");
    char magic[8]; if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, "FEECCSR1", 8)) die("bad csr magic");
    int64_t hdr[4]; if (std::fread(hdr, 8, 4, f) != 4) die("short csr");
    Csr m; m.n = hdr[0]; m.ncols = hdr[1]; m.nnz = hdr[2]; m.pdim = hdr[3];
    m.A.resize(m.n + 1); m.C.resize(m.nnz); m.V.resize(m.nnz); m.pos.resize(m.n * m.pdim);
    if (std::fread(m.A.data(), 4, m.n + 1, f) != (size_t)(m.n + 1)) die("short A");
    if (std::fread(m.C.data(), 4, m.nnz, f) != (size_t)m.nnz) die("short C");
    if (std::fread(m.V.data(), 8, m.nnz, f) != (size_t)m.nnz) die("short V");
    std::fclose(f);
    return m;
}

static std::vector<double> read_vec(const char* path, int64_t n) {
    std::vector<double> v(n);
    FILE* f = std::fopen(path, "rb"); if (!f) die("cannot read vec");
    if (std::fread(v.data(), 8, n, f) != (size_t)n) die("short vec");
    std::fclose(f);
    return v;
}

static void write_raw(FILE* f, const void* p, size_t bytes) { if (bytes && std::fwrite(p, 1, bytes, f) != bytes) die("write"); }

static SparseMatrix read_coo(const char* path) {
    FILE* f = std::fopen(path, "rb"); if (!f) die("cannot read coo");
    char magic[8]; if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, "FEECCOO1", 8)) die("bad coo magic");
    int64_t hdr[3]; if (std::fread(hdr, 8, 3, f) != 3) die("short coo");
    std::vector<int> r(hdr[2]), c(hdr[2]); std::vector<double> v(hdr[2]);
    if (std::fread(r.data(), 4, hdr[2], f) != (size_t)hdr[2] || std::fread(c.data(), 4, hdr[2], f) != (size_t)hdr[2] ||
        std::fread(v.data(), 8, hdr[2], f) != (size_t)hdr[2]) die("short coo data");
    std::fclose(f);
    std::vector<SparseMatrix::MatrixEntry> e(hdr[2]);
    for (int64_t i = 0; i < hdr[2]; i++) e[i] = SparseMatrix::MatrixEntry{r[i], c[i], v[i]};
    return SparseMatrix((int)hdr[0], (int)hdr[1], e);
}

static void write_coo(const char* path, const SparseMatrix& m) {
    FILE* f = std::fopen(path, "wb"); if (!f) die("cannot write coo");
    const auto& e = m.getentries();
    const int64_t hdr[3] = {m.getdimout(), m.getdimin(), (int64_t)e.size()};
    std::vector<int> r(e.size()), c(e.size()); std::vector<double> v(e.size());
    for (size_t i = 0; i < e.size(); i++) { r[i] = e[i].row; c[i] = e[i].column; v[i] = e[i].value; }
    write_raw(f, "FEECCOO1", 8); write_raw(f, hdr, sizeof(hdr));
    write_raw(f, r.data(), 4 * r.size()); write_raw(f, c.data(), 4 * c.size()); write_raw(f, v.data(), 8 * v.size());
    std::fclose(f);
}

static MatrixCSR to_matrix(const Csr& m) {
    std::vector<int> A(m.A), C(m.C); std::vector<Float> V(m.V.begin(), m.V.end());
    return MatrixCSR((int)m.n, (int)m.ncols, std::move(A), std::move(C), std::move(V));
}

static Csr from_matrix(const MatrixCSR& mat) {
    Csr m; m.n = mat.getdimout(); m.ncols = mat.getdimin(); m.nnz = mat.getnumberofentries();
    m.A.assign(mat.getA(), mat.getA() + m.n + 1);
    m.C.assign(mat.getC(), mat.getC() + m.nnz);
    m.V.assign(mat.getV(), mat.getV() + m.nnz);
    return m;
}

// SplitMix64 -> uniform double in [lo, hi); same generator as the package's workload module.
static uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double unit_double(uint64_t& s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

// Coefficient of the cell whose vertex coordinates (in units of the finest
// lattice spacing) sum to (sx, sy, sz): 10^(2u-1), u uniform in [0,1).
static double cell_coefficient(uint64_t seed, int64_t sx, int64_t sy, int64_t sz) {
    uint64_t s = seed ^ ((uint64_t)sx * 0x9E3779B97F4A7C15ull) ^ ((uint64_t)sy * 0xC2B2AE3D27D4EB4Full) ^ ((uint64_t)sz * 0x165667B19E3779F9ull);
    return std::pow(10.0, 2.0 * unit_double(s) - 1.0);
}

template <class MeshT>
static Csr assemble_on(MeshT& M, int n, int r, int L, uint64_t coef_seed) {
    SparseMatrix M0 = FEECBrokenMassMatrix(M, n, 0, r);
    SparseMatrix M1 = FEECBrokenMassMatrix(M, n, 1, r - 1);
    SparseMatrix D  = FEECBrokenDiffMatrix(M, n, 0, r);
    SparseMatrix I  = FEECSullivanInclusionMatrix(M, n, 0, r);
    const int nvol = M.count_simplices(n);
    const int localdim = (int)M0.getdimout() / nvol;
    if (coef_seed != 0) {
        // Log-uniform [0.1, 10] per cell. The factor is a hash of the cell's
        // vertex-coordinate sum on the 2^L lattice, so that any numbering of the
        // same mesh draws the same field (the package's lattice assembler uses
        // the identical rule).
        const auto& cc = M.getCoordinates();
        const double scale = std::ldexp(1.0, L);
        for (auto& e : M0.getentries()) {
            const int s = e.row / localdim;
            const IndexMap verts = M.get_subsimplices(n, 0, s);
            int64_t S[3] = {0, 0, 0};
            for (int v = 0; v <= n; v++)
                for (int d = 0; d < n; d++) S[d] += (int64_t)std::llround(cc.getdata(verts.at(v), d) * scale);
            e.value *= cell_coefficient(coef_seed, S[0], S[1], S[2]);
        }
    }
    M0.sortandcompressentries();
    M1.sortandcompressentries();
    SparseMatrix opr = D & I;
    SparseMatrix opl = opr.getTranspose();
    SparseMatrix stiff = opl & (M1 & opr);
    stiff.sortentries();
    SparseMatrix It = I.getTranspose();
    SparseMatrix mass = It & (M0 & I);
    mass.sortentries();
    MatrixCSR sum = MatrixCSR(stiff) + MatrixCSR(mass);
    Csr out = from_matrix(sum);

    // Positions of the global degrees of freedom, read off the inclusion matrix:
    // broken row s*localdim + a carries the Bernstein multi-index multis[a] on cell s.
    const auto multis = generateMultiIndices(IndexRange(0, n), r);
    if ((int)multis.size() != localdim) die("localdim mismatch");
    out.pdim = n;
    out.pos.assign(out.n * n, std::nan(""));
    const auto& coords = M.getCoordinates();
    for (const auto& e : I.getentries()) {
        const int s = e.row / localdim, a = e.row % localdim;
        const IndexMap verts = M.get_subsimplices(n, 0, s);
        for (int d = 0; d < n; d++) {
            double p = 0.0;
            for (int v = 0; v <= n; v++) p += multis[a].at(v) * coords.getdata(verts.at(v), d);
            out.pos[(int64_t)e.column * n + d] = p / r;
        }
    }
    return out;
}

int main(int argc, char** argv) {
    if (argc < 2) die("usage: see header");
    const std::string cmd = argv[1];
    if (cmd == "assemble") {
        if (argc != 7) die("assemble <dim> <r> <L> <coef_seed> <out.csr>");
        const int dim = std::atoi(argv[2]), r = std::atoi(argv[3]), L = std::atoi(argv[4]);
        const uint64_t seed = std::strtoull(argv[5], nullptr, 10);
        Csr m;
        if (dim == 2) { auto M = UnitSquare2D_simple(); for (int l = 0; l < L; l++) M.uniformrefinement(); m = assemble_on(M, 2, r, L, seed); }
        else if (dim == 3) { auto M = UnitCube3D(); for (int l = 0; l < L; l++) M.uniformrefinement(); m = assemble_on(M, 3, r, L, seed); }
        else die("dim must be 2 or 3");
        write_csr(argv[6], m);
        std::printf("N=%lld nnz=%lld\n", (long long)m.n, (long long)m.nnz);
        return 0;
    }
    if (cmd == "solve") {
        if (argc != 9) die("solve <kind> <in.csr> <b.vec> <x0.vec> <precision> <omega> <out.sol>");
        const std::string kind = argv[2];
        Csr m = read_csr(argv[3]);
        std::vector<double> b = read_vec(argv[4], m.n), x = read_vec(argv[5], m.n);
        const double precision = std::atof(argv[6]), omega = std::atof(argv[7]);
        std::vector<double> res(b);
        MatrixCSR mat = to_matrix(m);
        int K = -1;
        double secs = 0.0;
        if (kind == "cg") {
            auto t0 = std::chrono::steady_clock::now();
            K = ConjugateGradientSolverCSR((int)m.n, x.data(), b.data(), mat.getA(), mat.getC(), mat.getV(), res.data(), precision, -3);
            secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        } else if (kind == "ssor") {
            FloatVector diag = mat.getDiagonal();
            auto t0 = std::chrono::steady_clock::now();
            K = ConjugateGradientSolverCSR_SSOR((int)m.n, x.data(), b.data(), mat.getA(), mat.getC(), mat.getV(), res.data(), precision, -3, diag.raw(), omega);
            secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        } else if (kind == "rainbow") {
            FloatVector diag = mat.getDiagonal();
            Rainbow rb(mat);
            auto t0 = std::chrono::steady_clock::now();
            K = ConjugateGradientSolverCSR_Rainbow((int)m.n, x.data(), b.data(), mat.getA(), mat.getC(), mat.getV(), res.data(), precision, -3, diag.raw(), omega,
                                                   rb.num_colors, rb.F.data(), rb.B.data(), rb.R.data());
            secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        } else if (kind == "diag") {
            // the preconditioner the reference's callers pass: the inverse diagonal
            FloatVector diag = mat.getDiagonal();
            std::vector<double> precon(m.n);
            for (int64_t i = 0; i < m.n; i++) precon[i] = diag[i] != 0.0 ? 1.0 / diag[i] : 0.0;
            auto t0 = std::chrono::steady_clock::now();
            K = ConjugateGradientSolverCSR_DiagonalPreconditioner((int)m.n, x.data(), b.data(), mat.getA(), mat.getC(), mat.getV(), res.data(), precision, -3, precon.data());
            secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        } else if (kind == "eisenstat") {
            FloatVector diag = mat.getDiagonal();
            auto t0 = std::chrono::steady_clock::now();
            K = ConjugateGradientSolverCSR_SSOR_Eisenstat((int)m.n, x.data(), b.data(), mat.getA(), mat.getC(), mat.getV(), res.data(), precision, -3, diag.raw(), omega);
            secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        } else if (kind == "eisenstat_rainbow") {
            FloatVector diag = mat.getDiagonal();
            Rainbow rb(mat);
            auto t0 = std::chrono::steady_clock::now();
            K = ConjugateGradientSolverCSR_Eisenstat_Rainbow((int)m.n, x.data(), b.data(), mat.getA(), mat.getC(), mat.getV(), res.data(), precision, -3, diag.raw(), omega,
                                                             rb.num_colors, rb.F.data(), rb.B.data(), rb.R.data());
            secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        } else if (kind == "cr" || kind == "cr_textbook" || kind == "minres") {
            auto t0 = std::chrono::steady_clock::now();
            if (kind == "cr")
                K = ConjugateResidualSolverCSR((int)m.n, x.data(), b.data(), mat.getA(), mat.getC(), mat.getV(), res.data(), precision, -3);
            else if (kind == "cr_textbook")
                K = ConjugateResidualSolverCSR_textbook((int)m.n, x.data(), b.data(), mat.getA(), mat.getC(), mat.getV(), res.data(), precision, -3);
            else
                K = MINRESCSR((int)m.n, x.data(), b.data(), mat.getA(), mat.getC(), mat.getV(), res.data(), precision, -3);
            secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        } else if (kind == "chebyshev") {
            // the omega argument carries the spectral bounds as "lower:upper"; precon = 1/diagonal
            double lower = 0.0, upper = 0.0;
            if (std::sscanf(argv[7], "%lf:%lf", &lower, &upper) != 2) die("chebyshev wants <lower:upper> as omega");
            FloatVector diag = mat.getDiagonal();
            std::vector<double> precon(m.n);
            for (int64_t i = 0; i < m.n; i++) precon[i] = diag[i] != 0.0 ? 1.0 / diag[i] : 0.0;
            auto t0 = std::chrono::steady_clock::now();
            K = ChebyshevIteration_DiagonalPreconditioner((int)m.n, x.data(), b.data(), mat.getA(), mat.getC(), mat.getV(), res.data(), precision, -3,
                                                          precon.data(), lower, upper);
            secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        } else die("unknown solver kind");
        FILE* f = std::fopen(argv[8], "wb"); if (!f) die("cannot write sol");
        int64_t hdr[2] = {m.n, K};
        write_raw(f, hdr, 16); write_raw(f, &secs, 8);
        write_raw(f, x.data(), 8 * m.n); write_raw(f, res.data(), 8 * m.n);
        std::fclose(f);
        std::printf("K=%d secs=%.6f\n", K, secs);
        return 0;
    }
    if (cmd == "rainbow") {
        if (argc != 4) die("rainbow <in.csr> <out.rb>");
        Csr m = read_csr(argv[2]);
        MatrixCSR mat = to_matrix(m);
        auto t0 = std::chrono::steady_clock::now();
        Rainbow rb(mat);
        double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        FILE* f = std::fopen(argv[3], "wb"); if (!f) die("cannot write rb");
        int64_t hdr[2] = {m.n, rb.num_colors};
        write_raw(f, hdr, 16);
        write_raw(f, rb.F.data(), 4 * m.n); write_raw(f, rb.B.data(), 4 * (rb.num_colors + 1)); write_raw(f, rb.R.data(), 4 * m.n);
        std::fclose(f);
        std::printf("colors=%d secs=%.6f\n", rb.num_colors, secs);
        return 0;
    }
    if (cmd == "apply") {
        if (argc != 6) die("apply <in.csr> <in.vec> <scaling> <out.vec>");
        Csr m = read_csr(argv[2]);
        MatrixCSR mat = to_matrix(m);
        std::vector<double> src = read_vec(argv[3], m.ncols);
        FloatVector s(std::vector<Float>(src.begin(), src.end())), d((int)m.n, 0.0);
        mat.apply(d, s, std::atof(argv[4]));
        FILE* f = std::fopen(argv[5], "wb"); if (!f) die("cannot write vec");
        write_raw(f, d.raw(), 8 * m.n); std::fclose(f);
        return 0;
    }
    if (cmd == "diag") {
        if (argc != 4) die("diag <in.csr> <out.vec>");
        Csr m = read_csr(argv[2]);
        MatrixCSR mat = to_matrix(m);
        FloatVector d = mat.getDiagonal();
        FILE* f = std::fopen(argv[3], "wb"); if (!f) die("cannot write vec");
        write_raw(f, d.raw(), 8 * m.n); std::fclose(f);
        return 0;
    }
    if (cmd == "csradd") {
        if (argc != 7) die("csradd <a.csr> <b.csr> <s1> <s2> <out.csr>");
        MatrixCSR a = to_matrix(read_csr(argv[2])), b = to_matrix(read_csr(argv[3]));
        write_csr(argv[6], from_matrix(MatrixCSRAddition(a, b, std::atof(argv[4]), std::atof(argv[5]))));
        return 0;
    }
    if (cmd == "csrmul") {
        if (argc != 5) die("csrmul <a.csr> <b.csr> <out.csr>");
        MatrixCSR a = to_matrix(read_csr(argv[2])), b = to_matrix(read_csr(argv[3]));
        write_csr(argv[4], from_matrix(MatrixCSRMultiplication(a, b)));
        return 0;
    }
    if (cmd == "csrtrans") {
        if (argc != 4) die("csrtrans <a.csr> <out.csr>");
        write_csr(argv[3], from_matrix(to_matrix(read_csr(argv[2])).getTranspose()));
        return 0;
    }
    if (cmd == "coo2csr") {
        if (argc != 4) die("coo2csr <in.coo> <out.csr>");
        write_csr(argv[3], from_matrix(MatrixCSR(read_coo(argv[2]))));
        return 0;
    }
    if (cmd == "hodge") {
        if (argc != 11) die("hodge <variant> <A.csr> <B.csr> <Bt.csr> <C.csr> <b.vec> <precision> <inner_precision> <out.sol>");
        const std::string kind = argv[2];
        Csr A = read_csr(argv[3]), B = read_csr(argv[4]), Bt = read_csr(argv[5]), C = read_csr(argv[6]);
        const int N = (int)C.n, L = (int)A.n;
        std::vector<double> b = read_vec(argv[7], N), x(N, 0.0), res(N, 0.0);
        const double precision = std::atof(argv[8]), inner = std::atof(argv[9]);
        int K = -1;
        auto t0 = std::chrono::steady_clock::now();
        auto call = [&](auto fn) {
            return fn(N, L, x.data(), b.data(), A.A.data(), A.C.data(), A.V.data(), B.A.data(), B.C.data(), B.V.data(),
                      Bt.A.data(), Bt.C.data(), Bt.V.data(), C.A.data(), C.C.data(), C.V.data(), res.data(), precision, -3,
                      inner, -3);
        };
        if (kind == "diagonal") K = call(HodgeConjugateResidualSolverCSR_diagonal);
        else if (kind == "ssor") K = call(HodgeConjugateResidualSolverCSR_SSOR);
        else if (kind == "textbook") K = call(HodgeConjugateResidualSolverCSR_textbook);
        else if (kind == "plain") K = call(HodgeConjugateResidualSolverCSR);
        else die("unknown hodge variant");
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        FILE* f = std::fopen(argv[10], "wb"); if (!f) die("cannot write sol");
        int64_t hdr[2] = {N, K};
        write_raw(f, hdr, 16); write_raw(f, &secs, 8);
        write_raw(f, x.data(), 8 * (size_t)N); write_raw(f, res.data(), 8 * (size_t)N);
        std::fclose(f);
        std::printf("K=%d secs=%.6f\n", K, secs);
        return 0;
    }
    if (cmd == "hhs") {
        if (argc != 13) die("hhs <A> <B> <Bt> <C> <PA|-> <PC|-> <bA> <bC> <precision> <inner_precision> <out>");
        Csr A = read_csr(argv[2]), B = read_csr(argv[3]), Bt = read_csr(argv[4]), C = read_csr(argv[5]);
        const bool pa = std::string(argv[6]) != "-", pc = std::string(argv[7]) != "-";
        Csr PA = pa ? read_csr(argv[6]) : Csr(), PC = pc ? read_csr(argv[7]) : Csr();
        const int dA = (int)A.n, dC = (int)C.n;
        std::vector<double> bA = read_vec(argv[8], dA), bC = read_vec(argv[9], dC), xA(dA, 0.0), xC(dC, 0.0);
        const int K = HodgeHerzogSoodhalterMethod(
            dA, dC, xA.data(), xC.data(), bA.data(), bC.data(), A.A.data(), A.C.data(), A.V.data(), B.A.data(),
            B.C.data(), B.V.data(), Bt.A.data(), Bt.C.data(), Bt.V.data(), C.A.data(), C.C.data(), C.V.data(),
            std::atof(argv[10]), -3, pa ? PA.A.data() : nullptr, pa ? PA.C.data() : nullptr, pa ? PA.V.data() : nullptr,
            pc ? PC.A.data() : nullptr, pc ? PC.C.data() : nullptr, pc ? PC.V.data() : nullptr, std::atof(argv[11]), -3);
        FILE* f = std::fopen(argv[12], "wb"); if (!f) die("cannot write hhs");
        int64_t hdr[3] = {dA, dC, K};
        write_raw(f, hdr, 24); write_raw(f, xA.data(), 8 * (size_t)dA); write_raw(f, xC.data(), 8 * (size_t)dC);
        std::fclose(f);
        std::printf("K=%d\n", K);
        return 0;
    }
    if (cmd == "coomul") {
        if (argc != 5) die("coomul <a.coo> <b.coo> <out.coo>");
        const SparseMatrix a = read_coo(argv[2]), b = read_coo(argv[3]);
        write_coo(argv[4], SparseMatrixMultiplication(a, b));
        return 0;
    }
    die("unknown command");
}

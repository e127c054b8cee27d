// A FEEC++-style caller of the CSR Krylov drivers, linked against libfeec_dropin.so
// only. It declares the three drivers exactly as the reference's solver header does
// (solver/sparsesolver.hpp:11-19, 33-43, 59-70, with Float = double), so the calls
// below bind to the reference's C++ symbol names and run through the shim on the GPU.
//
// Usage: dropin_driver <input> <output>
//   input : int32 N, nnz, num_colors, print_modulo; float64 precision, omega;
//           int32 A[N+1], C[nnz]; float64 V[nnz], b[N], diagonal[N];
//           int32 F[N], B[num_colors+1], R[N]
//   output: for CG, SSOR, Rainbow in that order: int32 K; float64 x[N], residual[N]
// Each solve starts from x = 0 and residual = 0, as the reference's tests do.
#include <cstdio>
#include <cstdlib>
#include <vector>

int ConjugateGradientSolverCSR(const int N, double* x, const double* b, const int* csrrows, const int* csrcolumns,
                               const double* csrvalues, double* residual, double precision, int print_modulo);

int ConjugateGradientSolverCSR_SSOR(const int N, double* x, const double* b, const int* csrrows,
                                    const int* csrcolumns, const double* csrvalues, double* residual,
                                    double precision, int print_modulo, const double* diagonal, double omega);

int ConjugateGradientSolverCSR_Rainbow(const int N, double* x, const double* b, const int* csrrows,
                                       const int* csrcolumns, const double* csrvalues, double* residual,
                                       double precision, int print_modulo, const double* diagonal, double omega,
                                       int num_colors, const int* F, const int* B, const int* R);

template <typename T>
static void read_into(FILE* f, std::vector<T>& v, size_t count) {
    v.resize(count);
    if (count && std::fread(v.data(), sizeof(T), count, f) != count) {
        std::fprintf(stderr, "dropin_driver: short input\n");
        std::exit(2);
    }
}

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: dropin_driver <input> <output>\n");
        return 2;
    }
    FILE* in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    int hdr[4];
    double prm[2];
    if (std::fread(hdr, sizeof(int), 4, in) != 4 || std::fread(prm, sizeof(double), 2, in) != 2) return 2;
    const int N = hdr[0], nnz = hdr[1], nc = hdr[2], print_modulo = hdr[3];
    if (N <= 0 || nnz < 0 || nc <= 0) return 2;
    std::vector<int> A, C, F, B, R;
    std::vector<double> V, b, diag;
    read_into(in, A, (size_t)N + 1);
    read_into(in, C, (size_t)nnz);
    read_into(in, V, (size_t)nnz);
    read_into(in, b, (size_t)N);
    read_into(in, diag, (size_t)N);
    read_into(in, F, (size_t)N);
    read_into(in, B, (size_t)nc + 1);
    read_into(in, R, (size_t)N);
    std::fclose(in);

    FILE* out = std::fopen(argv[2], "wb");
    if (!out) return 2;
    for (int which = 0; which < 3; which++) {
        std::vector<double> x(N, 0.0), residual(N, 0.0);
        int K = 0;
        if (which == 0)
            K = ConjugateGradientSolverCSR(N, x.data(), b.data(), A.data(), C.data(), V.data(), residual.data(),
                                           prm[0], print_modulo);
        else if (which == 1)
            K = ConjugateGradientSolverCSR_SSOR(N, x.data(), b.data(), A.data(), C.data(), V.data(),
                                                residual.data(), prm[0], print_modulo, diag.data(), prm[1]);
        else
            K = ConjugateGradientSolverCSR_Rainbow(N, x.data(), b.data(), A.data(), C.data(), V.data(),
                                                   residual.data(), prm[0], print_modulo, diag.data(), prm[1], nc,
                                                   F.data(), B.data(), R.data());
        std::fwrite(&K, sizeof(int), 1, out);
        std::fwrite(x.data(), sizeof(double), (size_t)N, out);
        std::fwrite(residual.data(), sizeof(double), (size_t)N, out);
    }
    std::fclose(out);
    return 0;
}

// Host-side integer preprocessing for the SSOR sweeps.
//
// rainbow_host: the greedy multicolor ordering of sparse/rainbow.cpp:14-130
// (do_shuffle = false), bit-identical F / B / R. Rows are visited in index
// order; a row receives the smallest color that none of its off-diagonal
// neighbours holds at that moment, where neighbours not yet visited still hold
// their initial color 0 (this is what the reference's restart-on-conflict scan
// computes: the scan only ever moves to the next color, and neighbour colors do
// not change while a row is painted). Colors are then counted, B is the prefix
// sum of the counts, and R lists each color's rows from the top of its range
// downwards, so rows appear in descending index order within a color.
//
// triangular_levels: level schedule for the index-order SSOR sweeps of
// solver/sparsesolver.cpp:528-568 and :647-692. A row's forward value depends
// on its lower-index neighbours only, so rows of equal level can be swept at
// once; the backward sweep uses the mirrored rule.
#include <algorithm>
#include <vector>

#include "feec_internal.h"

namespace feec {

int rainbow_host(int n, const int* A, const int* C, int* F, int* B, int* R) {
    if (n <= 0) return 0;
    std::fill(F, F + n, 0);
    std::vector<int> seen;  // seen[c] == r + 1  <=>  color c is held by a neighbour of r
    int num_colors = 1;
    for (int r = 0; r < n; r++) {
        int maxc = -1;
        for (int k = A[r]; k < A[r + 1]; k++) {
            const int j = C[k];
            if (j == r) continue;
            const int c = F[j];
            if (c >= (int)seen.size()) seen.resize((size_t)c + 1, 0);
            seen[c] = r + 1;
            if (c > maxc) maxc = c;
        }
        int color = 0;
        while (color <= maxc && seen[color] == r + 1) color++;
        F[r] = color;
        if (color == num_colors) num_colors++;
    }
    std::vector<int> count((size_t)num_colors, 0);
    for (int r = 0; r < n; r++) count[F[r]]++;
    B[0] = 0;
    for (int c = 0; c < num_colors; c++) B[c + 1] = B[c] + count[c];
    for (int r = 0; r < n; r++) {
        const int c = F[r];
        R[B[c] + (--count[c])] = r;
    }
    return num_colors;
}

void triangular_levels(int n, const int* A, const int* C, bool lower, std::vector<int>& level, int& nlevels) {
    level.assign((size_t)n, 0);
    nlevels = 0;
    if (lower) {
        for (int r = 0; r < n; r++) {
            int lv = 0;
            for (int k = A[r]; k < A[r + 1]; k++) {
                const int j = C[k];
                if (j < r && level[j] + 1 > lv) lv = level[j] + 1;
            }
            level[r] = lv;
            if (lv + 1 > nlevels) nlevels = lv + 1;
        }
    } else {
        for (int r = n - 1; r >= 0; r--) {
            int lv = 0;
            for (int k = A[r]; k < A[r + 1]; k++) {
                const int j = C[k];
                if (j > r && level[j] + 1 > lv) lv = level[j] + 1;
            }
            level[r] = lv;
            if (lv + 1 > nlevels) nlevels = lv + 1;
        }
    }
}

}  // namespace feec

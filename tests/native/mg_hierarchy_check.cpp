// Reads lines "p n U_0 .. U_{n-1}" (a fine knot vector) and prints the
// library's coarsened knot vector (coarsen_knots), whether a knot was
// dropped, and the prolongation from the coarse to the fine spline space
// (boehm_prolongation) as "row col value" triples. Linked against
// libtdz.so; run by tests/test_mg_hierarchy_native.py.
#include <cstdio>
#include <vector>

#include "mg.h"

int main() {
    int p, n;
    while (std::scanf("%d %d", &p, &n) == 2) {
        std::vector<double> F(n);
        for (int i = 0; i < n; ++i)
            if (std::scanf("%lf", &F[i]) != 1) return 2;
        bool dropped = false;
        const std::vector<double> C = tdz::coarsen_knots(F, &dropped);
        std::printf("%d %d", (int)C.size(), dropped ? 1 : 0);
        for (double v : C) std::printf(" %.17g", v);
        std::printf("\n");
        const tdz::RowSparse P = tdz::boehm_prolongation(C, F, p);
        int nnz = 0;
        for (size_t k = 0; k < P.col.size(); ++k) nnz += P.col[k] >= 0;
        std::printf("%d %d %d\n", P.rows, P.cols, nnz);
        for (int r = 0; r < P.rows; ++r)
            for (int w = 0; w < P.width; ++w) {
                const int c = P.col[(size_t)r * P.width + w];
                if (c >= 0) std::printf("%d %d %.17g\n", r, c, P.val[(size_t)r * P.width + w]);
            }
    }
    return 0;
}

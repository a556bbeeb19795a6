// Reads lines "p nq n U_0 .. U_{n-1}" and prints the eigenbasis that the FDM
// preconditioner takes for an inner axis (gen_eig, fdm.cu): the generalised
// eigenpairs of the stiffness band S = (B', B') against the mass band M =
// (B, B) of the library's host axis, as "n", the n eigenvalues, then V row
// by row. Linked against libtdz.so; run by tests/test_axis_eig_native.py.
#include <cstdio>
#include <vector>

#include "fdm.h"
#include "space.h"

int main() {
    int p, nq, n;
    while (std::scanf("%d %d %d", &p, &nq, &n) == 3) {
        std::vector<double> U(n);
        for (int i = 0; i < n; ++i)
            if (std::scanf("%lf", &U[i]) != 1) return 2;
        tdz::Axis1D a;
        a.setup(U.data(), n, p, nq);
        std::vector<double> V, lam;
        tdz::gen_eig(a.band(nullptr, 1, 1), a.band(nullptr, 0, 0), V, lam);
        const int m = (int)lam.size();
        std::printf("%d\n", m);
        for (int i = 0; i < m; ++i) std::printf(i ? " %.17g" : "%.17g", lam[i]);
        std::printf("\n");
        for (int i = 0; i < m; ++i) {
            for (int j = 0; j < m; ++j) std::printf(j ? " %.17g" : "%.17g", V[(size_t)i * m + j]);
            std::printf("\n");
        }
    }
    return 0;
}

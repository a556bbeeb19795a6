// Reads lines "p nq n U_0 .. U_{n-1}" and prints, for the library's host
// axis (space.cpp) on those knots, the 1D band matrices the operators are
// built from -- mass, stiffness, position, and the x^2 potential -- and the
// Galerkin coarse mass P^T M P on the coarsened knots (mg_setup.cpp), each
// as "name rows cols" followed by the dense rows. Linked against libtdz.so;
// run by tests/test_axis_bands_native.py.
#include <cstdio>
#include <vector>

#include "mg.h"
#include "space.h"

static void dump(const char *name, const tdz::BandD &B) {
    std::printf("%s %d %d\n", name, B.n, B.n);
    for (int i = 0; i < B.n; ++i) {
        for (int j = 0; j < B.n; ++j) {
            const double v = (j >= i - B.p && j <= i + B.p) ? B.at(i, j) : 0.0;
            std::printf(j ? " %.17g" : "%.17g", v);
        }
        std::printf("\n");
    }
}

int main() {
    int p, nq, n;
    while (std::scanf("%d %d %d", &p, &nq, &n) == 3) {
        std::vector<double> U(n);
        for (int i = 0; i < n; ++i)
            if (std::scanf("%lf", &U[i]) != 1) return 2;
        tdz::Axis1D a;
        a.setup(U.data(), n, p, nq);
        std::vector<double> f(a.xq.size());
        for (size_t k = 0; k < f.size(); ++k) f[k] = a.xq[k] * a.xq[k];
        dump("M", a.band(nullptr, 0, 0));
        dump("S", a.band(nullptr, 1, 1));
        dump("X", a.band_x());
        dump("V", a.band(f.data(), 0, 0));
        bool dropped = false;
        const std::vector<double> C = tdz::coarsen_knots(U, &dropped);
        const tdz::RowSparse P = tdz::boehm_prolongation(C, U, p);
        dump("G", tdz::galerkin(P, a.band(nullptr, 0, 0)));
    }
    return 0;
}

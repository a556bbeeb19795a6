// Reads lines "pmin pmax split dp_in dp_out np p_1 .. p_np" and prints the
// energy nodes, then for every p the first node and the four weights
// (tsurff_nodes.h). Built and run by tests/test_end_nodes_native.py.
#include <cstdio>
#include <vector>

#include "tsurff_nodes.h"

int main() {
    double pmin, pmax, split, dpi, dpo;
    int np;
    while (std::scanf("%lf %lf %lf %lf %lf %d", &pmin, &pmax, &split, &dpi, &dpo, &np) == 6) {
        std::vector<double> ps(np);
        for (int i = 0; i < np; ++i)
            if (std::scanf("%lf", &ps[i]) != 1) return 2;
        const std::vector<double> node = tdz::energy_nodes(pmin, pmax, split, dpi, dpo);
        std::printf("%d", (int)node.size());
        for (double v : node) std::printf(" %.17g", v);
        std::printf("\n");
        for (double p : ps) {
            double w[4] = {0, 0, 0, 0};
            const int j0 = tdz::lagrange_weights(node, p, w);
            std::printf("%d %.17g %.17g %.17g %.17g\n", j0, w[0], w[1], w[2], w[3]);
        }
    }
    return 0;
}

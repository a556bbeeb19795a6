// Energy nodes and Lagrange weights of the t-SURFF end term (host,
// header-only so that a host test can check them against the oracle).
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

namespace tdz {

// Energy nodes in p = |k + A(T)| (src/tsurff.cpp:700-723): spacing dp_in
// from p_min up to split = min(max(2 k_cap, p_min), p_max), below which the
// absorber reflects and the box's quasi-modes set the scale, then dp_out up
// to p_max; halved until there are four nodes (the cubic weights need them).
// A segment ends exactly at its end point: a last node a + (b - a) cnt / cnt
// one rounding below b would open a second segment of one node next to it,
// whose Lagrange weights divide by the rounding difference.
inline std::vector<double> energy_nodes(double pmin, double pmax, double split, double dp_in, double dp_out) {
    std::vector<double> node;
    if (!(pmax > pmin)) return {pmin};
    auto segment = [&](double a, double b, double dp) {
        if (!(b > a)) return;
        const int cnt = std::max(1, (int)std::ceil((b - a) / dp - 1e-9));
        for (int i = node.empty() ? 0 : 1; i <= cnt; ++i) node.push_back(i == cnt ? b : a + (b - a) * i / cnt);
    };
    segment(pmin, split, dp_in);
    segment(node.empty() ? pmin : node.back(), pmax, dp_out);
    while (node.size() < 4) {
        std::vector<double> finer;
        for (size_t i = 0; i + 1 < node.size(); ++i) {
            finer.push_back(node[i]);
            finer.push_back(0.5 * (node[i] + node[i + 1]));
        }
        finer.push_back(node.back());
        node.swap(finer);
    }
    return node;
}

// Four-point Lagrange interpolation in p on the nodes around p
// (src/tsurff.cpp:725-756): returns the first node j0 and fills w[0 ..
// min(n, 4)) (one node: weight 1)
inline int lagrange_weights(const std::vector<double> &node, double p, double w[4]) {
    const int nn = (int)node.size();
    if (nn == 1) {
        w[0] = 1.0;
        return 0;
    }
    const int m = std::min(nn, 4);
    const int below = (int)(std::upper_bound(node.begin(), node.end(), p) - node.begin()) - 1;
    const int j0 = std::max(0, std::min(nn - m, below - 1));
    for (int a = 0; a < m; ++a) {
        w[a] = 1.0;
        for (int b = 0; b < m; ++b)
            if (b != a) w[a] *= (p - node[j0 + b]) / (node[j0 + a] - node[j0 + b]);
    }
    return j0;
}

}  // namespace tdz

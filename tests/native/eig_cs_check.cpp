// Check of the complex symmetric axis eigenbasis (gen_eig_complex) on bands
// read from a file: prints ok, |V^T S V - diag(lam)|_max / max|lam|,
// |V^T M V - I|_max. Built and run by tests/test_eig_cs.py.
#include <cstdio>

#include "fdm.h"

using namespace tdz;

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    FILE *f = std::fopen(argv[1], "r");
    if (!f) return 2;
    int n, p;
    if (std::fscanf(f, "%d %d", &n, &p) != 2) return 2;
    const int bw = 2 * p + 1;
    BandD M(n, p);
    std::vector<cd> S((size_t)n * bw);
    for (int i = 0; i < n; ++i)
        for (int o = 0; o < bw; ++o) {
            double m, a, b;
            if (std::fscanf(f, "%lf %lf %lf", &m, &a, &b) != 3) return 2;
            M.v[(size_t)i * bw + o] = m;
            S[(size_t)i * bw + o] = cd(a, b);
        }
    std::fclose(f);
    std::vector<cd> V, lam;
    const bool ok = gen_eig_complex(S, p, M, V, lam);
    double es = 0.0, em = 0.0, lmax = 0.0;
    if (ok) {
        auto s_at = [&](int i, int j) { return std::abs(i - j) <= p ? S[(size_t)i * bw + (j - i + p)] : cd(0.0); };
        auto m_at = [&](int i, int j) { return std::abs(i - j) <= p ? M.at(i, j) : 0.0; };
        for (const cd &l : lam) lmax = std::max(lmax, std::abs(l));
        for (int a = 0; a < n; ++a)
            for (int b = 0; b < n; ++b) {
                cd ss = 0.0, mm = 0.0;
                for (int i = 0; i < n; ++i)
                    for (int j = std::max(0, i - p); j <= std::min(n - 1, i + p); ++j) {
                        ss += V[(size_t)i * n + a] * s_at(i, j) * V[(size_t)j * n + b];
                        mm += V[(size_t)i * n + a] * m_at(i, j) * V[(size_t)j * n + b];
                    }
                es = std::max(es, std::abs(ss - (a == b ? lam[a] : cd(0.0))));
                em = std::max(em, std::abs(mm - (a == b ? 1.0 : 0.0)));
            }
    }
    std::printf("%d %.3e %.3e\n", ok ? 1 : 0, ok ? es / lmax : 0.0, em);
    return 0;
}

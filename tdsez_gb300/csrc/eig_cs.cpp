// Generalised eigenproblem of a complex symmetric band S (an axis operator
// with its absorbing layer, S = K + V - i W) against the real SPD overlap M,
// for the fast-diagonalisation preconditioner. Host, FP64, dense O(n^3).
//
// With M = L L^T, C = L^-1 S L^-T is complex symmetric. Its eigenvectors are
// computed from the complex Schur form C = Z T Z^H (Householder reduction to
// Hessenberg form, then single-shift QR sweeps with Wilkinson shifts and
// Givens rotations), by back-substitution in T and the back-transform with Z.
// For distinct eigenvalues the eigenvectors of a complex symmetric matrix
// are orthogonal in the bilinear form x^T y; scaled to x^T x = 1 they give
// Q^T C Q = diag(lam), Q^T Q = I, and V = L^-T Q satisfies V^T M V = I,
// V^T S V = diag(lam). Clusters of equal eigenvalues (the mirror-image
// modes of two absorbing layers) get an orthonormal basis of their invariant
// subspace in that form. Both identities are checked before the result is
// used.
#include <algorithm>
#include <cmath>
#include <functional>

#include "fdm.h"

namespace tdz {

namespace {

using Mat = std::vector<cd>;   // n x n, row-major

// Householder reduction to upper Hessenberg form: A <- Z^H A Z, Z accumulated.
void to_hessenberg(Mat &A, Mat &Z, int n) {
    std::vector<cd> v(n), w(n);
    for (int k = 0; k + 2 < n; ++k) {
        double norm2 = 0.0;
        for (int i = k + 1; i < n; ++i) norm2 += std::norm(A[(size_t)i * n + k]);
        const double norm = std::sqrt(norm2);
        if (norm == 0.0) continue;
        const cd x0 = A[(size_t)(k + 1) * n + k];
        const cd phase = std::abs(x0) > 0.0 ? x0 / std::abs(x0) : cd(1.0);
        const cd alpha = -phase * norm;
        std::fill(v.begin(), v.end(), cd(0.0));
        for (int i = k + 1; i < n; ++i) v[i] = A[(size_t)i * n + k];
        v[k + 1] -= alpha;
        double vn2 = 0.0;
        for (int i = k + 1; i < n; ++i) vn2 += std::norm(v[i]);
        if (vn2 == 0.0) continue;
        const double vs = 1.0 / std::sqrt(vn2);
        for (int i = k + 1; i < n; ++i) v[i] *= vs;
        // A <- (I - 2 v v^H) A
        for (int j = 0; j < n; ++j) {
            cd s = 0.0;
            for (int i = k + 1; i < n; ++i) s += std::conj(v[i]) * A[(size_t)i * n + j];
            s *= 2.0;
            for (int i = k + 1; i < n; ++i) A[(size_t)i * n + j] -= v[i] * s;
        }
        // A <- A (I - 2 v v^H), Z <- Z (I - 2 v v^H)
        for (Mat *M : {&A, &Z})
            for (int i = 0; i < n; ++i) {
                cd s = 0.0;
                for (int j = k + 1; j < n; ++j) s += (*M)[(size_t)i * n + j] * v[j];
                s *= 2.0;
                for (int j = k + 1; j < n; ++j) (*M)[(size_t)i * n + j] -= s * std::conj(v[j]);
            }
        for (int i = k + 2; i < n; ++i) A[(size_t)i * n + k] = 0.0;
    }
}

// Givens rotation G = [c s; -conj(s) c] (c real) with G [x; y] = [r; 0].
void givens(cd x, cd y, double &c, cd &s) {
    const double ax = std::abs(x), r = std::hypot(ax, std::abs(y));
    if (r == 0.0) { c = 1.0; s = 0.0; return; }
    if (ax == 0.0) { c = 0.0; s = 1.0; return; }
    c = ax / r;
    s = (x / ax) * std::conj(y) / r;
}

// Complex Schur form of an upper Hessenberg H: H <- G H G^H sweeps until
// upper triangular, Z <- Z G^H.
void schur(Mat &H, Mat &Z, int n) {
    const double eps = 2.220446049250313e-16;
    int hi = n - 1, iter = 0, total = 0;
    while (hi > 0) {
        int l = hi;
        while (l > 0) {
            const double sub = std::abs(H[(size_t)l * n + l - 1]);
            const double diag = std::abs(H[(size_t)l * n + l]) + std::abs(H[(size_t)(l - 1) * n + l - 1]);
            if (sub <= eps * (diag > 0.0 ? diag : 1.0)) break;
            --l;
        }
        if (l > 0) H[(size_t)l * n + l - 1] = 0.0;
        if (l == hi) {
            --hi;
            iter = 0;
            continue;
        }
        TDZ_CHECK(++total <= 60 * n, TDZ_ERR_INTERNAL, "complex Schur iteration did not converge");
        // Wilkinson shift: the eigenvalue of the trailing 2x2 block closer to its last entry
        const cd a = H[(size_t)(hi - 1) * n + hi - 1], b = H[(size_t)(hi - 1) * n + hi];
        const cd c2 = H[(size_t)hi * n + hi - 1], d = H[(size_t)hi * n + hi];
        const cd half = 0.5 * (a + d), disc = std::sqrt(0.25 * (a - d) * (a - d) + b * c2);
        const cd m1 = half + disc, m2 = half - disc;
        cd mu = std::abs(m1 - d) < std::abs(m2 - d) ? m1 : m2;
        if (++iter % 12 == 0) mu = d + 0.75 * std::abs(c2);   // exceptional shift
        cd x = H[(size_t)l * n + l] - mu, y = H[(size_t)(l + 1) * n + l];
        for (int k = l; k < hi; ++k) {
            double c;
            cd s;
            givens(x, y, c, s);
            // rows k, k+1 (from column k-1, or l, to the right edge)
            for (int j = std::max(l, k - 1); j < n; ++j) {
                const cd hk = H[(size_t)k * n + j], hk1 = H[(size_t)(k + 1) * n + j];
                H[(size_t)k * n + j] = c * hk + s * hk1;
                H[(size_t)(k + 1) * n + j] = -std::conj(s) * hk + c * hk1;
            }
            // columns k, k+1 (from the top to row min(k+2, hi)), and of Z
            const int rmax = std::min(k + 2, hi);
            for (int i = 0; i <= rmax; ++i) {
                const cd hk = H[(size_t)i * n + k], hk1 = H[(size_t)i * n + k + 1];
                H[(size_t)i * n + k] = hk * c + hk1 * std::conj(s);
                H[(size_t)i * n + k + 1] = -hk * s + hk1 * c;
            }
            for (int i = 0; i < n; ++i) {
                const cd zk = Z[(size_t)i * n + k], zk1 = Z[(size_t)i * n + k + 1];
                Z[(size_t)i * n + k] = zk * c + zk1 * std::conj(s);
                Z[(size_t)i * n + k + 1] = -zk * s + zk1 * c;
            }
            if (k + 1 < hi) {
                x = H[(size_t)(k + 1) * n + k];
                y = H[(size_t)(k + 2) * n + k];
            }
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) H[(size_t)i * n + j] = 0.0;
}

}  // namespace

bool gen_eig_complex(const std::vector<cd> &S, int p, const BandD &M, std::vector<cd> &V, std::vector<cd> &lam) {
    const int n = M.n, bw = 2 * p + 1;
    TDZ_CHECK(M.p == p && S.size() == (size_t)n * bw, TDZ_ERR_INTERNAL, "band shapes differ");
    auto s_at = [&](int i, int j) { return std::abs(i - j) <= p ? S[(size_t)i * bw + (j - i + p)] : cd(0.0); };
    // M = L L^T (dense lower factor of the band)
    std::vector<double> L((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int j = std::max(0, i - p); j <= i; ++j) {
            double v = M.at(i, j);
            for (int k = std::max(0, i - p); k < j; ++k) v -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
            if (i == j) {
                TDZ_CHECK(v > 0, TDZ_ERR_INTERNAL, "mass band not positive definite");
                L[(size_t)i * n + i] = std::sqrt(v);
            } else L[(size_t)i * n + j] = v / L[(size_t)j * n + j];
        }
    // C = L^-1 S L^-T
    Mat W((size_t)n * n), C((size_t)n * n);
    for (int c = 0; c < n; ++c)
        for (int i = 0; i < n; ++i) {
            cd v = s_at(i, c);
            for (int k = std::max(0, i - p); k < i; ++k) v -= L[(size_t)i * n + k] * W[(size_t)k * n + c];
            W[(size_t)i * n + c] = v / L[(size_t)i * n + i];
        }
    for (int r = 0; r < n; ++r)
        for (int i = 0; i < n; ++i) {
            cd v = W[(size_t)r * n + i];
            for (int k = std::max(0, i - p); k < i; ++k) v -= L[(size_t)i * n + k] * C[(size_t)r * n + k];
            C[(size_t)r * n + i] = v / L[(size_t)i * n + i];
        }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) C[(size_t)i * n + j] = C[(size_t)j * n + i] = 0.5 * (C[(size_t)i * n + j] + C[(size_t)j * n + i]);
    const Mat C0 = C;
    double cnorm = 0.0;
    for (const cd &v : C0) cnorm = std::max(cnorm, std::abs(v));

    Mat Z((size_t)n * n, cd(0.0));
    for (int i = 0; i < n; ++i) Z[(size_t)i * n + i] = 1.0;
    to_hessenberg(C, Z, n);
    schur(C, Z, n);

    // eigenvectors of T by back-substitution, then Q = Z Y
    lam.resize(n);
    for (int k = 0; k < n; ++k) lam[k] = C[(size_t)k * n + k];
    const double small = 1e-14 * std::max(cnorm, 1e-300);
    Mat Q((size_t)n * n, cd(0.0));
    std::vector<cd> y(n);
    for (int k = 0; k < n; ++k) {
        std::fill(y.begin(), y.end(), cd(0.0));
        y[k] = 1.0;
        for (int i = k - 1; i >= 0; --i) {
            cd sum = 0.0;
            for (int j = i + 1; j <= k; ++j) sum += C[(size_t)i * n + j] * y[j];
            cd den = C[(size_t)i * n + i] - lam[k];
            if (std::abs(den) < small) den = small;
            y[i] = -sum / den;
        }
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) {
            cd v = 0.0;
            for (int j = 0; j <= k; ++j) v += Z[(size_t)i * n + j] * y[j];
            Q[(size_t)i * n + k] = v;
            nrm += std::norm(v);
        }
        nrm = 1.0 / std::sqrt(nrm);
        for (int i = 0; i < n; ++i) Q[(size_t)i * n + k] *= nrm;
    }
    auto col_dot = [&](int a, int b) {   // bilinear q_a^T q_b
        cd g = 0.0;
        for (int i = 0; i < n; ++i) g += Q[(size_t)i * n + a] * Q[(size_t)i * n + b];
        return g;
    };
    // Clusters of (nearly) equal eigenvalues: mirror-image modes of the two
    // absorbing layers come in pairs whose splitting is at rounding level, so
    // the computed vectors of a pair are arbitrary mixtures. Each cluster
    // gets a bilinear-orthonormal basis of its invariant subspace (pivoted
    // Gram-Schmidt in the form x^T y), and the cluster block Q_c^T C Q_c is
    // diagonalised by complex symmetric Jacobi rotations.
    std::vector<int> cl(n);
    for (int k = 0; k < n; ++k) cl[k] = k;
    std::function<int(int)> root = [&](int k) { return cl[k] == k ? k : cl[k] = root(cl[k]); };
    for (int a = 0; a < n; ++a)
        for (int b = a + 1; b < n; ++b)
            if (std::abs(lam[a] - lam[b]) <= 1e-6 * std::max({std::abs(lam[a]), std::abs(lam[b]), 1e-300}))
                cl[root(a)] = root(b);
    double coupling = 0.0;   // largest off-diagonal entry left in a cluster block
    std::vector<std::vector<int>> groups(n);
    for (int k = 0; k < n; ++k) groups[root(k)].push_back(k);
    for (const std::vector<int> &g : groups) {
        if (g.empty()) continue;
        const int m = (int)g.size();
        // pivoted bilinear Gram-Schmidt
        std::vector<int> left = g, done;
        while (!left.empty()) {
            int best = -1;
            double bq = -1.0;
            for (int k : left) {
                double nn = 0.0;
                for (int i = 0; i < n; ++i) nn += std::norm(Q[(size_t)i * n + k]);
                const double r = std::abs(col_dot(k, k)) / std::max(nn, 1e-300);
                if (r > bq) { bq = r; best = k; }
            }
            if (!(bq > 1e-6)) return false;   // isotropic subspace: no bilinear-orthonormal basis
            const cd sc = 1.0 / std::sqrt(col_dot(best, best));
            for (int i = 0; i < n; ++i) Q[(size_t)i * n + best] *= sc;
            left.erase(std::find(left.begin(), left.end(), best));
            for (int k : left) {
                const cd h = col_dot(best, k);
                for (int i = 0; i < n; ++i) Q[(size_t)i * n + k] -= h * Q[(size_t)i * n + best];
            }
            done.push_back(best);
        }
        if (m == 1) continue;
        // G = Q_c^T C0 Q_c, diagonalised by rotations R = [c s; -s c], c^2 + s^2 = 1
        Mat G((size_t)m * m), CQ((size_t)n * m);
        for (int b = 0; b < m; ++b)
            for (int i = 0; i < n; ++i) {
                cd v = 0.0;
                for (int j = 0; j < n; ++j) v += C0[(size_t)i * n + j] * Q[(size_t)j * n + g[b]];
                CQ[(size_t)i * m + b] = v;
            }
        for (int a = 0; a < m; ++a)
            for (int b = 0; b < m; ++b) {
                cd v = 0.0;
                for (int i = 0; i < n; ++i) v += Q[(size_t)i * n + g[a]] * CQ[(size_t)i * m + b];
                G[(size_t)a * m + b] = v;
            }
        for (int a = 0; a < m; ++a)
            for (int b = 0; b < a; ++b) G[(size_t)a * m + b] = G[(size_t)b * m + a] = 0.5 * (G[(size_t)a * m + b] + G[(size_t)b * m + a]);
        // near an exceptional point (coalescing eigenvectors) the rotations
        // blow up: the cluster then keeps its orthonormal basis and the
        // diagonal of G, and the off-diagonal coupling (at most the
        // cluster's eigenvalue spread) is left to the Krylov method
        const Mat G0 = G;
        Mat Qsave((size_t)n * m);
        for (int b = 0; b < m; ++b)
            for (int i = 0; i < n; ++i) Qsave[(size_t)i * m + b] = Q[(size_t)i * n + g[b]];
        bool ep = false;
        for (int sweep = 0; sweep < 30 && !ep; ++sweep) {
            double off = 0.0, tot = 0.0;
            for (int a = 0; a < m; ++a)
                for (int b = 0; b < m; ++b) {
                    tot += std::norm(G[(size_t)a * m + b]);
                    if (a != b) off += std::norm(G[(size_t)a * m + b]);
                }
            if (off <= 1e-28 * tot) break;
            for (int pa = 0; pa < m - 1 && !ep; ++pa) {
                for (int qa = pa + 1; qa < m; ++qa) {
                    const cd gpq = G[(size_t)pa * m + qa];
                    // rounding-level coupling of (numerically) equal eigenvalues: nothing to rotate
                    if (std::abs(gpq) <= 1e-14 * (std::abs(G[(size_t)pa * m + pa]) + std::abs(G[(size_t)qa * m + qa])))
                        continue;
                    const cd dg = G[(size_t)pa * m + pa] - G[(size_t)qa * m + qa];
                    const cd root2 = std::sqrt(dg * dg + 4.0 * gpq * gpq);
                    const cd den = std::abs(dg + root2) >= std::abs(dg - root2) ? dg + root2 : dg - root2;
                    const cd t = std::abs(den) > 0.0 ? 2.0 * gpq / den : cd(0.0);   // smaller root of gpq t^2 - dg t - gpq
                    const cd w = 1.0 + t * t;
                    if (!(std::abs(den) > 0.0) || std::abs(w) < 1e-3 || std::abs(t) > 1e3) {
                        ep = true;
                        break;
                    }
                    const cd c = 1.0 / std::sqrt(w), sn = t * c;
                    // G <- R^T G R, Q_c <- Q_c R
                    for (int k = 0; k < m; ++k) {
                        const cd gkp = G[(size_t)k * m + pa], gkq = G[(size_t)k * m + qa];
                        G[(size_t)k * m + pa] = c * gkp - sn * gkq;
                        G[(size_t)k * m + qa] = sn * gkp + c * gkq;
                    }
                    for (int k = 0; k < m; ++k) {
                        const cd gpk = G[(size_t)pa * m + k], gqk = G[(size_t)qa * m + k];
                        G[(size_t)pa * m + k] = c * gpk - sn * gqk;
                        G[(size_t)qa * m + k] = sn * gpk + c * gqk;
                    }
                    for (int i = 0; i < n; ++i) {
                        const cd qp = Q[(size_t)i * n + g[pa]], qq = Q[(size_t)i * n + g[qa]];
                        Q[(size_t)i * n + g[pa]] = c * qp - sn * qq;
                        Q[(size_t)i * n + g[qa]] = sn * qp + c * qq;
                    }
                }
            }
        }
        if (ep) {
            G = G0;
            for (int b = 0; b < m; ++b)
                for (int i = 0; i < n; ++i) Q[(size_t)i * n + g[b]] = Qsave[(size_t)i * m + b];
            for (int a = 0; a < m; ++a)
                for (int b = 0; b < m; ++b)
                    if (a != b) coupling = std::max(coupling, std::abs(G[(size_t)a * m + b]));
        }
        for (int a = 0; a < m; ++a) lam[g[a]] = G[(size_t)a * m + a];
    }
    // checks: Q^T Q = I and C Q = Q diag(lam)
    double orth = 0.0, res = 0.0;
    for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) {
            cd g = 0.0, r = 0.0;
            for (int i = 0; i < n; ++i) {
                g += Q[(size_t)i * n + a] * Q[(size_t)i * n + b];
                r += C0[(size_t)a * n + i] * Q[(size_t)i * n + b];
            }
            orth = std::max(orth, std::abs(g - (a == b ? cd(1.0) : cd(0.0))));
            res = std::max(res, std::abs(r - Q[(size_t)a * n + b] * lam[b]));
        }
    if (!(coupling <= 1e-6 * std::max(cnorm, 1e-300))) return false;
    if (!(orth <= 1e-6) || !(res <= 1e-10 * std::max(cnorm, 1e-300) * std::sqrt((double)n) + 2.0 * coupling))
        return false;
    // V = L^-T Q (back-substitution with L^T, column by column)
    V.assign((size_t)n * n, cd(0.0));
    for (int c = 0; c < n; ++c)
        for (int i = n - 1; i >= 0; --i) {
            cd v = Q[(size_t)i * n + c];
            for (int k = i + 1; k <= std::min(n - 1, i + p); ++k) v -= L[(size_t)k * n + i] * V[(size_t)k * n + c];
            V[(size_t)i * n + c] = v / L[(size_t)i * n + i];
        }
    return true;
}

}  // namespace tdz

// Cyclic complex Jacobi eigensolver for small Hermitian matrices.
#include "host_eig.h"

#include <algorithm>
#include <cmath>
#include <numeric>

// Eigen-decomposition of a Hermitian n x n matrix (column-major, A[j * n + i]
// = A(i, j)) by cyclic complex Jacobi rotations: each rotation is the phase
// that makes A(p, q) real followed by the real Jacobi rotation that zeroes
// it.  Eigenvalues ascending; column c of vecs is the unit eigenvector.
void hermitian_eig(int n, std::vector<std::complex<double>> A, std::vector<double>& vals,
                   std::vector<std::complex<double>>& vecs) {
    using C = std::complex<double>;
    std::vector<C> V((size_t)n * n, C(0, 0));
    for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
    auto a = [&](int i, int j) -> C& { return A[(size_t)j * n + i]; };
    double fro = 0;
    for (auto& z : A) fro += std::norm(z);
    fro = std::sqrt(fro);
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0;
        for (int q = 0; q < n; ++q)
            for (int p = 0; p < q; ++p) off += std::norm(a(p, q));
        if (std::sqrt(off) <= 1e-16 * fro || fro == 0) break;
        for (int q = 1; q < n; ++q) {
            for (int p = 0; p < q; ++p) {
                const C apq = a(p, q);
                const double h = std::abs(apq);
                if (h <= 1e-300) continue;
                const C ph = apq / h;  // e^{i phi}
                const double app = a(p, p).real(), aqq = a(q, q).real();
                const double theta = (aqq - app) / (2 * h);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::abs(theta) + std::sqrt(theta * theta + 1));
                const double c = 1 / std::sqrt(t * t + 1), s = t * c;
                // R on (p, q): R_pp = c, R_pq = s, R_qp = -s conj(ph), R_qq = c conj(ph)
                const C rpp = c, rpq = s, rqp = -s * std::conj(ph), rqq = c * std::conj(ph);
                for (int i = 0; i < n; ++i) {  // columns: A <- A R
                    const C x = a(i, p), y = a(i, q);
                    a(i, p) = x * rpp + y * rqp;
                    a(i, q) = x * rpq + y * rqq;
                }
                for (int j = 0; j < n; ++j) {  // rows: A <- R^H A
                    const C x = a(p, j), y = a(q, j);
                    a(p, j) = std::conj(rpp) * x + std::conj(rqp) * y;
                    a(q, j) = std::conj(rpq) * x + std::conj(rqq) * y;
                }
                a(p, q) = 0.0;
                a(q, p) = 0.0;
                for (int i = 0; i < n; ++i) {
                    const C x = V[(size_t)p * n + i], y = V[(size_t)q * n + i];
                    V[(size_t)p * n + i] = x * rpp + y * rqp;
                    V[(size_t)q * n + i] = x * rpq + y * rqq;
                }
            }
        }
    }
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](int x, int y) { return a(x, x).real() < a(y, y).real(); });
    vals.resize(n);
    vecs.assign((size_t)n * n, C(0, 0));
    for (int c = 0; c < n; ++c) {
        vals[c] = a(idx[c], idx[c]).real();
        for (int i = 0; i < n; ++i) vecs[(size_t)c * n + i] = V[(size_t)idx[c] * n + i];
    }
}

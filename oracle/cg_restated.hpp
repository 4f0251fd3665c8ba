// Restatement of the Jacobi-preconditioned conjugate gradient that
// Eigen::ConjugateGradient<SparseMatrix<double>> runs with its defaults
// (reference call site: src/mps.cpp:452-460).  TEST INFRASTRUCTURE ONLY.
//
// Third-party dependency: Eigen (https://gitlab.com/libeigen/eigen.git, the
// reference's submodule is empty so its pinned commit is unknown).  The
// published algorithm restated here, in this project's own code:
//   * zero initial guess (solve() without a guess);
//   * diagonal (Jacobi) preconditioner: 1/a_jj, or 1 where the diagonal is
//     missing or zero;
//   * stop when ||r||^2 < max(tol^2 ||b||^2, DBL_MIN) on the recursively
//     updated residual, or after max_iter iterations (default 2n);
//   * return immediately with x = 0 when ||b|| = 0.
// The matrix is symmetric by construction, so y = A p is evaluated over the
// full rows instead of Eigen's lower-triangle self-adjoint view; the result
// differs from Eigen only in summation order.
#pragma once
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <vector>

namespace orc {

struct CgResult {
    int64_t iterations = 0;
    double error = 0.0;
};

// CSR with ascending columns inside each row.
inline CgResult cg_restated(int64_t n, const int64_t* row_ptr, const int32_t* col,
                            const double* val, const double* b, double* x, double tol,
                            int64_t max_iter) {
    CgResult res;
    std::vector<double> r(n), p(n), z(n), q(n), inv_diag(n);
    for (int64_t i = 0; i < n; i++) {
        double d = 0.0;
        bool found = false;
        for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; k++)
            if (col[k] == i) {
                d = val[k];
                found = true;
                break;
            }
        inv_diag[i] = (found && d != 0.0) ? 1.0 / d : 1.0;
    }
    double rhs_norm2 = 0.0;
    for (int64_t i = 0; i < n; i++) {
        x[i] = 0.0;
        r[i] = b[i];
        rhs_norm2 += b[i] * b[i];
    }
    if (rhs_norm2 == 0.0) return res;
    double threshold = std::max(tol * tol * rhs_norm2, DBL_MIN);
    double r_norm2 = rhs_norm2;
    if (r_norm2 < threshold) {
        res.error = std::sqrt(r_norm2 / rhs_norm2);
        return res;
    }
    double abs_new = 0.0;
    for (int64_t i = 0; i < n; i++) {
        p[i] = inv_diag[i] * r[i];
        abs_new += r[i] * p[i];
    }
    int64_t it = 0;
    while (it < max_iter) {
        double pq = 0.0;
        for (int64_t i = 0; i < n; i++) {
            double s = 0.0;
            for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; k++) s += val[k] * p[col[k]];
            q[i] = s;
            pq += p[i] * s;
        }
        double alpha = abs_new / pq;
        r_norm2 = 0.0;
        for (int64_t i = 0; i < n; i++) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
            r_norm2 += r[i] * r[i];
        }
        if (r_norm2 < threshold) break;
        double abs_old = abs_new;
        abs_new = 0.0;
        for (int64_t i = 0; i < n; i++) {
            z[i] = inv_diag[i] * r[i];
            abs_new += r[i] * z[i];
        }
        double beta = abs_new / abs_old;
        for (int64_t i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
        it++;
    }
    res.iterations = it;
    res.error = std::sqrt(r_norm2 / rhs_norm2);
    return res;
}

}  // namespace orc

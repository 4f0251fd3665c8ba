// Stand-in for the parts of Eigen that the reference's hot-path sources use
// (src/mps.cpp, src/mps.hpp, src/particle.hpp, src/settings.hpp).  TEST
// INFRASTRUCTURE ONLY: it lets oracle/ compile those sources unmodified so
// that they can produce golden vectors for the oracle restatement.  This is
// project-written code, not Eigen: fixed 3-vectors with component-wise
// IEEE operations in the order the expressions are written, a triplet-built
// sparse matrix, and a restatement of Eigen's published Jacobi-CG algorithm.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../cg_restated.hpp"

namespace Eigen {

enum ComputationInfo { Success = 0, NumericalIssue = 1, NoConvergence = 2, InvalidInput = 3 };
enum StorageOptions { ColMajor = 0, RowMajor = 1 };

class Vector3d {
public:
    double v[3];
    Vector3d() : v{0.0, 0.0, 0.0} {}
    Vector3d(double a, double b, double c) : v{a, b, c} {}
    static Vector3d Zero() { return Vector3d(0.0, 0.0, 0.0); }
    void setZero() { v[0] = v[1] = v[2] = 0.0; }
    double& x() { return v[0]; }
    double& y() { return v[1]; }
    double& z() { return v[2]; }
    double x() const { return v[0]; }
    double y() const { return v[1]; }
    double z() const { return v[2]; }
    // (x + y) + z, the summation order the oracle restatement also uses
    double squaredNorm() const { return (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]; }
    double norm() const { return std::sqrt(squaredNorm()); }
    double dot(const Vector3d& o) const { return (v[0] * o.v[0] + v[1] * o.v[1]) + v[2] * o.v[2]; }
    Vector3d normalized() const {
        double z2 = squaredNorm();
        if (z2 > 0.0) {
            double r = std::sqrt(z2);
            return Vector3d(v[0] / r, v[1] / r, v[2] / r);
        }
        return *this;
    }
    Vector3d& operator+=(const Vector3d& o) { v[0] += o.v[0]; v[1] += o.v[1]; v[2] += o.v[2]; return *this; }
    Vector3d& operator-=(const Vector3d& o) { v[0] -= o.v[0]; v[1] -= o.v[1]; v[2] -= o.v[2]; return *this; }
    Vector3d& operator*=(double s) { v[0] *= s; v[1] *= s; v[2] *= s; return *this; }
};
inline Vector3d operator+(const Vector3d& a, const Vector3d& b) { return Vector3d(a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]); }
inline Vector3d operator-(const Vector3d& a, const Vector3d& b) { return Vector3d(a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]); }
inline Vector3d operator*(const Vector3d& a, double s) { return Vector3d(a.v[0] * s, a.v[1] * s, a.v[2] * s); }
inline Vector3d operator*(double s, const Vector3d& a) { return Vector3d(s * a.v[0], s * a.v[1], s * a.v[2]); }
inline Vector3d operator/(const Vector3d& a, double s) { return Vector3d(a.v[0] / s, a.v[1] / s, a.v[2] / s); }

class VectorXd {
public:
    std::vector<double> d;
    VectorXd() = default;
    explicit VectorXd(int64_t n) : d(n, 0.0) {}
    void resize(int64_t n) { d.assign(n, 0.0); }
    int64_t size() const { return (int64_t)d.size(); }
    double& operator[](int64_t i) { return d[i]; }
    double operator[](int64_t i) const { return d[i]; }
    double& operator()(int64_t i) { return d[i]; }
};

template <typename Scalar>
class Triplet {
public:
    int64_t r, c;
    Scalar v;
    Triplet(int64_t r_, int64_t c_, Scalar v_) : r(r_), c(c_), v(v_) {}
    int64_t row() const { return r; }
    int64_t col() const { return c; }
    Scalar value() const { return v; }
};

// Compressed by rows regardless of the requested storage order; the hot path
// only builds it from triplets, edits single coefficients and hands it to CG.
template <typename Scalar, int Options = ColMajor>
class SparseMatrix {
public:
    int64_t nrows = 0, ncols = 0;
    std::vector<int64_t> outer{0};
    std::vector<int32_t> inner;
    std::vector<Scalar> values;

    SparseMatrix() = default;
    SparseMatrix(int64_t r, int64_t c) { resize(r, c); }
    template <int O2>
    SparseMatrix(const SparseMatrix<Scalar, O2>& o)
        : nrows(o.nrows), ncols(o.ncols), outer(o.outer), inner(o.inner), values(o.values) {}
    void resize(int64_t r, int64_t c) {
        nrows = r;
        ncols = c;
        outer.assign(r + 1, 0);
        inner.clear();
        values.clear();
    }
    int64_t rows() const { return nrows; }
    int64_t cols() const { return ncols; }
    template <typename It>
    void setFromTriplets(It begin, It end) {
        std::vector<std::vector<std::pair<int32_t, Scalar>>> rowsv(nrows);
        for (It it = begin; it != end; ++it) rowsv[it->row()].push_back({(int32_t)it->col(), it->value()});
        outer.assign(nrows + 1, 0);
        inner.clear();
        values.clear();
        for (int64_t i = 0; i < nrows; i++) {
            auto& rv = rowsv[i];
            std::stable_sort(rv.begin(), rv.end(), [](auto& a, auto& b) { return a.first < b.first; });
            for (size_t k = 0; k < rv.size(); k++) {
                if (k > 0 && rv[k].first == rv[k - 1].first) {
                    values.back() += rv[k].second;  // duplicates are summed
                    continue;
                }
                inner.push_back(rv[k].first);
                values.push_back(rv[k].second);
            }
            outer[i + 1] = (int64_t)inner.size();
        }
    }
    Scalar coeff(int64_t i, int64_t j) const {
        for (int64_t k = outer[i]; k < outer[i + 1]; k++)
            if (inner[k] == j) return values[k];
        return Scalar(0);
    }
    Scalar& coeffRef(int64_t i, int64_t j) {
        for (int64_t k = outer[i]; k < outer[i + 1]; k++)
            if (inner[k] == j) return values[k];
        // insertion keeps the row sorted
        int64_t k = outer[i];
        while (k < outer[i + 1] && inner[k] < j) k++;
        inner.insert(inner.begin() + k, (int32_t)j);
        values.insert(values.begin() + k, Scalar(0));
        for (int64_t r = i + 1; r <= nrows; r++) outer[r]++;
        return values[k];
    }
    SparseMatrix transpose() const {
        std::vector<Triplet<Scalar>> t;
        for (int64_t i = 0; i < nrows; i++)
            for (int64_t k = outer[i]; k < outer[i + 1]; k++) t.emplace_back(inner[k], i, values[k]);
        SparseMatrix m(ncols, nrows);
        m.setFromTriplets(t.begin(), t.end());
        return m;
    }
    double squaredNorm() const {
        double s = 0;
        for (auto v : values) s += v * v;
        return s;
    }
    // Eigen's isApprox: ||a - b||^2 <= prec^2 * min(||a||^2, ||b||^2), prec = 1e-12
    bool isApprox(const SparseMatrix& o) const {
        if (nrows != o.nrows || ncols != o.ncols) return false;
        double diff = 0.0;
        for (int64_t i = 0; i < nrows; i++) {
            int64_t a = outer[i], b = o.outer[i];
            while (a < outer[i + 1] || b < o.outer[i + 1]) {
                if (b >= o.outer[i + 1] || (a < outer[i + 1] && inner[a] < o.inner[b])) {
                    diff += values[a] * values[a];
                    a++;
                } else if (a >= outer[i + 1] || o.inner[b] < inner[a]) {
                    diff += o.values[b] * o.values[b];
                    b++;
                } else {
                    double d = values[a] - o.values[b];
                    diff += d * d;
                    a++;
                    b++;
                }
            }
        }
        double prec = 1e-12;
        return diff <= prec * prec * std::min(squaredNorm(), o.squaredNorm());
    }
};

template <typename MatrixType>
class ConjugateGradient {
public:
    SparseMatrix<double, RowMajor> A;
    int64_t iters = 0;
    double err = 0.0;
    ComputationInfo inf = Success;
    template <typename M>
    void compute(const M& m) {
        A = SparseMatrix<double, RowMajor>(m);
    }
    VectorXd solve(const VectorXd& b) {
        VectorXd x(A.rows());
        orc::CgResult r = orc::cg_restated(A.rows(), A.outer.data(), A.inner.data(), A.values.data(),
                                           b.d.data(), x.d.data(), 2.220446049250313e-16, 2 * A.cols());
        iters = r.iterations;
        err = r.error;
        inf = (r.error <= 2.220446049250313e-16) ? Success : NoConvergence;
        return x;
    }
    ComputationInfo info() const { return inf; }
    int64_t iterations() const { return iters; }
    double error() const { return err; }
};

}  // namespace Eigen

// Vec3: the subset of Eigen::Vector3d that the reference's classes expose
// (src/particle.hpp:33-34, src/settings.hpp:54).  Component-wise IEEE
// arithmetic; norm and dot sum as (x + y) + z.
#pragma once
#include <cmath>

class Vec3 {
public:
    double v[3] = {0.0, 0.0, 0.0};
    Vec3() = default;
    Vec3(double x, double y, double z) : v{x, y, z} {}
    static Vec3 Zero() { return Vec3(); }
    void setZero() { v[0] = v[1] = v[2] = 0.0; }
    double& x() { return v[0]; }
    double& y() { return v[1]; }
    double& z() { return v[2]; }
    double x() const { return v[0]; }
    double y() const { return v[1]; }
    double z() const { return v[2]; }
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
    double squaredNorm() const { return (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]; }
    double norm() const { return std::sqrt(squaredNorm()); }
    double dot(const Vec3& o) const { return (v[0] * o.v[0] + v[1] * o.v[1]) + v[2] * o.v[2]; }
    Vec3 normalized() const {
        double z2 = squaredNorm();
        if (z2 > 0.0) {
            double r = std::sqrt(z2);
            return Vec3(v[0] / r, v[1] / r, v[2] / r);
        }
        return *this;
    }
    Vec3& operator+=(const Vec3& o) {
        for (int i = 0; i < 3; i++) v[i] += o.v[i];
        return *this;
    }
    Vec3& operator-=(const Vec3& o) {
        for (int i = 0; i < 3; i++) v[i] -= o.v[i];
        return *this;
    }
    Vec3& operator*=(double s) {
        for (double& c : v) c *= s;
        return *this;
    }
    friend Vec3 operator+(const Vec3& a, const Vec3& b) { return Vec3(a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]); }
    friend Vec3 operator-(const Vec3& a, const Vec3& b) { return Vec3(a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]); }
    friend Vec3 operator*(const Vec3& a, double s) { return Vec3(a.v[0] * s, a.v[1] * s, a.v[2] * s); }
    friend Vec3 operator*(double s, const Vec3& a) { return Vec3(s * a.v[0], s * a.v[1], s * a.v[2]); }
    friend Vec3 operator/(const Vec3& a, double s) { return Vec3(a.v[0] / s, a.v[1] / s, a.v[2] / s); }
};

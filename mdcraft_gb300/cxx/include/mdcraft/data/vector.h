// Drop-in data types for MDcraft's C++ API over libmdg.
//
// mdcraft::data::vector / matrix are the 3-vector and 3x3 matrix of
// mdcraft/data/vector.h:7 and mdcraft/data/matrix.h:7 (Eigen fixed-size
// types in the reference). These are small own types with the same storage
// (3 doubles; 9 doubles column-major) and the subset of the Eigen API that
// MDcraft callers use on atoms: comma initialisation, (i), [i], x()/y()/z(),
// squaredNorm, norm, dot, arithmetic, Zero/Identity, trace, isZero.
#pragma once

#include <cmath>
#include <cstddef>

namespace mdcraft {
namespace data {

class vector {
public:
    vector() = default;
    vector(double x, double y, double z) : v_{x, y, z} {}

    static vector Zero() { return vector(0.0, 0.0, 0.0); }

    double& operator()(int i) { return v_[i]; }
    double operator()(int i) const { return v_[i]; }
    double& operator[](int i) { return v_[i]; }
    double operator[](int i) const { return v_[i]; }
    double& x() { return v_[0]; }
    double& y() { return v_[1]; }
    double& z() { return v_[2]; }
    double x() const { return v_[0]; }
    double y() const { return v_[1]; }
    double z() const { return v_[2]; }
    double* data() { return v_; }
    const double* data() const { return v_; }

    // ((x*x + y*y) + z*z), the order of a 3-term Eigen reduction
    double squaredNorm() const { return v_[0] * v_[0] + v_[1] * v_[1] + v_[2] * v_[2]; }
    double norm() const { return std::sqrt(squaredNorm()); }
    double dot(const vector& o) const { return v_[0] * o.v_[0] + v_[1] * o.v_[1] + v_[2] * o.v_[2]; }
    bool isZero(double eps = 0.0) const {
        return std::fabs(v_[0]) <= eps && std::fabs(v_[1]) <= eps && std::fabs(v_[2]) <= eps;
    }

    vector& operator+=(const vector& o) { for (int i = 0; i < 3; ++i) v_[i] += o.v_[i]; return *this; }
    vector& operator-=(const vector& o) { for (int i = 0; i < 3; ++i) v_[i] -= o.v_[i]; return *this; }
    vector& operator*=(double s) { for (int i = 0; i < 3; ++i) v_[i] *= s; return *this; }
    vector& operator/=(double s) { for (int i = 0; i < 3; ++i) v_[i] /= s; return *this; }
    friend vector operator+(vector a, const vector& b) { return a += b; }
    friend vector operator-(vector a, const vector& b) { return a -= b; }
    friend vector operator-(vector a) { return a *= -1.0; }
    friend vector operator*(vector a, double s) { return a *= s; }
    friend vector operator*(double s, vector a) { return a *= s; }
    friend vector operator/(vector a, double s) { return a /= s; }

    // comma initialiser: v << x, y, z;
    class Comma {
    public:
        Comma(vector& v, double x) : v_(v), i_(1) { v_.v_[0] = x; }
        Comma& operator,(double x) {
            if (i_ < 3) v_.v_[i_++] = x;
            return *this;
        }

    private:
        vector& v_;
        int i_;
    };
    Comma operator<<(double x) { return Comma(*this, x); }

private:
    double v_[3] = {0.0, 0.0, 0.0};
};

class matrix {
public:
    matrix() = default;
    static matrix Zero() { return matrix(); }
    static matrix Identity() {
        matrix m;
        m(0, 0) = m(1, 1) = m(2, 2) = 1.0;
        return m;
    }
    double& operator()(int r, int c) { return m_[r + 3 * c]; }
    double operator()(int r, int c) const { return m_[r + 3 * c]; }
    double trace() const { return m_[0] + m_[4] + m_[8]; }
    double* data() { return m_; }
    const double* data() const { return m_; }
    bool isZero(double eps = 0.0) const {
        for (double x : m_)
            if (std::fabs(x) > eps) return false;
        return true;
    }
    matrix& operator+=(const matrix& o) { for (int i = 0; i < 9; ++i) m_[i] += o.m_[i]; return *this; }
    matrix& operator*=(double s) { for (int i = 0; i < 9; ++i) m_[i] *= s; return *this; }
    friend matrix operator+(matrix a, const matrix& b) { return a += b; }
    friend matrix operator*(double s, matrix a) { return a *= s; }

private:
    double m_[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // column-major
};

}  // namespace data
}  // namespace mdcraft

// Oracle (test infrastructure only): FP64 CPU restatement of ptarmigan's
// geometry module.  Used by tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg as the checker; never linked into the product library.
//
// Follows src/geometry/four_vector.rs:22-110, three_vector.rs:24-130 and
// polarization.rs:44-155 (metric (+,-,-,-), Stokes vector [I,Q,U,V]).
#pragma once
#include <cmath>
#include <cassert>

namespace orc {

struct V3 {
    double x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(double a, double b, double c) : x(a), y(b), z(c) {}
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    V3 operator+(const V3& o) const { return V3(x + o.x, y + o.y, z + o.z); }
    V3 operator-(const V3& o) const { return V3(x - o.x, y - o.y, z - o.z); }
    V3 operator-() const { return V3(-x, -y, -z); }
    double operator*(const V3& o) const { return x * o.x + y * o.y + z * o.z; }
    V3 operator*(double s) const { return V3(x * s, y * s, z * s); }
    V3 operator/(double s) const { return V3(x / s, y / s, z / s); }
    V3 cross(const V3& o) const {
        return V3(y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x);
    }
    double norm_sqr() const { return (*this) * (*this); }
    V3 normalize() const {
        double mag = std::sqrt(norm_sqr());
        return (*this) / mag;
    }
    // three_vector.rs:77-95 (right-handed rotation about a unit axis)
    V3 rotate_around(const V3& a, double theta) const {
        double s = std::sin(theta), c = std::cos(theta);
        return V3((c + a.x * a.x * (1.0 - c)) * x + (a.x * a.y * (1.0 - c) - a.z * s) * y +
                      (a.x * a.z * (1.0 - c) + a.y * s) * z,
                  (a.y * a.x * (1.0 - c) + a.z * s) * x + (c + a.y * a.y * (1.0 - c)) * y +
                      (a.y * a.z * (1.0 - c) - a.x * s) * z,
                  (a.z * a.x * (1.0 - c) - a.y * s) * x + (a.z * a.y * (1.0 - c) + a.x * s) * y +
                      (c + a.z * a.z * (1.0 - c)) * z);
    }
    // three_vector.rs:111-119
    V3 rotate_around_z(double theta) const {
        double s = std::sin(theta), c = std::cos(theta);
        return V3(c * x - s * y, c * y + s * x, z);
    }
    V3 rotate_around_y(double theta) const { return rotate_around(V3(0, 1, 0), theta); }
};
inline V3 operator*(double s, const V3& v) { return v * s; }

struct V4 {
    double t, x, y, z;
    V4() : t(0), x(0), y(0), z(0) {}
    V4(double a, double b, double c, double d) : t(a), x(b), y(c), z(d) {}
    double operator[](int i) const { return i == 0 ? t : (i == 1 ? x : (i == 2 ? y : z)); }
    V4 operator+(const V4& o) const { return V4(t + o.t, x + o.x, y + o.y, z + o.z); }
    V4 operator-(const V4& o) const { return V4(t - o.t, x - o.x, y - o.y, z - o.z); }
    double operator*(const V4& o) const { return t * o.t - x * o.x - y * o.y - z * o.z; }
    V4 operator*(double s) const { return V4(t * s, x * s, y * s, z * s); }
    V4 operator/(double s) const { return V4(t / s, x / s, y / s, z / s); }
    V3 spatial() const { return V3(x, y, z); }
    // four_vector.rs:37-45
    V4 unitize() const { return V4(std::sqrt(1.0 + x * x + y * y + z * z), x, y, z); }
    static V4 lightlike(double x, double y, double z) {
        return V4(std::sqrt(x * x + y * y + z * z), x, y, z);
    }
    // four_vector.rs:96-106
    V4 rotate_around_z(double theta) const {
        double s = std::sin(theta), c = std::cos(theta);
        return V4(t, c * x - s * y, c * y + s * x, z);
    }
    // four_vector.rs:68-81
    V4 boost_by(const V4& u) const {
        double gamma = u.t;
        double beta = std::sqrt(1.0 - 1.0 / (gamma * gamma));
        V3 n = u.spatial().normalize();
        double a = t;
        V3 zz = spatial();
        double nz = n * zz;
        return V4(gamma * (a - beta * nz), zz.x + (gamma - 1.0) * nz * n.x - gamma * beta * a * n.x,
                  zz.y + (gamma - 1.0) * nz * n.y - gamma * beta * a * n.y,
                  zz.z + (gamma - 1.0) * nz * n.z - gamma * beta * a * n.z);
    }
};
inline V4 operator*(double s, const V4& v) { return v * s; }

inline double signum(double v) {
    // Rust f64::signum: 1.0 for +0.0 and positive, -1.0 for -0.0 and negative
    return std::signbit(v) ? -1.0 : 1.0;
}

struct Stokes {
    double i, q, u, v;
    Stokes() : i(1), q(0), u(0), v(0) {}
    Stokes(double a, double b, double c, double d) : i(a), q(b), u(c), v(d) {}
    double operator[](int k) const { return k == 0 ? i : (k == 1 ? q : (k == 2 ? u : v)); }
    static Stokes unpolarized() { return Stokes(1, 0, 0, 0); }
    // polarization.rs:44-52
    Stokes rotate_by(double theta) const {
        double s = std::sin(2.0 * theta), c = std::cos(2.0 * theta);
        return Stokes(i, c * q + s * u, -s * q + c * u, v);
    }
    // polarization.rs:58-97: Stokes parameters in the basis whose principal
    // axis is `a` (perpendicular to `k`); returns cos 2θ and sin 2θ too.
    Stokes in_basis(const V3& a, const V3& k, double* cos_2theta, double* sin_2theta) const {
        double k_mag = std::hypot(k.x, k.z);
        double a_mag = std::sqrt(a.norm_sqr());
        double cos_theta = (k_mag == 0.0) ? a.x / a_mag : (k.z * a.x - k.x * a.z) / (k_mag * a_mag);
        double det = (k_mag == 0.0) ? (-k.y * a.z + k.z * a.y)
                                    : (a.y * (k.x * k.x + k.z * k.z) - k.y * (a.x * k.x + a.z * k.z));
        double sign = -signum(det);
        cos_theta = std::fmin(std::fmax(cos_theta, -1.0), 1.0);
        double sin_theta = sign * std::sqrt(1.0 - cos_theta * cos_theta);
        double c2 = cos_theta * cos_theta - sin_theta * sin_theta;
        double s2 = 2.0 * cos_theta * sin_theta;
        *cos_2theta = c2;
        *sin_2theta = s2;
        return Stokes(i, c2 * q - s2 * u, s2 * q + c2 * u, v);
    }
    // polarization.rs:101-114
    static void lma_basis_rotation(const V4& k, double* sin_theta, double* cos_theta) {
        double k_minus = k.t - k.z;
        double c = (k.z * k_minus - k.x * k.x) / (k_minus * std::hypot(k.x, k.z));
        double det = k.x * k.y;
        double sign = signum(det);
        c = std::fmin(std::fmax(c, -1.0), 1.0);
        *sin_theta = sign * std::sqrt(1.0 - c * c);
        *cos_theta = c;
    }
    // polarization.rs:117-130
    Stokes in_lma_basis(const V4& k) const {
        double s, c;
        lma_basis_rotation(k, &s, &c);
        double c2 = c * c - s * s, s2 = 2.0 * c * s;
        return Stokes(i, c2 * q - s2 * u, s2 * q + c2 * u, v);
    }
    // polarization.rs:141-155
    Stokes from_lma_basis(const V4& k) const {
        double s, c;
        lma_basis_rotation(k, &s, &c);
        s = -s;
        double c2 = c * c - s * s, s2 = 2.0 * c * s;
        return Stokes(i, c2 * q - s2 * u, s2 * q + c2 * u, v);
    }
};

}  // namespace orc

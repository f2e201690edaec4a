// Titan/vec.h -- 3-vector of doubles with the interface of Titan's Vec
// (include/Titan/vec.h:33-163 in the reference): componentwise arithmetic,
// bounds-checked operator[], norm() = sqrt(x^2 + y^2 + z^2), dot, cross.
// Host-only here: device code uses the engine's own structure-of-arrays.
#ifndef TITAN_GB300_VEC_H
#define TITAN_GB300_VEC_H

#include <cmath>
#include <cstdio>
#include <iostream>
#include <vector>

namespace titan {

class Vec {
public:
    Vec() = default;
    Vec(const Vec &v) = default;
    Vec(double x, double y, double z) : data{x, y, z} {}
    Vec(const std::vector<double> &v) : data{v[0], v[1], v[2]} {}
    Vec &operator=(const Vec &v) = default;

    Vec &operator+=(const Vec &v) {
        data[0] += v.data[0];
        data[1] += v.data[1];
        data[2] += v.data[2];
        return *this;
    }
    Vec &operator-=(const Vec &v) {
        data[0] -= v.data[0];
        data[1] -= v.data[1];
        data[2] -= v.data[2];
        return *this;
    }
    Vec operator-() const { return Vec(-data[0], -data[1], -data[2]); }

    double &operator[](int n) {
        if (n < 0 || n >= 3) {
            std::printf("%s\n", "Out of bounds!");
            return data[0];
        }
        return data[n];
    }
    const double &operator[](int n) const {
        if (n < 0 || n >= 3) {
            std::printf("%s\n", "Out of bounds!");
            return data[0];
        }
        return data[n];
    }

    friend Vec operator+(const Vec &a, const Vec &b) { return Vec(a.data[0] + b.data[0], a.data[1] + b.data[1], a.data[2] + b.data[2]); }
    friend Vec operator-(const Vec &a, const Vec &b) { return Vec(a.data[0] - b.data[0], a.data[1] - b.data[1], a.data[2] - b.data[2]); }
    friend Vec operator*(const double x, const Vec &v) { return Vec(v.data[0] * x, v.data[1] * x, v.data[2] * x); }
    friend Vec operator*(const Vec &v, const double x) { return x * v; }
    friend bool operator==(const Vec &a, const Vec &b) { return a[0] == b[0] && a[1] == b[1] && a[2] == b[2]; }
    friend Vec operator*(const Vec &a, const Vec &b) { return Vec(a.data[0] * b.data[0], a.data[1] * b.data[1], a.data[2] * b.data[2]); }
    friend Vec operator/(const Vec &v, const double x) { return Vec(v.data[0] / x, v.data[1] / x, v.data[2] / x); }
    friend Vec operator/(const Vec &a, const Vec &b) { return Vec(a.data[0] / b.data[0], a.data[1] / b.data[1], a.data[2] / b.data[2]); }
    friend std::ostream &operator<<(std::ostream &s, const Vec &v) {
        return s << "(" << v[0] << ", " << v[1] << ", " << v[2] << ")";
    }

    void print() { std::printf("(%3f, %3f, %3f)\n", data[0], data[1], data[2]); }
    double norm() const {
        double a = data[0] * data[0], b = data[1] * data[1], c = data[2] * data[2];
        return std::sqrt((a + b) + c);
    }
    double sum() const { return data[0] + data[1] + data[2]; }
    Vec normalize() const { return *this / norm(); }

private:
    double data[3] = {0, 0, 0};
};

inline double dot(const Vec &a, const Vec &b) { return (a * b).sum(); }
inline Vec cross(const Vec &v1, const Vec &v2) {
    return Vec(v1[1] * v2[2] - v1[2] * v2[1], v2[0] * v1[2] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]);
}

}  // namespace titan

#endif

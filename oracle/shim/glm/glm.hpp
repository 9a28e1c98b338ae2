// Minimal stand-in for the subset of the OpenGL Mathematics (glm) API that the
// tensor-voting CPU path of tiralib uses.  It exists only so that the oracle
// can compile the reference's own `tira::cpu` functions in this container,
// where glm is not installed.  Test infrastructure, not part of the product.
//
// Semantics follow glm's documented conventions:
//   * vecN are plain aggregates of N components (x, y, z) with operator[].
//   * mat3 is COLUMN-major: mat3(c0, c1, c2) stores three columns, M[i] is
//     column i, M[i][j] is column i / row j.
//   * mat3 * vec3 and mat3 * mat3 are the usual linear-algebra products in
//     that convention; transpose swaps rows and columns.
//   * mat3(s) puts s on the diagonal (glm's scalar constructor).
#pragma once
#include <cmath>
#include <cstddef>

namespace glm {

struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    vec2(float a, float b) : x(a), y(b) {}
    float& operator[](int i) { return i == 0 ? x : y; }
    const float& operator[](int i) const { return i == 0 ? x : y; }
};

struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    int& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const int& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct vec3 {
    float x, y, z;
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const float& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
};

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }

inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(const vec3& a) { return std::sqrt(dot(a, a)); }
// glm::normalize multiplies by the inverse square root of the squared length.
inline vec3 normalize(const vec3& a) { return a * (1.0f / std::sqrt(dot(a, a))); }

struct mat3 {
    vec3 c[3];
    mat3() { c[0] = vec3(1, 0, 0); c[1] = vec3(0, 1, 0); c[2] = vec3(0, 0, 1); }
    explicit mat3(float s) { c[0] = vec3(s, 0, 0); c[1] = vec3(0, s, 0); c[2] = vec3(0, 0, s); }
    mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
    mat3& operator+=(const mat3& o) { c[0] += o.c[0]; c[1] += o.c[1]; c[2] += o.c[2]; return *this; }
};

inline mat3 operator*(float s, const mat3& m) { return mat3(s * m[0], s * m[1], s * m[2]); }
inline mat3 operator*(const mat3& m, float s) { return mat3(m[0] * s, m[1] * s, m[2] * s); }
inline mat3 operator+(const mat3& a, const mat3& b) { return mat3(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }

// (M v)[r] = sum_c M[c][r] * v[c]
inline vec3 operator*(const mat3& m, const vec3& v) {
    return vec3(m[0][0] * v.x + m[1][0] * v.y + m[2][0] * v.z,
                m[0][1] * v.x + m[1][1] * v.y + m[2][1] * v.z,
                m[0][2] * v.x + m[1][2] * v.y + m[2][2] * v.z);
}

// (A B)[c] = A * (column c of B)
inline mat3 operator*(const mat3& a, const mat3& b) { return mat3(a * b[0], a * b[1], a * b[2]); }

inline mat3 transpose(const mat3& m) {
    return mat3(vec3(m[0][0], m[1][0], m[2][0]),
                vec3(m[0][1], m[1][1], m[2][1]),
                vec3(m[0][2], m[1][2], m[2][2]));
}

}  // namespace glm

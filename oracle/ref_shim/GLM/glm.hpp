// Project-written subset of the GLM vector/matrix API, only as much as the
// reference's CPU smoothers and evaluators use, so that their unmodified
// sources compile into the checker library oracle/_ref.  TEST
// INFRASTRUCTURE ONLY.
//
// Semantics follow GLM 0.9.7 (the version the reference was written
// against): column-major matrices (m[c] is column c, m * v sums columns),
// vectors default-construct to zero and matrices to the identity (which
// AbstractSampler's constructor relies on), normalize(v) = v * (1/sqrt(v.v)),
// sign() returns -1 / 0 / +1, scalar functions are templates so that they
// never compete with the C library overloads.
#pragma once

// standard headers the reference's sources reach through their external
// includes in the original build
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <string>
#include <vector>

namespace glm {

template <class T> struct tvec4;

template <class T>
struct tvec2
{
    T x, y;
    tvec2() : x(0), y(0) {}
    template <class U> explicit tvec2(U s) : x(T(s)), y(T(s)) {}
    template <class A, class B> tvec2(A a, B b) : x(T(a)), y(T(b)) {}
    template <class U> tvec2(const tvec2<U>& o) : x(T(o.x)), y(T(o.y)) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
};

template <class T>
struct tvec3
{
    T x, y, z;
    tvec3() : x(0), y(0), z(0) {}
    template <class U> explicit tvec3(U s) : x(T(s)), y(T(s)), z(T(s)) {}
    template <class A, class B, class C> tvec3(A a, B b, C c) : x(T(a)), y(T(b)), z(T(c)) {}
    template <class U> tvec3(const tvec3<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    template <class U> explicit tvec3(const tvec4<U>& o);
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
    tvec3& operator+=(const tvec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    tvec3& operator-=(const tvec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    tvec3& operator*=(T s) { x *= s; y *= s; z *= s; return *this; }
    tvec3& operator/=(T s) { x /= s; y /= s; z /= s; return *this; }
};

template <class T>
struct tvec4
{
    T x, y, z, w;
    tvec4() : x(0), y(0), z(0), w(0) {}
    template <class U> explicit tvec4(U s) : x(T(s)), y(T(s)), z(T(s)), w(T(s)) {}
    template <class A, class B, class C, class D> tvec4(A a, B b, C c, D d) : x(T(a)), y(T(b)), z(T(c)), w(T(d)) {}
    template <class U, class W> tvec4(const tvec3<U>& v, W w_) : x(T(v.x)), y(T(v.y)), z(T(v.z)), w(T(w_)) {}
    template <class U> tvec4(const tvec4<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
};

template <class T> template <class U> tvec3<T>::tvec3(const tvec4<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}

// ---- vector arithmetic (component-wise) ----
#define GLMSHIM_VOPS(V, N)                                                                         \
    template <class T> V<T> operator+(const V<T>& a, const V<T>& b) { V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] + b[i]; return r; } \
    template <class T> V<T> operator-(const V<T>& a, const V<T>& b) { V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] - b[i]; return r; } \
    template <class T> V<T> operator*(const V<T>& a, const V<T>& b) { V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] * b[i]; return r; } \
    template <class T> V<T> operator/(const V<T>& a, const V<T>& b) { V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] / b[i]; return r; } \
    template <class T> V<T> operator*(const V<T>& a, T s) { V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] * s; return r; } \
    template <class T> V<T> operator*(T s, const V<T>& a) { V<T> r; for (int i = 0; i < N; ++i) r[i] = s * a[i]; return r; } \
    template <class T> V<T> operator/(const V<T>& a, T s) { V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] / s; return r; } \
    template <class T> V<T> operator+(const V<T>& a, T s) { V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] + s; return r; } \
    template <class T> V<T> operator-(const V<T>& a, T s) { V<T> r; for (int i = 0; i < N; ++i) r[i] = a[i] - s; return r; } \
    template <class T> V<T> operator-(const V<T>& a) { V<T> r; for (int i = 0; i < N; ++i) r[i] = -a[i]; return r; } \
    template <class T> bool operator==(const V<T>& a, const V<T>& b) { for (int i = 0; i < N; ++i) if (!(a[i] == b[i])) return false; return true; } \
    template <class T> bool operator!=(const V<T>& a, const V<T>& b) { return !(a == b); }
GLMSHIM_VOPS(tvec2, 2)
GLMSHIM_VOPS(tvec3, 3)
GLMSHIM_VOPS(tvec4, 4)
#undef GLMSHIM_VOPS

// ---- matrices: m[c] is column c ----
template <class T> struct tmat4;

template <class T>
struct tmat2
{
    tvec2<T> c[2];
    tmat2() { c[0] = tvec2<T>(1, 0); c[1] = tvec2<T>(0, 1); }
    explicit tmat2(T s) { c[0] = tvec2<T>(s, 0); c[1] = tvec2<T>(0, s); }
    tmat2(const tvec2<T>& a, const tvec2<T>& b) { c[0] = a; c[1] = b; }
    tmat2(T a, T b, T d, T e) { c[0] = tvec2<T>(a, b); c[1] = tvec2<T>(d, e); }
    tvec2<T>& operator[](int i) { return c[i]; }
    const tvec2<T>& operator[](int i) const { return c[i]; }
};

template <class T>
struct tmat3
{
    tvec3<T> c[3];
    tmat3() { c[0] = tvec3<T>(1, 0, 0); c[1] = tvec3<T>(0, 1, 0); c[2] = tvec3<T>(0, 0, 1); }
    explicit tmat3(T s) { c[0] = tvec3<T>(s, 0, 0); c[1] = tvec3<T>(0, s, 0); c[2] = tvec3<T>(0, 0, s); }
    tmat3(const tvec3<T>& a, const tvec3<T>& b, const tvec3<T>& d) { c[0] = a; c[1] = b; c[2] = d; }
    template <class U> tmat3(const tmat3<U>& o) { for (int i = 0; i < 3; ++i) c[i] = tvec3<T>(o[i]); }
    template <class U> explicit tmat3(const tmat4<U>& o);
    tvec3<T>& operator[](int i) { return c[i]; }
    const tvec3<T>& operator[](int i) const { return c[i]; }
};

template <class T>
struct tmat4
{
    tvec4<T> c[4];
    tmat4() { for (int i = 0; i < 4; ++i) { c[i] = tvec4<T>(0, 0, 0, 0); c[i][i] = 1; } }
    explicit tmat4(T s) { for (int i = 0; i < 4; ++i) { c[i] = tvec4<T>(0, 0, 0, 0); c[i][i] = s; } }
    template <class U> explicit tmat4(const tmat3<U>& m)
    {
        for (int i = 0; i < 3; ++i) c[i] = tvec4<T>(tvec3<T>(m[i]), 0);
        c[3] = tvec4<T>(0, 0, 0, 1);
    }
    template <class U> tmat4(const tmat4<U>& o) { for (int i = 0; i < 4; ++i) c[i] = tvec4<T>(o[i]); }
    tvec4<T>& operator[](int i) { return c[i]; }
    const tvec4<T>& operator[](int i) const { return c[i]; }
};

template <class T> template <class U> tmat3<T>::tmat3(const tmat4<U>& o)
{
    for (int i = 0; i < 3; ++i) c[i] = tvec3<T>(T(o[i].x), T(o[i].y), T(o[i].z));
}

template <class T> tvec3<T> operator*(const tmat3<T>& m, const tvec3<T>& v)
{
    return tvec3<T>(m[0][0] * v.x + m[1][0] * v.y + m[2][0] * v.z, m[0][1] * v.x + m[1][1] * v.y + m[2][1] * v.z,
                    m[0][2] * v.x + m[1][2] * v.y + m[2][2] * v.z);
}
template <class T> tmat3<T> operator*(const tmat3<T>& a, const tmat3<T>& b)
{
    tmat3<T> r;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) r[j][i] = a[0][i] * b[j][0] + a[1][i] * b[j][1] + a[2][i] * b[j][2];
    return r;
}
template <class T> tmat3<T> operator*(const tmat3<T>& a, T s) { tmat3<T> r; for (int i = 0; i < 3; ++i) r[i] = a[i] * s; return r; }
template <class T> tmat3<T> operator*(T s, const tmat3<T>& a) { return a * s; }
template <class T> tmat3<T> operator+(const tmat3<T>& a, const tmat3<T>& b) { tmat3<T> r; for (int i = 0; i < 3; ++i) r[i] = a[i] + b[i]; return r; }
template <class T> tmat3<T> operator-(const tmat3<T>& a, const tmat3<T>& b) { tmat3<T> r; for (int i = 0; i < 3; ++i) r[i] = a[i] - b[i]; return r; }

template <class T> tvec2<T> operator*(const tmat2<T>& m, const tvec2<T>& v)
{
    return tvec2<T>(m[0][0] * v.x + m[1][0] * v.y, m[0][1] * v.x + m[1][1] * v.y);
}
template <class T> tmat2<T> operator*(const tmat2<T>& a, const tmat2<T>& b)
{
    tmat2<T> r;
    for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i) r[j][i] = a[0][i] * b[j][0] + a[1][i] * b[j][1];
    return r;
}

// ---- functions ----
template <class T> T abs(T x) { return x < T(0) ? -x : x; }
template <class T> T sqrt(T x) { return std::sqrt(x); }
template <class T> T pow(T a, T b) { return std::pow(a, b); }
template <class T> T cos(T x) { return std::cos(x); }
template <class T> T ceil(T x) { return std::ceil(x); }
template <class T> T sign(T x) { return T((T(0) < x) - (x < T(0))); }
template <class T> T min(T a, T b) { return (b < a) ? b : a; }
template <class T> T max(T a, T b) { return (a < b) ? b : a; }
template <class T> T clamp(T x, T lo, T hi) { return min(max(x, lo), hi); }
template <class T> tvec3<T> min(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
template <class T> tvec3<T> max(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<T>(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }

template <class T> T dot(const tvec2<T>& a, const tvec2<T>& b) { return a.x * b.x + a.y * b.y; }
template <class T> T dot(const tvec3<T>& a, const tvec3<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> T dot(const tvec4<T>& a, const tvec4<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
template <class V> auto length(const V& v) -> decltype(dot(v, v)) { return std::sqrt(dot(v, v)); }
template <class V> auto distance(const V& a, const V& b) -> decltype(dot(a, b)) { return length(b - a); }
template <class V> V normalize(const V& v) { return v * (decltype(dot(v, v))(1) / std::sqrt(dot(v, v))); }
template <class T> tvec3<T> cross(const tvec3<T>& x, const tvec3<T>& y)
{
    return tvec3<T>(x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y);
}

template <class T> T determinant(const tmat3<T>& m)
{
    return +m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) - m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2]) +
           m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
}
template <class T> tmat3<T> inverse(const tmat3<T>& m)
{
    T ood = T(1) / (+m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) - m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2]) +
                    m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]));
    tmat3<T> r;
    r[0][0] = +(m[1][1] * m[2][2] - m[2][1] * m[1][2]) * ood;
    r[1][0] = -(m[1][0] * m[2][2] - m[2][0] * m[1][2]) * ood;
    r[2][0] = +(m[1][0] * m[2][1] - m[2][0] * m[1][1]) * ood;
    r[0][1] = -(m[0][1] * m[2][2] - m[2][1] * m[0][2]) * ood;
    r[1][1] = +(m[0][0] * m[2][2] - m[2][0] * m[0][2]) * ood;
    r[2][1] = -(m[0][0] * m[2][1] - m[2][0] * m[0][1]) * ood;
    r[0][2] = +(m[0][1] * m[1][2] - m[1][1] * m[0][2]) * ood;
    r[1][2] = -(m[0][0] * m[1][2] - m[1][0] * m[0][2]) * ood;
    r[2][2] = +(m[0][0] * m[1][1] - m[1][0] * m[0][1]) * ood;
    return r;
}
template <class T> tmat3<T> transpose(const tmat3<T>& m)
{
    tmat3<T> r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r[i][j] = m[j][i];
    return r;
}
template <class T> tmat2<T> transpose(const tmat2<T>& m) { return tmat2<T>(m[0][0], m[1][0], m[0][1], m[1][1]); }
template <class T> tmat3<T> mix(const tmat3<T>& a, const tmat3<T>& b, T t) { return a + (b - a) * t; }
template <class T> T mix(T a, T b, T t) { return a + t * (b - a); }
template <class T> tvec3<T> mix(const tvec3<T>& a, const tvec3<T>& b, const tvec3<T>& t) { return a + t * (b - a); }
template <class T> tvec3<T> mix(const tvec3<T>& a, const tvec3<T>& b, T t) { return a + t * (b - a); }

// rotation by `angle` radians about `axis`, composed on the right of m
template <class T> tmat4<T> rotate(const tmat4<T>& m, T angle, const tvec3<T>& v)
{
    const T a = angle, c = std::cos(a), s = std::sin(a);
    tvec3<T> axis = normalize(v);
    tvec3<T> temp = (T(1) - c) * axis;
    tmat3<T> R;
    R[0][0] = c + temp[0] * axis[0];
    R[0][1] = temp[0] * axis[1] + s * axis[2];
    R[0][2] = temp[0] * axis[2] - s * axis[1];
    R[1][0] = temp[1] * axis[0] - s * axis[2];
    R[1][1] = c + temp[1] * axis[1];
    R[1][2] = temp[1] * axis[2] + s * axis[0];
    R[2][0] = temp[2] * axis[0] + s * axis[1];
    R[2][1] = temp[2] * axis[1] - s * axis[0];
    R[2][2] = c + temp[2] * axis[2];
    tmat4<T> r;
    r[0] = m[0] * R[0][0] + m[1] * R[0][1] + m[2] * R[0][2];
    r[1] = m[0] * R[1][0] + m[1] * R[1][1] + m[2] * R[1][2];
    r[2] = m[0] * R[2][0] + m[1] * R[2][1] + m[2] * R[2][2];
    r[3] = m[3];
    return r;
}

// ---- used by TextureSampler ----
template <class T> bool operator==(const tmat3<T>& a, const tmat3<T>& b) { return a[0] == b[0] && a[1] == b[1] && a[2] == b[2]; }
template <class T> bool operator!=(const tmat3<T>& a, const tmat3<T>& b) { return !(a == b); }
// round half away from zero per component (std::round)
template <class T> tvec3<T> round(const tvec3<T>& v) { return tvec3<T>(std::round(v.x), std::round(v.y), std::round(v.z)); }
template <class T> tvec3<bool> lessThan(const tvec3<T>& a, const tvec3<T>& b) { return tvec3<bool>(a.x < b.x, a.y < b.y, a.z < b.z); }
inline bool all(const tvec3<bool>& v) { return v.x && v.y && v.z; }
template <class T> tmat4<T> operator*(const tmat4<T>& a, const tmat4<T>& b)
{
    tmat4<T> r;
    for (int j = 0; j < 4; ++j)
        for (int i = 0; i < 4; ++i)
            r[j][i] = a[0][i] * b[j][0] + a[1][i] * b[j][1] + a[2][i] * b[j][2] + a[3][i] * b[j][3];
    return r;
}
template <class T> tmat4<T>& operator*=(tmat4<T>& a, const tmat4<T>& b) { a = a * b; return a; }
// gtc/matrix_transform: m * S(v), m * T(v)
template <class T> tmat4<T> scale(const tmat4<T>& m, const tvec3<T>& v)
{
    tmat4<T> r;
    r[0] = tvec4<T>(m[0].x * v.x, m[0].y * v.x, m[0].z * v.x, m[0].w * v.x);
    r[1] = tvec4<T>(m[1].x * v.y, m[1].y * v.y, m[1].z * v.y, m[1].w * v.y);
    r[2] = tvec4<T>(m[2].x * v.z, m[2].y * v.z, m[2].z * v.z, m[2].w * v.z);
    r[3] = m[3];
    return r;
}
template <class T> tmat4<T> translate(const tmat4<T>& m, const tvec3<T>& v)
{
    tmat4<T> r(m);
    for (int i = 0; i < 4; ++i) r[3][i] = m[0][i] * v.x + m[1][i] * v.y + m[2][i] * v.z + m[3][i];
    return r;
}

typedef tvec2<double> dvec2;
typedef tvec3<double> dvec3;
typedef tvec4<double> dvec4;
typedef tvec2<float> vec2;
typedef tvec3<float> vec3;
typedef tvec4<float> vec4;
typedef tvec2<int> ivec2;
typedef tvec3<int> ivec3;
typedef tvec2<unsigned int> uvec2;
typedef tvec3<unsigned int> uvec3;
typedef tmat2<double> dmat2;
typedef tmat3<double> dmat3;
typedef tmat4<double> dmat4;
typedef tmat3<float> mat3;
typedef tmat4<float> mat4;

}  // namespace glm

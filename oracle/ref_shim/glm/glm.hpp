// Oracle (test infrastructure only): stand-in for the part of glm that the reference's
// include/lm/math.h, include/lm/surface.h and the accel, material, light and camera sources
// compiled into oracle/_ref use, so that they compile unmodified. glm itself (a third-party header library; the reference's
// environment.yml and conda/meta.yaml list it without a version, the 0.9.9 series at the time) is
// absent here.
//
// Written from glm's documented API. The arithmetic follows glm's generic (non-SIMD) code paths,
// which are the ones taken for the reference's double-precision vectors even under
// GLM_FORCE_INTRINSICS:
//   min(x, y) = (y < x) ? y : x          max(x, y) = (x < y) ? y : x     (per component)
//   abs(x)    = x >= 0 ? x : -x
//   dot(a, b) = t.x + t.y + t.z with t = a * b (left to right)
//   cross(x, y) = (x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x, x.x*y.y - y.x*x.y)
//   normalize(v) = v * inversesqrt(dot(v, v)), inversesqrt(s) = 1 / sqrt(s)
//   mat3 * vec3: row r = (m[0][r]*v.x + m[1][r]*v.y) + m[2][r]*v.z
//   mat4 * vec4: (m[0]*v.x + m[1]*v.y) + (m[2]*v.z + m[3]*v.w)
//   mat4 * mat4: column i = ((A[0]*B[i].x + A[1]*B[i].y) + A[2]*B[i].z) + A[3]*B[i].w
//   determinant(mat3): cofactor expansion along the first column
// inverse(mat4) is a cofactor inverse; it feeds only normal transforms, which no pinned output
// depends on.
#pragma once
#include <cmath>
#include <cstddef>

namespace glm {

template <typename T> struct tvec2;
template <typename T> struct tvec3;
template <typename T> struct tvec4;

template <typename T> struct tvec2 {
    T x{}, y{};
    tvec2() = default;
    explicit tvec2(T s) : x(s), y(s) {}
    tvec2(T a, T b) : x(a), y(b) {}
    template <typename U> explicit tvec2(const tvec2<U>& v) : x(T(v.x)), y(T(v.y)) {}
    tvec2(const tvec3<T>& v);  // drops z (implicit, as glm's is by default)
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
};

template <typename T> struct tvec3 {
    T x{}, y{}, z{};
    tvec3() = default;
    explicit tvec3(T s) : x(s), y(s), z(s) {}
    tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    tvec3(const tvec4<T>& v);  // drops w (glm's converting constructor is implicit)
    template <typename U> explicit tvec3(const tvec3<U>& v) : x(T(v.x)), y(T(v.y)), z(T(v.z)) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
};

template <typename T> struct tvec4 {
    // glm's storage: the components alias an array member `data.data`
    struct Storage { T data[4]; };
    union {
        struct { T x, y, z, w; };
        Storage data;
    };
    tvec4() : x(0), y(0), z(0), w(0) {}
    explicit tvec4(T s) : x(s), y(s), z(s), w(s) {}
    tvec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    tvec4(const tvec3<T>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
    tvec4(const tvec2<T>& a, const tvec2<T>& b) : x(a.x), y(a.y), z(b.x), w(b.y) {}
    T& operator[](int i) { return data.data[i]; }
    const T& operator[](int i) const { return data.data[i]; }
};

template <typename T> inline tvec3<T>::tvec3(const tvec4<T>& v) : x(v.x), y(v.y), z(v.z) {}
template <typename T> inline tvec2<T>::tvec2(const tvec3<T>& v) : x(v.x), y(v.y) {}

// -- component-wise arithmetic -------------------------------------------------------------------
#define LMREF_GLM_BINOP(V, N, OP)                                                                  \
    template <typename T> inline V<T> operator OP(const V<T>& a, const V<T>& b) {                  \
        V<T> r; for (int i = 0; i < N; i++) r[i] = a[i] OP b[i]; return r; }                       \
    template <typename T> inline V<T> operator OP(const V<T>& a, T s) {                            \
        V<T> r; for (int i = 0; i < N; i++) r[i] = a[i] OP s; return r; }                          \
    template <typename T> inline V<T> operator OP(T s, const V<T>& a) {                            \
        V<T> r; for (int i = 0; i < N; i++) r[i] = s OP a[i]; return r; }                          \
    template <typename T> inline V<T>& operator OP##=(V<T>& a, const V<T>& b) { a = a OP b; return a; } \
    template <typename T> inline V<T>& operator OP##=(V<T>& a, T s) { a = a OP s; return a; }
#define LMREF_GLM_VEC(V, N)                                                                        \
    LMREF_GLM_BINOP(V, N, +) LMREF_GLM_BINOP(V, N, -) LMREF_GLM_BINOP(V, N, *) LMREF_GLM_BINOP(V, N, /) \
    template <typename T> inline V<T> operator-(const V<T>& a) {                                   \
        V<T> r; for (int i = 0; i < N; i++) r[i] = -a[i]; return r; }                              \
    template <typename T> inline bool operator==(const V<T>& a, const V<T>& b) {                   \
        for (int i = 0; i < N; i++) if (!(a[i] == b[i])) return false; return true; }              \
    template <typename T> inline bool operator!=(const V<T>& a, const V<T>& b) { return !(a == b); }
LMREF_GLM_VEC(tvec2, 2)
LMREF_GLM_VEC(tvec3, 3)
LMREF_GLM_VEC(tvec4, 4)
#undef LMREF_GLM_VEC
#undef LMREF_GLM_BINOP

using ivec2 = tvec2<int>;

// -- common functions -----------------------------------------------------------------------------
template <typename T> inline T min(T x, T y) { return (y < x) ? y : x; }
template <typename T> inline T max(T x, T y) { return (x < y) ? y : x; }
template <typename T> inline T clamp(T x, T lo, T hi) { return min(max(x, lo), hi); }
template <typename T> inline T abs(T x) { return x >= T(0) ? x : -x; }
template <typename T> inline tvec2<T> min(const tvec2<T>& a, const tvec2<T>& b) { return {min(a.x, b.x), min(a.y, b.y)}; }
template <typename T> inline tvec2<T> max(const tvec2<T>& a, const tvec2<T>& b) { return {max(a.x, b.x), max(a.y, b.y)}; }
template <typename T> inline tvec3<T> min(const tvec3<T>& a, const tvec3<T>& b) { return {min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)}; }
template <typename T> inline tvec3<T> max(const tvec3<T>& a, const tvec3<T>& b) { return {max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)}; }
template <typename T> inline tvec3<T> abs(const tvec3<T>& a) { return {abs(a.x), abs(a.y), abs(a.z)}; }
template <typename T> inline T sin(T x) { return std::sin(x); }
template <typename T> inline T cos(T x) { return std::cos(x); }
template <typename T> inline T sqrt(T x) { return std::sqrt(x); }
template <typename T> inline T inversesqrt(T x) { return T(1) / std::sqrt(x); }

// -- geometric functions --------------------------------------------------------------------------
template <typename T> inline T dot(const tvec2<T>& a, const tvec2<T>& b) { const tvec2<T> t = a * b; return t.x + t.y; }
template <typename T> inline T dot(const tvec3<T>& a, const tvec3<T>& b) { const tvec3<T> t = a * b; return t.x + t.y + t.z; }
template <typename T> inline T dot(const tvec4<T>& a, const tvec4<T>& b) { const tvec4<T> t = a * b; return (t.x + t.y) + (t.z + t.w); }
template <typename T> inline tvec3<T> cross(const tvec3<T>& x, const tvec3<T>& y) {
    return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y};
}
template <typename T> inline T length(const tvec3<T>& v) { return std::sqrt(dot(v, v)); }
template <typename T> inline T length2(const tvec3<T>& v) { return dot(v, v); }
template <typename T> inline T distance(const tvec3<T>& a, const tvec3<T>& b) { return length(b - a); }
template <typename T> inline T distance2(const tvec3<T>& a, const tvec3<T>& b) { return length2(b - a); }
template <typename T> inline tvec3<T> normalize(const tvec3<T>& v) { return v * inversesqrt(dot(v, v)); }
template <typename T> inline T compMax(const tvec3<T>& v) { return max(max(v.x, v.y), v.z); }
template <typename T> inline T compMin(const tvec3<T>& v) { return min(min(v.x, v.y), v.z); }

// -- vector relational ----------------------------------------------------------------------------
template <typename V> struct tbvec { bool b[4] = {false, false, false, false}; int n = 0; };
template <typename T> inline tbvec<tvec2<T>> equal(const tvec2<T>& a, const tvec2<T>& b) {
    tbvec<tvec2<T>> r; r.n = 2; for (int i = 0; i < 2; i++) r.b[i] = a[i] == b[i]; return r;
}
template <typename T> inline tbvec<tvec3<T>> equal(const tvec3<T>& a, const tvec3<T>& b) {
    tbvec<tvec3<T>> r; r.n = 3; for (int i = 0; i < 3; i++) r.b[i] = a[i] == b[i]; return r;
}
template <typename V> inline bool all(const tbvec<V>& v) {
    for (int i = 0; i < v.n; i++) if (!v.b[i]) return false;
    return true;
}

// -- matrices (column-major, m[column][row]) ------------------------------------------------------
template <typename T> struct tmat4x4;

template <typename T> struct tmat3x3 {
    tvec3<T> c[3];
    tmat3x3() : tmat3x3(T(1)) {}
    explicit tmat3x3(T s) { c[0] = {s, 0, 0}; c[1] = {0, s, 0}; c[2] = {0, 0, s}; }
    tmat3x3(const tvec3<T>& a, const tvec3<T>& b, const tvec3<T>& d) { c[0] = a; c[1] = b; c[2] = d; }
    explicit tmat3x3(const tmat4x4<T>& m);
    tvec3<T>& operator[](int i) { return c[i]; }
    const tvec3<T>& operator[](int i) const { return c[i]; }
};

template <typename T> struct tmat4x4 {
    tvec4<T> c[4];
    tmat4x4() : tmat4x4(T(1)) {}
    explicit tmat4x4(T s) { c[0] = {s, 0, 0, 0}; c[1] = {0, s, 0, 0}; c[2] = {0, 0, s, 0}; c[3] = {0, 0, 0, s}; }
    tmat4x4(const tvec4<T>& a, const tvec4<T>& b, const tvec4<T>& d, const tvec4<T>& e) { c[0] = a; c[1] = b; c[2] = d; c[3] = e; }
    tvec4<T>& operator[](int i) { return c[i]; }
    const tvec4<T>& operator[](int i) const { return c[i]; }
};

template <typename T> inline tmat3x3<T>::tmat3x3(const tmat4x4<T>& m) {
    for (int i = 0; i < 3; i++) c[i] = tvec3<T>(m[i].x, m[i].y, m[i].z);
}

template <typename T> inline tvec3<T> operator*(const tmat3x3<T>& m, const tvec3<T>& v) {
    tvec3<T> r;
    for (int k = 0; k < 3; k++) r[k] = m[0][k] * v.x + m[1][k] * v.y + m[2][k] * v.z;
    return r;
}
template <typename T> inline tvec4<T> operator*(const tmat4x4<T>& m, const tvec4<T>& v) {
    const tvec4<T> add0 = m[0] * v.x + m[1] * v.y;
    const tvec4<T> add1 = m[2] * v.z + m[3] * v.w;
    return add0 + add1;
}
template <typename T> inline tmat4x4<T> operator*(const tmat4x4<T>& a, const tmat4x4<T>& b) {
    tmat4x4<T> r;
    for (int i = 0; i < 4; i++) r[i] = a[0] * b[i].x + a[1] * b[i].y + a[2] * b[i].z + a[3] * b[i].w;
    return r;
}
template <typename T> inline tmat3x3<T> operator*(const tmat3x3<T>& a, const tmat3x3<T>& b) {
    tmat3x3<T> r;
    for (int i = 0; i < 3; i++) r[i] = a[0] * b[i].x + a[1] * b[i].y + a[2] * b[i].z;
    return r;
}

template <typename T> inline tmat3x3<T> transpose(const tmat3x3<T>& m) {
    tmat3x3<T> r;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) r[i][j] = m[j][i];
    return r;
}
template <typename T> inline tmat4x4<T> transpose(const tmat4x4<T>& m) {
    tmat4x4<T> r;
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) r[i][j] = m[j][i];
    return r;
}
template <typename T> inline T determinant(const tmat3x3<T>& m) {
    return m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2])
         - m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2])
         + m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
}
template <typename T> inline tmat4x4<T> inverse(const tmat4x4<T>& m) {
    // Adjugate over the determinant; minor(r, c) deletes row r and column c (m[col][row]).
    auto minor3 = [&](int r, int c) {
        T a[9];
        int k = 0;
        for (int cc = 0; cc < 4; cc++) {
            if (cc == c) continue;
            for (int rr = 0; rr < 4; rr++) {
                if (rr == r) continue;
                a[k++] = m[cc][rr];
            }
        }
        return a[0] * (a[4] * a[8] - a[7] * a[5]) - a[3] * (a[1] * a[8] - a[7] * a[2]) + a[6] * (a[1] * a[5] - a[4] * a[2]);
    };
    tmat4x4<T> adj;
    T det = T(0);
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) {
            const T cof = ((r + c) % 2 ? T(-1) : T(1)) * minor3(r, c);
            adj[r][c] = cof;  // transpose of the cofactor matrix
            if (r == 0) det += m[c][0] * cof;
        }
    for (int i = 0; i < 4; i++) adj[i] = adj[i] / det;
    return adj;
}

// Camera matrices (right-handed, clip depth in [-1, 1]); no pinned output depends on them.
template <typename T> inline T radians(T degrees) { return degrees * T(0.01745329251994329576923690768489); }
template <typename T> inline T tan(T x) { return std::tan(x); }
template <typename T> inline tmat4x4<T> lookAt(const tvec3<T>& eye, const tvec3<T>& center, const tvec3<T>& up) {
    const tvec3<T> f = normalize(center - eye);
    const tvec3<T> s = normalize(cross(f, up));
    const tvec3<T> u = cross(s, f);
    tmat4x4<T> r(T(1));
    r[0][0] = s.x; r[1][0] = s.y; r[2][0] = s.z;
    r[0][1] = u.x; r[1][1] = u.y; r[2][1] = u.z;
    r[0][2] = -f.x; r[1][2] = -f.y; r[2][2] = -f.z;
    r[3][0] = -dot(s, eye); r[3][1] = -dot(u, eye); r[3][2] = dot(f, eye);
    return r;
}
template <typename T> inline tmat4x4<T> perspective(T fovy, T aspect, T znear, T zfar) {
    const T th = std::tan(fovy / T(2));
    tmat4x4<T> r(T(0));
    r[0][0] = T(1) / (aspect * th);
    r[1][1] = T(1) / th;
    r[2][2] = -(zfar + znear) / (zfar - znear);
    r[2][3] = -T(1);
    r[3][2] = -(T(2) * zfar * znear) / (zfar - znear);
    return r;
}

template <typename T> inline T* value_ptr(tvec3<T>& v) { return &v.x; }
template <typename T> inline const T* value_ptr(const tvec3<T>& v) { return &v.x; }
template <typename T> inline T* value_ptr(tmat4x4<T>& m) { return &m[0].x; }
template <typename T> inline const T* value_ptr(const tmat4x4<T>& m) { return &m[0].x; }

}  // namespace glm

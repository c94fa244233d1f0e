// Oracle (test infrastructure only): CPU restatement of Lightmetrica v3's math layer.
//
// This header is part of the CPU oracle that the tests and the benchmark's CPU-baseline leg use
// to check the CUDA path. Nothing in the product links it.
//
// Follows include/lm/math.h of the reference (glm-based). glm is not available here, so the
// vector and matrix operations are written out with glm's operation order made explicit:
//   dot(a,b)   = (a.x*b.x + a.y*b.y) + a.z*b.z            (glm compute_dot: tmp = a*b; x+y+z)
//   cross(a,b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
//   normalize  = v * (1 / sqrt(dot(v,v)))                  (glm inversesqrt)
//   mat3*vec3  = row-wise ((m0*x + m1*y) + m2*z)
//   mat4*vec4  = (m0*x + m1*y) + (m2*z + m3*w)             (glm's Mul/Add pairing)
// These orders are an assumption about glm 0.9.9 that cannot be confirmed without glm. The
// product follows the same orders, so the fp32 parity gate is self-consistent either way.
// The oracle is compiled with -ffp-contract=off so no FMA changes the rounding.
#pragma once
#include <cmath>
#include <cstdint>
#include <algorithm>
#include <vector>
#include <limits>

namespace lmo {

template <typename F> struct V2 {
    F x = 0, y = 0;
    V2() = default;
    V2(F x_, F y_) : x(x_), y(y_) {}
    F operator[](int i) const { return i == 0 ? x : y; }
};

template <typename F> struct V3 {
    F x = 0, y = 0, z = 0;
    V3() = default;
    explicit V3(F s) : x(s), y(s), z(s) {}
    V3(F x_, F y_, F z_) : x(x_), y(y_), z(z_) {}
    F operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    F& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};

template <typename F> struct V4 {
    F x = 0, y = 0, z = 0, w = 0;
    V4() = default;
    V4(F x_, F y_, F z_, F w_) : x(x_), y(y_), z(z_), w(w_) {}
    V4(V3<F> v, F w_) : x(v.x), y(v.y), z(v.z), w(w_) {}
    F operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

template <typename F> inline V3<F> operator+(V3<F> a, V3<F> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename F> inline V3<F> operator-(V3<F> a, V3<F> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename F> inline V3<F> operator-(V3<F> a) { return {-a.x, -a.y, -a.z}; }
template <typename F> inline V3<F> operator*(V3<F> a, V3<F> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <typename F> inline V3<F> operator*(V3<F> a, F s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename F> inline V3<F> operator*(F s, V3<F> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename F> inline V3<F> operator/(V3<F> a, F s) { return {a.x / s, a.y / s, a.z / s}; }
template <typename F> inline V3<F> operator/(V3<F> a, V3<F> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <typename F> inline V3<F>& operator+=(V3<F>& a, V3<F> b) { a = a + b; return a; }
template <typename F> inline V3<F>& operator*=(V3<F>& a, V3<F> b) { a = a * b; return a; }
template <typename F> inline V3<F>& operator*=(V3<F>& a, F s) { a = a * s; return a; }
template <typename F> inline V3<F>& operator/=(V3<F>& a, F s) { a = a / s; return a; }

template <typename F> inline V2<F> operator+(V2<F> a, V2<F> b) { return {a.x + b.x, a.y + b.y}; }
template <typename F> inline V2<F> operator-(V2<F> a, V2<F> b) { return {a.x - b.x, a.y - b.y}; }
template <typename F> inline V2<F> operator*(V2<F> a, F s) { return {a.x * s, a.y * s}; }
template <typename F> inline V2<F> operator*(F s, V2<F> a) { return {s * a.x, s * a.y}; }

template <typename F> inline F dot(V3<F> a, V3<F> b) {
    const F tx = a.x * b.x, ty = a.y * b.y, tz = a.z * b.z;
    return (tx + ty) + tz;
}
template <typename F> inline V3<F> cross(V3<F> x, V3<F> y) {
    return {x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y};
}
template <typename F> inline F length(V3<F> v) { return std::sqrt(dot(v, v)); }
template <typename F> inline F distance(V3<F> a, V3<F> b) { return length(b - a); }
template <typename F> inline V3<F> normalize(V3<F> v) {
    const F inv = F(1) / std::sqrt(dot(v, v));
    return v * inv;
}
template <typename F> inline V3<F> vabs(V3<F> v) { return {std::abs(v.x), std::abs(v.y), std::abs(v.z)}; }
template <typename F> inline V3<F> vmin(V3<F> a, V3<F> b) {
    // glm::min(a,b) per component is (b < a ? b : a)
    return {b.x < a.x ? b.x : a.x, b.y < a.y ? b.y : a.y, b.z < a.z ? b.z : a.z};
}
template <typename F> inline V3<F> vmax(V3<F> a, V3<F> b) {
    // glm::max(a,b) per component is (a < b ? b : a)
    return {a.x < b.x ? b.x : a.x, a.y < b.y ? b.y : a.y, a.z < b.z ? b.z : a.z};
}
template <typename F> inline F comp_max(V3<F> v) { return std::max(std::max(v.x, v.y), v.z); }
template <typename F> inline bool is_zero(V3<F> v) { return v.x == F(0) && v.y == F(0) && v.z == F(0); }

// Column-major 3x3 matrix (c[i] is column i), as glm::tmat3x3.
template <typename F> struct M3 {
    V3<F> c[3];
    M3() { c[0] = {1, 0, 0}; c[1] = {0, 1, 0}; c[2] = {0, 0, 1}; }
    M3(V3<F> a, V3<F> b, V3<F> d) { c[0] = a; c[1] = b; c[2] = d; }
};
template <typename F> inline V3<F> operator*(const M3<F>& m, V3<F> v) {
    return {
        (m.c[0].x * v.x + m.c[1].x * v.y) + m.c[2].x * v.z,
        (m.c[0].y * v.x + m.c[1].y * v.y) + m.c[2].y * v.z,
        (m.c[0].z * v.x + m.c[1].z * v.y) + m.c[2].z * v.z,
    };
}
template <typename F> inline M3<F> transpose(const M3<F>& m) {
    return M3<F>({m.c[0].x, m.c[1].x, m.c[2].x}, {m.c[0].y, m.c[1].y, m.c[2].y}, {m.c[0].z, m.c[1].z, m.c[2].z});
}
template <typename F> inline F determinant(const M3<F>& m) {
    // Cofactor expansion along the first column (glm's formula order for mat3).
    return m.c[0].x * (m.c[1].y * m.c[2].z - m.c[2].y * m.c[1].z)
         - m.c[1].x * (m.c[0].y * m.c[2].z - m.c[2].y * m.c[0].z)
         + m.c[2].x * (m.c[0].y * m.c[1].z - m.c[1].y * m.c[0].z);
}

// Column-major 4x4 matrix.
template <typename F> struct M4 {
    V4<F> c[4];
    M4() { c[0] = {1, 0, 0, 0}; c[1] = {0, 1, 0, 0}; c[2] = {0, 0, 1, 0}; c[3] = {0, 0, 0, 1}; }
    static M4 from_colmajor(const double* m) {
        M4 r;
        for (int i = 0; i < 4; i++) r.c[i] = {F(m[4 * i]), F(m[4 * i + 1]), F(m[4 * i + 2]), F(m[4 * i + 3])};
        return r;
    }
    bool is_identity() const {
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
                if (c[i][j] != F(i == j ? 1 : 0)) return false;
        return true;
    }
};
template <typename F> inline V4<F> operator*(const M4<F>& m, V4<F> v) {
    V4<F> r;
    const F* col[4] = {&m.c[0].x, &m.c[1].x, &m.c[2].x, &m.c[3].x};
    F out[4];
    for (int i = 0; i < 4; i++) {
        const F mul0 = col[0][i] * v.x, mul1 = col[1][i] * v.y;
        const F mul2 = col[2][i] * v.z, mul3 = col[3][i] * v.w;
        out[i] = (mul0 + mul1) + (mul2 + mul3);
    }
    r = {out[0], out[1], out[2], out[3]};
    return r;
}
template <typename F> inline M4<F> operator*(const M4<F>& a, const M4<F>& b) {
    // glm mat4*mat4: column i = A0*B[i][0] + A1*B[i][1] + A2*B[i][2] + A3*B[i][3], left to right.
    M4<F> r;
    const F* A[4] = {&a.c[0].x, &a.c[1].x, &a.c[2].x, &a.c[3].x};
    for (int i = 0; i < 4; i++) {
        F out[4];
        for (int k = 0; k < 4; k++)
            out[k] = ((A[0][k] * b.c[i].x + A[1][k] * b.c[i].y) + A[2][k] * b.c[i].z) + A[3][k] * b.c[i].w;
        r.c[i] = {out[0], out[1], out[2], out[3]};
    }
    return r;
}
template <typename F> inline M3<F> upper3(const M4<F>& m) {
    return M3<F>({m.c[0].x, m.c[0].y, m.c[0].z}, {m.c[1].x, m.c[1].y, m.c[1].z}, {m.c[2].x, m.c[2].y, m.c[2].z});
}
// Inverse of a 4x4 matrix by cofactors (any exact-arithmetic-equivalent method; used only for
// normal transforms, which do not enter the hit-parity gate).
template <typename F> inline M4<F> inverse(const M4<F>& m) {
    F a[16];
    for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) a[4 * i + j] = m.c[i][j];
    F inv[16];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    F det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    M4<F> r;
    for (int i = 0; i < 4; i++) r.c[i] = {inv[4 * i] / det, inv[4 * i + 1] / det, inv[4 * i + 2] / det, inv[4 * i + 3] / det};
    return r;
}
template <typename F> inline M4<F> transpose(const M4<F>& m) {
    M4<F> r;
    for (int i = 0; i < 4; i++) r.c[i] = {m.c[0][i], m.c[1][i], m.c[2][i], m.c[3][i]};
    return r;
}

// include/lm/math.h:54-56
template <typename F> struct C {
    static constexpr F Inf = F(1e+10);
    static constexpr F Eps = F(1e-3);
    static constexpr F Pi = F(3.14159265358979323846);
};

// include/lm/math.h:67-77
template <typename F> struct Ray { V3<F> o, d; };

// include/lm/math.h:82-179 (Bound). isect_range is the reference slab test; `robust` widens the
// far distance by (1 + 2*gamma(3)) after the loop (Ize 2013, "Robust BVH ray traversal") so the
// fp32 parity build culls no triangle whose Moller-Trumbore test accepts the ray.
template <typename F> struct Bound {
    V3<F> min = V3<F>(C<F>::Inf);
    V3<F> max = V3<F>(-C<F>::Inf);
    V3<F> center() const { return (min + max) * F(.5); }
    F surface_area() const {
        const auto d = max - min;
        return F(2) * (d.x * d.y + d.y * d.z + d.z * d.x);
    }
    bool isect(const Ray<F>& r, F tmin, F tmax, bool robust) const {
        for (int i = 0; i < 3; i++) {
            const F vd = F(1) / r.d[i];
            F t1 = (min[i] - r.o[i]) * vd;
            F t2 = (max[i] - r.o[i]) * vd;
            if (vd < 0) std::swap(t1, t2);
            if (robust) t2 = t2 * F(1.0000004);
            // glm::max(t1, tmin) = (t1 < tmin ? tmin : t1); glm::min(t2, tmax) = (tmax < t2 ? tmax : t2)
            tmin = t1 < tmin ? tmin : t1;
            tmax = tmax < t2 ? tmax : t2;
            if (tmax < tmin) return false;
        }
        return true;
    }
};
template <typename F> inline Bound<F> merge(Bound<F> b, V3<F> p) { return {vmin(b.min, p), vmax(b.max, p)}; }
template <typename F> inline Bound<F> merge(Bound<F> a, Bound<F> b) { return {vmin(a.min, b.min), vmax(a.max, b.max)}; }

// include/lm/math.h:724-746
template <typename F> struct Transform {
    M4<F> M;
    M3<F> normal_M;
    F J = 1;
    Transform() = default;
    explicit Transform(const M4<F>& m) : M(m) {
        normal_M = upper3(transpose(inverse(m)));
        J = std::abs(determinant(upper3(m)));
    }
};

// include/lm/math.h:310-371 (Dist)
template <typename F> struct Dist {
    std::vector<F> c{F(0)};
    void clear() { c.clear(); c.push_back(F(0)); }
    bool empty() const { return c.size() == 1; }
    void add(F v) { c.push_back(c.back() + v); }
    void norm() {
        const auto sum = c.back();
        for (auto& v : c) v /= sum;
    }
    F pmf(int i) const { return (i < 0 || i + 1 >= int(c.size())) ? F(0) : c[i + 1] - c[i]; }
    int sample(F u) const {
        const auto it = std::upper_bound(c.begin(), c.end(), u);
        return std::clamp(int(std::distance(c.begin(), it)) - 1, 0, int(c.size()) - 2);
    }
};

// include/lm/math.h:378-432 (Dist2)
template <typename F> struct Dist2 {
    std::vector<Dist<F>> ds;
    Dist<F> m;
    int w = 0, h = 0;
    void init(const std::vector<F>& v, int cols, int rows) {
        w = cols; h = rows;
        ds.assign(h, {});
        m.clear();
        for (int i = 0; i < h; i++) {
            auto& d = ds[i];
            for (int j = 0; j < w; j++) d.add(v[i * w + j]);
            m.add(d.c.back());
            d.norm();
        }
        m.norm();
    }
    F pdf(F u, F v) const {
        const int y = std::min(int(v * h), h - 1);
        return m.pmf(y) * ds[y].pmf(int(u * w)) * w * h;
    }
    V2<F> sample(F u0, F u1, F u2, F u3) const {
        const int y = m.sample(u0);
        const int x = ds[y].sample(u1);
        return V2<F>((x + u2) / w, (y + u3) / h);
    }
};

// include/lm/math.h:478-702 (math:: helpers)
template <typename F> inline F safe_sqrt(F v) { return std::sqrt(std::max(F(0), v)); }
template <typename F> inline F sq(F v) { return v * v; }
template <typename F> inline V3<F> reflection(V3<F> w, V3<F> n) { return F(2) * dot(w, n) * n - w; }
template <typename F> struct RefractionResult { V3<F> wt; bool total; };
template <typename F> inline RefractionResult<F> refraction(V3<F> wi, V3<F> n, F eta) {
    const auto t = dot(wi, n);
    const auto t2 = F(1) - eta * eta * (F(1) - t * t);
    if (t2 <= F(0)) return {{}, true};
    return {eta * (n * t - wi) - n * safe_sqrt(t2), false};
}
template <typename F> inline void orthonormal_basis(V3<F> n, V3<F>& u, V3<F>& v) {
    const auto s = std::copysign(F(1), n.z);
    const auto a = F(-1) / (s + n.z);
    const auto b = n.x * n.y * a;
    u = V3<F>(F(1) + s * n.x * n.x * a, s * b, -s * n.x);
    v = V3<F>(b, s + n.y * n.y * a, -n.y);
}
template <typename F> inline V3<F> geometry_normal(V3<F> p1, V3<F> p2, V3<F> p3) {
    return normalize(cross(p2 - p1, p3 - p1));
}
template <typename F> inline V3<F> mix_barycentric(V3<F> a, V3<F> b, V3<F> c, V2<F> uv) {
    return a * (F(1) - uv.x - uv.y) + b * uv.x + c * uv.y;
}
// the same for texture coordinates (mesh_raw.cpp:97: math::mix_barycentric on Vec2)
template <typename F> inline V2<F> mix_barycentric2(V2<F> a, V2<F> b, V2<F> c, V2<F> uv) {
    const F w = F(1) - uv.x - uv.y;
    return V2<F>(a.x * w + b.x * uv.x + c.x * uv.y, a.y * w + b.y * uv.x + c.y * uv.y);
}
template <typename F> inline V2<F> sample_uniform_disk(V2<F> u) {
    const auto r = safe_sqrt(u.x);
    const auto t = F(2) * C<F>::Pi * u.y;
    return {r * std::cos(t), r * std::sin(t)};
}
template <typename F> inline V3<F> sample_cosine_weighted(V2<F> u) {
    const auto r = safe_sqrt(u.x);
    const auto t = F(2) * C<F>::Pi * u.y;
    const auto x = r * std::cos(t);
    const auto y = r * std::sin(t);
    return {x, y, safe_sqrt(F(1) - x * x - y * y)};
}
template <typename F> inline V3<F> sample_uniform_sphere(V2<F> u) {
    const auto z = F(1) - F(2) * u.x;
    const auto r = safe_sqrt(F(1) - z * z);
    const auto t = F(2) * C<F>::Pi * u.y;
    return {r * std::cos(t), r * std::sin(t), z};
}
template <typename F> inline F pdf_uniform_sphere() { return F(1) / (F(4) * C<F>::Pi); }
template <typename F> inline F balance_heuristic(F p1, F p2) {
    if (p1 == F(0) && p2 == F(0)) return F(0);
    return p1 / (p1 + p2);
}

}  // namespace lmo

// The hit distance the accel API reports: the reference's fp64 Möller–Trumbore distance of the
// hit triangle (accel_sahbvh.cpp:58-75, glm's dot and cross order) from the fp32 ray and triangle
// record (p1, e1, e2), rounded once to float.
//
// GB300 runs double-precision arithmetic at a small fraction of its single-precision rate, and the
// fp64 chain (about 30 double operations, a division and 13 conversions per hit) took a third of
// the raycast probe's device time. hit_t() therefore first evaluates the same formula in
// double-float arithmetic (pairs of floats carrying about 48 significant bits; exact products by
// fma, exact sums by TwoSum) together with a bound on how far that value can be from the fp64
// chain's quotient. When every real number within the bound rounds to the same float, that float
// is the fp64 chain's result rounded to float; otherwise (a near-tie with a rounding boundary, a
// badly conditioned grazing hit, inputs outside the range where the float products are exact)
// it runs the fp64 chain itself. The result is the fp64 chain's, bit for bit, in every case.
//
// Plain C++ as well as CUDA: the host build is the unit test's (same IEEE single and double
// operations, round to nearest, no contraction).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define LMGPU_HT_FN __host__ __device__ __forceinline__
#else
#define LMGPU_HT_FN inline
#endif

namespace lmgpu_ht {

#if defined(__CUDA_ARCH__)
LMGPU_HT_FN float fadd(float a, float b) { return __fadd_rn(a, b); }
LMGPU_HT_FN float fsub(float a, float b) { return __fsub_rn(a, b); }
LMGPU_HT_FN float fmul(float a, float b) { return __fmul_rn(a, b); }
LMGPU_HT_FN float fdiv(float a, float b) { return __fdiv_rn(a, b); }
LMGPU_HT_FN float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
LMGPU_HT_FN double dadd(double a, double b) { return __dadd_rn(a, b); }
LMGPU_HT_FN double dsub(double a, double b) { return __dsub_rn(a, b); }
LMGPU_HT_FN double dmul(double a, double b) { return __dmul_rn(a, b); }
LMGPU_HT_FN double ddiv(double a, double b) { return __ddiv_rn(a, b); }
LMGPU_HT_FN float d2f(double a) { return __double2float_rn(a); }
LMGPU_HT_FN int32_t fbits(float a) { return __float_as_int(a); }
LMGPU_HT_FN float bitsf(int32_t b) { return __int_as_float(b); }
LMGPU_HT_FN float fabs_(float a) { return fabsf(a); }
LMGPU_HT_FN bool finite_(float a) { return isfinite(a); }
#else
// host: compiled with -ffp-contract=off, so each expression is one IEEE operation
inline float fadd(float a, float b) { return a + b; }
inline float fsub(float a, float b) { return a - b; }
inline float fmul(float a, float b) { return a * b; }
inline float fdiv(float a, float b) { return a / b; }
inline float ffma(float a, float b, float c) { return std::fmaf(a, b, c); }
inline double dadd(double a, double b) { return a + b; }
inline double dsub(double a, double b) { return a - b; }
inline double dmul(double a, double b) { return a * b; }
inline double ddiv(double a, double b) { return a / b; }
inline float d2f(double a) { return float(a); }
inline int32_t fbits(float a) { int32_t b; std::memcpy(&b, &a, 4); return b; }
inline float bitsf(int32_t b) { float a; std::memcpy(&a, &b, 4); return a; }
inline float fabs_(float a) { return std::fabs(a); }
inline bool finite_(float a) { return std::isfinite(a); }
#endif

// The fp64 chain: accel_sahbvh.cpp:58-75 with explicit IEEE double operations.
LMGPU_HT_FN float hit_t_fp64(const float o[3], const float d[3], const float p1[3], const float e1[3], const float e2[3]) {
    const double ox = o[0], oy = o[1], oz = o[2], dx = d[0], dy = d[1], dz = d[2];
    const double e1x = e1[0], e1y = e1[1], e1z = e1[2], e2x = e2[0], e2y = e2[1], e2z = e2[2];
    const double px = dsub(dmul(dy, e2z), dmul(e2y, dz));
    const double py = dsub(dmul(dz, e2x), dmul(e2z, dx));
    const double pz = dsub(dmul(dx, e2y), dmul(e2x, dy));
    const double tx = dsub(ox, double(p1[0])), ty = dsub(oy, double(p1[1])), tz = dsub(oz, double(p1[2]));
    const double qx = dsub(dmul(ty, e1z), dmul(e1y, tz));
    const double qy = dsub(dmul(tz, e1x), dmul(e1z, tx));
    const double qz = dsub(dmul(tx, e1y), dmul(e1x, ty));
    const double det = dadd(dadd(dmul(e1x, px), dmul(e1y, py)), dmul(e1z, pz));
    const double num = dadd(dadd(dmul(e2x, qx), dmul(e2y, qy)), dmul(e2z, qz));
    return d2f(ddiv(num, det));
}

// A double-float: the unevaluated sum hi + lo.
struct DF {
    float hi, lo;
};
// Knuth's TwoSum: s + e == a + b exactly.
LMGPU_HT_FN DF two_sum(float a, float b) {
    const float s = fadd(a, b);
    const float bb = fsub(s, a);
    return {s, fadd(fsub(a, fsub(s, bb)), fsub(b, bb))};
}
// p + e == a * b exactly, while the product and its error stay normal.
LMGPU_HT_FN DF two_prod(float a, float b) {
    const float p = fmul(a, b);
    return {p, ffma(a, b, -p)};
}
LMGPU_HT_FN DF df_add(DF a, DF b) {
    const DF s = two_sum(a.hi, b.hi);
    const DF t = two_sum(a.lo, b.lo);
    const DF u = two_sum(s.hi, fadd(s.lo, t.hi));
    return two_sum(u.hi, fadd(u.lo, t.lo));
}
LMGPU_HT_FN DF df_neg(DF a) { return {-a.hi, -a.lo}; }
LMGPU_HT_FN DF df_mul(DF a, float b) {
    const DF p = two_prod(a.hi, b);
    return two_sum(p.hi, ffma(a.lo, b, p.lo));
}
// a * b - c * e for floats: both products exact, one rounding to a double-float.
LMGPU_HT_FN DF df_cross(float a, float b, float c, float e) { return df_add(two_prod(a, b), df_neg(two_prod(c, e))); }
// a * b - c * e for double-floats a, c.
LMGPU_HT_FN DF df_cross(DF a, float b, DF c, float e) { return df_add(df_mul(a, b), df_neg(df_mul(c, e))); }

LMGPU_HT_FN bool in_range(float x) {
    const float ax = fabs_(x);
    return ax == 0.f || (ax >= 0x1p-30f && ax <= 0x1p30f);
}

// The fast evaluation; false when it cannot decide (the caller then runs hit_t_fp64).
//
// Error bound. Each component below is a sum of magnitudes m (of the products that form it). The
// fp64 chain's value of p, q, det and num is within a few units of 2^-53 m of the exact value
// (products of two floats are exact in double; each later operation adds one rounding), and the
// double-float value within a few units of 2^-47 m (TwoSum and the fma products are exact; each
// df_add / df_mul rounds once at about 2^-48). eps = 2^-40 bounds the distance between the two
// values of det and num with a wide margin. With eN, eD those distances,
//   |N64 / D64 - N / D| <= (eN + |t| eD) / (|D| - eD),
// and the division (a float quotient corrected by its double-float residual) and fp64's own
// rounding of the quotient add at most 2^-39 |t|. The inputs are limited to magnitudes in
// [2^-30, 2^30] (or zero) so that every fma product and its error term stay normal floats.
LMGPU_HT_FN bool hit_t_fast(const float o[3], const float d[3], const float p1[3], const float e1[3], const float e2[3],
                            float& out) {
    for (int i = 0; i < 3; i++)
        if (!in_range(o[i]) || !in_range(d[i]) || !in_range(p1[i]) || !in_range(e1[i]) || !in_range(e2[i])) return false;
    // p = d x e2
    const DF px = df_cross(d[1], e2[2], e2[1], d[2]);
    const DF py = df_cross(d[2], e2[0], e2[2], d[0]);
    const DF pz = df_cross(d[0], e2[1], e2[0], d[1]);
    const float mpx = fadd(fabs_(fmul(d[1], e2[2])), fabs_(fmul(e2[1], d[2])));
    const float mpy = fadd(fabs_(fmul(d[2], e2[0])), fabs_(fmul(e2[2], d[0])));
    const float mpz = fadd(fabs_(fmul(d[0], e2[1])), fabs_(fmul(e2[0], d[1])));
    // tv = o - p1, exactly
    const DF tx = two_sum(o[0], -p1[0]), ty = two_sum(o[1], -p1[1]), tz = two_sum(o[2], -p1[2]);
    if (!in_range(tx.hi) || !in_range(ty.hi) || !in_range(tz.hi)) return false;
    // q = tv x e1
    const DF qx = df_cross(ty, e1[2], tz, e1[1]);
    const DF qy = df_cross(tz, e1[0], tx, e1[2]);
    const DF qz = df_cross(tx, e1[1], ty, e1[0]);
    const float mqx = fadd(fabs_(fmul(ty.hi, e1[2])), fabs_(fmul(e1[1], tz.hi)));
    const float mqy = fadd(fabs_(fmul(tz.hi, e1[0])), fabs_(fmul(e1[2], tx.hi)));
    const float mqz = fadd(fabs_(fmul(tx.hi, e1[1])), fabs_(fmul(e1[0], ty.hi)));
    // det = (e1x px + e1y py) + e1z pz, num = (e2x qx + e2y qy) + e2z qz
    const DF D = df_add(df_add(df_mul(px, e1[0]), df_mul(py, e1[1])), df_mul(pz, e1[2]));
    const DF N = df_add(df_add(df_mul(qx, e2[0]), df_mul(qy, e2[1])), df_mul(qz, e2[2]));
    const float mD = fadd(fadd(fmul(fabs_(e1[0]), mpx), fmul(fabs_(e1[1]), mpy)), fmul(fabs_(e1[2]), mpz));
    const float mN = fadd(fadd(fmul(fabs_(e2[0]), mqx), fmul(fabs_(e2[1]), mqy)), fmul(fabs_(e2[2]), mqz));
    const float eps = 0x1p-40f;
    const float eD = fmul(fmul(eps, mD), 1.01f), eN = fmul(fmul(eps, mN), 1.01f);
    const float aD = fabs_(D.hi);
    if (!(aD > fmul(4.f, eD)) || !finite_(D.hi) || !finite_(N.hi)) return false;
    // t = N / D: a float quotient and its correction from the residual N - q0 D
    const float q0 = fdiv(N.hi, D.hi);
    const DF r = df_add(N, df_neg(df_mul(D, q0)));
    const float q1 = fdiv(fadd(r.hi, r.lo), D.hi);
    const float f = fadd(q0, q1);
    if (!finite_(f) || !(f > 0.f) || f < 0x1p-100f || f > 0x1p100f) return false;
    const float at = fabs_(q0);
    const float B = fadd(fdiv(fmul(fadd(eN, fmul(at, eD)), 1.01f), fsub(aD, fmul(2.f, eD))), fmul(0x1p-39f, at));
    // distance from t = q0 + q1 to f, and half the smaller float gap around f
    const float diff = fabs_(fadd(fsub(q0, f), q1));
    const int32_t fb = fbits(f);
    const float up = fsub(bitsf(fb + 1), f), dn = fsub(f, bitsf(fb - 1));
    const float half_gap = fmul(0.5f, up < dn ? up : dn);
    if (!(fadd(diff, B) < fmul(half_gap, 0.999f))) return false;
    out = f;
    return true;
}

LMGPU_HT_FN float hit_t(const float o[3], const float d[3], const float p1[3], const float e1[3], const float e2[3]) {
    float t;
    if (hit_t_fast(o, d, p1, e1, e2, t)) return t;
    return hit_t_fp64(o, d, p1, e1, e2);
}

}  // namespace lmgpu_ht

// Device building blocks shared by the trace and render kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace lmgpu {

constexpr float kInf = 1e10f;  // include/lm/math.h:54
constexpr float kEps = 1e-3f;  // include/lm/math.h:55
constexpr float kPi = 3.14159265358979323846f;

// ---------------------------------------------------------------------------------------------
// fp32 vector math. The `ieee` namespace spells out every multiply and add with the _rn
// intrinsics, which the compiler never contracts into FMA, in glm's operation order; it is used
// wherever results must match the host restatement bit for bit (ray generation, triangle test).
struct f3 { float x, y, z; };
__host__ __device__ inline f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ inline f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ inline f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ inline f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ inline f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ inline f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ inline f3 operator*(float s, f3 a) { return {a.x * s, a.y * s, a.z * s}; }
__device__ inline f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
// Shading math fuses with explicit fmaf (the library is compiled with --fmad=false, so nothing is
// fused implicitly and every kernel inlining these gets the same bits).
__device__ inline float dot(f3 a, f3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
__device__ inline f3 cross(f3 a, f3 b) {
    return {fmaf(a.y, b.z, -(b.y * a.z)), fmaf(a.z, b.x, -(b.z * a.x)), fmaf(a.x, b.y, -(b.x * a.y))};
}
// a*s + b*t + c*r per component (barycentric interpolation, basis expansion)
__device__ inline f3 mix3(f3 a, float s, f3 b, float t, f3 c, float r) {
    return {fmaf(c.x, r, fmaf(b.x, t, a.x * s)), fmaf(c.y, r, fmaf(b.y, t, a.y * s)), fmaf(c.z, r, fmaf(b.z, t, a.z * s))};
}
__device__ inline f3 normalize(f3 v) { return v * (1.0f / sqrtf(dot(v, v))); }
__device__ inline float length(f3 v) { return sqrtf(dot(v, v)); }
__device__ inline float cmax(f3 v) { return fmaxf(fmaxf(v.x, v.y), v.z); }
__device__ inline bool is_zero(f3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }

namespace ieee {
__device__ inline float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ inline float add(float a, float b) { return __fadd_rn(a, b); }
__device__ inline float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ inline float div(float a, float b) { return __fdiv_rn(a, b); }
__device__ inline f3 sub3(f3 a, f3 b) { return {sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z)}; }
__device__ inline f3 add3(f3 a, f3 b) { return {add(a.x, b.x), add(a.y, b.y), add(a.z, b.z)}; }
__device__ inline f3 scale3(f3 a, float s) { return {mul(a.x, s), mul(a.y, s), mul(a.z, s)}; }
// glm compute_dot: (x*x' + y*y') + z*z'
__device__ inline float dot3(f3 a, f3 b) { return add(add(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z)); }
// glm cross: (x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x, x.x*y.y - y.x*x.y)
__device__ inline f3 cross3(f3 x, f3 y) {
    return {sub(mul(x.y, y.z), mul(y.y, x.z)), sub(mul(x.z, y.x), mul(y.z, x.x)), sub(mul(x.x, y.y), mul(y.x, x.y))};
}
// glm normalize: v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x)
__device__ inline f3 normalize3(f3 v) { return scale3(v, div(1.0f, __fsqrt_rn(dot3(v, v)))); }
}  // namespace ieee

// ---------------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC 2011), keyed per path:
//   key = (seed, 0x6c6d6770), counter = (4*vertex + slot/4, path_lo, path_hi, 0)
// Slots of one vertex: 0-7 light sample, 8-11 direction, 12 Russian roulette, 13-14 component.
struct U4 { float v[4]; };
#ifndef LMGPU_PHILOX_UNROLL
#define LMGPU_PHILOX_UNROLL 10
#endif
constexpr int kPhiloxUnroll = LMGPU_PHILOX_UNROLL;  // rounds unrolled per loop trip (code size vs loop overhead)
__device__ inline U4 philox_block(uint32_t seed, uint64_t path, uint32_t block) {
    uint32_t c0 = block, c1 = uint32_t(path), c2 = uint32_t(path >> 32), c3 = 0u;
    uint32_t k0 = seed, k1 = 0x6c6d6770u;
#pragma unroll kPhiloxUnroll
    for (int r = 0; r < 10; r++) {
        const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    const float s = 1.0f / 16777216.0f;
    return U4{{float(c0 >> 8) * s, float(c1 >> 8) * s, float(c2 >> 8) * s, float(c3 >> 8) * s}};
}

// ---------------------------------------------------------------------------------------------
// 8-wide BVH (layout in bvh_build.h).
struct Bvh8 {
    const uint4* nodes;   // 5 words per node
    const float4* tris;   // 3 words per triangle
    int32_t depth;        // levels; bounds the traversal stack
    uint32_t num_nodes;   // node index bound
    // Two-level trees (instancing): per instance 4 float4, the rows of its local-from-world
    // transform and {root node, first hit index, 0, 0} as bits; null for single-level trees.
    const float4* inst;
    uint32_t max_visits;  // node visits one ray can make; more flag corruption
};

struct TraceHit {
    float t, u, v;
    int32_t id;
};

// Moller-Trumbore exactly as accel_sahbvh.cpp:58-75 in fp32 (IEEE ops, no FMA). Returns true and
// fills t/u/v if accepted in [tl, th].
__device__ inline bool tri_test(f3 o, f3 d, f3 p1, f3 e1, f3 e2, float tl, float th, float& t, float& u, float& v) {
    using ieee::add; using ieee::mul; using ieee::div;
    const f3 p = ieee::cross3(d, e2);
    const f3 tv = ieee::sub3(o, p1);
    const f3 q = ieee::cross3(tv, e1);
    const float det = ieee::dot3(e1, p);
    const float ad = fabsf(det);
    const float s = copysignf(1.0f, det);
    const float uu = mul(ieee::dot3(tv, p), s);
    const float vv = mul(ieee::dot3(d, q), s);
    if (ad < 1e-8f || uu < 0.0f || vv < 0.0f || add(uu, vv) > ad) return false;
    const float tt = div(ieee::dot3(e2, q), det);
    if (tt < tl || th < tt) return false;
    t = tt;
    u = div(uu, ad);
    v = div(vv, ad);
    return true;
}

__device__ inline uint32_t byte_of(uint32_t w, int k) { return (w >> (8 * k)) & 0xffu; }

// Three-input min / max (one instruction each on sm_100 and later; exact, like the two-input
// forms, so the slab test's result does not change).
#ifndef LMGPU_TRAV_SPLIT
// persistent traversal steps: 0 = a node and all its entered leaf triangles per step (trav_step);
// 1 = a node or one triangle per step (trav_step_split); 2 = as 1, and a closest-hit step that
// tests a node's last pending triangle goes on to the next node (measured on the displaced-sphere
// frame: extension 70.7 -> 64.5 ms, shadow 27.5 -> 27.2 ms per 64-spp frame)
#define LMGPU_TRAV_SPLIT 2
#endif

#ifndef LMGPU_NO_MINMAX3
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
#else
__device__ __forceinline__ float fmax3(float a, float b, float c) { return fmaxf(fmaxf(a, b), c); }
__device__ __forceinline__ float fmin3(float a, float b, float c) { return fminf(fminf(a, b), c); }
#endif

// Permutes the 8 slot bits of `m` so that bit (s ^ oct) holds slot s.
__device__ inline uint32_t oct_permute(uint32_t m, uint32_t oct) {
    if (oct & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (oct & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (oct & 4u) m = ((m & 0x0fu) << 4) | ((m >> 4) & 0x0fu);
    return m;
}

// Ray traversal of the 8-wide BVH. Closest hit: the smallest t over every triangle whose test
// accepts the ray in [tmin, tmax], ties broken toward the smaller flattened index. Any hit
// (`any_hit`): ends at the first accepted triangle. The per-thread stack of sibling groups
// lives in shared memory: stk[i * stride] for i < bvh.depth. Child boxes carry a margin of one
// quantum and the slab comparison widens by 2^-18 relative, which bounds the rounding of the
// one-FMA slab distances (see the node visit below), so no triangle the exact test would accept
// is culled.
//
// The traversal is a resumable state (Trav) advanced one node visit at a time by trav_step, so
// a persistent kernel can interleave rays on a lane (dynamic ray fetch); trace_bvh8 runs one ray
// to the end. Either way a ray's visits, tests and result are the same.
//
// Two-level trees (kTwoLevel): a top-level child whose node carries the instance marker
// (exponent byte 0xFF) stands for one instance. Visiting it saves the world ray, moves the ray
// into the instance's local frame (o' = M^-1 o, d' = M^-1 d, not renormalized, so t keeps its
// meaning and best.t stays valid), records the stack level and continues at the instance's BLAS
// root; hit indices get the instance's first hit index added. When the traversal pops back to
// the recorded level the world ray is restored and the top level resumes. One instancing level,
// as accel::embreeinstanced builds (accel_embree_instanced.cpp:84-230).
struct Trav {
    f3 o, d, inv;
    float tmin;
    uint32_t oct;
    int sp;
    uint32_t node;
    uint32_t nvis, ntri;
    TraceHit best;
    // two-level only (never read, so never allocated, in single-level code)
    f3 wo, wd;
    int inst_sp;
    int32_t id_base;
#if LMGPU_TRAV_SPLIT
    // split steps: the entered leaf triangles of the last node, tested one per step
    uint32_t tri_base, tri_mask;
#endif
};

__device__ inline void trav_set_ray(Trav& s, f3 o, f3 d) {
    s.o = o;
    s.d = d;
    // Slab reciprocals from a direction whose zero (or tiny) components are replaced by +-1e-20,
    // keeping the sign: every slab distance stays finite (an exact zero would give infinities and
    // then NaN in the one-FMA form, which would disable culling on that axis). The triangle test
    // still uses the true direction.
    const float dxs = fabsf(d.x) > 1e-20f ? d.x : copysignf(1e-20f, d.x);
    const float dys = fabsf(d.y) > 1e-20f ? d.y : copysignf(1e-20f, d.y);
    const float dzs = fabsf(d.z) > 1e-20f ? d.z : copysignf(1e-20f, d.z);
    s.inv = {1.0f / dxs, 1.0f / dys, 1.0f / dzs};
    s.oct = (signbit(d.x) ? 1u : 0u) | (signbit(d.y) ? 2u : 0u) | (signbit(d.z) ? 4u : 0u);
}

__device__ inline void trav_init(Trav& s, f3 o, f3 d, float tmin, float tmax) {
    trav_set_ray(s, o, d);
    s.tmin = tmin;
    s.best = TraceHit{tmax, 0.f, 0.f, -1};
    s.sp = 0;
    s.node = 0;
    s.nvis = 0;
    s.ntri = 0;
    s.inst_sp = -1;
    s.id_base = 0;
#if LMGPU_TRAV_SPLIT
    s.tri_mask = 0u;
#endif
}

// Visits s.node (testing the triangles of every leaf child the ray enters) and moves to the next
// node. Returns true when the traversal has ended; s.best is then the result. Sets *err (and
// ends) on a stack overflow (1) or a visit count above the node count (2), which only a corrupt
// BVH can cause.
template <bool kAnyHit, bool kCount, bool kTwoLevel = false>
__device__ __forceinline__ bool trav_step(const Bvh8& bvh, Trav& s, uint32_t* stk_base, uint32_t* stk_bits, int stride,
                                          int* err) {
    if (s.node >= bvh.num_nodes || s.nvis >= bvh.max_visits) { *err = 2; return true; }
    const uint4* np = bvh.nodes + size_t(s.node) * 5;
    const uint4 w0 = __ldg(np), w1 = __ldg(np + 1);
    s.nvis++;
    if (kTwoLevel && (w0.w & 0xffu) == 0xffu) {
        // instance pseudo-node: continue in the instance's frame at its BLAS root
        const float4* ip = bvh.inst + size_t(w1.x) * 4;
        const float4 r0 = __ldg(ip), r1 = __ldg(ip + 1), r2 = __ldg(ip + 2);
        const uint4 m = __ldg(reinterpret_cast<const uint4*>(ip + 3));
        s.wo = s.o;
        s.wd = s.d;
        const f3 lo = {r0.x * s.o.x + r0.y * s.o.y + r0.z * s.o.z + r0.w, r1.x * s.o.x + r1.y * s.o.y + r1.z * s.o.z + r1.w,
                       r2.x * s.o.x + r2.y * s.o.y + r2.z * s.o.z + r2.w};
        const f3 ld = {r0.x * s.d.x + r0.y * s.d.y + r0.z * s.d.z, r1.x * s.d.x + r1.y * s.d.y + r1.z * s.d.z,
                       r2.x * s.d.x + r2.y * s.d.y + r2.z * s.d.z};
        trav_set_ray(s, lo, ld);
        s.inst_sp = s.sp;
        s.id_base = int32_t(m.y);
        s.node = m.x;
        return false;
    }
    const uint4 w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
    const uint32_t oct = s.oct;
    // Slab distances with one FMA per plane. Plane q of an axis lies at p + q*s; with
    // a = s*inv and b = (p - o)*inv, t = q*a + b. The byte is unpacked straight into the float
    // X = 2^23 + 256*q (one byte permute), so t = fma(X, a/256, b - 2^15*a): the large offset
    // cancels exactly inside the FMA. Error: about 5 ulp relative plus 0.003 quanta absolute;
    // the builder leaves one quantum of margin around every child box and the comparison
    // widens by 2^-18 relative, so the test never culls a box the exact ray enters.
    const float sx = __uint_as_float((w0.w & 0xffu) << 23);
    const float sy = __uint_as_float(((w0.w >> 8) & 0xffu) << 23);
    const float sz = __uint_as_float(((w0.w >> 16) & 0xffu) << 23);
    const uint32_t imask = w0.w >> 24;
    const float ax = sx * s.inv.x, ay = sy * s.inv.y, az = sz * s.inv.z;
    const float bx = (__uint_as_float(w0.x) - s.o.x) * s.inv.x;
    const float by = (__uint_as_float(w0.y) - s.o.y) * s.inv.y;
    const float bz = (__uint_as_float(w0.z) - s.o.z) * s.inv.z;
    const float ax8 = ax * 0.00390625f, ay8 = ay * 0.00390625f, az8 = az * 0.00390625f;
    const float bx8 = fmaf(-32768.0f, ax, bx), by8 = fmaf(-32768.0f, ay, by), bz8 = fmaf(-32768.0f, az, bz);
    // near/far plane bytes per axis, chosen by the ray's octant
    const uint32_t lx0 = w2.x, lx1 = w2.y, ly0 = w2.z, ly1 = w2.w, lz0 = w3.x, lz1 = w3.y;
    const uint32_t hx0 = w3.z, hx1 = w3.w, hy0 = w4.x, hy1 = w4.y, hz0 = w4.z, hz1 = w4.w;
    const uint32_t nx0 = (oct & 1u) ? hx0 : lx0, nx1 = (oct & 1u) ? hx1 : lx1;
    const uint32_t fx0 = (oct & 1u) ? lx0 : hx0, fx1 = (oct & 1u) ? lx1 : hx1;
    const uint32_t ny0 = (oct & 2u) ? hy0 : ly0, ny1 = (oct & 2u) ? hy1 : ly1;
    const uint32_t fy0 = (oct & 2u) ? ly0 : hy0, fy1 = (oct & 2u) ? ly1 : hy1;
    const uint32_t nz0 = (oct & 4u) ? hz0 : lz0, nz1 = (oct & 4u) ? hz1 : lz1;
    const uint32_t fz0 = (oct & 4u) ? lz0 : hz0, fz1 = (oct & 4u) ? lz1 : hz1;
    uint32_t hitmask = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const uint32_t sel = 0x5404u | (uint32_t(k & 3) << 4);  // bytes: 00, q, 00, 4B
        const float qnx = __uint_as_float(__byte_perm(k < 4 ? nx0 : nx1, 0x4B00u, sel));
        const float qfx = __uint_as_float(__byte_perm(k < 4 ? fx0 : fx1, 0x4B00u, sel));
        const float qny = __uint_as_float(__byte_perm(k < 4 ? ny0 : ny1, 0x4B00u, sel));
        const float qfy = __uint_as_float(__byte_perm(k < 4 ? fy0 : fy1, 0x4B00u, sel));
        const float qnz = __uint_as_float(__byte_perm(k < 4 ? nz0 : nz1, 0x4B00u, sel));
        const float qfz = __uint_as_float(__byte_perm(k < 4 ? fz0 : fz1, 0x4B00u, sel));
        const float tn = fmax3(fmaf(qnx, ax8, bx8), fmaf(qny, ay8, by8), fmaxf(fmaf(qnz, az8, bz8), s.tmin));
        const float tf0 = fmin3(fmaf(qfx, ax8, bx8), fmaf(qfy, ay8, by8), fminf(fmaf(qfz, az8, bz8), s.best.t));
        // Widening the far side by 2^-18 covers the relative error of both sides. Empty slots
        // hold inverted boxes (qlo = 255, qhi = 0) that no ray enters; one accepted through
        // rounding is a leaf of zero triangles.
        if (tn <= tf0 * 1.0000038f) hitmask |= 1u << k;
    }
    // ---- leaf children: test their triangles now -----------------------------------------------
    uint32_t leaves = hitmask & ~imask;
    while (leaves) {
        const int k = __ffs(leaves) - 1;
        leaves &= leaves - 1;
        const uint32_t meta = byte_of(k < 4 ? w1.z : w1.w, k & 3);
        const uint32_t cnt = meta >> 5, off = meta & 31u;
        for (uint32_t j = 0; j < cnt; j++) {
            const float4* tp = bvh.tris + size_t(w1.y + off + j) * 3;
            const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
            if (kCount) s.ntri++;
            float t, u, v;
            if (tri_test(s.o, s.d, mk(a.x, a.y, a.z), mk(a.w, b.x, b.y), mk(b.z, b.w, c.x), s.tmin, s.best.t, t, u, v)) {
                const int32_t id = (kTwoLevel ? s.id_base : 0) + int32_t(__float_as_uint(c.y));
                if (kAnyHit) {
                    s.best = TraceHit{t, u, v, id};
                    return true;
                }
                if (t < s.best.t || s.best.id < 0 || id < s.best.id) s.best = TraceHit{t, u, v, id};
            }
        }
    }
    // ---- next node: nearest-first by octant order ----------------------------------------------
    uint32_t inner = oct_permute(hitmask & imask, oct);
    uint32_t g_base = w1.x, g_imask = imask;
    if (inner == 0u) {
        if (kTwoLevel && s.sp == s.inst_sp) {  // the instance is done: back to the world ray
            trav_set_ray(s, s.wo, s.wd);
            s.inst_sp = -1;
            s.id_base = 0;
        }
        if (s.sp == 0) return true;
        s.sp--;
        g_base = stk_base[s.sp * stride];
        const uint32_t bits = stk_bits[s.sp * stride];
        g_imask = bits >> 8;
        inner = bits & 0xffu;
    }
    const int k = __ffs(inner) - 1;
    inner &= inner - 1;
    const uint32_t slot = uint32_t(k) ^ s.oct;
    s.node = g_base + __popc(g_imask & ((1u << slot) - 1u));
    if (inner != 0u) {
        if (s.sp >= bvh.depth) { *err = 1; return true; }
        stk_base[s.sp * stride] = g_base;
        stk_bits[s.sp * stride] = (g_imask << 8) | inner;
        s.sp++;
    }
    return false;
}

#if LMGPU_TRAV_SPLIT
// trav_step with finer steps (after the triangle-postponing traversal of Ylitie et al., HPG 2017):
// a node step records the triangles of the leaf children the ray enters as a mask; each later
// step tests one of them; the next node is visited once the mask is empty. The order of tests is
// trav_step's, so the result is the same; a warp's lanes now diverge between a node step and
// one triangle test instead of waiting for the lane with the most triangles.
template <bool kAnyHit, bool kCount, bool kTwoLevel = false>
__device__ __forceinline__ bool trav_step_split(const Bvh8& bvh, Trav& s, uint32_t* stk_base, uint32_t* stk_bits, int stride,
                                                int* err) {
    if (s.tri_mask) {
        const int j = __ffs(s.tri_mask) - 1;
        s.tri_mask &= s.tri_mask - 1u;
        const float4* tp = bvh.tris + size_t(s.tri_base + uint32_t(j)) * 3;
        const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
        if (kCount) s.ntri++;
        float t, u, v;
        if (tri_test(s.o, s.d, mk(a.x, a.y, a.z), mk(a.w, b.x, b.y), mk(b.z, b.w, c.x), s.tmin, s.best.t, t, u, v)) {
            const int32_t id = (kTwoLevel ? s.id_base : 0) + int32_t(__float_as_uint(c.y));
            if (kAnyHit) {
                s.best = TraceHit{t, u, v, id};
                return true;
            }
            if (t < s.best.t || s.best.id < 0 || id < s.best.id) s.best = TraceHit{t, u, v, id};
        }
        // closest hit (mode 2): after the last pending triangle go on to the next node in the same
        // step; any hit keeps one triangle per step (measured faster for shadow rays)
        if (kAnyHit || LMGPU_TRAV_SPLIT != 2) return s.tri_mask == 0u && s.node == 0xffffffffu;
        if (s.tri_mask != 0u) return false;
    }
    if (s.node == 0xffffffffu) return true;
    if (s.node >= bvh.num_nodes || s.nvis >= bvh.max_visits) { *err = 2; return true; }
    const uint4* np = bvh.nodes + size_t(s.node) * 5;
    const uint4 w0 = __ldg(np), w1 = __ldg(np + 1);
    s.nvis++;
    if (kTwoLevel && (w0.w & 0xffu) == 0xffu) {
        const float4* ip = bvh.inst + size_t(w1.x) * 4;
        const float4 r0 = __ldg(ip), r1 = __ldg(ip + 1), r2 = __ldg(ip + 2);
        const uint4 m = __ldg(reinterpret_cast<const uint4*>(ip + 3));
        s.wo = s.o;
        s.wd = s.d;
        const f3 lo = {r0.x * s.o.x + r0.y * s.o.y + r0.z * s.o.z + r0.w, r1.x * s.o.x + r1.y * s.o.y + r1.z * s.o.z + r1.w,
                       r2.x * s.o.x + r2.y * s.o.y + r2.z * s.o.z + r2.w};
        const f3 ld = {r0.x * s.d.x + r0.y * s.d.y + r0.z * s.d.z, r1.x * s.d.x + r1.y * s.d.y + r1.z * s.d.z,
                       r2.x * s.d.x + r2.y * s.d.y + r2.z * s.d.z};
        trav_set_ray(s, lo, ld);
        s.inst_sp = s.sp;
        s.id_base = int32_t(m.y);
        s.node = m.x;
        return false;
    }
    const uint4 w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
    const uint32_t oct = s.oct;
    const float sx = __uint_as_float((w0.w & 0xffu) << 23);
    const float sy = __uint_as_float(((w0.w >> 8) & 0xffu) << 23);
    const float sz = __uint_as_float(((w0.w >> 16) & 0xffu) << 23);
    const uint32_t imask = w0.w >> 24;
    const float ax = sx * s.inv.x, ay = sy * s.inv.y, az = sz * s.inv.z;
    const float bx = (__uint_as_float(w0.x) - s.o.x) * s.inv.x;
    const float by = (__uint_as_float(w0.y) - s.o.y) * s.inv.y;
    const float bz = (__uint_as_float(w0.z) - s.o.z) * s.inv.z;
    const float ax8 = ax * 0.00390625f, ay8 = ay * 0.00390625f, az8 = az * 0.00390625f;
    const float bx8 = fmaf(-32768.0f, ax, bx), by8 = fmaf(-32768.0f, ay, by), bz8 = fmaf(-32768.0f, az, bz);
    const uint32_t lx0 = w2.x, lx1 = w2.y, ly0 = w2.z, ly1 = w2.w, lz0 = w3.x, lz1 = w3.y;
    const uint32_t hx0 = w3.z, hx1 = w3.w, hy0 = w4.x, hy1 = w4.y, hz0 = w4.z, hz1 = w4.w;
    const uint32_t nx0 = (oct & 1u) ? hx0 : lx0, nx1 = (oct & 1u) ? hx1 : lx1;
    const uint32_t fx0 = (oct & 1u) ? lx0 : hx0, fx1 = (oct & 1u) ? lx1 : hx1;
    const uint32_t ny0 = (oct & 2u) ? hy0 : ly0, ny1 = (oct & 2u) ? hy1 : ly1;
    const uint32_t fy0 = (oct & 2u) ? ly0 : hy0, fy1 = (oct & 2u) ? ly1 : hy1;
    const uint32_t nz0 = (oct & 4u) ? hz0 : lz0, nz1 = (oct & 4u) ? hz1 : lz1;
    const uint32_t fz0 = (oct & 4u) ? lz0 : hz0, fz1 = (oct & 4u) ? lz1 : hz1;
    uint32_t hitmask = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const uint32_t sel = 0x5404u | (uint32_t(k & 3) << 4);
        const float qnx = __uint_as_float(__byte_perm(k < 4 ? nx0 : nx1, 0x4B00u, sel));
        const float qfx = __uint_as_float(__byte_perm(k < 4 ? fx0 : fx1, 0x4B00u, sel));
        const float qny = __uint_as_float(__byte_perm(k < 4 ? ny0 : ny1, 0x4B00u, sel));
        const float qfy = __uint_as_float(__byte_perm(k < 4 ? fy0 : fy1, 0x4B00u, sel));
        const float qnz = __uint_as_float(__byte_perm(k < 4 ? nz0 : nz1, 0x4B00u, sel));
        const float qfz = __uint_as_float(__byte_perm(k < 4 ? fz0 : fz1, 0x4B00u, sel));
        const float tn = fmax3(fmaf(qnx, ax8, bx8), fmaf(qny, ay8, by8), fmaxf(fmaf(qnz, az8, bz8), s.tmin));
        const float tf0 = fmin3(fmaf(qfx, ax8, bx8), fmaf(qfy, ay8, by8), fminf(fmaf(qfz, az8, bz8), s.best.t));
        if (tn <= tf0 * 1.0000038f) hitmask |= 1u << k;
    }
    // the entered leaf children's triangles, in trav_step's order (children ascending, then the
    // triangles of each): one mask bit per triangle slot after the node's first triangle
    uint32_t leaves = hitmask & ~imask, tmask = 0u;
    while (leaves) {
        const int k = __ffs(leaves) - 1;
        leaves &= leaves - 1;
        const uint32_t meta = byte_of(k < 4 ? w1.z : w1.w, k & 3);
        const uint32_t cnt = meta >> 5, off = meta & 31u;
        tmask |= ((1u << cnt) - 1u) << off;
    }
    s.tri_base = w1.y;
    s.tri_mask = tmask;
    // next node (visited after these triangles)
    uint32_t inner = oct_permute(hitmask & imask, oct);
    uint32_t g_base = w1.x, g_imask = imask;
    if (inner == 0u) {
        if (kTwoLevel && s.sp == s.inst_sp) {
            // the instance is done once its last node's triangles are: test them in this frame
            // first (a node sentinel would lose the frame switch), so finish them here
            while (s.tri_mask) {
                const int j = __ffs(s.tri_mask) - 1;
                s.tri_mask &= s.tri_mask - 1u;
                const float4* tp = bvh.tris + size_t(s.tri_base + uint32_t(j)) * 3;
                const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                if (kCount) s.ntri++;
                float t, u, v;
                if (tri_test(s.o, s.d, mk(a.x, a.y, a.z), mk(a.w, b.x, b.y), mk(b.z, b.w, c.x), s.tmin, s.best.t, t, u, v)) {
                    const int32_t id = s.id_base + int32_t(__float_as_uint(c.y));
                    if (kAnyHit) {
                        s.best = TraceHit{t, u, v, id};
                        return true;
                    }
                    if (t < s.best.t || s.best.id < 0 || id < s.best.id) s.best = TraceHit{t, u, v, id};
                }
            }
            trav_set_ray(s, s.wo, s.wd);
            s.inst_sp = -1;
            s.id_base = 0;
        }
        if (s.sp == 0) {
            s.node = 0xffffffffu;  // no node left: done after the pending triangles
            return s.tri_mask == 0u;
        }
        s.sp--;
        g_base = stk_base[s.sp * stride];
        const uint32_t bits = stk_bits[s.sp * stride];
        g_imask = bits >> 8;
        inner = bits & 0xffu;
    }
    const int k = __ffs(inner) - 1;
    inner &= inner - 1;
    const uint32_t slot = uint32_t(k) ^ s.oct;
    s.node = g_base + __popc(g_imask & ((1u << slot) - 1u));
    if (inner != 0u) {
        if (s.sp >= bvh.depth) { *err = 1; return true; }
        stk_base[s.sp * stride] = g_base;
        stk_bits[s.sp * stride] = (g_imask << 8) | inner;
        s.sp++;
    }
    return false;
}
#endif

// One ray to the end. Adds the node visits and triangle tests to *nodes_visited / *tris_tested
// when kCount.
template <bool kAnyHit, bool kCount, bool kTwoLevel = false>
__device__ inline TraceHit trace_bvh8(const Bvh8& bvh, f3 o, f3 d, float tmin, float tmax, uint32_t* stk_base,
                                      uint32_t* stk_bits, int stride, uint32_t* nodes_visited, uint32_t* tris_tested,
                                      int* err) {
    Trav s;
    trav_init(s, o, d, tmin, tmax);
    while (!trav_step<kAnyHit, kCount, kTwoLevel>(bvh, s, stk_base, stk_bits, stride, err)) {
    }
    if (kCount) { *nodes_visited += s.nvis; *tris_tested += s.ntri; }
    return s.best;
}

// Dynamic ray fetch for the persistent trace kernels: `self` hands out queue entries (zero at
// launch); `other`, when set, is the counter of another trace kernel that this launch resets for
// that kernel's next launch (the path tracers' extension and shadow kernels alternate on one
// stream, so neither counter is in use while the other kernel runs). refill: see Tuning.
struct Fetch {
    int* self;
    int* other;
    int refill;
};

// Persistent traversal with dynamic ray fetch (Aila & Laine, HPG 2009): every lane of a warp
// holds one ray in flight; once fewer than f.refill lanes still trace, the idle lanes take the
// next entries of the queue (one atomic per warp), so a warp no longer waits for its slowest
// ray. begin(k, s, B) loads entry k into the traversal state (and B, the BVH it traverses);
// end(k, s) consumes the finished traversal. Called by every thread of full warps.
template <bool kAnyHit, bool kCount, bool kTwoLevel, typename Begin, typename End>
__device__ __forceinline__ void fetch_loop(int n, const Fetch& f, const Bvh8& bvh0, uint32_t* sb, uint32_t* sbits,
                                           int stride, int* lerr, Begin begin, End end) {
    const int lane = int(threadIdx.x & 31u);
    const unsigned below = (1u << lane) - 1u;
    Trav s;
    Bvh8 B = bvh0;
    int k = 0;
    bool active = false, exhausted = false;
    while (true) {
        if (!exhausted) {
            const unsigned idle = __ballot_sync(0xffffffffu, !active);
            if (idle) {
                const int leader = __ffs(idle) - 1;
                int base = 0;
                if (lane == leader) base = atomicAdd(f.self, __popc(idle));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (base + __popc(idle) >= n) exhausted = true;  // warp-uniform
                if (!active) {
                    k = base + __popc(idle & below);
                    if (k < n) {
                        begin(k, s, B);
                        active = true;
                    }
                }
            }
        }
        if (__ballot_sync(0xffffffffu, active) == 0u) break;
        const int keep = exhausted ? 1 : f.refill;
        do {
#if LMGPU_TRAV_SPLIT
            // two-level trees keep whole-node steps (measured faster on the instanced frame)
            if (active && (kTwoLevel ? trav_step<kAnyHit, kCount, kTwoLevel>(B, s, sb, sbits, stride, lerr)
                                     : trav_step_split<kAnyHit, kCount, kTwoLevel>(B, s, sb, sbits, stride, lerr))) {
#else
            if (active && trav_step<kAnyHit, kCount, kTwoLevel>(B, s, sb, sbits, stride, lerr)) {
#endif
                end(k, s);
                active = false;
            }
        } while (__popc(__ballot_sync(0xffffffffu, active)) >= keep);
    }
}

}  // namespace lmgpu

// Scene, film and renderer C-ABI (include/lmgpu.h): renderer::raycast as one kernel, renderer::pt
// as a wavefront of generate -> [extend -> shade -> shadow] x (max_verts - 1) kernels over
// structure-of-arrays queues whose lengths stay on the device.
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>

#include "lmgpu_dev.cuh"
#include "runtime.h"

namespace cg = cooperative_groups;

namespace lmgpu {

Bvh8 device_view(const lmgpu_accel* a);
size_t trace_smem(const lmgpu_accel* a);

// ---------------------------------------------------------------------------------------------
// Device scene
struct DevMaterial {
    int32_t type;
    float c[3];
    float ax, ay, ni;
    float ks[3];  // mixture: the glossy lobe's Ks
    int32_t map_kd, mask;  // texture indices or -1 (diffuse / mixture mapKd; mixture alpha mask)
    float alpha;           // mixture: the alpha mask's value at the shaded point (1 without a mask)
};
// texture::bitmap (texture_bitmap.cpp): w x h texels of c (3 or 4) floats at texels + off, row 0
// at the bottom
struct DevTexture {
    int32_t w, h, c, pad;
    int64_t off;
};
struct DevLight {
    int32_t type;
    float ke[3];
    int32_t tri_off, tri_cnt, cdf_off;
    float invA_J;  // (1 / mesh-local area) / |det M|, light_area.cpp:41-46
    int32_t env_w, env_h, tex_off, marg_off, cond_off;
    float rot, scale;
    float v[3];    // point: position; directional: the normalized direction it travels
};
// Scene features that select a specialised shade kernel: code for a feature the scene lacks is
// left out of it (the shade kernels are bound by instruction fetch)
constexpr uint32_t kFeatEnvTex = 1u;    // a textured environment light (light::env)
constexpr uint32_t kFeatMixture = 2u;   // material::mixture_wavefrontobj
constexpr uint32_t kFeatTwoLevel = 4u;  // a two-level (instanced) tree
constexpr uint32_t kFeatDelta = 8u;     // light::point or light::directional
constexpr uint32_t kFeatTexture = 16u;  // an image texture on a material (mapKd, alpha mask)
constexpr uint32_t kFeatAll = 31u;

struct DevScene {
    Bvh8 bvh;
    const float4* shade;   // 6 words per triangle: p1 p2 p3 n1 n2 n3 gn prim
    const int2* prim_ml;   // (material, light) per primitive
    const DevMaterial* mats;
    const DevLight* lights;
    int32_t num_lights;
    int32_t env_light;     // index into lights or -1
    const float4* ltri;    // 3 words per light triangle: (a, b.x) (b.yz, c.xy) (c.z, gn)
    const float* cdf;      // area-light CDFs (tri_cnt + 1 entries each)
    const float* env;      // env texels, marginal and conditional CDFs
    f3 cam_p, cam_u, cam_v, cam_w;
    float tf, aspect;
    int32_t has_camera;
    // Two-level scenes: shading records are per BLAS in the BLAS's frame; per instance 7 float4:
    // world-from-local rows (3), normal-matrix rows (3), {first hit index, first shading record}.
    const float4* inst;
    int32_t num_inst;      // 0: records are in world space, indexed by hit index
    // bounding sphere of the scene's triangles (scene.cpp:288-311, light_envconst.cpp:38-43): where
    // light tracing starts the rays of an environment light; radius 0 without triangles
    f3 bound_c;
    float bound_r;
    uint32_t feat;  // kFeat* bits present in the scene
    // image textures (kFeatTexture): per shading record the three corners' texture coordinates
    const float* uv;
    const DevTexture* tex;
    const float* texels;
};

}  // namespace lmgpu

struct lmgpu_scene {
    lmgpu_accel* accel = nullptr;
    lmgpu::DevScene dev{};
    lmgpu::DevBuf shade, prim_ml, mats, lights, ltri, cdf, env, uv, tex, texels;
    lmgpu::DevBuf inst;      // two-level scenes: per-instance shading transforms
    lmgpu::DevBuf counters;  // raycast error flag
};

struct lmgpu_film {
    int32_t w = 0, h = 0;
    lmgpu::DevBuf sum, out;
    double scale = 1.0;
    int64_t accumulated_spp = 0;
    // split passes (lmgpu_pt_params::split_passes): odd global passes accumulate in sum_odd
    lmgpu::DevBuf sum_odd;
    lmgpu::DevBuf mse_acc;  // lmgpu_film_rel_mse's accumulator, allocated once
    bool split = false;
    int64_t passes_even = 0, passes_odd = 0;
};

namespace lmgpu {

// ---------------------------------------------------------------------------------------------
// Geometry (include/lm/surface.h)
struct Geom {
    f3 p, n, gn, wo;
    f3 u, v;
    bool degenerated, infinite;
};

// math::orthonormal_basis (Duff et al. 2017), include/lm/math.h:540-547
__device__ inline void onb(f3 n, f3& u, f3& v) {
    const float s = copysignf(1.f, n.z);
    const float a = -1.f / (s + n.z);
    const float b = n.x * n.y * a;
    u = mk(1.f + s * n.x * n.x * a, s * b, -s * n.x);
    v = mk(b, s + n.y * n.y * a, -n.y);
}
__device__ inline Geom on_surface(f3 p, f3 n, f3 gn) {
    Geom g;
    g.p = p; g.n = n; g.gn = gn; g.wo = mk(0, 0, 0);
    g.degenerated = false; g.infinite = false;
    onb(n, g.u, g.v);
    return g;
}
__device__ inline Geom infinite_point(f3 wo) {
    Geom g;
    g.p = mk(0, 0, 0); g.n = mk(0, 0, 0); g.gn = g.n; g.u = g.n; g.v = g.n;
    g.wo = wo; g.degenerated = false; g.infinite = true;
    return g;
}
__device__ inline Geom degenerate_point(f3 p) {
    Geom g;
    g.p = p; g.n = mk(0, 0, 0); g.gn = g.n; g.u = g.n; g.v = g.n; g.wo = g.n;
    g.degenerated = true; g.infinite = false;
    return g;
}
__device__ inline bool opposite(const Geom& g, f3 a, f3 b) { return dot(a, g.n) * dot(b, g.n) <= 0.f; }

// surface.h:329-348 for a finite or degenerate s1 and any s2
__device__ inline float geometry_term(const Geom& s1, const Geom& s2) {
    f3 d;
    float L2;
    if (s2.infinite) {
        d = -s2.wo;
        L2 = 1.f;
    } else {
        d = s2.p - s1.p;
        L2 = dot(d, d);
        d = d / sqrtf(L2);
    }
    const float c1 = s1.degenerated ? 1.f : fabsf(dot(s1.n, d));
    const float c2 = (s2.degenerated || s2.infinite) ? 1.f : fabsf(dot(s2.n, -d));
    return c1 * c2 / L2;
}
// surface.h:377-390
__device__ inline float pdf_sa_to_projsa(float pdf, const Geom& g, f3 d) {
    if (g.degenerated) return pdf;
    const float J = fabsf(dot(g.n, d));
    return J == 0.f ? 0.f : pdf / J;
}
// surface.h:424-438, transport direction EL
__device__ inline float sn_correction(const Geom& g, f3 wi, f3 wo) {
    const float wi_ng = dot(wi, g.gn), wo_ng = dot(wo, g.gn);
    const float wi_ns = dot(wi, g.n), wo_ns = dot(wo, g.n);
    return (wi_ng * wi_ns <= 0.f || wo_ng * wo_ns <= 0.f) ? 0.f : 1.f;
}

// surface.h:424-438, transport direction LE: wi.ns wo.ng / (wo.ns wi.ng)
__device__ inline float sn_correction_le(const Geom& g, f3 wi, f3 wo) {
    const float wi_ng = dot(wi, g.gn), wo_ng = dot(wo, g.gn);
    const float wi_ns = dot(wi, g.n), wo_ns = dot(wo, g.n);
    if (wi_ng * wi_ns <= 0.f || wo_ng * wo_ns <= 0.f) return 0.f;
    return wi_ns * wo_ng / (wo_ns * wi_ng);
}

template <uint32_t kF = kFeatAll>
__device__ inline Geom surface_at(const DevScene& S, int32_t id, float u, float v, int32_t& prim, int64_t* rec_out = nullptr) {
    if ((kF & kFeatTwoLevel) && S.num_inst > 0) {
        // instance holding hit index id (the last whose first hit index is <= id), then the local
        // surface point moved to world space as scene.cpp:335-343 does with the hit's transform
        int lo = 0, hi = S.num_inst;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (int32_t(__float_as_uint(__ldg(S.inst + 7 * size_t(mid) + 6).x)) <= id) lo = mid; else hi = mid;
        }
        const float4* ip = S.inst + 7 * size_t(lo);
        const float4 m0 = __ldg(ip), m1 = __ldg(ip + 1), m2 = __ldg(ip + 2);
        const float4 q0 = __ldg(ip + 3), q1 = __ldg(ip + 4), q2 = __ldg(ip + 5), mt = __ldg(ip + 6);
        const int64_t rec = int64_t(__float_as_uint(mt.y)) + (id - int32_t(__float_as_uint(mt.x)));
        if (rec_out) *rec_out = rec;
        const float4* sp = S.shade + size_t(rec) * 6;
        const float4 s0 = __ldg(sp), s1 = __ldg(sp + 1), s2 = __ldg(sp + 2), s3 = __ldg(sp + 3), s4 = __ldg(sp + 4),
                     s5 = __ldg(sp + 5);
        const f3 p1 = mk(s0.x, s0.y, s0.z), p2 = mk(s0.w, s1.x, s1.y), p3 = mk(s1.z, s1.w, s2.x);
        const f3 n1 = mk(s2.y, s2.z, s2.w), n2 = mk(s3.x, s3.y, s3.z), n3 = mk(s3.w, s4.x, s4.y);
        const f3 gl = mk(s4.z, s4.w, s5.x);
        prim = int32_t(__float_as_uint(s5.y));
        const float b0 = 1.f - u - v;
        const f3 pl = mix3(p1, b0, p2, u, p3, v);
        const f3 nl = normalize(mix3(n1, b0, n2, u, n3, v));
        const f3 p = mk(m0.x * pl.x + m0.y * pl.y + m0.z * pl.z + m0.w, m1.x * pl.x + m1.y * pl.y + m1.z * pl.z + m1.w,
                        m2.x * pl.x + m2.y * pl.y + m2.z * pl.z + m2.w);
        const f3 n = normalize(mk(dot(mk(q0.x, q0.y, q0.z), nl), dot(mk(q1.x, q1.y, q1.z), nl), dot(mk(q2.x, q2.y, q2.z), nl)));
        const f3 gn = normalize(mk(dot(mk(q0.x, q0.y, q0.z), gl), dot(mk(q1.x, q1.y, q1.z), gl), dot(mk(q2.x, q2.y, q2.z), gl)));
        return on_surface(p, n, gn);
    }
    if (rec_out) *rec_out = id;
    const float4* sp = S.shade + size_t(id) * 6;
    const float4 s0 = __ldg(sp), s1 = __ldg(sp + 1), s2 = __ldg(sp + 2), s3 = __ldg(sp + 3), s4 = __ldg(sp + 4),
                 s5 = __ldg(sp + 5);
    const f3 p1 = mk(s0.x, s0.y, s0.z), p2 = mk(s0.w, s1.x, s1.y), p3 = mk(s1.z, s1.w, s2.x);
    const f3 n1 = mk(s2.y, s2.z, s2.w), n2 = mk(s3.x, s3.y, s3.z), n3 = mk(s3.w, s4.x, s4.y);
    const f3 gn = mk(s4.z, s4.w, s5.x);
    prim = int32_t(__float_as_uint(s5.y));
    const float b0 = 1.f - u - v;  // mix_barycentric, math.h:572-575
    const f3 p = mix3(p1, b0, p2, u, p3, v);
    const f3 n = normalize(mix3(n1, b0, n2, u, n3, v));
    return on_surface(p, n, gn);
}

// ---------------------------------------------------------------------------------------------
// Image textures (texture_bitmap.cpp:68-85): the nearest texel of the wrapped coordinate.
__device__ inline int64_t tex_index(const DevTexture& T, float tu, float tv) {
    const float uu = tu - floorf(tu), vv = tv - floorf(tv);
    const int x = min(max(int(uu * float(T.w)), 0), T.w - 1);
    const int y = min(max(int(vv * float(T.h)), 0), T.h - 1);
    return T.off + int64_t(T.c) * (int64_t(T.w) * y + x);
}
// The material at a shaded point: mapKd's texel becomes Kd (material_diffuse.cpp:70, 79, 88; the
// mixture's diffuse lobe), the alpha mask's value its alpha (model_wavefrontobj.cpp:365-368).
// Texture coordinates: mix_barycentric of the record's corners (mesh_raw.cpp:97).
__device__ inline void resolve_textures(const DevScene& S, DevMaterial& m, int64_t rec, float u, float v) {
    const float* t = S.uv + size_t(rec) * 6;
    const float b0 = 1.f - u - v;
    const float tu = fmaf(__ldg(t + 4), v, fmaf(__ldg(t + 2), u, __ldg(t) * b0));
    const float tv = fmaf(__ldg(t + 5), v, fmaf(__ldg(t + 3), u, __ldg(t + 1) * b0));
    if (m.map_kd >= 0) {
        const int64_t i = tex_index(S.tex[m.map_kd], tu, tv);
        m.c[0] = __ldg(S.texels + i);
        m.c[1] = __ldg(S.texels + i + 1);
        m.c[2] = __ldg(S.texels + i + 2);
    }
    if (m.mask >= 0) m.alpha = __ldg(S.texels + tex_index(S.tex[m.mask], tu, tv) + 3);
}

// ---------------------------------------------------------------------------------------------
// Camera (camera_pinhole.cpp)
__device__ inline f3 primary_dir(const DevScene& S, float rx, float ry) {
    using ieee::mul; using ieee::sub;
    const float x = sub(mul(2.f, rx), 1.f), y = sub(mul(2.f, ry), 1.f);
    const f3 d = ieee::normalize3(mk(mul(mul(S.aspect, S.tf), x), mul(S.tf, y), -1.f));
    return ieee::add3(ieee::add3(ieee::scale3(S.cam_u, d.x), ieee::scale3(S.cam_v, d.y)), ieee::scale3(S.cam_w, d.z));
}
__device__ inline bool raster_pos(const DevScene& S, f3 wo, float& rx, float& ry) {
    const float ex = dot(S.cam_u, wo), ey = dot(S.cam_v, wo), ez = dot(S.cam_w, wo);
    if (ez >= 0.f) return false;
    rx = (-ex / ez / S.tf / S.aspect) * .5f + .5f;
    ry = (-ey / ez / S.tf) * .5f + .5f;
    return !(rx < 0.f || rx > 1.f || ry < 0.f || ry > 1.f);
}
__device__ inline float cam_J(const DevScene& S, f3 wo) {
    const float c = -dot(S.cam_w, wo);
    const float ic = 1.f / c;
    return ic * ic * ic / (S.tf * S.tf * S.aspect * 4.f);
}
__device__ inline float cam_pdf(const DevScene& S, f3 wo) {
    float rx, ry;
    return raster_pos(S, wo, rx, ry) ? cam_J(S, wo) : 0.f;
}

// ---------------------------------------------------------------------------------------------
// Materials (material_{diffuse,glossy,glass,mirror}.cpp)
__device__ inline void basis2(const Geom& g, f3 wi, f3& n, f3& u, f3& v) {
    const bool i = dot(wi, g.n) > 0.f;
    n = i ? g.n : -g.n;
    u = g.u;
    v = i ? g.v : -g.v;
}
__device__ inline float ggx_d(const DevMaterial& m, f3 wh, f3 u, f3 v, f3 n) {
    const float a = dot(wh, u) / m.ax, b = dot(wh, v) / m.ay, c = dot(wh, n);
    const float s = a * a + b * b + c * c;
    return 1.f / (kPi * m.ax * m.ay * s * s);
}
__device__ inline float ggx_g1(const DevMaterial& m, f3 w, f3 u, f3 v, f3 n) {
    const float c = dot(w, n);
    const float s = fmaxf(kEps, sqrtf(fmaxf(0.f, 1.f - c * c)));
    const float cp = dot(w, u) / s, cs = dot(w, v) / s;
    const float a2 = (cp * m.ax) * (cp * m.ax) + (cs * m.ay) * (cs * m.ay);
    const float sc = s / c;
    return c == 0.f ? 0.f : 2.f / (1.f + sqrtf(fmaxf(0.f, 1.f + a2 * sc * sc)));
}
__device__ inline void glass_fresnel(const DevMaterial& m, const Geom& g, f3 wi, f3& wt, bool& total, float& eta, float& Fr) {
    const bool in = dot(wi, g.n) > 0.f;
    const f3 n = in ? g.n : -g.n;
    eta = in ? 1.f / m.ni : m.ni;
    const float t = dot(wi, n);
    const float t2 = 1.f - eta * eta * (1.f - t * t);
    total = t2 <= 0.f;
    if (total) {
        wt = mk(0, 0, 0);
        Fr = 1.f;
        return;
    }
    wt = eta * (n * t - wi) - n * sqrtf(fmaxf(0.f, t2));
    const float cs = in ? dot(wi, g.n) : dot(wt, g.n);
    const float r = (1.f - m.ni) / (1.f + m.ni);
    const float r2 = r * r;
    Fr = r2 + (1.f - r2) * powf(1.f - cs, 5.f);
}
__device__ inline bool mat_specular(const DevMaterial& m, int comp = 0) {
    // the mixture's component 1 is the alpha mask's pass-through (model_wavefrontobj.cpp:513-515)
    return m.type == LMGPU_MAT_GLASS || m.type == LMGPU_MAT_MIRROR || (m.type == LMGPU_MAT_MIXTURE && comp != 0);
}

// Lobes shared by the glossy and mixture materials (material_glossy.cpp:35-113) and the diffuse
// and mixture materials (material_diffuse.cpp:55-95).
__device__ inline f3 glossy_eval(const DevMaterial& m, f3 ks, const Geom& g, f3 wi, f3 wo) {
    if (opposite(g, wi, wo)) return mk(0, 0, 0);
    const f3 wh = normalize(wi + wo);
    f3 n, u, v;
    basis2(g, wi, n, u, v);
    const float f5 = powf(1.f - dot(wo, wh), 5.f);
    const f3 Fr = ks + (mk(1, 1, 1) - ks) * f5;
    const float k = ggx_d(m, wh, u, v, n) * (ggx_g1(m, wi, u, v, n) * ggx_g1(m, wo, u, v, n)) / (4.f * dot(wi, n) * dot(wo, n));
    return ks * Fr * k;
}
__device__ inline float glossy_pdf(const DevMaterial& m, const Geom& g, f3 wi, f3 wo) {
    if (opposite(g, wi, wo)) return 0.f;
    const f3 wh = normalize(wi + wo);
    f3 n, u, v;
    basis2(g, wi, n, u, v);
    return ggx_d(m, wh, u, v, n) * dot(wh, n) / (4.f * dot(wo, wh) * dot(wo, n));
}
__device__ inline bool glossy_dir(const DevMaterial& m, const Geom& g, f3 wi, float u0, float u1, f3& wo) {
    f3 n, u, v;
    basis2(g, wi, n, u, v);
    const float a1 = u0 * 2.f * kPi;
    float s1, c1;
    sincosf(a1, &s1, &c1);
    const f3 wh = normalize(sqrtf(fmaxf(0.f, u1 / (1.f - u1))) * (m.ax * c1 * u + m.ay * s1 * v) + n);
    wo = 2.f * dot(wi, wh) * wh - wi;
    return !opposite(g, wi, wo);
}
__device__ inline f3 diffuse_dir(const Geom& g, f3 wi, float u0, float u1) {
    f3 n, u, v;
    basis2(g, wi, n, u, v);
    const float r = sqrtf(fmaxf(0.f, u0)), t = 2.f * kPi * u1;
    float st, ct;
    sincosf(t, &st, &ct);
    const float x = r * ct, y = r * st;
    const float z = sqrtf(fmaxf(0.f, 1.f - x * x - y * y));
    return mix3(u, x, v, y, n, z);
}
// material::mixture_wavefrontobj: probability of the diffuse lobe, max(Kd) / (max(Kd) + max(Ks))
// (model_wavefrontobj.cpp:427-435)
__device__ inline float mixture_w(const DevMaterial& m) {
    const float wd = fmaxf(fmaxf(m.c[0], m.c[1]), m.c[2]), wg = fmaxf(fmaxf(m.ks[0], m.ks[1]), m.ks[2]);
    return (wd == 0.f && wg == 0.f) ? 1.f : wd / (wd + wg);
}

// le: transport direction LE (light tracing): refraction carries no eta^2 (material_glass.cpp:85-87)
template <uint32_t kF = kFeatAll>
__device__ inline f3 mat_eval(const DevMaterial& m, const Geom& g, f3 wi, f3 wo, int comp, bool eval_delta, bool le = false) {
    switch (m.type) {
    case LMGPU_MAT_DIFFUSE:
        if (opposite(g, wi, wo)) return mk(0, 0, 0);
        return mk(m.c[0], m.c[1], m.c[2]) / kPi;
    case LMGPU_MAT_GLOSSY:
        return glossy_eval(m, mk(m.c[0], m.c[1], m.c[2]), g, wi, wo);
    case LMGPU_MAT_MIXTURE: {  // model_wavefrontobj.cpp:496-507: the two lobes summed, times alpha
        if (!(kF & kFeatMixture)) return mk(0, 0, 0);  // not in this scene
        if ((kF & kFeatTexture) && comp != 0) {
            const float r = eval_delta ? 0.f : 1.f - m.alpha;
            return mk(r, r, r);
        }
        const f3 fd = opposite(g, wi, wo) ? mk(0, 0, 0) : mk(m.c[0], m.c[1], m.c[2]) / kPi;
        const f3 f = fd + glossy_eval(m, mk(m.ks[0], m.ks[1], m.ks[2]), g, wi, wo);
        return (kF & kFeatTexture) ? f * m.alpha : f;
    }
    case LMGPU_MAT_GLASS: {
        if (eval_delta) return mk(0, 0, 0);
        f3 wt; bool total; float eta, Fr;
        glass_fresnel(m, g, wi, wt, total, eta, Fr);
        if (comp == 0) return mk(Fr, Fr, Fr);
        const float r = le ? 1.f - Fr : (1.f - Fr) * eta * eta;
        return mk(r, r, r);
    }
    default:
        return eval_delta ? mk(0, 0, 0) : mk(1, 1, 1);
    }
}
template <uint32_t kF = kFeatAll>
__device__ inline float mat_pdf(const DevMaterial& m, const Geom& g, f3 wi, f3 wo, bool eval_delta) {
    switch (m.type) {
    case LMGPU_MAT_DIFFUSE:
        return opposite(g, wi, wo) ? 0.f : 1.f / kPi;
    case LMGPU_MAT_GLOSSY:
        return glossy_pdf(m, g, wi, wo);
    case LMGPU_MAT_MIXTURE: {  // model_wavefrontobj.cpp:484-494: the lobes' pdfs by selection probability
        if (!(kF & kFeatMixture)) return 0.f;
        const float w = mixture_w(m);
        const float pd = opposite(g, wi, wo) ? 0.f : 1.f / kPi;
        return w * pd + (1.f - w) * glossy_pdf(m, g, wi, wo);
    }
    default:
        return eval_delta ? 0.f : 1.f;
    }
}
// Returns false when no direction is produced (glossy below the surface). uc: the component
// random number of the direction sample (DirectionSampleU::udc.x), used by the mixture.
template <uint32_t kF = kFeatAll>
__device__ inline bool mat_sample(const DevMaterial& m, const Geom& g, f3 wi, int comp, float u0, float u1, float uc, f3& wo,
                                  f3& w, bool le = false) {
    switch (m.type) {
    case LMGPU_MAT_DIFFUSE:
        wo = diffuse_dir(g, wi, u0, u1);
        w = mk(m.c[0], m.c[1], m.c[2]);
        return true;
    case LMGPU_MAT_GLOSSY: {
        if (!glossy_dir(m, g, wi, u0, u1, wo)) return false;
        const f3 f = mat_eval<kF>(m, g, wi, wo, 0, false);
        const float p = mat_pdf<kF>(m, g, wi, wo, false);
        w = f / p;
        return true;
    }
    case LMGPU_MAT_MIXTURE: {  // model_wavefrontobj.cpp:437-461: one lobe sampled, weight f / p of the sum
        if (!(kF & kFeatMixture)) return false;
        if ((kF & kFeatTexture) && comp != 0) {
            // the alpha mask's pass-through (model_wavefrontobj.cpp:462-471): the reference returns
            // weight 1, not its f / p, so the path keeps only the component weight 1 / (1 - alpha)
            wo = -wi;
            w = mk(1, 1, 1);
            return true;
        }
        if (uc < mixture_w(m)) wo = diffuse_dir(g, wi, u0, u1);
        else if (!glossy_dir(m, g, wi, u0, u1, wo)) return false;
        const f3 f = mat_eval<kF>(m, g, wi, wo, 0, false);
        const float p = mat_pdf<kF>(m, g, wi, wo, false);
        w = f / p;
        return true;
    }
    case LMGPU_MAT_GLASS: {
        if (comp == 0) {
            wo = 2.f * dot(wi, g.n) * g.n - wi;
        } else {
            f3 wt; bool total; float eta, Fr;
            glass_fresnel(m, g, wi, wt, total, eta, Fr);
            wo = wt;
        }
        w = mat_eval<kF>(m, g, wi, wo, comp, false, le);  // pdf of a component direction is 1
        return true;
    }
    default:
        wo = 2.f * dot(wi, g.n) * g.n - wi;
        w = mk(1, 1, 1);
        return true;
    }
}

// ---------------------------------------------------------------------------------------------
// Lights (light_area.cpp, light_envconst.cpp, light_env.cpp)
__device__ inline int cdf_sample(const float* c, int n, float u) {
    // upper_bound over c[0..n], then clamp(index - 1, 0, n - 1)  (math.h:367-370)
    int lo = 0, hi = n + 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (u < __ldg(c + mid)) hi = mid; else lo = mid + 1;
    }
    return min(max(lo - 1, 0), n - 1);
}
__device__ inline float cdf_pmf(const float* c, int n, int i) {
    return (i < 0 || i + 1 >= n + 1) ? 0.f : __ldg(c + i + 1) - __ldg(c + i);
}
__device__ inline void env_uv(const DevLight& L, f3 d, float& u, float& v) {
    float at = atan2f(d.x, d.z);
    at = at < 0.f ? at + 2.f * kPi : at;
    const float t = (at - L.rot) * .5f / kPi;
    u = t - floorf(t);
    v = acosf(fminf(1.f, fmaxf(-1.f, d.y))) / kPi;
}
template <uint32_t kF = kFeatAll>
__device__ inline f3 env_eval(const DevScene& S, const DevLight& L, f3 gwo) {
    if (!(kF & kFeatEnvTex) || L.type == LMGPU_LIGHT_ENVCONST) return mk(L.ke[0], L.ke[1], L.ke[2]);
    const f3 d = -gwo;
    float u, v;
    env_uv(L, d, u, v);
    const int x = min(max(int(u * L.env_w), 0), L.env_w - 1);
    const int y = min(max(int(v * L.env_h), 0), L.env_h - 1);
    const float* t = S.env + L.tex_off + 3 * (size_t(y) * L.env_w + x);
    return mk(__ldg(t), __ldg(t + 1), __ldg(t + 2)) * L.scale;
}
// pdf_direct of an infinite light endpoint with direction gwo, seen from g (projected solid angle)
template <uint32_t kF = kFeatAll>
__device__ inline float env_pdf_direct(const DevScene& S, const DevLight& L, const Geom& g, f3 gwo) {
    const f3 d = -gwo;
    if (!(kF & kFeatEnvTex) || L.type == LMGPU_LIGHT_ENVCONST) return pdf_sa_to_projsa(1.f / (4.f * kPi), g, d);
    float u, v;
    env_uv(L, d, u, v);
    const float st = sqrtf(fmaxf(0.f, 1.f - d.y * d.y));
    if (st == 0.f) return 0.f;
    const float* marg = S.env + L.marg_off;
    const int y = min(int(v * L.env_h), L.env_h - 1);
    const float pdf2 = cdf_pmf(marg, L.env_h, y) * cdf_pmf(S.env + L.cond_off + size_t(y) * (L.env_w + 1), L.env_w, int(u * L.env_w)) *
                       float(L.env_w) * float(L.env_h);
    return pdf_sa_to_projsa(pdf2 / (2.f * kPi * kPi * st), g, d);
}
__device__ inline float area_pdf_direct(const DevLight& L, const Geom& g, const Geom& gL, f3 wo) {
    if (dot(wo, gL.n) <= 0.f) return 0.f;
    const float G = geometry_term(g, gL);
    return G == 0.f ? 0.f : L.invA_J / G;
}

struct LightSample {
    Geom gL;
    f3 wo;      // direction from the light toward the shading point
    f3 weight;  // Le / (p_sel * pdf)
    int light;
};

// path::sample_direct(LE), path.h:493-530, with u = {up(0,1), upc(2,3), ud(4,5), udc(6,7)}
template <uint32_t kF = kFeatAll>
__device__ inline bool sample_direct(const DevScene& S, const Geom& g, const float* u, LightSample& out) {
    const int n = S.num_lights;
    const int li = min(max(int(u[2] * float(n)), 0), n - 1);
    const float p_sel = 1.f / float(n);
    const DevLight L = S.lights[li];
    out.light = li;
    if (L.type == LMGPU_LIGHT_AREA) {
        const int ti = cdf_sample(S.cdf + L.cdf_off, L.tri_cnt, u[3]);
        const float4* tp = S.ltri + size_t(L.tri_off + ti) * 3;
        const float4 a4 = __ldg(tp), b4 = __ldg(tp + 1), c4 = __ldg(tp + 2);
        const f3 a = mk(a4.x, a4.y, a4.z), b = mk(a4.w, b4.x, b4.y), c = mk(b4.z, b4.w, c4.x), gn = mk(c4.y, c4.z, c4.w);
        const float s = sqrtf(fmaxf(0.f, u[0]));
        const float bu = 1.f - s, bv = u[1] * s;
        const f3 p = a * (1.f - bu - bv) + b * bu + c * bv;
        out.gL = on_surface(p, gn, gn);
        out.wo = normalize(g.p - p);
        const float pL = area_pdf_direct(L, g, out.gL, out.wo);
        if (pL == 0.f) return false;
        const f3 Le = dot(out.wo, out.gL.n) <= 0.f ? mk(0, 0, 0) : mk(L.ke[0], L.ke[1], L.ke[2]);
        out.weight = Le / pL / p_sel;
        return true;
    }
    if ((kF & kFeatDelta) && L.type == LMGPU_LIGHT_POINT) {  // light_point.cpp:84-100: pdf 1 / G
        const f3 pl = mk(L.v[0], L.v[1], L.v[2]);
        out.gL = degenerate_point(pl);
        out.wo = normalize(g.p - pl);
        const float G = geometry_term(g, out.gL);
        if (G == 0.f) return false;
        out.weight = mk(L.ke[0], L.ke[1], L.ke[2]) / (1.f / G) / p_sel;
        return true;
    }
    if ((kF & kFeatDelta) && L.type == LMGPU_LIGHT_DIRECTIONAL) {  // light_directional.cpp:109-124
        out.wo = mk(L.v[0], L.v[1], L.v[2]);
        out.gL = infinite_point(out.wo);
        const float pL = pdf_sa_to_projsa(1.f, g, -out.wo);
        if (pL == 0.f) return false;
        out.weight = mk(L.ke[0], L.ke[1], L.ke[2]) / pL / p_sel;
        return true;
    }
    f3 wo;
    if (!(kF & kFeatEnvTex) || L.type == LMGPU_LIGHT_ENVCONST) {
        const float z = 1.f - 2.f * u[4];
        const float r = sqrtf(fmaxf(0.f, 1.f - z * z));
        float st, ct;
        sincosf(2.f * kPi * u[5], &st, &ct);
        wo = mk(r * ct, r * st, z);
    } else {
        const float* marg = S.env + L.marg_off;
        const int y = cdf_sample(marg, L.env_h, u[4]);
        const int x = cdf_sample(S.env + L.cond_off + size_t(y) * (L.env_w + 1), L.env_w, u[5]);
        const float su = (float(x) + u[0]) / float(L.env_w), sv = (float(y) + u[1]) / float(L.env_h);
        const float t = kPi * sv;
        const float st = sinf(t);
        const float ph = 2.f * kPi * su + L.rot;
        wo = -mk(st * sinf(ph), cosf(t), st * cosf(ph));
    }
    out.gL = infinite_point(wo);
    out.wo = wo;
    const float pL = env_pdf_direct<kF>(S, L, g, wo);
    if (pL == 0.f) return false;
    out.weight = env_eval<kF>(S, L, wo) / pL / p_sel;
    return true;
}

// path::sample_primary_ray(LE), path.h:101-118: a light by u[2], then its sample_ray with
// u = {up(0,1), upc(2,3), ud(4,5), udc(6,7)}. Area lights (light_area.cpp:78-100): a point as in
// sample_direct, a cosine-weighted direction about its normal, weight Le / (pA / pi). Environment
// lights (light_envconst.cpp:47-68, light_env.cpp:86-107): a uniform direction d, a point on the
// disk of the scene's bounding sphere facing d, weight Le(-d) / (1 / (4 pi) / (pi R^2)). Point
// lights (light_point.cpp:39-49): a uniform direction from the position, weight Le / (1 / (4 pi)).
// Directional lights (light_directional.cpp:49-70): the light's direction from a point of that
// disk, weight Le / (1 / (pi R^2)). Returns false when nothing can be hit (an environment or
// directional light in a scene without triangles). li_out: the light chosen; n_out: an area
// light's normal at the sampled point.
__device__ inline bool sample_light_ray(const DevScene& S, const float* u, f3& o, f3& d, f3& w, int* li_out = nullptr,
                                        f3* n_out = nullptr) {
    const int n = S.num_lights;
    const int li = min(max(int(u[2] * float(n)), 0), n - 1);
    const float p_sel = 1.f / float(n);
    const DevLight L = S.lights[li];
    if (li_out) *li_out = li;
    if (L.type == LMGPU_LIGHT_AREA) {
        const int ti = cdf_sample(S.cdf + L.cdf_off, L.tri_cnt, u[3]);
        const float4* tp = S.ltri + size_t(L.tri_off + ti) * 3;
        const float4 a4 = __ldg(tp), b4 = __ldg(tp + 1), c4 = __ldg(tp + 2);
        const f3 a = mk(a4.x, a4.y, a4.z), b = mk(a4.w, b4.x, b4.y), c = mk(b4.z, b4.w, c4.x), gn = mk(c4.y, c4.z, c4.w);
        const float s = sqrtf(fmaxf(0.f, u[0]));
        const float bu = 1.f - s, bv = u[1] * s;
        o = a * (1.f - bu - bv) + b * bu + c * bv;
        f3 tu, tv;
        onb(gn, tu, tv);
        const float r = sqrtf(fmaxf(0.f, u[4]));
        float st, ct;
        sincosf(2.f * kPi * u[5], &st, &ct);
        const float x = r * ct, y = r * st;
        const float z = sqrtf(fmaxf(0.f, 1.f - x * x - y * y));
        d = tu * x + tv * y + gn * z;
        if (n_out) *n_out = gn;
        const f3 Le = dot(d, gn) <= 0.f ? mk(0, 0, 0) : mk(L.ke[0], L.ke[1], L.ke[2]);
        w = Le / (L.invA_J * (1.f / kPi)) / p_sel;
        return true;
    }
    if (L.type == LMGPU_LIGHT_POINT) {
        o = mk(L.v[0], L.v[1], L.v[2]);
        const float z = 1.f - 2.f * u[4];
        const float r = sqrtf(fmaxf(0.f, 1.f - z * z));
        float st, ct;
        sincosf(2.f * kPi * u[5], &st, &ct);
        d = mk(r * ct, r * st, z);
        w = mk(L.ke[0], L.ke[1], L.ke[2]) / (1.f / (4.f * kPi)) / p_sel;
        return true;
    }
    if (!(S.bound_r > 0.f)) return false;
    if (L.type == LMGPU_LIGHT_DIRECTIONAL) {
        d = mk(L.v[0], L.v[1], L.v[2]);
        const float rd = sqrtf(fmaxf(0.f, u[0]));
        float sd, cd;
        sincosf(2.f * kPi * u[1], &sd, &cd);
        f3 tu, tv;
        onb(d, tu, tv);
        o = S.bound_c + (-d) * S.bound_r + (tu * (rd * cd * S.bound_r) + tv * (rd * sd * S.bound_r));
        w = mk(L.ke[0], L.ke[1], L.ke[2]) / (1.f / (kPi * S.bound_r * S.bound_r)) / p_sel;
        return true;
    }
    const float z = 1.f - 2.f * u[4];
    const float r = sqrtf(fmaxf(0.f, 1.f - z * z));
    float st, ct;
    sincosf(2.f * kPi * u[5], &st, &ct);
    d = mk(r * ct, r * st, z);
    const float rd = sqrtf(fmaxf(0.f, u[0]));
    float sd, cd;
    sincosf(2.f * kPi * u[1], &sd, &cd);
    const float px = rd * cd * S.bound_r, py = rd * sd * S.bound_r;
    f3 tu, tv;
    onb(d, tu, tv);
    o = S.bound_c + (-d) * S.bound_r + (tu * px + tv * py);
    const float pdf = (1.f / (4.f * kPi)) * (1.f / (kPi * S.bound_r * S.bound_r));
    w = env_eval(S, L, d) / pdf / p_sel;
    return true;
}

// ---------------------------------------------------------------------------------------------
// Film splats: one atomic add per channel. Lanes of a warp almost never share a pixel (the
// wavefront starts paths sample-major, so neighbouring queue entries belong to different
// pixels), and grouping them by pixel first (match + three reductions) measured slower: shade
// 44.2 -> 37.1 ms and shadow 27.1 -> 24.5 ms per 64-spp displaced-sphere frame without it.
__device__ inline void splat(float* film, uint32_t pixel, f3 c) {
    float* px = film + 3 * size_t(pixel);
    atomicAdd(px, c.x);
    atomicAdd(px + 1, c.y);
    atomicAdd(px + 2, c.z);
}

// ---------------------------------------------------------------------------------------------
// Wavefront state
struct ExtQ {
    float4* o;     // origin (w unused)
    float4* d;     // direction (w unused)
    float4* thr;   // throughput, pdf of the sampled direction (projected solid angle)
    float4* nrm;   // shading normal of the origin vertex, flags (bit 0 NEE-samplable, bit 1 camera, bits 8-15 vertex)
    uint2* ids;    // path index (RNG key pixel * spp + sample), film pixel
    uint32_t* job; // job of each entry (job-table mode only)
};
struct ShadowQ {
    float4* o;     // origin, tmax
    float4* d;
    float4* c;     // contribution, pixel
    uint32_t* job; // job of each entry (job-table mode only)
};
struct PtConst {
    uint32_t seed;
    int32_t max_verts;
    int64_t spp;
    int32_t mode;      // LMGPU_SAMPLING_*
    int32_t image;     // 1: image primary-ray mode
    int32_t w, h;
};
// One job of a shared wavefront: its scene, renderer parameters and film. Its npix * spp paths
// are started in sample-major order (all pixels of sample 0 first), so pass s of the job is
// complete when pass_done[pass_off + s] reaches npix. path_begin: paths submitted before it.
struct JobDev {
    DevScene S;
    PtConst P;
    float* film;
    float* film_odd;   // split passes: odd global passes splat here (else null)
    int64_t path_begin;
    int64_t npix;
    int64_t limit;     // paths the planner starts: npix * the job's current spp (lmgpu_batch_job_set_spp)
    uint32_t pass_off;
    uint32_t parity0;  // parity of the job's first pass among the film's passes
};

constexpr int kBlock = 256;
// Shadow-queue pixel word: bit 31 marks an odd pass of a split-pass film (pixels stay below 2^31).
constexpr uint32_t kOddPass = 0x80000000u;
constexpr int64_t kRenderQueue = int64_t(1) << 25;  // paths in flight of lmgpu_render_pt by default (2^24: 1.2 % slower; 2^26: no faster)
#ifndef LMGPU_TRACE_MINBLOCKS
#define LMGPU_TRACE_MINBLOCKS 4  // resident 256-thread blocks per SM of the closest-hit kernel (3 and 5 measured slower)
#endif
#ifndef LMGPU_SHADOW_MINBLOCKS
#define LMGPU_SHADOW_MINBLOCKS 5  // the any-hit kernel (shadow rays): 5 measured faster than 4 (24.6 -> 23.4 ms per frame)
#endif

#ifndef LMGPU_RNG_LOOP_UNROLL
#define LMGPU_RNG_LOOP_UNROLL 4
#endif
constexpr int kRngLoopUnroll = LMGPU_RNG_LOOP_UNROLL;
__device__ inline void rng_slots(uint32_t seed, uint64_t path, uint32_t vertex, int first_block, int nblocks, float* u) {
#pragma unroll kRngLoopUnroll
    for (int b = 0; b < nblocks; b++) {
        const U4 r = philox_block(seed, path, vertex * 4u + uint32_t(first_block + b));
        u[4 * b] = r.v[0]; u[4 * b + 1] = r.v[1]; u[4 * b + 2] = r.v[2]; u[4 * b + 3] = r.v[3];
    }
}

// Queue slot for the calling lane: one atomic per warp (the lanes that push together take
// consecutive slots, so their stores coalesce).
__device__ inline int queue_slot(int* count) {
    cg::coalesced_group g = cg::coalesced_threads();
    int base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(count, int(g.size()));
    return g.shfl(base, 0) + int(g.thread_rank());
}

template <bool kBatched>
__device__ inline void push_shadow(const ShadowQ& sq, int* count, f3 o, f3 d, float tmax, f3 c, uint32_t pixel, uint32_t job) {
    const int k = queue_slot(count);
    sq.o[k] = make_float4(o.x, o.y, o.z, tmax);
    sq.d[k] = make_float4(d.x, d.y, d.z, 0.f);
    sq.c[k] = make_float4(c.x, c.y, c.z, __uint_as_float(pixel));
    if (kBatched) sq.job[k] = job;
}

__device__ inline uint32_t pixel_of(const PtConst& P, float rx, float ry) {
    const int x = min(max(int(rx * float(P.w)), 0), P.w - 1);
    const int y = min(max(int(ry * float(P.h)), 0), P.h - 1);
    return uint32_t(y) * uint32_t(P.w) + uint32_t(x);
}

// NEE connection from vertex g (material m, or the camera if m == nullptr); pushes a shadow ray
// with the contribution it carries when the connection is nonzero (renderer_pt.cpp:142-192).
template <bool kBatched, uint32_t kF = kFeatAll>
__device__ inline void nee(const DevScene& S, const PtConst& P, const Geom& g, const DevMaterial* m, f3 wi, int comp, f3 thr,
                           const float* u8, uint32_t pixel, const ShadowQ& sq, int* scount, uint32_t job) {
    LightSample sL;
    if (!sample_direct<kF>(S, g, u8, sL)) return;
    const f3 wo = -sL.wo;
    uint32_t px = pixel;
    f3 fs;
    if (m == nullptr) {
        float rx, ry;
        if (!raster_pos(S, wo, rx, ry)) return;
        px = pixel_of(P, rx, ry) | (pixel & kOddPass);  // the camera vertex keeps the pass bit
        fs = mk(cam_J(S, wo), cam_J(S, wo), cam_J(S, wo));
    } else {
        fs = mat_eval<kF>(*m, g, wi, wo, comp, true) * sn_correction(g, wi, wo);
    }
    if (is_zero(fs)) return;
    float mis = 1.f;
    // renderer_pt.cpp:172-179: a light BSDF sampling cannot reach (point, directional) keeps weight 1
    const bool delta = (kF & kFeatDelta) && (sL.gL.degenerated || S.lights[sL.light].type == LMGPU_LIGHT_DIRECTIONAL);
    if (P.mode == LMGPU_SAMPLING_MIS && !delta) {
        const DevLight L = S.lights[sL.light];
        const float pl = (1.f / float(S.num_lights)) *
                         (L.type == LMGPU_LIGHT_AREA ? area_pdf_direct(L, g, sL.gL, sL.wo) : env_pdf_direct<kF>(S, L, g, sL.gL.wo));
        const float pb = m == nullptr ? cam_pdf(S, wo) : mat_pdf<kF>(*m, g, wi, wo, true);
        mis = (pl == 0.f && pb == 0.f) ? 0.f : pl / (pl + pb);
    }
    const f3 C = thr * fs * sL.weight * mis;
    if (is_zero(C)) return;
    f3 dir;
    float tmax;
    if (sL.gL.infinite) {
        dir = -sL.gL.wo;
        tmax = kInf - 1.f;
    } else {
        dir = normalize(sL.gL.p - g.p);
        tmax = length(sL.gL.p - g.p) * (1.f - kEps);
    }
    push_shadow<kBatched>(sq, scount, g.p, dir, tmax, C, px, job);
}

template <bool kBatched>
__device__ inline void push_ext(const ExtQ& q, int* count, f3 o, f3 d, f3 thr, float pdf, f3 n, uint32_t flags, uint32_t path,
                                uint32_t pixel, uint32_t job) {
    const int k = queue_slot(count);
    q.o[k] = make_float4(o.x, o.y, o.z, 0.f);
    q.d[k] = make_float4(d.x, d.y, d.z, 0.f);
    q.thr[k] = make_float4(thr.x, thr.y, thr.z, pdf);
    q.nrm[k] = make_float4(n.x, n.y, n.z, __uint_as_float(flags));
    q.ids[k] = make_uint2(path, pixel);
    if (kBatched) q.job[k] = job;
}

// Camera vertex of one path: renderer_pt.cpp:95-116 and the first pass of the loop (NEE in image
// mode, the jittered primary direction, raster position caching). `path` is the RNG key
// pixel * spp + sample; `pix` the pixel whose window is sampled.
template <bool kBatched>
__device__ __forceinline__ void generate_path(const DevScene& S, const PtConst& P, uint64_t path, int64_t pix, const ExtQ& q,
                                              int* qcount, const ShadowQ& sq, int* scount, uint32_t job, uint32_t odd_bit) {
    float wx = 0.f, wy = 0.f, ww = 1.f, wh = 1.f;
    if (!P.image) {
        const int x = int(pix % P.w), y = int(pix / P.w);
        ww = 1.f / float(P.w);
        wh = 1.f / float(P.h);
        wx = ww * float(x);
        wy = wh * float(y);
    }
    Geom g;
    g.p = S.cam_p; g.n = mk(0, 0, 0); g.gn = g.n; g.u = g.n; g.v = g.n; g.wo = g.n;
    g.degenerated = true; g.infinite = false;
    const bool nee_ok = P.mode != LMGPU_SAMPLING_NAIVE && P.image;
    float u[16];
    rng_slots(P.seed, path, 1u, 0, 4, u);
    if (nee_ok) nee<kBatched>(S, P, g, nullptr, mk(0, 0, 0), 0, mk(1, 1, 1), u, odd_bit, sq, scount, job);
    const f3 d = primary_dir(S, wx + ww * u[8], wy + wh * u[9]);
    float rx = 0.f, ry = 0.f;
    raster_pos(S, d, rx, ry);
    const uint32_t pixel = pixel_of(P, rx, ry);
    const float pdf = nee_ok ? cam_pdf(S, d) : 0.f;
    push_ext<kBatched>(q, qcount, S.cam_p, d, mk(1, 1, 1), pdf, mk(0, 0, 0), (nee_ok ? 1u : 0u) | 2u | (1u << 8),
                       uint32_t(path), pixel, job);
}

// Single scene: paths [start, start + count) enumerated pixel-major (path = pixel * spp + sample).
__global__ void __launch_bounds__(kBlock) k_pt_generate(const __grid_constant__ DevScene S, const __grid_constant__ PtConst P,
                                                        int64_t start, int64_t count, ExtQ q, int* qcount, ShadowQ sq,
                                                        int* scount) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x) {
        const uint64_t path = uint64_t(start + i);
        generate_path<false>(S, P, path, int64_t(path / uint64_t(P.spp)), q, qcount, sq, scount, 0u, 0u);
    }
}

// Shared wavefront: the planner's allocation list. Entry e gives queue slots [slot_e, slot_{e+1})
// to job `job`, starting at its path `local` (sample-major: local = sample * npix + pixel).
struct AllocEntry {
    int64_t local, slot;
    int32_t job, pad;
};
// Planner's view of a job that still has paths to start (its end is read from the job table,
// where the host may move it between runs).
struct ActiveJob {
    int64_t npix, total;
    int32_t job, pad;
};

// New paths for the slots the planner handed out this iteration (ctl[3] of them, in ctl[22]
// allocation entries; both read here, not baked into a captured launch).
__global__ void __launch_bounds__(kBlock) k_wf_generate(const JobDev* __restrict__ jobs, const AllocEntry* __restrict__ alloc,
                                                        const int64_t* __restrict__ ctl, ExtQ q, int* qcount, ShadowQ sq,
                                                        int* scount) {
    const int64_t count = ctl[3];
    const int na = int(ctl[22]);
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x) {
        int lo = 0, hi = na;  // last entry with slot <= i
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (alloc[mid].slot <= i) lo = mid; else hi = mid;
        }
        const AllocEntry e = alloc[lo];
        const JobDev& J = jobs[e.job];
        const int64_t local = e.local + (i - e.slot);
        const int64_t sample = local / J.npix, pix = local - sample * J.npix;
        const uint32_t odd = (J.film_odd && ((uint32_t(sample) + J.parity0) & 1u)) ? kOddPass : 0u;
        generate_path<true>(J.S, J.P, uint64_t(pix * J.P.spp + sample), pix, q, qcount, sq, scount, uint32_t(e.job), odd);
    }
}

// Instrumented runs: keeps the largest per-ray node count in *maxv and (racily, for diagnosis)
// the ray that produced it in worst[0..7].
__device__ inline void record_worst(unsigned long long* maxv, float* worst, uint32_t visits, float4 o, float4 d,
                                    float tmin, float tmax) {
    if (visits > *reinterpret_cast<volatile unsigned long long*>(maxv)) {
        const unsigned long long prev = atomicMax(maxv, (unsigned long long)visits);
        if (prev < visits) {
            worst[0] = o.x; worst[1] = o.y; worst[2] = o.z; worst[3] = tmin;
            worst[4] = d.x; worst[5] = d.y; worst[6] = d.z; worst[7] = tmax;
        }
    }
}

// Extension rays: closest hit over [Eps, Inf]. kCount: rays with (k & count_mask) == 0 also count
// node visits and triangle tests into sums[0..2] (instrumented runs only). kBatched: each entry
// traverses its own job's BVH; bvh.depth is then the largest depth of the table (stack size).
// f.refill > 0: persistent with dynamic fetch; 0: one ray per thread, grid-stride.
template <bool kCount, bool kBatched = false, bool kTwoLevel = false>
__global__ void __launch_bounds__(kBlock, LMGPU_TRACE_MINBLOCKS) k_pt_extend(Bvh8 bvh, const float4* __restrict__ qo, const float4* __restrict__ qd,
                                                      const int* __restrict__ qcount, float4* __restrict__ hits,
                                                      unsigned long long* rays, int* err, unsigned long long* sums,
                                                      int count_mask, float* worst, Fetch f, const JobDev* __restrict__ jobs = nullptr,
                                                      const uint32_t* __restrict__ qjob = nullptr) {
    extern __shared__ uint32_t smem[];
    const int n = *qcount;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(rays, (unsigned long long)n);
        if (f.other) *f.other = 0;
    }
    uint32_t* sb = smem + threadIdx.x;
    uint32_t* sbits = smem + blockDim.x * bvh.depth + threadIdx.x;
    int lerr = 0;
    uint32_t cn = 0, ct = 0, cc = 0;
    if (f.refill > 0) {
        fetch_loop<false, kCount, kTwoLevel>(
            n, f, bvh, sb, sbits, int(blockDim.x), &lerr,
            [&](int k, Trav& s, Bvh8& B) {
                const float4 o = qo[k], d = qd[k];
                if (kBatched) B = jobs[qjob[k]].S.bvh;
                trav_init(s, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), kEps, kInf);
            },
            [&](int k, const Trav& s) {
                hits[k] = make_float4(s.best.t, s.best.u, s.best.v, __int_as_float(s.best.id));
                if (kCount && (k & count_mask) == 0) {
                    cn += s.nvis;
                    ct += s.ntri;
                    cc++;
                    record_worst(sums + 6, worst, s.nvis, make_float4(s.o.x, s.o.y, s.o.z, 0.f),
                                 make_float4(s.d.x, s.d.y, s.d.z, 0.f), kEps, kInf);
                }
            });
    } else {
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
            const float4 o = qo[k], d = qd[k];
            const Bvh8& B = kBatched ? jobs[qjob[k]].S.bvh : bvh;
            TraceHit h;
            if (kCount && (k & count_mask) == 0) {
                const uint32_t before = cn;
                h = trace_bvh8<false, true, kTwoLevel>(B, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), kEps, kInf, sb, sbits, blockDim.x, &cn,
                                            &ct, &lerr);
                cc++;
                record_worst(sums + 6, worst, cn - before, o, d, kEps, kInf);
            } else {
                h = trace_bvh8<false, false, kTwoLevel>(B, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), kEps, kInf, sb, sbits, blockDim.x,
                                             nullptr, nullptr, &lerr);
            }
            hits[k] = make_float4(h.t, h.u, h.v, __int_as_float(h.id));
        }
    }
    if (kCount && cc) {
        atomicAdd(sums + 0, (unsigned long long)cn);
        atomicAdd(sums + 1, (unsigned long long)ct);
        atomicAdd(sums + 2, (unsigned long long)cc);
    }
    if (lerr) atomicOr(err, lerr);
}

// Shadow rays: any hit over [Eps, tmax]; unoccluded contributions go to the film. kCount,
// kBatched and f as in k_pt_extend; counts into sums[3..5].
template <bool kCount, bool kBatched = false, bool kTwoLevel = false>
__global__ void __launch_bounds__(kBlock, LMGPU_SHADOW_MINBLOCKS) k_pt_shadow(Bvh8 bvh, ShadowQ sq, const int* __restrict__ scount, float* film,
                                                      unsigned long long* rays, int* err, unsigned long long* sums,
                                                      int count_mask, float* worst, Fetch f, const JobDev* __restrict__ jobs = nullptr,
                                                      float* film_odd = nullptr) {
    extern __shared__ uint32_t smem[];
    const int n = *scount;
    // the accumulator of an unoccluded contribution: the pixel word's bit 31 marks an odd pass
    auto target = [&](uint32_t job, uint32_t pw) -> float* {
        if (pw & kOddPass) return kBatched ? jobs[job].film_odd : film_odd;
        return kBatched ? jobs[job].film : film;
    };
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(rays, (unsigned long long)n);
        if (f.other) *f.other = 0;
    }
    uint32_t* sb = smem + threadIdx.x;
    uint32_t* sbits = smem + blockDim.x * bvh.depth + threadIdx.x;
    int lerr = 0;
    uint32_t cn = 0, ct = 0, cc = 0;
    if (f.refill > 0) {
        fetch_loop<true, kCount, kTwoLevel>(
            n, f, bvh, sb, sbits, int(blockDim.x), &lerr,
            [&](int k, Trav& s, Bvh8& B) {
                const float4 o = sq.o[k], d = sq.d[k];
                if (kBatched) B = jobs[sq.job[k]].S.bvh;
                trav_init(s, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), kEps, o.w);
            },
            [&](int k, const Trav& s) {
                if (s.best.id < 0) {
                    const float4 c = sq.c[k];
                    const uint32_t pw = __float_as_uint(c.w);
                    splat(target(kBatched ? sq.job[k] : 0u, pw), pw & ~kOddPass, mk(c.x, c.y, c.z));
                }
                if (kCount && (k & count_mask) == 0) {
                    cn += s.nvis;
                    ct += s.ntri;
                    cc++;
                    record_worst(sums + 7, worst + 8, s.nvis, make_float4(s.o.x, s.o.y, s.o.z, 0.f),
                                 make_float4(s.d.x, s.d.y, s.d.z, 0.f), kEps, s.best.t);
                }
            });
    } else {
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
            const float4 o = sq.o[k], d = sq.d[k];
            const uint32_t job = kBatched ? sq.job[k] : 0u;
            const Bvh8& B = kBatched ? jobs[job].S.bvh : bvh;
            TraceHit h;
            if (kCount && (k & count_mask) == 0) {
                const uint32_t before = cn;
                h = trace_bvh8<true, true, kTwoLevel>(B, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), kEps, o.w, sb, sbits, blockDim.x, &cn,
                                           &ct, &lerr);
                cc++;
                record_worst(sums + 7, worst + 8, cn - before, o, d, kEps, o.w);
            } else {
                h = trace_bvh8<true, false, kTwoLevel>(B, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), kEps, o.w, sb, sbits, blockDim.x,
                                            nullptr, nullptr, &lerr);
            }
            if (h.id < 0) {
                const float4 c = sq.c[k];
                const uint32_t pw = __float_as_uint(c.w);
                splat(target(job, pw), pw & ~kOddPass, mk(c.x, c.y, c.z));
            }
        }
    }
    if (kCount && cc) {
        atomicAdd(sums + 3, (unsigned long long)cn);
        atomicAdd(sums + 4, (unsigned long long)ct);
        atomicAdd(sums + 5, (unsigned long long)cc);
    }
    if (lerr) atomicOr(err, lerr);
}

// One pass of the loop body after the intersection (renderer_pt.cpp:221-300) for one path whose
// ray left vertex nv (flags bits 8-15), then NEE and direction sampling at the new vertex nv+1.
// Returns false when the path ends here.
template <bool kBatched, uint32_t kF = kFeatAll>
__device__ __forceinline__ bool shade_path(const DevScene& S, const PtConst& P, float* film, float* film_odd, uint32_t parity0,
                                           uint32_t job, float4 o4, float4 d4, float4 t4, float4 n4, float4 h4, uint2 ids,
                                           const ExtQ& qo, int* qocount, const ShadowQ& sq, int* scount) {
    // split passes: the path's pass (sample index) picks the accumulator; NEE carries it in the
    // shadow entry's pixel word
    uint32_t odd_bit = 0u;
    if (film_odd && ((ids.x % uint32_t(P.spp) + parity0) & 1u)) {
        film = film_odd;
        odd_bit = kOddPass;
    }
    const uint32_t flags = __float_as_uint(n4.w);
    const int it = int((flags >> 8) & 0xffu);
    const bool prev_nee = flags & 1u;
    const f3 d = mk(d4.x, d4.y, d4.z);
    f3 thr = mk(t4.x, t4.y, t4.z);
    const float prev_pdf = t4.w;
    Geom gp;  // the vertex the ray left from
    gp.p = mk(o4.x, o4.y, o4.z);
    gp.n = mk(n4.x, n4.y, n4.z);
    gp.degenerated = (flags & 2u) != 0;
    gp.infinite = false;
    const bool direct_ok = P.mode == LMGPU_SAMPLING_NEE ? !prev_nee : true;
    const bool use_mis = P.mode != LMGPU_SAMPLING_NAIVE && prev_nee;
    const int32_t id = __float_as_int(h4.w);
    if (id < 0) {
        // miss: the environment light endpoint (scene.cpp:321-331), then the env-hit break
        if (S.env_light >= 0 && direct_ok) {
            const DevLight L = S.lights[S.env_light];
            const f3 gwo = -d;
            float mis = 1.f;
            if (use_mis) {
                const float pl = (1.f / float(S.num_lights)) * env_pdf_direct<kF>(S, L, gp, gwo);
                mis = (prev_pdf == 0.f && pl == 0.f) ? 0.f : prev_pdf / (prev_pdf + pl);
            }
            const f3 C = thr * env_eval<kF>(S, L, gwo) * mis;
            if (!is_zero(C)) splat(film, ids.y, C);
        }
        return false;
    }
    int32_t prim;
    int64_t rec = 0;
    const Geom g = surface_at<kF>(S, id, h4.y, h4.z, prim, (kF & kFeatTexture) ? &rec : nullptr);
    const int2 ml = __ldg(S.prim_ml + prim);
    const f3 wi = -d;
    if (ml.y >= 0 && direct_ok) {
        const DevLight L = S.lights[ml.y];
        const f3 woL = wi;
        if (dot(woL, g.n) > 0.f) {
            float mis = 1.f;
            if (use_mis) {
                const float pl = (1.f / float(S.num_lights)) * area_pdf_direct(L, gp, g, woL);
                mis = (prev_pdf == 0.f && pl == 0.f) ? 0.f : prev_pdf / (prev_pdf + pl);
            }
            const f3 C = thr * mk(L.ke[0], L.ke[1], L.ke[2]) * mis;
            if (!is_zero(C)) splat(film, ids.y, C);
        }
    }
    float u[16];
    rng_slots(P.seed, ids.x, uint32_t(it), 3, 1, u + 12);
    if (it > 5) {
        const float qrr = fmaxf(.2f, 1.f - cmax(thr));
        if (u[12] < qrr) return false;
        thr = thr / (1.f - qrr);
    }
    DevMaterial m = S.mats[ml.x];
    if ((kF & kFeatTexture) && (m.map_kd >= 0 || m.mask >= 0)) resolve_textures(S, m, rec, h4.y, h4.z);
    int comp = 0;
    if (m.type == LMGPU_MAT_GLASS) {
        f3 wt; bool total; float eta, Fr;
        glass_fresnel(m, g, wi, wt, total, eta, Fr);
        comp = u[13] < Fr ? 0 : 1;
        thr = thr * (1.f / (comp == 0 ? Fr : 1.f - Fr));
    } else if ((kF & kFeatTexture) && m.type == LMGPU_MAT_MIXTURE && m.mask >= 0) {
        // model_wavefrontobj.cpp:413-420: the surface with probability alpha, else the pass-through
        comp = u[13] < m.alpha ? 0 : 1;
        thr = thr * (1.f / (comp == 0 ? m.alpha : 1.f - m.alpha));
    }
    const int nv = it + 1;
    if (nv >= P.max_verts) return false;
    const bool spec = mat_specular(m, comp);
    const bool nee_ok = P.mode != LMGPU_SAMPLING_NAIVE && !spec;
    rng_slots(P.seed, ids.x, uint32_t(nv), 0, 3, u);
    if (nee_ok) nee<kBatched, kF>(S, P, g, &m, wi, comp, thr, u, ids.y | odd_bit, sq, scount, job);
    f3 wo, w;
    if (!mat_sample<kF>(m, g, wi, comp, u[8], u[9], u[10], wo, w)) return false;
    w = w * sn_correction(g, wi, wo);
    const float pdf = (P.mode == LMGPU_SAMPLING_MIS && nee_ok) ? mat_pdf<kF>(m, g, wi, wo, true) : 0.f;
    thr = thr * w;
    push_ext<kBatched>(qo, qocount, g.p, wo, thr, pdf, g.n, (nee_ok ? 1u : 0u) | (uint32_t(nv) << 8), ids.x, ids.y, job);
    return true;
}

// kMinBlocks: resident 256-thread blocks per SM the register allocation must allow (2: up to 128
// registers; 3: 80; 4: 64), selected at run time by the "shade_minblocks" tuning key.
template <int kMinBlocks>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_pt_shade(const __grid_constant__ DevScene S, const __grid_constant__ PtConst P,
                                                     ExtQ qi, const float4* __restrict__ hits, const int* __restrict__ qicount,
                                                     ExtQ qo, int* qocount, ShadowQ sq, int* scount, float* film) {
    const int n = *qicount;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        shade_path<false>(S, P, film, nullptr, 0u, 0u, qi.o[k], qi.d[k], qi.thr[k], qi.nrm[k], hits[k], qi.ids[k], qo, qocount,
                          sq, scount);
}

// ---------------------------------------------------------------------------------------------
// renderer::lt (renderer_lt.cpp:50-160) on the same queues: light paths start at a light, every
// surface vertex connects to the pinhole camera (a shadow ray whose unoccluded contribution
// lands on the pixel the connection passes through), and the walk continues in transport
// direction LE. Random numbers: philox keyed (seed, path); vertex 1 slots 0-7 the primary ray;
// the ray that left vertex k takes its roulette (k > 5) from slot 12 and the hit's component from
// slots 13-14 of vertex k; vertex k's direction from slots 8-11 (slots 0-7 would be the camera
// sample, which the pinhole camera does not use).

// Light paths [start, start + count): the primary ray from a sampled light (path = its index).
__global__ void __launch_bounds__(kBlock) k_lt_generate(const __grid_constant__ DevScene S, const __grid_constant__ PtConst P,
                                                        int64_t start, int64_t count, ExtQ q, int* qcount) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x) {
        const uint64_t path = uint64_t(start + i);
        float u[8];
        rng_slots(P.seed, path, 1u, 0, 2, u);
        f3 o, d, w;
        if (!sample_light_ray(S, u, o, d, w)) continue;
        if (is_zero(w)) continue;  // contributes nothing
        push_ext<false>(q, qcount, o, d, w, 0.f, mk(0, 0, 0), 1u << 8, uint32_t(path), 0u, 0u);
    }
}

// One light path after its extension ray: roulette and component at the hit (vertex k + 1), the
// camera connection of that vertex (camera_pinhole.cpp:178-203: weight J(wo) G; the raster
// position is tested before the shadow ray is queued), and the next direction.
template <int kMinBlocks, uint32_t kF = kFeatAll>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_lt_shade(const __grid_constant__ DevScene S, const __grid_constant__ PtConst P,
                                                     ExtQ qi, const float4* __restrict__ hits, const int* __restrict__ qicount,
                                                     ExtQ qo, int* qocount, ShadowQ sq, int* scount) {
    const int n = *qicount;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const float4 h4 = hits[k];
        const int32_t id = __float_as_int(h4.w);
        if (id < 0) continue;  // no surface (or the environment): the walk ends
        const float4 d4 = qi.d[k], t4 = qi.thr[k], n4 = qi.nrm[k];
        const uint2 ids = qi.ids[k];
        const int it = int((__float_as_uint(n4.w) >> 8) & 0xffu);
        f3 thr = mk(t4.x, t4.y, t4.z);
        float u[16];
        rng_slots(P.seed, ids.x, uint32_t(it), 3, 1, u + 12);
        if (it > 5) {
            const float qrr = fmaxf(.2f, 1.f - cmax(thr));
            if (u[12] < qrr) continue;
            thr = thr / (1.f - qrr);
        }
        int32_t prim;
        const Geom g = surface_at<kF>(S, id, h4.y, h4.z, prim);
        const DevMaterial m = S.mats[__ldg(S.prim_ml + prim).x];
        const f3 wi = -mk(d4.x, d4.y, d4.z);
        int comp = 0;
        if (m.type == LMGPU_MAT_GLASS) {
            f3 wt; bool total; float eta, Fr;
            glass_fresnel(m, g, wi, wt, total, eta, Fr);
            comp = u[13] < Fr ? 0 : 1;
            thr = thr * (1.f / (comp == 0 ? Fr : 1.f - Fr));
        }
        const int nv = it + 1;
        if (nv >= P.max_verts) continue;
        if (!mat_specular(m)) {  // a specular vertex's connection evaluates to 0
            const f3 wE = normalize(g.p - S.cam_p);
            float rx, ry;
            if (raster_pos(S, wE, rx, ry)) {
                const f3 dc = S.cam_p - g.p;
                const float L2 = dot(dc, dc);
                const float len = sqrtf(L2);
                const float G = fabsf(dot(g.n, dc / len)) / L2;
                if (G != 0.f) {
                    const f3 wo = -wE;
                    const f3 fs = mat_eval<kF>(m, g, wi, wo, comp, true, true) * sn_correction_le(g, wi, wo);
                    const f3 C = thr * fs * (cam_J(S, wE) * G);
                    if (!is_zero(C)) push_shadow<false>(sq, scount, g.p, normalize(dc), len * (1.f - kEps), C, pixel_of(P, rx, ry), 0u);
                }
            }
        }
        if (nv + 1 >= P.max_verts) continue;  // the next vertex would not connect
        rng_slots(P.seed, ids.x, uint32_t(nv), 2, 1, u + 8);
        f3 wo, w;
        if (!mat_sample<kF>(m, g, wi, comp, u[8], u[9], u[10], wo, w, true)) continue;
        thr = thr * (w * sn_correction_le(g, wi, wo));
        if (is_zero(thr)) continue;
        push_ext<false>(qo, qocount, g.p, wo, thr, 0.f, g.n, uint32_t(nv) << 8, ids.x, 0u, 0u);
    }
}

// ---------------------------------------------------------------------------------------------
// renderer::bdpt (renderer_bdpt.cpp:297-413 over include/lm/bidir.h): per sample one eye and one
// light subpath, then every strategy (s light vertices, t eye vertices) with its power-heuristic
// weight. Subpaths are traced on the shared extend kernel (eye and light rays in one queue) and
// their vertices kept in records; k_bd_connect evaluates the strategies, queues one visibility
// ray per connection (s, t >= 1) for k_pt_shadow and splats s = 0 directly.
// The weight is the reference's (bidir.h:460-479: 1 / sum over strategies s' of (p_s' / p_s)^2
// with pdf_bidir, bidir.h:397-449). p_s' is a product over the path's vertices of their local
// pdfs, sampled from the light side (qL) for the first s' vertices and from the eye side (qE)
// for the rest, so p_{s'+1} / p_s' = qL(s') / qE(s'). Each vertex keeps the local pdf of the
// direction its subpath sampled it from (qf) and the factors of the opposite direction that its
// subpath already fixes (pc_out, prev_rev, G); a strategy evaluates only the four local pdfs next
// to its connection and sweeps the ratios: O(n) per strategy instead of O(n^2).
// Philox: eye vertex i draws from "vertex" kBdEyeBase + i, light vertex i from kBdLightBase + i;
// slots 0-7 the primary ray (the camera uses 4-5), 8-11 the direction sampled at the vertex,
// 13-14 the component of the vertex the ray that leaves it hits.
constexpr uint32_t kBdEyeBase = 1, kBdLightBase = 129;
constexpr int kBdMaxVerts = 64;
// kinds (2 bits): kBdArea a light endpoint at a finite position (light::area, light::point),
// kBdInfinite an environment or directional light endpoint, or the environment hit by a subpath.
// kBdDelta marks a point or directional light endpoint: degenerate or specular, so the strategy
// that would reach it by tracing (s = 0) does not exist (bidir.h:187-191).
enum : uint32_t { kBdSurface = 0, kBdCamera = 1, kBdArea = 2, kBdInfinite = 3 };
constexpr uint32_t kBdDelta = 4u;
// ext-queue flags of the BDPT subpaths: bits 8-15 the vertex the ray leaves, then these
constexpr uint32_t kBdLightSub = 1u << 16, kBdInfOrigin = 1u << 17, kBdDegOrigin = 1u << 18;

// A subpath vertex. p: position (an infinite vertex: its direction wo, surface.h:90-110);
// a: the subpath weight of the vertices before it (eval_subpath_sampling_weight, bidir.h:233-275)
// without its own component pdf pc. qf: pc * pdf_direction(previous vertex) * G(previous, this),
// the local pdf its subpath sampled it with (the endpoints: pdf_position, or 1). pc_out: the
// component pdf toward the next vertex of the subpath; prev_rev: pdf_direction of this vertex
// toward the previous one given the next one, times G(previous, this); G: that geometry term.
struct BdVtx {
    f3 p, n, gn, a;
    uint32_t kind, comp;
    int32_t light, mat;
    float pc, qf, pc_out, prev_rev, G;
    bool spec;
    bool delta;  // a point or directional light endpoint
};
// Records: 5 float4 per vertex, [subpath][vertex][sample] so that consecutive samples read
// consecutive records. r4 = (qf, +-pc_out, prev_rev, pc) alone carries what the weight sweep
// reads (the sign of pc_out marks a specular vertex). nv: vertices per subpath, [subpath][sample].
struct BdRec {
    float4* r;
    int32_t* nv;
    int64_t W;
    int32_t mv;          // record rows per subpath
    int32_t max_e, max_l;  // vertices the eye / light subpath may reach (0: not sampled)
    int32_t mode;        // LMGPU_BDPT_*
};
constexpr int kBdRecWords = 5;
__device__ inline size_t bd_at(const BdRec& R, int sub, int j, int64_t k) {
    return ((size_t(sub) * R.mv + j) * size_t(R.W) + k) * kBdRecWords;
}
__device__ inline void bd_store(const BdRec& R, int sub, int j, int64_t k, const BdVtx& v) {
    float4* q = R.r + bd_at(R, sub, j, k);
    const uint32_t word = v.kind | (v.delta ? kBdDelta : 0u) | (v.comp << 4) | (uint32_t(v.light + 1) << 8);
    q[0] = make_float4(v.p.x, v.p.y, v.p.z, __uint_as_float(word));
    q[1] = make_float4(v.n.x, v.n.y, v.n.z, __int_as_float(v.mat));
    q[2] = make_float4(v.gn.x, v.gn.y, v.gn.z, v.pc);
    q[3] = make_float4(v.a.x, v.a.y, v.a.z, v.G);
    q[4] = make_float4(v.qf, v.spec ? -v.pc_out : v.pc_out, v.prev_rev, v.pc);
}
// the direction-sampling part of a vertex, written once its next direction is known
__device__ inline void bd_store_out(const BdRec& R, int sub, int j, int64_t k, const BdVtx& v) {
    R.r[bd_at(R, sub, j, k) + 4] = make_float4(v.qf, v.spec ? -v.pc_out : v.pc_out, v.prev_rev, v.pc);
}
__device__ inline BdVtx bd_load(const BdRec& R, int sub, int j, int64_t k) {
    const float4* q = R.r + bd_at(R, sub, j, k);
    const float4 r0 = q[0], r1 = q[1], r2 = q[2], r3 = q[3], r4 = q[4];
    BdVtx v;
    const uint32_t word = __float_as_uint(r0.w);
    v.p = mk(r0.x, r0.y, r0.z);
    v.kind = word & 3u;
    v.delta = (word & kBdDelta) != 0u;
    v.comp = (word >> 4) & 15u;
    v.light = int32_t(word >> 8) - 1;
    v.n = mk(r1.x, r1.y, r1.z);
    v.mat = __float_as_int(r1.w);
    v.gn = mk(r2.x, r2.y, r2.z);
    v.pc = r2.w;
    v.a = mk(r3.x, r3.y, r3.z);
    v.G = r3.w;
    v.qf = r4.x;
    v.pc_out = fabsf(r4.y);
    v.spec = signbit(r4.y);
    v.prev_rev = r4.z;
    return v;
}
__device__ inline float4 bd_pdfs(const BdRec& R, int sub, int j, int64_t k) { return R.r[bd_at(R, sub, j, k) + 4]; }
// bidir.h:140-155: the direction from `from` toward record j (an infinite vertex: back along its wo)
__device__ inline f3 bd_toward(const BdRec& R, int sub, int j, int64_t k, f3 from) {
    const float4 r0 = R.r[bd_at(R, sub, j, k)];
    if ((__float_as_uint(r0.w) & 3u) == kBdInfinite) return -mk(r0.x, r0.y, r0.z);
    return normalize(mk(r0.x, r0.y, r0.z) - from);
}
__device__ inline Geom bd_geom(const BdVtx& v) { return on_surface(v.p, v.n, v.gn); }
// path.h:228-234 with material_glass.cpp:143-158
__device__ inline float bd_pcomp(const DevMaterial& m, const Geom& g, int comp, f3 wi) {
    if (m.type != LMGPU_MAT_GLASS) return 1.f;
    f3 wt; bool total; float eta, Fr;
    glass_fresnel(m, g, wi, wt, total, eta, Fr);
    return comp == 0 ? Fr : 1.f - Fr;
}
// pdf_primary_ray of an environment light (light_envconst.cpp:70-74), selection included
__device__ inline float bd_env_pray(const DevScene& S) {
    return (1.f / float(S.num_lights)) * (1.f / (4.f * kPi)) * (1.f / (kPi * S.bound_r * S.bound_r));
}
// pdf_position of an area light endpoint (light_area.cpp:142, selection included)
__device__ inline float bd_area_pa(const DevScene& S, int light) { return (1.f / float(S.num_lights)) * S.lights[light].invA_J; }

// Samples [start, start + count) of a wave (record slot = index in the wave): the camera endpoint
// and its primary ray over the whole image (camera_pinhole.cpp:134-140), the light endpoint and
// its ray (sample_light_ray). Both rays go to one queue; thr.w carries the pdf_direction of the
// ray at its origin, nrm.xyz the origin's normal.
__global__ void __launch_bounds__(kBlock) k_bd_generate(const __grid_constant__ DevScene S, const __grid_constant__ PtConst P,
                                                        BdRec R, int64_t start, int64_t count, ExtQ q, int* qcount) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += int64_t(gridDim.x) * blockDim.x) {
        const uint64_t path = uint64_t(start + i);
        float u[8];
        rng_slots(P.seed, path, kBdEyeBase, 1, 1, u + 4);
        BdVtx c;
        c.p = S.cam_p; c.n = c.gn = mk(0, 0, 0); c.a = mk(1, 1, 1);
        c.kind = kBdCamera; c.comp = 0; c.light = -1; c.mat = -1; c.pc = 1.f;
        c.qf = 1.f; c.pc_out = 1.f; c.prev_rev = 0.f; c.G = 0.f; c.spec = false; c.delta = false;
        bd_store(R, 0, 0, i, c);
        R.nv[i] = 1;
        const f3 de = primary_dir(S, u[4], u[5]);
        if (R.max_e >= 2)
            push_ext<false>(q, qcount, S.cam_p, de, mk(1, 1, 1), cam_pdf(S, de), mk(0, 0, 0), kBdDegOrigin, uint32_t(path), uint32_t(i),
                            0u);
        if (R.max_l == 0) {  // renderer::pt_naive_path samples no light subpath
            R.nv[R.W + i] = 0;
            continue;
        }
        rng_slots(P.seed, path, kBdLightBase, 0, 2, u);
        f3 o, d, w, ln = mk(0, 0, 0);
        int li = 0;
        if (!sample_light_ray(S, u, o, d, w, &li, &ln)) {
            R.nv[R.W + i] = 0;
            continue;
        }
        BdVtx l;
        l.comp = 0; l.light = li; l.mat = -1; l.pc = 1.f; l.pc_out = 1.f; l.prev_rev = 0.f; l.G = 0.f; l.spec = false;
        float pdir;
        const int32_t ltype = S.lights[li].type;
        l.delta = ltype == LMGPU_LIGHT_POINT || ltype == LMGPU_LIGHT_DIRECTIONAL;
        if (ltype == LMGPU_LIGHT_AREA || ltype == LMGPU_LIGHT_POINT) {
            // connectable endpoints: qf = pdf_position (light_area.cpp:142; light_point.cpp:78-80: 1),
            // the first direction's pdf cosine-weighted, or uniform from a point (light_point.cpp:64-66)
            l.kind = kBdArea; l.p = o; l.n = l.gn = ln;
            l.qf = ltype == LMGPU_LIGHT_AREA ? bd_area_pa(S, li) : 1.f / float(S.num_lights);
            const float ia = 1.f / l.qf;
            l.a = mk(ia, ia, ia);
            pdir = ltype == LMGPU_LIGHT_POINT ? 1.f / (4.f * kPi) : (dot(d, ln) <= 0.f ? 0.f : 1.f / kPi);
        } else {
            // pdf_primary_ray of the endpoint (light_directional.cpp:72-75 without eval_delta)
            l.kind = kBdInfinite; l.p = d; l.n = l.gn = mk(0, 0, 0); l.a = mk(0, 0, 0);
            l.qf = 1.f;
            pdir = ltype == LMGPU_LIGHT_DIRECTIONAL ? (1.f / float(S.num_lights)) * (1.f / (kPi * S.bound_r * S.bound_r)) : bd_env_pray(S);
        }
        bd_store(R, 1, 0, i, l);
        R.nv[R.W + i] = 1;
        if (is_zero(w) || R.max_l < 2) continue;
        const uint32_t oflag = l.kind == kBdInfinite ? kBdInfOrigin : (ltype == LMGPU_LIGHT_POINT ? kBdDegOrigin : 0u);
        push_ext<false>(q, qcount, o, d, w, pdir, l.n, kBdLightSub | oflag, uint32_t(path), uint32_t(i), 0u);
    }
}

// One subpath step (bidir.h:507-569): the hit becomes vertex j + 1 with the component sampled
// there; then, while the subpath has fewer than max_verts vertices, the next direction in the
// subpath's transport direction. The queue carries the subpath weight up to the hit.
template <int kMinBlocks, uint32_t kF = kFeatAll>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_bd_shade(const __grid_constant__ DevScene S, const __grid_constant__ PtConst P,
                                                     BdRec R, ExtQ qi, const float4* __restrict__ hits, const int* __restrict__ qicount,
                                                     ExtQ qo, int* qocount) {
    const int n = *qicount;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const float4 h4 = hits[k], o4 = qi.o[k], d4 = qi.d[k], t4 = qi.thr[k], n4 = qi.nrm[k];
        const uint2 ids = qi.ids[k];
        const uint32_t flags = __float_as_uint(n4.w);
        const int j = int((flags >> 8) & 0xffu);
        const int sub = (flags & kBdLightSub) ? 1 : 0;
        const uint32_t base = sub ? kBdLightBase : kBdEyeBase;
        const int64_t slot = int64_t(ids.y);
        const f3 o = mk(o4.x, o4.y, o4.z), d = mk(d4.x, d4.y, d4.z), thr = mk(t4.x, t4.y, t4.z), no = mk(n4.x, n4.y, n4.z);
        const int32_t id = __float_as_int(h4.w);
        BdVtx v;
        v.a = thr; v.pc = 1.f; v.comp = 0; v.pc_out = 1.f; v.prev_rev = 0.f; v.spec = false; v.delta = false;
        if (id < 0) {
            if (S.env_light < 0) continue;  // nothing hit: the subpath ends
            // the environment as a vertex (scene.cpp:321-331); G with an infinite end: |n_o . d|
            v.kind = kBdInfinite; v.p = -d; v.n = v.gn = mk(0, 0, 0); v.light = S.env_light; v.mat = -1;
            v.G = (flags & (kBdDegOrigin | kBdInfOrigin)) ? 1.f : fabsf(dot(no, d));
            v.qf = t4.w * v.G;
            bd_store(R, sub, j + 1, slot, v);
            R.nv[sub * R.W + slot] = j + 2;
            continue;
        }
        int32_t prim;
        const Geom g = surface_at<kF>(S, id, h4.y, h4.z, prim);
        const int2 ml = __ldg(S.prim_ml + prim);
        const DevMaterial m = S.mats[ml.x];
        float u[16];
        rng_slots(P.seed, ids.x, base + uint32_t(j), 3, 1, u + 12);
        if (m.type == LMGPU_MAT_GLASS) {
            f3 wt; bool total; float eta, Fr;
            glass_fresnel(m, g, -d, wt, total, eta, Fr);
            v.comp = u[13] < Fr ? 0u : 1u;
            v.pc = v.comp == 0 ? Fr : 1.f - Fr;
        }
        // geometry term of the edge just traced (surface.h:329-348), from the positions
        {
            f3 dd;
            float L2, c1;
            if (flags & kBdInfOrigin) {
                dd = d; L2 = 1.f; c1 = 1.f;
            } else {
                dd = g.p - o; L2 = dot(dd, dd); dd = dd / sqrtf(L2);
                c1 = (flags & kBdDegOrigin) ? 1.f : fabsf(dot(no, dd));
            }
            v.G = c1 * fabsf(dot(g.n, -dd)) / L2;
        }
        v.qf = v.pc * (t4.w * v.G);
        v.kind = kBdSurface; v.p = g.p; v.n = g.n; v.gn = g.gn; v.light = ml.y; v.mat = ml.x;
        v.spec = mat_specular(m);
        bd_store(R, sub, j + 1, slot, v);
        R.nv[sub * R.W + slot] = j + 2;
        if (j + 2 >= (sub ? R.max_l : R.max_e)) continue;
        rng_slots(P.seed, ids.x, base + uint32_t(j + 1), 2, 1, u + 8);
        // toward the previous vertex (bidir.h:530): from the positions, or back along an
        // infinite origin's direction
        const f3 wi = (flags & kBdInfOrigin) ? -d : normalize(o - g.p);
        f3 wo, w;
        if (!mat_sample<kF>(m, g, wi, int(v.comp), u[8], u[9], u[10], wo, w, sub == 1)) continue;
        w = w * (sub ? sn_correction_le(g, wi, wo) : sn_correction(g, wi, wo));
        const f3 next = (thr / v.pc) * w;
        if (is_zero(next)) continue;  // every strategy through the next vertex weighs 0
        v.pc_out = bd_pcomp(m, g, int(v.comp), wo);
        v.prev_rev = mat_pdf<kF>(m, g, wo, wi, false) * v.G;
        bd_store_out(R, sub, j + 1, slot, v);
        push_ext<false>(qo, qocount, g.p, wo, next, mat_pdf<kF>(m, g, wi, wo, false), g.n, (uint32_t(j + 1) << 8) | (sub ? kBdLightSub : 0u),
                        ids.x, ids.y, 0u);
    }
}

// The strategies of the wave's samples as a dense work list (renderer_bdpt.cpp:347-355): item
// (sample, s | t << 8) for s <= n_L, 1 <= t <= n_E and min_verts <= s + t <= max_verts. One warp
// takes 32 consecutive samples: their item count in closed form, one atomic for the warp's range,
// then the items in (t, s) order across the lanes (ballot ranks), so neighbouring items share
// their strategy and their samples' records.
__global__ void __launch_bounds__(kBlock) k_bd_items(BdRec R, int64_t count, int32_t min_verts, int32_t max_verts, uint2* items,
                                                     int* icount, int64_t icap, int* err) {
    const unsigned full = 0xffffffffu;
    const int lane = int(threadIdx.x & 31u);
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t w = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; w * 32 < count; w += nwarps) {
        const int64_t k = w * 32 + lane;
        // strategy bounds of the mode: lt_nee_path connects only to the camera (t = 1),
        // pt_nee_path only the light endpoint or nothing (s <= 1)
        const int nE = k < count ? (R.mode == LMGPU_BDPT_LT_NEE ? min(R.nv[k], 1) : R.nv[k]) : 0;
        const int nL = k < count ? (R.mode == LMGPU_BDPT_PT_NEE ? min(R.nv[R.W + k], 1) : R.nv[R.W + k]) : 0;
        int mine = 0;
        for (int t = 1; t <= nE; t++) mine += max(0, min(nL, max_verts - t) - max(0, min_verts - t) + 1);
        int tot = mine, tmax = nE, smax = nL;
        for (int o = 16; o > 0; o >>= 1) {
            tot += __shfl_xor_sync(full, tot, o);
            tmax = max(tmax, __shfl_xor_sync(full, tmax, o));
            smax = max(smax, __shfl_xor_sync(full, smax, o));
        }
        int base = 0;
        if (lane == 0 && tot > 0) base = atomicAdd(icount, tot);
        base = __shfl_sync(full, base, 0);
        if (int64_t(base) + tot > icap) {  // cannot happen with the capacity the host sizes
            if (lane == 0) atomicOr(err, 4);
            continue;
        }
        int off = 0;
        for (int t = 1; t <= tmax; t++) {
            for (int s = 0; s <= smax; s++) {
                const bool have = t <= nE && s <= nL && s + t >= min_verts && s + t <= max_verts;
                const unsigned b = __ballot_sync(full, have);
                if (have) items[base + off + __popc(b & ((1u << lane) - 1u))] = make_uint2(uint32_t(k), uint32_t(s) | (uint32_t(t) << 8));
                off += __popc(b);
            }
        }
    }
}

// Strategy-major order of the items: a counting sort by (t, s), so that a warp of k_bd_connect
// runs one strategy (one path length, one pair of connection vertex roles) instead of a mix.
// Bucket key t * (max_verts + 1) + s; at most kBdSortBuckets buckets (max_verts <= 31).
constexpr int kBdSortBuckets = 1024;
__device__ __forceinline__ int bd_item_key(uint2 item, int32_t max_verts) {
    return int(item.y >> 8) * (max_verts + 1) + int(item.y & 0xffu);
}
__global__ void __launch_bounds__(kBlock) k_bd_sort_count(const uint2* __restrict__ items, const int* __restrict__ icount,
                                                          int32_t max_verts, int nbuckets, int* __restrict__ hist) {
    __shared__ int h[kBdSortBuckets];
    for (int i = threadIdx.x; i < nbuckets; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const int n = *icount;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&h[bd_item_key(items[i], max_verts)], 1);
    __syncthreads();
    for (int i = threadIdx.x; i < nbuckets; i += blockDim.x)
        if (h[i]) atomicAdd(hist + i, h[i]);
}
// One block: exclusive prefix of the bucket counts, in place (the scatter's cursors).
__global__ void k_bd_sort_scan(int* hist, int nbuckets) {
    if (threadIdx.x == 0) {
        int run = 0;
        for (int i = 0; i < nbuckets; i++) {
            const int c = hist[i];
            hist[i] = run;
            run += c;
        }
    }
}
// Each block takes one contiguous range of the items: it counts its range per bucket in shared
// memory, reserves one run per nonempty bucket with one global atomic, then places its items with
// shared-memory atomics (one global atomic per block and bucket instead of per warp and key).
__global__ void __launch_bounds__(kBlock) k_bd_sort_scatter(const uint2* __restrict__ items, const int* __restrict__ icount,
                                                            int32_t max_verts, int nbuckets, int* __restrict__ cursor,
                                                            uint2* __restrict__ out) {
    __shared__ int h[kBdSortBuckets];
    const int n = *icount;
    const int per = (n + int(gridDim.x) - 1) / int(gridDim.x);
    const int lo = int(blockIdx.x) * per, hi = min(n, lo + per);
    for (int b = threadIdx.x; b < nbuckets; b += blockDim.x) h[b] = 0;
    __syncthreads();
    for (int i = lo + int(threadIdx.x); i < hi; i += blockDim.x) atomicAdd(&h[bd_item_key(items[i], max_verts)], 1);
    __syncthreads();
    for (int b = threadIdx.x; b < nbuckets; b += blockDim.x) {
        const int c = h[b];
        h[b] = c ? atomicAdd(cursor + b, c) : 0;
    }
    __syncthreads();
    for (int i = lo + int(threadIdx.x); i < hi; i += blockDim.x) {
        const uint2 item = items[i];
        out[atomicAdd(&h[bd_item_key(item, max_verts)], 1)] = item;
    }
}

// One strategy of one sample per item: the connection (bidir.h:593-643), the unweighted
// contribution alpha_L * c_st * alpha_E (bidir.h:325-343) and the weight. s = 0 splats at the
// eye's raster position; s, t >= 1 queue a visibility ray from the light vertex to the eye
// vertex. Strategies whose own pdf is 0 contribute nothing.
template <int kMinBlocks, uint32_t kF = kFeatAll>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_bd_connect(const __grid_constant__ DevScene S, const __grid_constant__ PtConst P,
                                                       BdRec R, const uint2* __restrict__ items, const int* __restrict__ icount,
                                                       ShadowQ sq, int* scount, int64_t scap, float* film, int* err) {
    const int nitems = *icount;
    for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < nitems; it += gridDim.x * blockDim.x) {
        const uint2 item = items[it];
        const int64_t k = int64_t(item.x);
        const int s = int(item.y & 0xffu), t = int(item.y >> 8);
        const int n = s + t;
        const int nL = R.nv[R.W + k];
        const bool opt = R.mode == LMGPU_BDPT_OPT;
        const bool weighted = opt || R.mode == LMGPU_BDPT_ALL;  // the path-structure renderers take one strategy per length
        uint32_t eye_px = 0;
        if (t >= 2) {  // bidir.h:167-171: the raster position of the camera's first edge
            const float4 r0 = R.r[bd_at(R, 0, 1, k)];
            const f3 e1 = mk(r0.x, r0.y, r0.z);
            const f3 de = (__float_as_uint(r0.w) & 3u) == kBdInfinite ? -e1 : normalize(e1 - S.cam_p);
            float rx = 0.f, ry = 0.f;
            raster_pos(S, de, rx, ry);
            eye_px = pixel_of(P, rx, ry);
        }
        const uint32_t w0 = nL > 0 ? __float_as_uint(R.r[bd_at(R, 1, 0, k)].w) : 0u;
        const bool env_l0 = nL > 0 && (w0 & 3u) == kBdInfinite;
        const bool delta_l0 = (w0 & kBdDelta) != 0u;  // x_0 = L[0] cannot be reached by tracing
        const BdVtx vE = bd_load(R, 0, t - 1, k);
        f3 Cu;
        uint32_t px = eye_px;
        // fresh local pdfs next to the connection; x_i = L[i] for i < s, E[n-1-i] after
        float qLs = 0.f, qLs1 = 0.f, qEs1 = 0.f, qEs2 = 0.f, qE0 = 0.f;
        BdVtx vL;
        if (s == 0) {
            // the eye subpath ends on a light, which becomes the light endpoint x_0
            if (t < 2 || vE.light < 0) continue;
            const float4 e2 = bd_pdfs(R, 0, t - 2, k);
            // renderer::pt_nee_path takes s = 0 only in place of s = 1 when the eye vertex that
            // s = 1 would connect is specular (renderer_bdpt.cpp:160-172)
            if (R.mode == LMGPU_BDPT_PT_NEE && (nL < 1 || !signbit(e2.y))) continue;
            const DevLight L = S.lights[vE.light];
            f3 Le;
            float pdir;
            if (vE.kind == kBdInfinite) {
                Le = env_eval<kF>(S, L, vE.p);
                pdir = bd_env_pray(S);
                qLs = 1.f;
            } else {
                const f3 wo = bd_toward(R, 0, t - 2, k, vE.p);
                const bool front = dot(wo, vE.n) > 0.f;
                Le = front ? mk(L.ke[0], L.ke[1], L.ke[2]) : mk(0, 0, 0);
                pdir = front ? 1.f / kPi : 0.f;
                qLs = bd_area_pa(S, vE.light);
            }
            // alpha_L(0) = 1; alpha_E ends on the light endpoint, component pdf 1 (bidir.h); bdptopt
            // keeps the vertex's own component weight (renderer_bdptopt.cpp:265-270)
            Cu = opt ? Le * (vE.a / vE.pc) : Le * vE.a;
            qLs1 = (opt ? 1.f : fabsf(e2.y)) * (pdir * vE.G);
            qE0 = vE.qf / vE.pc;
        } else {
            vL = bd_load(R, 1, s - 1, k);
            if (vL.kind == kBdInfinite || vE.kind == kBdInfinite) continue;
            if (R.mode == LMGPU_BDPT_PT_NEE && vE.spec) continue;  // replaced by s = 0 (above)
            const f3 aL = vL.a / vL.pc, aE = vE.a / vE.pc;
            if (is_zero(aL) || is_zero(aE)) continue;
            const f3 dLE = normalize(vE.p - vL.p), dEL = -dLE;
            const float Gc = [&] {
                const f3 dv = vE.p - vL.p;
                const float L2 = dot(dv, dv);
                const f3 dn = dv / sqrtf(L2);
                const float c2 = vE.kind == kBdCamera ? 1.f : fabsf(dot(vE.n, -dn));
                const float c1 = vL.delta ? 1.f : fabsf(dot(vL.n, dn));  // a point light is degenerate
                return c1 * c2 / L2;
            }();
            f3 fL = mk(0, 0, 0), fE = mk(0, 0, 0);
            float pLf = 0.f, pcL = 1.f, pEf = 0.f, pcE = 1.f;
            if (s == 1) {
                // the light endpoint: Le toward the front of an area light (pdf_direction 1 / pi),
                // toward every direction from a point light (1 / (4 pi), light_point.cpp:64-66, 117-119)
                const DevLight L = S.lights[vL.light];
                const bool front = vL.delta || dot(dLE, vL.n) > 0.f;
                fL = front ? mk(L.ke[0], L.ke[1], L.ke[2]) : mk(0, 0, 0);
                pLf = vL.delta ? 1.f / (4.f * kPi) : (front ? 1.f / kPi : 0.f);
                if (is_zero(fL)) continue;
            }
            if (t == 1) {  // the camera endpoint
                float rx, ry;
                if (!raster_pos(S, dEL, rx, ry)) continue;
                const float J = cam_J(S, dEL);
                fE = mk(J, J, J);
                pEf = J;
                px = pixel_of(P, rx, ry);
            }
            // Surface connection vertices: the light side (transport LE) and the eye side (EL) run
            // through one code path, so the material code is emitted once (the kernel is bound by
            // instruction fetch). Per side: f, the pdf toward the other vertex, the component pdf
            // there, and the reverse pdf toward the subpath's previous vertex.
            bool dead = false;
#pragma unroll 1
            for (int side = s == 1 ? 1 : 0; side < (t == 1 ? 1 : 2); side++) {
                const bool le = side == 0;
                const f3 vp = le ? vL.p : vE.p, vn = le ? vL.n : vE.n, vgn = le ? vL.gn : vE.gn;
                const int comp = int(le ? vL.comp : vE.comp);
                const float vG = le ? vL.G : vE.G;
                const int sub = le ? 1 : 0, prev = (le ? s : t) - 2;
                const f3 wo = le ? dLE : dEL;
                const DevMaterial m = S.mats[le ? vL.mat : vE.mat];
                const Geom g = on_surface(vp, vn, vgn);
                const f3 wi = bd_toward(R, sub, prev, k, vp);
                const f3 f = mat_eval<kF>(m, g, wi, wo, comp, true, le) * (le ? sn_correction_le(g, wi, wo) : sn_correction(g, wi, wo));
                if (is_zero(f)) {
                    dead = true;
                    break;
                }
                const float pf = mat_pdf<kF>(m, g, wi, wo, false);
                const float pc = bd_pcomp(m, g, comp, wo);
                const float qrev = (opt ? 1.f : fabsf(bd_pdfs(R, sub, prev, k).y)) * (mat_pdf<kF>(m, g, wo, wi, false) * vG);
                if (le) {
                    fL = f; pLf = pf; pcL = pc; qEs2 = qrev;
                } else {
                    fE = f; pEf = pf; pcE = pc; qLs1 = qrev;
                }
            }
            if (dead) continue;
            Cu = aL * (fL * Gc * fE) * aE;
            qLs = (opt ? 1.f : pcE) * (pLf * Gc);
            qEs1 = (opt ? 1.f : pcL) * (pEf * Gc);
        }
        if (is_zero(Cu)) continue;

        // The ratio sweeps over x_i = L[i] (i < s) and E[n-1-i] (i >= s), one record row (r4:
        // qf, +-pc_out, prev_rev, G) loaded per step and the neighbours kept in registers.
        // qL(i): i < s stored (L[i].qf); s, s+1 fresh; beyond, the eye subpath's reverse factors
        // pc_out(E[e]) * prev_rev(E[e+1]). qE(i): i >= s stored (E[e].qf; x_0 as the endpoint:
        // qE0); s-1, s-2 fresh; below, pc_out(L[i]) * prev_rev(L[i+1]). Samplable (bidir.h:185-224):
        // x_{s'-1} and x_{s'} not specular (the sign of pc_out; endpoints never are), an infinite
        // light endpoint not connected (s' = 1), the camera endpoint degenerate (s' = n).
        const bool inf0 = s == 0 ? vE.kind == kBdInfinite : env_l0;
        auto spec_of = [](const float4& q) -> bool { return signbit(q.y); };
        // bdptopt's cached pdfs leave out the component pdfs (renderer_bdptopt.cpp:145-215)
        auto fwd = [&](const float4& q) -> float { return opt ? q.x / q.w : q.x; };
        auto cout = [&](const float4& q) -> float { return opt ? 1.f : fabsf(q.y); };
        bool ok = true;
        float inv = 1.f;
        if (weighted) {
            float r = 1.f;
            float4 prev = make_float4(0.f, 1.f, 0.f, 0.f);
            float4 cur = bd_pdfs(R, 0, t - 1, k);  // x_s = E[t-1]
            for (int j = s; j <= n - 2; j++) {     // p_{j+1} / p_s
                const int e = n - 1 - j;           // x_j = E[e]; x_{j+1} = E[e-1]
                const float4 nxt = bd_pdfs(R, 0, e - 1, k);
                const float den = (j == 0) ? qE0 : fwd(cur);
                if (den == 0.f) { ok = false; break; }
                const float num = j == s ? qLs : (j == s + 1 ? qLs1 : cout(cur) * prev.z);
                r *= num / den;
                const bool spec_j = j != 0 && spec_of(cur);
                const bool spec_j1 = (j + 1 != n - 1) && spec_of(nxt);
                if (r != 0.f && j + 1 < n && !(j + 1 == 1 && inf0) && !spec_j && !spec_j1) inv += opt ? r : r * r;
                prev = cur;
                cur = nxt;
            }
        }
        if (weighted && ok && s > 0) {
            float r = 1.f;
            float4 above = make_float4(0.f, 1.f, 0.f, 0.f);
            float4 cur = bd_pdfs(R, 1, s - 1, k);  // x_{s-1} = L[s-1]
            for (int j = s - 1; j >= 0; j--) {     // p_j / p_s
                const float4 below = j > 0 ? bd_pdfs(R, 1, j - 1, k) : make_float4(0.f, 1.f, 0.f, 0.f);
                const float den = fwd(cur);
                if (den == 0.f) { ok = false; break; }
                const float num = j == s - 1 ? qEs1 : (j == s - 2 ? qEs2 : cout(cur) * above.z);
                r *= num / den;
                // samplable(j): x_{j-1} (L[j-1]) and x_j (L[j]) not specular; x_0 an endpoint that
                // tracing reaches (not a point or directional light)
                const bool samp = j == 0 ? !delta_l0 : (!(j == 1 && inf0) && !(j - 1 != 0 && spec_of(below)) && !spec_of(cur));
                if (r != 0.f && samp) inv += opt ? r : r * r;
                above = cur;
                cur = below;
            }
        }
        if (!ok) continue;
        const f3 C = Cu * (1.f / inv);
        if (is_zero(C)) continue;
        if (s == 0) {
            splat(film, px, C);
            continue;
        }
        const int slot = queue_slot(scount);
        if (slot >= scap) {
            atomicOr(err, 2);
            continue;
        }
        // Scene::visible from the light vertex (include/lm/scene.h:343-364)
        const f3 dv = vE.p - vL.p;
        const f3 dn = normalize(dv);
        sq.o[slot] = make_float4(vL.p.x, vL.p.y, vL.p.z, length(dv) * (1.f - kEps));
        sq.d[slot] = make_float4(dn.x, dn.y, dn.z, 0.f);
        sq.c[slot] = make_float4(C.x, C.y, C.z, __uint_as_float(px));
    }
}

// Job table: as k_pt_shade with each entry's own job; a path that ends adds one to its job's pass
// counter (warp-aggregated per pass).
template <int kMinBlocks, bool kSingle, uint32_t kF = kFeatAll>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_wf_shade(const JobDev* __restrict__ jobs, ExtQ qi, const float4* __restrict__ hits,
                                                     const int* __restrict__ qicount, ExtQ qo, int* qocount, ShadowQ sq,
                                                     int* scount, unsigned int* pass_done) {
    const int n = *qicount;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        // kSingle: the batch holds one job, so no per-path job id is read
        const uint32_t job = kSingle ? 0u : qi.job[k];
        const JobDev& J = jobs[job];
        const uint2 ids = qi.ids[k];
        const bool alive = shade_path<true, kF>(J.S, J.P, J.film, J.film_odd, J.parity0, job, qi.o[k], qi.d[k], qi.thr[k], qi.nrm[k], hits[k], ids, qo,
                                            qocount, sq, scount);
        if (!alive) {
            const uint32_t key = J.pass_off + ids.x % uint32_t(J.P.spp);
            // the lanes that end paths of one pass share one atomic (sample-major order puts them
            // together; one atomic per lane on the same counter measured 3x slower shading)
            cg::coalesced_group g = cg::coalesced_threads();
            cg::coalesced_group peers = cg::labeled_partition(g, key);
            if (peers.thread_rank() == 0) atomicAdd(pass_done + key, peers.size());
        }
    }
}

// Device-side planner, one warp. Tops the next queue up to `cap` paths: with `first_pass`, first
// the remaining sample-0 paths of every job that has not started them all (in submission order),
// so a newly admitted job's first image does not wait behind older jobs' later samples; then
// paths in submission order. Only the order in which paths start changes, never a path's random
// stream. Keeps per job the next path to start (job_next) and the list of jobs with paths left
// (active, compacted in place). ctl: [0] paths started, [1] paths submitted, [3] slots handed
// out, [4] paths in flight or waiting (0 = done), [5] jobs submitted, [20] jobs seen, [21]
// active jobs, [22] allocation entries.
__global__ void __launch_bounds__(32) k_wf_plan(int64_t* ctl, const int* qcount, int64_t cap, const JobDev* __restrict__ jobs,
                                                int64_t* job_next, ActiveJob* active, AllocEntry* alloc, int first_pass) {
    const int lane = int(threadIdx.x);
    const unsigned below = (1u << lane) - 1u;
    const int64_t njobs = ctl[5], seen = ctl[20];
    int64_t nact = ctl[21];
    for (int64_t j = seen + lane; j < njobs; j += 32) {
        const JobDev& J = jobs[j];
        active[nact + (j - seen)] = ActiveJob{J.npix, J.limit, int32_t(j), 0};
    }
    nact += njobs > seen ? njobs - seen : 0;
    __syncwarp();
    const int64_t inq = *qcount;
    int64_t left = cap > inq ? cap - inq : 0;
    int64_t slot = 0, na = 0;
    for (int phase = first_pass ? 0 : 1; phase < 2 && left > 0; phase++) {
        for (int64_t base = 0; base < nact && left > 0; base += 32) {
            const int64_t a = base + lane;
            int64_t want = 0, nx = 0;
            int32_t j = 0;
            if (a < nact) {
                const ActiveJob A = active[a];
                j = A.job;
                nx = job_next[j];
                const int64_t total = jobs[j].limit;
                const int64_t end = phase == 0 ? min(A.npix, total) : total;
                want = end > nx ? end - nx : 0;
            }
            int64_t inc = want;  // inclusive scan of the wants across the warp
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            const int64_t before = inc - want;
            const int64_t take = min(want, left > before ? left - before : 0);
            const unsigned has = __ballot_sync(0xffffffffu, take > 0);
            if (take > 0) {
                alloc[na + __popc(has & below)] = AllocEntry{nx, slot + before, j, 0};
                job_next[j] = nx + take;
            }
            const int64_t chunk = __shfl_sync(0xffffffffu, inc, 31);
            const int64_t used = min(chunk, left);
            slot += used;
            left -= used;
            na += __popc(has);
            __syncwarp();
        }
    }
    // keep the jobs with paths still to start; entries move down only, and a chunk is read
    // completely before any of it is written
    int64_t k = 0;
    for (int64_t base = 0; base < nact; base += 32) {
        const int64_t a = base + lane;
        bool keep = false;
        ActiveJob A{};
        if (a < nact) {
            A = active[a];
            keep = job_next[A.job] < jobs[A.job].limit;
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) active[k + __popc(m & below)] = A;
        k += __popc(m);
        __syncwarp();
    }
    if (lane == 0) {
        ctl[20] = njobs;
        ctl[21] = k;
        ctl[22] = na;
        ctl[3] = slot;
        ctl[0] += slot;
        ctl[4] = inq + (ctl[1] - ctl[0]);
    }
}

__global__ void k_scale2(const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ out, int64_t n, float s) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        out[i] = (a[i] + b[i]) * s;
}

// Sum over pixels and channels of Var(I) / (I^2 + eps) from the even / odd accumulators (see
// lmgpu_film_rel_mse); u converts a per-pass sum into the estimate's units.
__global__ void k_rel_mse(const float* __restrict__ a, const float* __restrict__ b, int64_t n, double na, double nb, double u,
                          double eps, double* acc) {
    double s = 0.0;
    const double N = na + nb;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const double A = double(a[i]) * u / na, B = double(b[i]) * u / nb, I = (double(a[i]) + double(b[i])) * u / N;
        const double var = (A - B) * (A - B) * na * nb / (N * N);
        s += var / (I * I + eps);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(acc, s);
}

// L2 read bandwidth probe: every thread streams float4s of an L2-resident buffer with loads that
// bypass L1 (ld.global.cg); the sum only keeps the loads alive.
__global__ void k_l2_probe(const float4* __restrict__ buf, int64_t n, int iters, float* out) {
    float acc = 0.f;
    for (int it = 0; it < iters; it++)
        for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
            const float4 v = __ldcg(buf + i);
            acc += (v.x + v.y) + (v.z + v.w);
        }
    if (acc == 1234.5f) out[0] = acc;
}

__global__ void k_scale(const float* __restrict__ in, float* __restrict__ out, int64_t n, float s) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        out[i] = in[i] * s;
}

// renderer::raycast, one thread per pixel (renderer_raycast.cpp:70-98)
template <bool kTwoLevel>
__global__ void __launch_bounds__(kBlock) k_raycast(DevScene S, int w, int h, lmgpu_raycast_params prm, float* film, int* err) {
    extern __shared__ uint32_t smem[];
    uint32_t* sb = smem + threadIdx.x;
    uint32_t* sbits = smem + blockDim.x * S.bvh.depth + threadIdx.x;
    int lerr = 0;
    const int64_t n = int64_t(w) * h;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const int x = int(i % w), y = int(i / w);
        const float rx = ieee::div(ieee::add(float(x), .5f), float(w)), ry = ieee::div(ieee::add(float(y), .5f), float(h));
        const f3 d = primary_dir(S, rx, ry);
        const TraceHit hit =
            trace_bvh8<false, false, kTwoLevel>(S.bvh, S.cam_p, d, kEps, kInf, sb, sbits, blockDim.x, nullptr, nullptr, &lerr);
        f3 c;
        if (hit.id < 0) {
            if (S.env_light >= 0) {
                const DevLight L = S.lights[S.env_light];
                c = prm.visualize_normal ? mk(0, 0, 0) : env_eval(S, L, -d);
            } else {
                c = mk(prm.bg_color[0], prm.bg_color[1], prm.bg_color[2]);
            }
        } else {
            int32_t prim;
            int64_t rec = 0;
            const Geom g = surface_at(S, hit.id, hit.u, hit.v, prim, &rec);
            if (prm.visualize_normal) {
                c = mk(fabsf(g.n.x), fabsf(g.n.y), fabsf(g.n.z));
            } else {
                f3 R;
                if (prm.has_color) {
                    R = mk(prm.color[0], prm.color[1], prm.color[2]);
                } else {
                    DevMaterial m = S.mats[__ldg(S.prim_ml + prim).x];
                    if ((S.feat & kFeatTexture) && m.map_kd >= 0) resolve_textures(S, m, rec, hit.u, hit.v);
                    // Material::reflectance: Kd (diffuse, mixture), Ks (glossy), none for the specular ones
                    R = (m.type == LMGPU_MAT_DIFFUSE || m.type == LMGPU_MAT_GLOSSY || m.type == LMGPU_MAT_MIXTURE)
                            ? mk(m.c[0], m.c[1], m.c[2])
                            : mk(0, 0, 0);
                }
                c = prm.use_constant_color ? R : R * (.2f + .8f * fabsf(dot(g.n, -d)));
            }
        }
        film[3 * i] = c.x;
        film[3 * i + 1] = c.y;
        film[3 * i + 2] = c.z;
    }
    if (lerr) atomicOr(err, lerr);
}

template <typename K>
K pick_shade(K two, K three, K four, int minblocks) {
    return minblocks <= 2 ? two : (minblocks == 3 ? three : four);
}

template <typename K>
int grid_for(K kernel, int block, size_t smem) {
    if (smem > 48 * 1024) LMGPU_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = 0;
    LMGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem));
    return std::max(1, per_sm) * current_device().num_sms;
}

// Per-device state of lmgpu_render_pt, shared by every scene and held for the whole of a call (the
// call ends with its stream synchronized), so scenes cost only their own tables: the shared
// wavefront a render runs its job on, and the fixed-wave queues of instrumented renders. Grown on
// demand; kept for the life of the process.
struct Workspace {
    std::mutex m;
    int64_t cap = 0;
    DevBuf q_o[2], q_d[2], q_thr[2], q_nrm[2], q_ids[2], hits, s_o, s_d, s_c, counters;
    lmgpu_batch* batch = nullptr;  // the regenerating wavefront lmgpu_render_pt runs its job on
    int64_t batch_cap = 0;
    DevBuf bd_rec, bd_nv, bd_s_o, bd_s_d, bd_s_c, bd_items, bd_items_sorted, bd_hist;  // lmgpu_render_bdpt: subpath records,
    // connection rays, strategies (and in strategy-major order), the sort's bucket counts
};

Workspace& workspace(int device) {
    static std::mutex reg_m;
    static Workspace* reg[64] = {};
    if (device < 0 || device >= 64) throw Error(LMGPU_ERR_UNSUPPORTED, "device index above 63");
    std::lock_guard<std::mutex> lk(reg_m);
    if (!reg[device]) reg[device] = new Workspace();  // never freed: outlives the CUDA runtime's teardown order
    return *reg[device];
}

// Light-tracing and BDPT kernels specialised on the features they use: instances and mixture
// materials (shade), the textured environment and mixture materials (connect).
// Three resident blocks per SM (up to 80 registers) rather than four (64 registers, up to 48
// bytes of stack): the LT frame 16.04 -> 15.72 ms (A/B on one GB300, three alternating runs each).
using LtShadeK = decltype(&k_lt_shade<3, kFeatAll>);
LtShadeK lt_shade_for(uint32_t feat) {
    switch (feat & (kFeatMixture | kFeatTwoLevel)) {
    case 0: return k_lt_shade<3, 0u>;
    case kFeatMixture: return k_lt_shade<3, kFeatMixture>;
    case kFeatTwoLevel: return k_lt_shade<3, kFeatTwoLevel>;
    default: return k_lt_shade<3, kFeatMixture | kFeatTwoLevel>;
    }
}
// Three resident blocks per SM (up to 80 registers, no spills) rather than four (64 registers,
// 80 bytes of stack): shade + connect 5.91 -> 5.48 ms on the headline BDPT frame (A/B on one
// GB300, three alternating runs each).
using BdShadeK = decltype(&k_bd_shade<3, kFeatAll>);
BdShadeK bd_shade_for(uint32_t feat) {
    switch (feat & (kFeatMixture | kFeatTwoLevel)) {
    case 0: return k_bd_shade<3, 0u>;
    case kFeatMixture: return k_bd_shade<3, kFeatMixture>;
    case kFeatTwoLevel: return k_bd_shade<3, kFeatTwoLevel>;
    default: return k_bd_shade<3, kFeatMixture | kFeatTwoLevel>;
    }
}
// Two resident blocks per SM (up to 128 registers, no spills) rather than three (80 registers,
// 150-230 bytes of spills per thread): shade + connect 6.12 -> 5.84 ms on the headline BDPT frame
// (A/B on one GB300, three alternating runs each).
using BdConnectK = decltype(&k_bd_connect<2, kFeatAll>);
BdConnectK bd_connect_for(uint32_t feat) {
    switch (feat & (kFeatEnvTex | kFeatMixture)) {
    case 0: return k_bd_connect<2, 0u>;
    case kFeatEnvTex: return k_bd_connect<2, kFeatEnvTex>;
    case kFeatMixture: return k_bd_connect<2, kFeatMixture>;
    default: return k_bd_connect<2, kFeatEnvTex | kFeatMixture>;
    }
}

void ensure_queues(Workspace& w, int64_t cap) {
    if (!w.counters.p) w.counters.alloc(192);
    if (w.cap >= cap) return;
    for (int b = 0; b < 2; b++) {
        w.q_o[b].alloc(size_t(cap) * 16);
        w.q_d[b].alloc(size_t(cap) * 16);
        w.q_thr[b].alloc(size_t(cap) * 16);
        w.q_nrm[b].alloc(size_t(cap) * 16);
        w.q_ids[b].alloc(size_t(cap) * 8);
    }
    w.hits.alloc(size_t(cap) * 16);
    w.s_o.alloc(size_t(cap) * 16);
    w.s_d.alloc(size_t(cap) * 16);
    w.s_c.alloc(size_t(cap) * 16);
    w.cap = cap;
}

}  // namespace lmgpu

using namespace lmgpu;


// ---------------------------------------------------------------------------------------------
// Scene upload (Scene_::build, src/scene.cpp:274-317, for the GPU renderers)

namespace {

// camera_pinhole.cpp:86-96 in fp32 with glm's operation order (the same arithmetic as the
// restatement's fp32 mode, so primary rays agree bit for bit).
struct HostCam {
    float p[3], u[3], v[3], w[3], tf, aspect;
};
inline float hdot(const float* a, const float* b) {
    const float x = a[0] * b[0], y = a[1] * b[1], z = a[2] * b[2];
    return (x + y) + z;
}
inline void hcross(const float* x, const float* y, float* o) {
    o[0] = x[1] * y[2] - y[1] * x[2];
    o[1] = x[2] * y[0] - y[2] * x[0];
    o[2] = x[0] * y[1] - y[0] * x[1];
}
inline void hnormalize(float* v) {
    const float inv = 1.0f / std::sqrt(hdot(v, v));
    v[0] *= inv; v[1] *= inv; v[2] *= inv;
}
HostCam make_camera(const lmgpu_camera& c) {
    HostCam h;
    for (int i = 0; i < 3; i++) { h.p[i] = c.position[i]; h.w[i] = c.position[i] - c.center[i]; }
    hnormalize(h.w);
    hcross(c.up, h.w, h.u);
    hnormalize(h.u);
    hcross(h.w, h.u, h.v);
    const float pi = 3.14159265358979323846f;
    h.tf = std::tan(c.vfov * pi / 180.0f * 0.5f);
    h.aspect = c.aspect;
    return h;
}

void ensure_film(lmgpu_film* f) {
    if (f->sum.p) return;
    const size_t n = size_t(f->w) * f->h * 3;
    f->sum.alloc(n * 4);
    f->out.alloc(n * 4);
    LMGPU_CUDA_SYNC(cudaMemset(f->sum.p, 0, n * 4));
    LMGPU_CUDA_SYNC(cudaMemset(f->out.p, 0, n * 4));
}

}  // namespace

extern "C" {

int lmgpu_scene_create(lmgpu_scene** out, lmgpu_accel* accel, const lmgpu_scene_desc* D) {
    return guarded([&] {
        if (!out || !accel || !D) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        if (accel->num_nodes == 0) throw Error(LMGPU_ERR_UNINITIALIZED, "accel is not built");
        const bool two_level = accel->num_instances > 0;
        if (D->num_tris != (two_level ? accel->blas_offsets.back() : accel->num_tris))
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "scene triangle count differs from the accel's");
        if (D->num_tris > 0 && (!D->positions || !D->normals || !D->geo_normals || !D->tri_prim))
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "missing per-triangle arrays");
        if (D->num_prims < 0 || D->num_materials < 0 || D->num_lights < 0 || D->num_light_tris < 0)
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "negative table size");
        if ((D->num_prims > 0 && (!D->prim_material || !D->prim_light)) || (D->num_materials > 0 && !D->materials) ||
            (D->num_lights > 0 && !D->lights))
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "missing table");
        auto s = std::make_unique<lmgpu_scene>();
        s->accel = accel;
        const int64_t nt = D->num_tris;

        // per-triangle shading records: p1 p2 p3 n1 n2 n3 gn prim (24 floats)
        std::vector<float> shade(size_t(nt) * 24, 0.f);
        for (int64_t t = 0; t < nt; t++) {
            float* r = &shade[size_t(t) * 24];
            std::memcpy(r, D->positions + 9 * t, 9 * 4);
            std::memcpy(r + 9, D->normals + 9 * t, 9 * 4);
            std::memcpy(r + 18, D->geo_normals + 3 * t, 3 * 4);
            const int32_t p = D->tri_prim[t];
            if (p < 0 || p >= D->num_prims) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "tri_prim out of range");
            std::memcpy(r + 21, &p, 4);
        }
        s->shade.upload(shade.data(), shade.size());
        if (two_level) {
            // per instance: world-from-local rows, normal-matrix rows (inverse transpose of the
            // linear part, math.h:742-745), first hit index, first shading record of its BLAS
            std::vector<float4> it(size_t(7) * accel->num_instances);
            for (int32_t i = 0; i < accel->num_instances; i++) {
                const double* M = &accel->inst_xform[size_t(12) * i];
                const double a00 = M[0], a01 = M[1], a02 = M[2], a10 = M[4], a11 = M[5], a12 = M[6], a20 = M[8], a21 = M[9],
                             a22 = M[10];
                const double det = a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) + a02 * (a10 * a21 - a11 * a20);
                // inverse transpose: (A^-1)^T = cofactor(A) / det
                const double nm[9] = {(a11 * a22 - a12 * a21) / det, (a12 * a20 - a10 * a22) / det, (a10 * a21 - a11 * a20) / det,
                                      (a02 * a21 - a01 * a22) / det, (a00 * a22 - a02 * a20) / det, (a01 * a20 - a00 * a21) / det,
                                      (a01 * a12 - a02 * a11) / det, (a02 * a10 - a00 * a12) / det, (a00 * a11 - a01 * a10) / det};
                float4* r = &it[size_t(7) * i];
                for (int k = 0; k < 3; k++) {
                    r[k] = make_float4(float(M[4 * k]), float(M[4 * k + 1]), float(M[4 * k + 2]), float(M[4 * k + 3]));
                    r[3 + k] = make_float4(float(nm[3 * k]), float(nm[3 * k + 1]), float(nm[3 * k + 2]), 0.f);
                }
                const uint32_t meta[4] = {uint32_t(accel->inst_id_base[i]), uint32_t(accel->blas_offsets[accel->inst_blas[i]]), 0u, 0u};
                std::memcpy(&r[6], meta, sizeof(meta));
            }
            s->inst.upload(it.data(), it.size());
        }

        std::vector<int32_t> pml(size_t(D->num_prims) * 2);
        for (int32_t p = 0; p < D->num_prims; p++) {
            const int32_t m = D->prim_material[p], l = D->prim_light[p];
            if (m < 0 || m >= D->num_materials) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "prim_material out of range");
            if (l < -1 || l >= D->num_lights) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "prim_light out of range");
            pml[2 * p] = m;
            pml[2 * p + 1] = l;
        }
        s->prim_ml.upload(pml.data(), pml.size());

        std::vector<DevMaterial> mats(D->num_materials);
        for (int32_t i = 0; i < D->num_materials; i++) {
            const lmgpu_material& m = D->materials[i];
            if (m.type < LMGPU_MAT_DIFFUSE || m.type > LMGPU_MAT_MIXTURE) throw Error(LMGPU_ERR_UNSUPPORTED, "unknown material type");
            if (m.type == LMGPU_MAT_MIXTURE && !(m.ax > 0.f && m.ay > 0.f))
                throw Error(LMGPU_ERR_INVALID_ARGUMENT, "mixture roughness must be > 0");
            if (m.type == LMGPU_MAT_GLOSSY && !(m.ax > 0.f && m.ay > 0.f)) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "glossy roughness must be > 0");
            const bool takes_kd = m.type == LMGPU_MAT_DIFFUSE || m.type == LMGPU_MAT_MIXTURE;
            if (m.map_kd < -1 || m.map_kd >= D->num_textures || m.mask < -1 || m.mask >= D->num_textures ||
                (!takes_kd && m.map_kd >= 0) || (m.type != LMGPU_MAT_MIXTURE && m.mask >= 0))
                throw Error(LMGPU_ERR_INVALID_ARGUMENT, "material texture index out of range or on a material without one");
            if (m.mask >= 0 && D->textures[m.mask].c != 4)
                throw Error(LMGPU_ERR_INVALID_ARGUMENT, "alpha mask texture without an alpha channel");
            mats[i] = DevMaterial{m.type, {m.color[0], m.color[1], m.color[2]}, m.ax, m.ay, m.ni, {m.ks[0], m.ks[1], m.ks[2]},
                                  m.map_kd, m.mask, 1.f};
        }
        s->mats.upload(mats.data(), mats.size());

        // image textures: the table, the texels and per shading record the corners' coordinates
        bool textured = false;
        for (int32_t i = 0; i < D->num_materials; i++)
            textured = textured || D->materials[i].map_kd >= 0 || D->materials[i].mask >= 0;
        if (D->num_textures < 0 || D->num_texels < 0) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "negative texture table size");
        if (D->num_textures > 0 && (!D->textures || !D->texels)) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "missing texture table");
        if (textured && nt > 0 && !D->texcoords) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "textured materials need texcoords");
        if (D->num_textures > 0) {
            std::vector<DevTexture> tex(D->num_textures);
            for (int32_t i = 0; i < D->num_textures; i++) {
                const lmgpu_texture& t = D->textures[i];
                if (t.w <= 0 || t.h <= 0 || (t.c != 3 && t.c != 4) || t.offset < 0 ||
                    t.offset + int64_t(t.w) * t.h * t.c > D->num_texels)
                    throw Error(LMGPU_ERR_INVALID_ARGUMENT, "texture size or offset out of range");
                tex[i] = DevTexture{t.w, t.h, t.c, 0, t.offset};
            }
            s->tex.upload(tex.data(), tex.size());
            s->texels.upload(D->texels, size_t(D->num_texels));
        }
        if (textured && nt > 0) {
            for (int64_t k = 0; k < 6 * nt; k++)
                if (!std::isfinite(D->texcoords[k])) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "non-finite texture coordinate");
            s->uv.upload(D->texcoords, size_t(nt) * 6);
        }

        // lights: area CDFs and env tables are built here in double precision, then stored fp32
        std::vector<DevLight> lights(D->num_lights);
        std::vector<float> cdf, ltri, env;
        int32_t env_light = -1;
        bool has_directional = false;
        for (int32_t i = 0; i < D->num_lights; i++) {
            const lmgpu_light& L = D->lights[i];
            DevLight& dl = lights[i];
            std::memset(&dl, 0, sizeof(dl));
            dl.type = L.type;
            dl.ke[0] = L.ke[0]; dl.ke[1] = L.ke[1]; dl.ke[2] = L.ke[2];
            if (L.type == LMGPU_LIGHT_AREA) {
                if (L.tri_count <= 0 || L.tri_offset < 0 || L.tri_offset + L.tri_count > D->num_light_tris)
                    throw Error(LMGPU_ERR_INVALID_ARGUMENT, "area light triangle range out of bounds");
                dl.tri_off = int32_t(ltri.size() / 12);
                dl.tri_cnt = int32_t(L.tri_count);
                dl.cdf_off = int32_t(cdf.size());
                double sum = 0;
                std::vector<double> c(size_t(L.tri_count) + 1, 0.0);
                for (int64_t k = 0; k < L.tri_count; k++) {
                    sum += double(D->light_tri_area[L.tri_offset + k]);
                    c[k + 1] = sum;
                }
                if (!(sum > 0)) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "area light has zero area");
                for (double v : c) cdf.push_back(float(v / sum));
                dl.invA_J = float((1.0 / sum) / double(L.transform_j));
                for (int64_t k = 0; k < L.tri_count; k++) {
                    const float* p = D->light_tri_p + 9 * (L.tri_offset + k);
                    const float* g = D->light_tri_gn + 3 * (L.tri_offset + k);
                    const float rec[12] = {p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8], g[0], g[1], g[2]};
                    ltri.insert(ltri.end(), rec, rec + 12);
                }
            } else if (L.type == LMGPU_LIGHT_ENVCONST || L.type == LMGPU_LIGHT_ENV) {
                if (env_light >= 0) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "only one environment light is allowed");
                env_light = i;
                if (L.type == LMGPU_LIGHT_ENV) {
                    const int w = L.env_w, h = L.env_h;
                    if (w <= 0 || h <= 0 || !D->env_texels || L.env_offset < 0 || L.env_offset + int64_t(w) * h * 3 > D->num_env_texels)
                        throw Error(LMGPU_ERR_INVALID_ARGUMENT, "env texture out of bounds");
                    const float* tex = D->env_texels + L.env_offset;
                    dl.env_w = w; dl.env_h = h;
                    dl.rot = L.rot_deg * 3.14159265358979323846f / 180.0f;
                    dl.scale = L.scale;
                    dl.tex_off = int32_t(env.size());
                    env.insert(env.end(), tex, tex + size_t(w) * h * 3);
                    // light_env.cpp:65-71 then Dist2::init (math.h:396-409)
                    std::vector<double> rows(h + 1, 0.0);
                    std::vector<double> cond(size_t(h) * (w + 1), 0.0);
                    double msum = 0;
                    for (int y = 0; y < h; y++) {
                        double rs = 0;
                        for (int x = 0; x < w; x++) {
                            const int i2 = y * w + x;
                            const float* t = tex + 3 * size_t(i2);
                            const double m = std::max(std::max(double(t[0]) * L.scale, double(t[1]) * L.scale), double(t[2]) * L.scale);
                            rs += m * std::sin(3.14159265358979323846 * (double(i2) / w + .5) / h);
                            cond[size_t(y) * (w + 1) + x + 1] = rs;
                        }
                        for (int x = 0; x <= w; x++) cond[size_t(y) * (w + 1) + x] = rs > 0 ? cond[size_t(y) * (w + 1) + x] / rs : 0.0;
                        msum += rs;
                        rows[y + 1] = msum;
                    }
                    if (!(msum > 0)) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "env map is black");
                    dl.marg_off = int32_t(env.size());
                    for (int y = 0; y <= h; y++) env.push_back(float(rows[y] / msum));
                    dl.cond_off = int32_t(env.size());
                    for (double v : cond) env.push_back(float(v));
                }
            } else if (L.type == LMGPU_LIGHT_POINT) {
                dl.v[0] = L.vec[0]; dl.v[1] = L.vec[1]; dl.v[2] = L.vec[2];
                if (!std::isfinite(dl.v[0]) || !std::isfinite(dl.v[1]) || !std::isfinite(dl.v[2]))
                    throw Error(LMGPU_ERR_INVALID_ARGUMENT, "point light position is not finite");
            } else if (L.type == LMGPU_LIGHT_DIRECTIONAL) {
                // light_directional.cpp:36: the direction normalized (in double)
                const double x = L.vec[0], y = L.vec[1], z = L.vec[2];
                const double len = std::sqrt(x * x + y * y + z * z);
                if (!(len > 0) || !std::isfinite(len)) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "directional light needs a nonzero direction");
                dl.v[0] = float(x / len); dl.v[1] = float(y / len); dl.v[2] = float(z / len);
                has_directional = true;
            } else {
                throw Error(LMGPU_ERR_UNSUPPORTED, "unknown light type");
            }
        }
        s->lights.upload(lights.data(), lights.size());
        s->ltri.upload(ltri.data(), ltri.size());
        s->cdf.upload(cdf.data(), cdf.size());
        s->env.upload(env.data(), env.size());

        // scene.cpp:288-311 and light_envconst.cpp:38-43: the bound of every triangle in world space
        // (two-level scenes: each instance's BLAS triangles moved by its transform), as a sphere
        // of radius 1.01 |max - center| (light_directional.cpp:40-45 alike); environment and
        // directional lights use it
        const bool need_bound = env_light >= 0 || has_directional;
        double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
        auto grow = [&](double x, double y, double z) {
            lo[0] = std::min(lo[0], x); lo[1] = std::min(lo[1], y); lo[2] = std::min(lo[2], z);
            hi[0] = std::max(hi[0], x); hi[1] = std::max(hi[1], y); hi[2] = std::max(hi[2], z);
        };
        if (need_bound && !two_level) {
            for (int64_t k = 0; k < 3 * nt; k++) grow(D->positions[3 * k], D->positions[3 * k + 1], D->positions[3 * k + 2]);
        } else if (need_bound) {
            for (int32_t i = 0; i < accel->num_instances; i++) {
                const double* M = &accel->inst_xform[size_t(12) * i];
                const int b = accel->inst_blas[i];
                for (int64_t k = 3 * accel->blas_offsets[b]; k < 3 * accel->blas_offsets[b + 1]; k++) {
                    const double x = D->positions[3 * k], y = D->positions[3 * k + 1], z = D->positions[3 * k + 2];
                    grow(M[0] * x + M[1] * y + M[2] * z + M[3], M[4] * x + M[5] * y + M[6] * z + M[7], M[8] * x + M[9] * y + M[10] * z + M[11]);
                }
            }
        }
        f3 bound_c = mk(0, 0, 0);
        float bound_r = 0.f;
        if (lo[0] <= hi[0]) {
            const double c[3] = {(hi[0] + lo[0]) * .5, (hi[1] + lo[1]) * .5, (hi[2] + lo[2]) * .5};
            const double e[3] = {hi[0] - c[0], hi[1] - c[1], hi[2] - c[2]};
            bound_c = mk(float(c[0]), float(c[1]), float(c[2]));
            bound_r = float(std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) * 1.01);
        }

        DevScene& ds = s->dev;
        ds.bvh = device_view(accel);
        ds.bound_c = bound_c;
        ds.bound_r = bound_r;
        ds.feat = two_level ? kFeatTwoLevel : 0u;
        for (int32_t i = 0; i < D->num_lights; i++)
            if (D->lights[i].type == LMGPU_LIGHT_ENV) ds.feat |= kFeatEnvTex;
            else if (D->lights[i].type == LMGPU_LIGHT_POINT || D->lights[i].type == LMGPU_LIGHT_DIRECTIONAL) ds.feat |= kFeatDelta;
        for (int32_t i = 0; i < D->num_materials; i++) {
            if (D->materials[i].type == LMGPU_MAT_MIXTURE) ds.feat |= kFeatMixture;
            if (D->materials[i].map_kd >= 0 || D->materials[i].mask >= 0) ds.feat |= kFeatTexture;
        }
        ds.uv = s->uv.as<const float>();
        ds.tex = s->tex.as<const DevTexture>();
        ds.texels = s->texels.as<const float>();
        ds.shade = s->shade.as<const float4>();
        ds.prim_ml = s->prim_ml.as<const int2>();
        ds.mats = s->mats.as<const DevMaterial>();
        ds.lights = s->lights.as<const DevLight>();
        ds.num_lights = D->num_lights;
        ds.env_light = env_light;
        ds.ltri = s->ltri.as<const float4>();
        ds.cdf = s->cdf.as<const float>();
        ds.env = s->env.as<const float>();
        ds.has_camera = D->has_camera;
        ds.inst = two_level ? s->inst.as<const float4>() : nullptr;
        ds.num_inst = two_level ? accel->num_instances : 0;
        if (D->has_camera) {
            const HostCam c = make_camera(D->camera);
            ds.cam_p = mk(c.p[0], c.p[1], c.p[2]);
            ds.cam_u = mk(c.u[0], c.u[1], c.u[2]);
            ds.cam_v = mk(c.v[0], c.v[1], c.v[2]);
            ds.cam_w = mk(c.w[0], c.w[1], c.w[2]);
            ds.tf = c.tf;
            ds.aspect = c.aspect;
        }
        s->counters.alloc(192);
        LMGPU_CUDA_SYNC(cudaMemset(s->counters.p, 0, 192));
        *out = s.release();
    });
}

int lmgpu_scene_destroy(lmgpu_scene* scene) {
    return guarded([&] { delete scene; });
}

int lmgpu_scene_device_bytes(const lmgpu_scene* s, int64_t* out) {
    return guarded([&] {
        if (!s || !out) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        const size_t b = s->shade.bytes + s->prim_ml.bytes + s->mats.bytes + s->lights.bytes + s->ltri.bytes + s->cdf.bytes +
                         s->env.bytes + s->inst.bytes + s->counters.bytes;
        *out = int64_t(b);
    });
}

// ---------------------------------------------------------------------------------------------
// Film

int lmgpu_film_create(lmgpu_film** out, int32_t w, int32_t h) {
    return guarded([&] {
        if (!out || w <= 0 || h <= 0) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "invalid film size");
        auto f = std::make_unique<lmgpu_film>();
        f->w = w;
        f->h = h;
        *out = f.release();  // device memory is allocated on first use
    });
}

int lmgpu_film_destroy(lmgpu_film* film) {
    return guarded([&] { delete film; });
}

int lmgpu_film_clear(lmgpu_film* f) {
    return guarded([&] {
        if (!f) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "film is null");
        ensure_film(f);
        const size_t n = size_t(f->w) * f->h * 3;
        LMGPU_CUDA_SYNC(cudaMemset(f->sum.p, 0, n * 4));
        LMGPU_CUDA_SYNC(cudaMemset(f->out.p, 0, n * 4));
        if (f->sum_odd.p) LMGPU_CUDA_SYNC(cudaMemset(f->sum_odd.p, 0, n * 4));
        f->accumulated_spp = 0;
        f->scale = 1.0;
        f->split = false;
        f->passes_even = f->passes_odd = 0;
    });
}

int lmgpu_film_rel_mse(lmgpu_film* f, double eps, double* rel_mse) {
    return guarded([&] {
        if (!f || !rel_mse || !(eps >= 0.0)) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "invalid argument");
        if (!f->split || f->passes_even < 1 || f->passes_odd < 1)
            throw Error(LMGPU_ERR_UNINITIALIZED, "film has no split passes (render with split_passes and spp >= 2)");
        const int64_t n = int64_t(f->w) * f->h * 3;
        const double N = double(f->passes_even + f->passes_odd);
        DevBuf& acc = f->mse_acc;
        acc.alloc(sizeof(double));
        LMGPU_CUDA_SYNC(cudaMemset(acc.p, 0, sizeof(double)));
        // the accumulators hold per-pass sums in the estimate's units (a render scales its film by
        // 1 / passes in both primary modes), so no further unit factor; N only fixes the pass count
        (void)N;
        k_rel_mse<<<256, 256>>>(f->sum.as<float>(), f->sum_odd.as<float>(), n, double(f->passes_even), double(f->passes_odd),
                                1.0, eps, acc.as<double>());
        LMGPU_CUDA(cudaGetLastError());
        double h = 0.0;
        LMGPU_CUDA_SYNC(cudaMemcpy(&h, acc.p, sizeof(double), cudaMemcpyDeviceToHost));
        *rel_mse = h / double(n);
    });
}

int lmgpu_probe_l2_bandwidth(int64_t bytes, int32_t iters, double* gbs) {
    return guarded([&] {
        if (!gbs || bytes < (int64_t(1) << 20) || iters < 1) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "invalid probe size");
        DevBuf buf, out;
        const int64_t n = bytes / 16;
        buf.alloc(size_t(n) * 16);
        out.alloc(16);
        LMGPU_CUDA_SYNC(cudaMemset(buf.p, 0, size_t(n) * 16));
        const int grid = 8 * current_device().num_sms;
        k_l2_probe<<<grid, 256>>>(buf.as<float4>(), n, 1, out.as<float>());  // brings the buffer into L2
        LMGPU_CUDA(cudaGetLastError());
        cudaEvent_t e0, e1;
        LMGPU_CUDA(cudaEventCreate(&e0));
        LMGPU_CUDA(cudaEventCreate(&e1));
        LMGPU_CUDA(cudaEventRecord(e0));
        k_l2_probe<<<grid, 256>>>(buf.as<float4>(), n, iters, out.as<float>());
        LMGPU_CUDA(cudaEventRecord(e1));
        LMGPU_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        LMGPU_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        LMGPU_CUDA(cudaGetLastError());
        *gbs = double(n) * 16.0 * iters / (double(ms) * 1e-3) / 1e9;
    });
}

int lmgpu_film_fill(lmgpu_film* f, const float* rgb) {
    return guarded([&] {
        if (!f || !rgb) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        ensure_film(f);
        const size_t n = size_t(f->w) * f->h;
        std::vector<float> px(n * 3);
        for (size_t i = 0; i < n; i++) {
            px[3 * i] = rgb[0];
            px[3 * i + 1] = rgb[1];
            px[3 * i + 2] = rgb[2];
        }
        LMGPU_CUDA_SYNC(cudaMemcpy(f->sum.p, px.data(), n * 3 * 4, cudaMemcpyHostToDevice));
        LMGPU_CUDA_SYNC(cudaMemcpy(f->out.p, px.data(), n * 3 * 4, cudaMemcpyHostToDevice));
        if (f->sum_odd.p) LMGPU_CUDA_SYNC(cudaMemset(f->sum_odd.p, 0, n * 3 * 4));
        f->accumulated_spp = 0;
        f->scale = 1.0;
        f->split = false;
        f->passes_even = f->passes_odd = 0;
    });
}

int lmgpu_film_read(lmgpu_film* f, float* out_rgb) {
    return guarded([&] {
        if (!f || !out_rgb) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        ensure_film(f);
        LMGPU_CUDA_SYNC(cudaMemcpy(out_rgb, f->out.p, size_t(f->w) * f->h * 3 * 4, cudaMemcpyDeviceToHost));
    });
}

int lmgpu_film_device_ptr(lmgpu_film* f, void** out) {
    return guarded([&] {
        if (!f || !out) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        ensure_film(f);
        *out = f->out.p;
    });
}

// ---------------------------------------------------------------------------------------------
// Renderers

int lmgpu_render_raycast(lmgpu_scene* s, lmgpu_film* f, const lmgpu_raycast_params* prm, void* stream) {
    return guarded([&] {
        if (!s || !f || !prm) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        if (!s->dev.has_camera) throw Error(LMGPU_ERR_UNSUPPORTED, "Missing camera primitive.");
        ensure_film(f);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const size_t smem = trace_smem(s->accel) * kBlock / 128;
        int* err = s->counters.as<int>() + 3;
        LMGPU_CUDA(cudaMemsetAsync(err, 0, 4, st));
        const int64_t n = int64_t(f->w) * f->h;
        auto rk = s->dev.num_inst > 0 ? k_raycast<true> : k_raycast<false>;
        int g = grid_for(rk, kBlock, smem);
        g = int(std::min<int64_t>(g, (n + kBlock - 1) / kBlock));
        rk<<<g, kBlock, smem, st>>>(s->dev, f->w, f->h, *prm, f->sum.as<float>(), err);
        LMGPU_CUDA(cudaGetLastError());
        k_scale<<<256, 256, 0, st>>>(f->sum.as<float>(), f->out.as<float>(), n * 3, 1.0f);
        int herr = 0;
        LMGPU_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaStreamSynchronize(st));
        if (herr) throw Error(LMGPU_ERR_INTERNAL, "traversal consistency check failed");
        f->scale = 1.0;
        f->accumulated_spp = 1;
    });
}

namespace {

void must(int rc) {
    if (rc != LMGPU_OK) throw Error(rc, lmgpu_last_error());
}

// Fixed waves of at most wave_paths paths, each run for max_verts - 1 bounces with one launch per
// kernel per bounce. Used for instrumented renders (node / triangle counts).
void render_pt_waves(lmgpu_scene* s, lmgpu_film* f, const lmgpu_pt_params* prm, void* stream, lmgpu_render_stats* stats) {
    {
        ensure_film(f);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const int64_t npix = int64_t(f->w) * f->h;
        const int64_t total = npix * prm->spp;
        if (total > (int64_t(1) << 32)) throw Error(LMGPU_ERR_UNSUPPORTED, "more than 2^32 paths in one render");
        int64_t wave = prm->wave_paths > 0 ? prm->wave_paths : (int64_t(1) << 22);
        wave = std::min(wave, total);
        Workspace& ws = workspace(current_device().device);
        std::lock_guard<std::mutex> ws_lock(ws.m);
        ensure_queues(ws, wave);

        PtConst P;
        P.seed = prm->seed;
        P.max_verts = prm->max_verts;
        P.spp = prm->spp;
        P.mode = prm->sampling_mode;
        P.image = prm->primary_mode == LMGPU_PRIMARY_IMAGE;
        P.w = f->w;
        P.h = f->h;

        ExtQ q[2];
        for (int b = 0; b < 2; b++)
            q[b] = ExtQ{ws.q_o[b].as<float4>(), ws.q_d[b].as<float4>(), ws.q_thr[b].as<float4>(), ws.q_nrm[b].as<float4>(),
                        ws.q_ids[b].as<uint2>()};
        ShadowQ sq{ws.s_o.as<float4>(), ws.s_d.as<float4>(), ws.s_c.as<float4>()};
        // [0],[1] extension queues, [2] shadow queue, [3] error, [4],[5] extension / shadow ray fetch
        int* cnt = ws.counters.as<int>();
        const int refill = tuning().trace_refill;
        const Fetch f_ext{cnt + 4, cnt + 5, refill}, f_sh{cnt + 5, cnt + 4, refill};
        unsigned long long* rays = reinterpret_cast<unsigned long long*>(ws.counters.as<char>() + 32);
        float* film = f->sum.as<float>();
        const Bvh8 bvh = s->dev.bvh;
        const size_t tsmem = size_t(2) * 4 * kBlock * size_t(bvh.depth);

        const bool inst = prm->instrument != 0;
        const bool two = s->dev.num_inst > 0;
        auto ext_k = inst ? (two ? k_pt_extend<true, false, true> : k_pt_extend<true, false, false>)
                          : (two ? k_pt_extend<false, false, true> : k_pt_extend<false, false, false>);
        auto sh_k = inst ? (two ? k_pt_shadow<true, false, true> : k_pt_shadow<true, false, false>)
                         : (two ? k_pt_shadow<false, false, true> : k_pt_shadow<false, false, false>);
        const int g_gen = grid_for(k_pt_generate, kBlock, 0);
        const int g_ext = grid_for(ext_k, kBlock, tsmem);
        const int g_sh = grid_for(sh_k, kBlock, tsmem);
        auto shade_k = pick_shade(k_pt_shade<2>, k_pt_shade<3>, k_pt_shade<4>, tuning().shade_minblocks);
        const int g_shade = grid_for(shade_k, kBlock, 0);
        unsigned long long* sums = reinterpret_cast<unsigned long long*>(ws.counters.as<char>() + 64);  // 8 counters
        float* worst = reinterpret_cast<float*>(ws.counters.as<char>() + 128);                           // 2 rays
        const int cmask = prm->instrument == 2 ? 0 : 63;

        // per-kernel device time: events bracket every launch when stats are requested
        enum { K_GEN = 0, K_EXT = 1, K_SHADE = 2, K_SHADOW = 3 };
        std::vector<std::pair<int, cudaEvent_t>> marks;
        const bool timed = stats != nullptr;
        auto mark = [&](int kind) {
            if (!timed) return;
            cudaEvent_t e;
            LMGPU_CUDA(cudaEventCreate(&e));
            LMGPU_CUDA(cudaEventRecord(e, st));
            marks.emplace_back(kind, e);
        };
        cudaEvent_t e0, e1;
        LMGPU_CUDA(cudaEventCreate(&e0));
        LMGPU_CUDA(cudaEventCreate(&e1));
        int64_t n_ext = 0, n_sh = 0;

        LMGPU_CUDA(cudaEventRecord(e0, st));
        if (!prm->accumulate) {
            LMGPU_CUDA(cudaMemsetAsync(film, 0, size_t(npix) * 3 * 4, st));
            f->accumulated_spp = 0;
        }
        LMGPU_CUDA(cudaMemsetAsync(ws.counters.p, 0, 192, st));
        for (int64_t start = 0; start < total; start += wave) {
            const int64_t n = std::min(wave, total - start);
            int cur = 0;
            LMGPU_CUDA(cudaMemsetAsync(cnt, 0, 12, st));
            LMGPU_CUDA(cudaMemsetAsync(cnt + 4, 0, 8, st));
            mark(K_GEN);
            k_pt_generate<<<std::min<int64_t>(g_gen, (n + kBlock - 1) / kBlock), kBlock, 0, st>>>(s->dev, P, start, n, q[0],
                                                                                               cnt + 0, sq, cnt + 2);
            mark(-1);
            LMGPU_CUDA(cudaGetLastError());
            if (P.image) {
                mark(K_SHADOW);
                sh_k<<<g_sh, kBlock, tsmem, st>>>(bvh, sq, cnt + 2, film, rays + 1, cnt + 3, sums, cmask, worst, f_sh, nullptr,
                                                  nullptr);
                mark(-1);
                n_sh++;
                LMGPU_CUDA(cudaMemsetAsync(cnt + 2, 0, 4, st));
            }
            for (int it = 1; it < P.max_verts; it++) {
                mark(K_EXT);
                ext_k<<<g_ext, kBlock, tsmem, st>>>(bvh, q[cur].o, q[cur].d, cnt + cur, ws.hits.as<float4>(), rays, cnt + 3, sums,
                                                    cmask, worst, f_ext, nullptr, nullptr);
                mark(-1);
                n_ext++;
                LMGPU_CUDA(cudaMemsetAsync(cnt + (1 - cur), 0, 4, st));
                LMGPU_CUDA(cudaMemsetAsync(cnt + 2, 0, 4, st));
                mark(K_SHADE);
                shade_k<<<g_shade, kBlock, 0, st>>>(s->dev, P, q[cur], ws.hits.as<float4>(), cnt + cur, q[1 - cur],
                                                      cnt + (1 - cur), sq, cnt + 2, film);
                mark(-1);
                mark(K_SHADOW);
                sh_k<<<g_sh, kBlock, tsmem, st>>>(bvh, sq, cnt + 2, film, rays + 1, cnt + 3, sums, cmask, worst, f_sh, nullptr,
                                                  nullptr);
                mark(-1);
                n_sh++;
                LMGPU_CUDA(cudaGetLastError());
                cur = 1 - cur;
            }
        }
        f->accumulated_spp += prm->spp;
        // renderer_pt.cpp:307-312: 1 / spp in pixel mode; w*h / (paths) = 1 / spp in image mode
        const double scale = 1.0 / double(f->accumulated_spp);
        f->scale = scale;
        k_scale<<<1024, 256, 0, st>>>(film, f->out.as<float>(), npix * 3, float(scale));
        LMGPU_CUDA(cudaEventRecord(e1, st));
        unsigned long long hr[2], hs[8];
        float hw[16];
        int herr = 0;
        LMGPU_CUDA(cudaMemcpyAsync(hr, rays, sizeof(hr), cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaMemcpyAsync(hs, sums, sizeof(hs), cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaMemcpyAsync(hw, worst, sizeof(hw), cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaMemcpyAsync(&herr, cnt + 3, 4, cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaStreamSynchronize(st));
        float ms = 0.f;
        LMGPU_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        double kms[4] = {0, 0, 0, 0};
        for (size_t i = 0; i + 1 < marks.size(); i++) {
            if (marks[i].first < 0) continue;
            float m = 0.f;
            LMGPU_CUDA(cudaEventElapsedTime(&m, marks[i].second, marks[i + 1].second));
            kms[marks[i].first] += m;
        }
        for (auto& e : marks) cudaEventDestroy(e.second);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (herr) throw Error(LMGPU_ERR_INTERNAL, "traversal consistency check failed");
        if (stats) {
            stats->paths = total;
            stats->extension_rays = int64_t(hr[0]);
            stats->shadow_rays = int64_t(hr[1]);
            stats->rays = int64_t(hr[0] + hr[1]);
            stats->elapsed_ms = ms;
            stats->generate_ms = kms[K_GEN];
            stats->extend_ms = kms[K_EXT];
            stats->shade_ms = kms[K_SHADE];
            stats->shadow_ms = kms[K_SHADOW];
            stats->trace_ms = kms[K_EXT] + kms[K_SHADOW];
            stats->extend_launches = n_ext;
            stats->shadow_launches = n_sh;
            stats->ext_nodes = hs[2] ? double(hs[0]) / double(hs[2]) : 0.0;
            stats->ext_tris = hs[2] ? double(hs[1]) / double(hs[2]) : 0.0;
            stats->shadow_nodes = hs[5] ? double(hs[3]) / double(hs[5]) : 0.0;
            stats->shadow_tris = hs[5] ? double(hs[4]) / double(hs[5]) : 0.0;
            stats->ext_max_nodes = int64_t(hs[6]);
            stats->shadow_max_nodes = int64_t(hs[7]);
            for (int i = 0; i < 8; i++) {
                stats->ext_worst_ray[i] = hw[i];
                stats->shadow_worst_ray[i] = hw[8 + i];
            }
        }
    }
}

}  // namespace

int lmgpu_render_pt(lmgpu_scene* s, lmgpu_film* f, const lmgpu_pt_params* prm, void* stream, lmgpu_render_stats* stats) {
    return guarded([&] {
        if (!s || !f || !prm) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        if (!s->dev.has_camera) throw Error(LMGPU_ERR_UNSUPPORTED, "Missing camera primitive.");
        if (s->dev.num_lights == 0) throw Error(LMGPU_ERR_UNSUPPORTED, "No light in the scene.");
        if (prm->spp <= 0 || prm->max_verts < 1) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "spp must be > 0 and max_verts >= 1");
        if (prm->max_verts > 255) throw Error(LMGPU_ERR_UNSUPPORTED, "max_verts above 255");
        if (prm->sampling_mode < 0 || prm->sampling_mode > 2 || prm->primary_mode < 0 || prm->primary_mode > 1)
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "unknown sampling mode");
        if (prm->instrument) {
            if (prm->split_passes) throw Error(LMGPU_ERR_UNSUPPORTED, "split_passes with instrument");
            render_pt_waves(s, f, prm, stream, stats);
            return;
        }
        // One job on the device's shared wavefront: finished paths are replaced by new ones of
        // the same job, so every bounce launch sees a full queue (a fixed wave thins out).
        Workspace& ws = workspace(current_device().device);
        std::lock_guard<std::mutex> ws_lock(ws.m);
        const int64_t cap = prm->wave_paths > 0 ? prm->wave_paths : kRenderQueue;
        if (!ws.batch || ws.batch_cap != cap) {
            if (ws.batch) must(lmgpu_batch_destroy(ws.batch));
            ws.batch = nullptr;
            must(lmgpu_batch_create(&ws.batch, cap));
            ws.batch_cap = cap;
        }
        lmgpu_batch* b = ws.batch;
        must(lmgpu_batch_reset(b));
        must(lmgpu_batch_set_timing(b, stats != nullptr));
        int32_t job = 0;
        must(lmgpu_batch_submit(b, s, f, prm, &job));
        int64_t left = 0;
        must(lmgpu_batch_run(b, 0, stream, &left));
        must(lmgpu_batch_resolve(b, job, stream));
        if (stats) must(lmgpu_batch_get_stats(b, stats));
    });
}

int lmgpu_render_lt(lmgpu_scene* s, lmgpu_film* f, const lmgpu_lt_params* prm, void* stream, lmgpu_render_stats* stats) {
    return guarded([&] {
        if (!s || !f || !prm) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        if (s->dev.feat & kFeatTexture)
            throw Error(LMGPU_ERR_UNSUPPORTED, "image textures are supported by renderer::pt and renderer::raycast");
        if (!s->dev.has_camera) throw Error(LMGPU_ERR_UNSUPPORTED, "Missing camera primitive.");
        if (s->dev.num_lights == 0) throw Error(LMGPU_ERR_UNSUPPORTED, "No light in the scene.");
        if (prm->num_samples <= 0 || prm->max_verts < 1 || prm->first_path < 0)
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "num_samples must be > 0, first_path >= 0 and max_verts >= 1");
        if (prm->max_verts > 255) throw Error(LMGPU_ERR_UNSUPPORTED, "max_verts above 255");
        if (prm->first_path + prm->num_samples > (int64_t(1) << 32))
            throw Error(LMGPU_ERR_UNSUPPORTED, "light path index above 2^32");
        if (prm->accumulate && f->split) throw Error(LMGPU_ERR_UNSUPPORTED, "film holds split passes");
        ensure_film(f);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const int64_t npix = int64_t(f->w) * f->h;
        const int64_t total = prm->num_samples;
        const int64_t wave = std::min(prm->wave_paths > 0 ? prm->wave_paths : kRenderQueue, total);
        Workspace& ws = workspace(current_device().device);
        std::lock_guard<std::mutex> ws_lock(ws.m);
        ensure_queues(ws, wave);

        PtConst P{};
        P.seed = prm->seed;
        P.max_verts = prm->max_verts;
        P.spp = 1;
        P.w = f->w;
        P.h = f->h;
        ExtQ q[2];
        for (int b = 0; b < 2; b++)
            q[b] = ExtQ{ws.q_o[b].as<float4>(), ws.q_d[b].as<float4>(), ws.q_thr[b].as<float4>(), ws.q_nrm[b].as<float4>(),
                        ws.q_ids[b].as<uint2>()};
        ShadowQ sq{ws.s_o.as<float4>(), ws.s_d.as<float4>(), ws.s_c.as<float4>()};
        // [0],[1] extension queues, [2] shadow queue, [3] error, [4],[5] extension / shadow ray fetch
        int* cnt = ws.counters.as<int>();
        const int refill = tuning().trace_refill;
        const Fetch f_ext{cnt + 4, cnt + 5, refill}, f_sh{cnt + 5, cnt + 4, refill};
        unsigned long long* rays = reinterpret_cast<unsigned long long*>(ws.counters.as<char>() + 32);
        float* film = f->sum.as<float>();
        const Bvh8 bvh = s->dev.bvh;
        const size_t tsmem = size_t(2) * 4 * kBlock * size_t(bvh.depth);
        const bool two = s->dev.num_inst > 0;
        auto ext_k = two ? k_pt_extend<false, false, true> : k_pt_extend<false, false, false>;
        auto sh_k = two ? k_pt_shadow<false, false, true> : k_pt_shadow<false, false, false>;
        // the default register budget runs a kernel specialised on the scene's features
        auto shade_k = tuning().shade_minblocks >= 4 ? lt_shade_for(s->dev.feat)
                                                      : pick_shade(k_lt_shade<2>, k_lt_shade<3>, k_lt_shade<4>, tuning().shade_minblocks);
        const int g_gen = grid_for(k_lt_generate, kBlock, 0);
        const int g_ext = grid_for(ext_k, kBlock, tsmem);
        const int g_sh = grid_for(sh_k, kBlock, tsmem);
        const int g_shade = grid_for(shade_k, kBlock, 0);

        enum { K_GEN = 0, K_EXT = 1, K_SHADE = 2, K_SHADOW = 3 };
        std::vector<std::pair<int, cudaEvent_t>> marks;
        const bool timed = stats != nullptr;
        auto mark = [&](int kind) {
            if (!timed) return;
            cudaEvent_t e;
            LMGPU_CUDA(cudaEventCreate(&e));
            LMGPU_CUDA(cudaEventRecord(e, st));
            marks.emplace_back(kind, e);
        };
        cudaEvent_t e0, e1;
        LMGPU_CUDA(cudaEventCreate(&e0));
        LMGPU_CUDA(cudaEventCreate(&e1));
        int64_t n_ext = 0, n_sh = 0;

        LMGPU_CUDA(cudaEventRecord(e0, st));
        if (!prm->accumulate) {
            LMGPU_CUDA(cudaMemsetAsync(film, 0, size_t(npix) * 3 * 4, st));
            f->accumulated_spp = 0;
            f->split = false;
            f->passes_even = f->passes_odd = 0;
        }
        LMGPU_CUDA(cudaMemsetAsync(ws.counters.p, 0, 192, st));
        // a path of max_verts <= 2 vertices cannot reach a camera connection (renderer_lt.cpp:89)
        for (int64_t start = 0; prm->max_verts > 2 && start < total; start += wave) {
            const int64_t n = std::min(wave, total - start);
            int cur = 0;
            LMGPU_CUDA(cudaMemsetAsync(cnt, 0, 12, st));
            LMGPU_CUDA(cudaMemsetAsync(cnt + 4, 0, 8, st));
            mark(K_GEN);
            k_lt_generate<<<int(std::min<int64_t>(g_gen, (n + kBlock - 1) / kBlock)), kBlock, 0, st>>>(
                s->dev, P, prm->first_path + start, n, q[0], cnt + 0);
            mark(-1);
            LMGPU_CUDA(cudaGetLastError());
            // the ray that leaves vertex it; its hit connects when it + 1 < max_verts
            for (int it = 1; it + 1 < P.max_verts; it++) {
                mark(K_EXT);
                ext_k<<<g_ext, kBlock, tsmem, st>>>(bvh, q[cur].o, q[cur].d, cnt + cur, ws.hits.as<float4>(), rays, cnt + 3, nullptr,
                                                    0, nullptr, f_ext, nullptr, nullptr);
                mark(-1);
                n_ext++;
                LMGPU_CUDA(cudaMemsetAsync(cnt + (1 - cur), 0, 4, st));
                LMGPU_CUDA(cudaMemsetAsync(cnt + 2, 0, 4, st));
                mark(K_SHADE);
                shade_k<<<g_shade, kBlock, 0, st>>>(s->dev, P, q[cur], ws.hits.as<float4>(), cnt + cur, q[1 - cur], cnt + (1 - cur),
                                                      sq, cnt + 2);
                mark(-1);
                mark(K_SHADOW);
                sh_k<<<g_sh, kBlock, tsmem, st>>>(bvh, sq, cnt + 2, film, rays + 1, cnt + 3, nullptr, 0, nullptr, f_sh, nullptr,
                                                  nullptr);
                mark(-1);
                n_sh++;
                LMGPU_CUDA(cudaGetLastError());
                cur = 1 - cur;
            }
        }
        f->accumulated_spp += total;
        const double scale = double(npix) / double(f->accumulated_spp);
        f->scale = scale;
        k_scale<<<1024, 256, 0, st>>>(film, f->out.as<float>(), npix * 3, float(scale));
        LMGPU_CUDA(cudaGetLastError());
        LMGPU_CUDA(cudaEventRecord(e1, st));
        unsigned long long hr[2];
        int herr = 0;
        LMGPU_CUDA(cudaMemcpyAsync(hr, rays, sizeof(hr), cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaMemcpyAsync(&herr, cnt + 3, 4, cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaStreamSynchronize(st));
        float ms = 0.f;
        LMGPU_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        double kms[4] = {0, 0, 0, 0};
        for (size_t i = 0; i + 1 < marks.size(); i++) {
            if (marks[i].first < 0) continue;
            float m = 0.f;
            LMGPU_CUDA(cudaEventElapsedTime(&m, marks[i].second, marks[i + 1].second));
            kms[marks[i].first] += m;
        }
        for (auto& e : marks) cudaEventDestroy(e.second);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (herr) throw Error(LMGPU_ERR_INTERNAL, "traversal consistency check failed");
        if (stats) {
            *stats = lmgpu_render_stats{};
            stats->paths = total;
            stats->extension_rays = int64_t(hr[0]);
            stats->shadow_rays = int64_t(hr[1]);
            stats->rays = int64_t(hr[0] + hr[1]);
            stats->elapsed_ms = ms;
            stats->generate_ms = kms[K_GEN];
            stats->extend_ms = kms[K_EXT];
            stats->shade_ms = kms[K_SHADE];
            stats->shadow_ms = kms[K_SHADOW];
            stats->trace_ms = kms[K_EXT] + kms[K_SHADOW];
            stats->extend_launches = n_ext;
            stats->shadow_launches = n_sh;
        }
    });
}

int lmgpu_render_bdpt(lmgpu_scene* s, lmgpu_film* f, const lmgpu_bdpt_params* prm, void* stream, lmgpu_render_stats* stats) {
    return guarded([&] {
        if (!s || !f || !prm) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        if (s->dev.feat & kFeatTexture)
            throw Error(LMGPU_ERR_UNSUPPORTED, "image textures are supported by renderer::pt and renderer::raycast");
        if (!s->dev.has_camera) throw Error(LMGPU_ERR_UNSUPPORTED, "Missing camera primitive.");
        if (s->dev.num_lights == 0) throw Error(LMGPU_ERR_UNSUPPORTED, "No light in the scene.");
        if (prm->num_samples <= 0 || prm->first_path < 0 || prm->max_verts < 2 || prm->min_verts < 0)
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "num_samples must be > 0, first_path >= 0, max_verts >= 2 and min_verts >= 0");
        if (prm->max_verts > kBdMaxVerts) throw Error(LMGPU_ERR_UNSUPPORTED, "max_verts above 64");
        if (prm->strategy < LMGPU_BDPT_ALL || prm->strategy > LMGPU_BDPT_OPT) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "unknown strategy");
        if (prm->first_path + prm->num_samples > (int64_t(1) << 32)) throw Error(LMGPU_ERR_UNSUPPORTED, "sample index above 2^32");
        if (prm->accumulate && f->split) throw Error(LMGPU_ERR_UNSUPPORTED, "film holds split passes");
        ensure_film(f);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const int64_t npix = int64_t(f->w) * f->h;
        const int64_t total = prm->num_samples;
        const int mv = prm->max_verts;
        const int64_t pairs = int64_t(mv) * (mv - 1) / 2;  // strategies with s, t >= 1 and s + t <= max_verts
        // default: 2^22 samples (about 21 GB of records and queues at max_verts 11; per bounce the
        // extend launch then stays full: 2^20 measured 20.3 ms per 2^22-sample frame, 2^21 17.5 ms,
        // 2^22 16.3 ms), fewer for long paths so the connection queue stays within 2^28 rays
        const int64_t wave = std::min(prm->wave_paths > 0 ? prm->wave_paths : std::min<int64_t>(int64_t(1) << 22, (int64_t(1) << 28) / pairs),
                                      total);
        const int64_t scap = wave * pairs;
        if (scap > (int64_t(1) << 31) - 1) throw Error(LMGPU_ERR_UNSUPPORTED, "wave_paths too large for max_verts");
        Workspace& ws = workspace(current_device().device);
        std::lock_guard<std::mutex> ws_lock(ws.m);
        ensure_queues(ws, 2 * wave);
        ws.bd_rec.alloc(size_t(2) * mv * size_t(wave) * kBdRecWords * 16);
        ws.bd_nv.alloc(size_t(2) * size_t(wave) * 4);
        ws.bd_s_o.alloc(size_t(scap) * 16);
        ws.bd_s_d.alloc(size_t(scap) * 16);
        ws.bd_s_c.alloc(size_t(scap) * 16);
        const int64_t icap = wave * (int64_t(mv) * (mv + 1) / 2);  // strategies with t >= 1, s + t <= max_verts
        ws.bd_items.alloc(size_t(icap) * 8);
        const int nbuckets = (mv + 1) * (mv + 1);
        const bool sort_items = nbuckets <= kBdSortBuckets;
        if (sort_items) {
            ws.bd_items_sorted.alloc(size_t(icap) * 8);
            ws.bd_hist.alloc(size_t(kBdSortBuckets) * 4);
        }

        PtConst P{};
        P.seed = prm->seed;
        P.max_verts = mv;
        P.spp = 1;
        P.w = f->w;
        P.h = f->h;
        // subpath lengths of the mode (the reference samples a 1-vertex-limited subpath up to its
        // first hit; that hit is never connected, so it is not traced here)
        const int max_e = prm->strategy == LMGPU_BDPT_LT_NEE ? 1 : mv;
        const int max_l = prm->strategy == LMGPU_BDPT_PT_NAIVE ? 0 : (prm->strategy == LMGPU_BDPT_PT_NEE ? 1 : mv);
        const BdRec R{ws.bd_rec.as<float4>(), ws.bd_nv.as<int32_t>(), wave, mv, max_e, max_l, prm->strategy};
        ExtQ q[2];
        for (int b = 0; b < 2; b++)
            q[b] = ExtQ{ws.q_o[b].as<float4>(), ws.q_d[b].as<float4>(), ws.q_thr[b].as<float4>(), ws.q_nrm[b].as<float4>(),
                        ws.q_ids[b].as<uint2>()};
        ShadowQ sq{ws.bd_s_o.as<float4>(), ws.bd_s_d.as<float4>(), ws.bd_s_c.as<float4>()};
        // [0],[1] extension queues, [2] connection rays, [3] error, [4],[5] ray fetch, [6] strategies
        int* cnt = ws.counters.as<int>();
        const int refill = tuning().trace_refill;
        const Fetch f_ext{cnt + 4, cnt + 5, refill}, f_sh{cnt + 5, cnt + 4, refill};
        unsigned long long* rays = reinterpret_cast<unsigned long long*>(ws.counters.as<char>() + 32);
        float* film = f->sum.as<float>();
        const Bvh8 bvh = s->dev.bvh;
        const size_t tsmem = size_t(2) * 4 * kBlock * size_t(bvh.depth);
        const bool two = s->dev.num_inst > 0;
        auto ext_k = two ? k_pt_extend<false, false, true> : k_pt_extend<false, false, false>;
        auto sh_k = two ? k_pt_shadow<false, false, true> : k_pt_shadow<false, false, false>;
        auto shade_k = tuning().shade_minblocks >= 4 ? bd_shade_for(s->dev.feat)
                                                      : pick_shade(k_bd_shade<2>, k_bd_shade<3>, k_bd_shade<4>, tuning().shade_minblocks);
        const int g_gen = grid_for(k_bd_generate, kBlock, 0);
        const int g_ext = grid_for(ext_k, kBlock, tsmem);
        const int g_sh = grid_for(sh_k, kBlock, tsmem);
        const int g_shade = grid_for(shade_k, kBlock, 0);
        const int g_items = grid_for(k_bd_items, kBlock, 0);
        const int g_sort = grid_for(k_bd_sort_scatter, kBlock, 0);
        // the "shade_minblocks" tuning key: 2 gives connect its full register budget, more gives 3 blocks
        auto con_k = tuning().shade_minblocks <= 2 ? k_bd_connect<2> : bd_connect_for(s->dev.feat);
        const int g_con = grid_for(con_k, kBlock, 0);

        enum { K_GEN = 0, K_EXT = 1, K_SHADE = 2, K_SHADOW = 3 };
        std::vector<std::pair<int, cudaEvent_t>> marks;
        const bool timed = stats != nullptr;
        auto mark = [&](int kind) {
            if (!timed) return;
            cudaEvent_t e;
            LMGPU_CUDA(cudaEventCreate(&e));
            LMGPU_CUDA(cudaEventRecord(e, st));
            marks.emplace_back(kind, e);
        };
        cudaEvent_t e0, e1;
        LMGPU_CUDA(cudaEventCreate(&e0));
        LMGPU_CUDA(cudaEventCreate(&e1));
        int64_t n_ext = 0, n_sh = 0;

        LMGPU_CUDA(cudaEventRecord(e0, st));
        if (!prm->accumulate) {
            LMGPU_CUDA(cudaMemsetAsync(film, 0, size_t(npix) * 3 * 4, st));
            f->accumulated_spp = 0;
            f->split = false;
            f->passes_even = f->passes_odd = 0;
        }
        LMGPU_CUDA(cudaMemsetAsync(ws.counters.p, 0, 192, st));
        for (int64_t start = 0; start < total; start += wave) {
            const int64_t n = std::min(wave, total - start);
            int cur = 0;
            LMGPU_CUDA(cudaMemsetAsync(cnt, 0, 12, st));
            LMGPU_CUDA(cudaMemsetAsync(cnt + 4, 0, 8, st));
            mark(K_GEN);
            k_bd_generate<<<int(std::min<int64_t>(g_gen, (n + kBlock - 1) / kBlock)), kBlock, 0, st>>>(
                s->dev, P, R, prm->first_path + start, n, q[0], cnt + 0);
            mark(-1);
            LMGPU_CUDA(cudaGetLastError());
            // the ray that leaves subpath vertex it creates vertex it + 1 (at most max_verts - 1)
            for (int it = 0; it + 1 < mv; it++) {
                // the extend kernel's fetch counter is otherwise reset by the shadow kernel, which
                // runs once per wave here
                LMGPU_CUDA(cudaMemsetAsync(cnt + 4, 0, 4, st));
                mark(K_EXT);
                ext_k<<<g_ext, kBlock, tsmem, st>>>(bvh, q[cur].o, q[cur].d, cnt + cur, ws.hits.as<float4>(), rays, cnt + 3, nullptr,
                                                    0, nullptr, f_ext, nullptr, nullptr);
                mark(-1);
                n_ext++;
                LMGPU_CUDA(cudaMemsetAsync(cnt + (1 - cur), 0, 4, st));
                mark(K_SHADE);
                shade_k<<<g_shade, kBlock, 0, st>>>(s->dev, P, R, q[cur], ws.hits.as<float4>(), cnt + cur, q[1 - cur], cnt + (1 - cur));
                mark(-1);
                LMGPU_CUDA(cudaGetLastError());
                cur = 1 - cur;
            }
            mark(K_SHADE);
            LMGPU_CUDA(cudaMemsetAsync(cnt + 6, 0, 4, st));
            k_bd_items<<<int(std::min<int64_t>(g_items, (n + kBlock - 1) / kBlock)), kBlock, 0, st>>>(
                R, n, prm->min_verts, mv, ws.bd_items.as<uint2>(), cnt + 6, icap, cnt + 3);
            const uint2* items = ws.bd_items.as<uint2>();
            if (sort_items) {
                int* hist = ws.bd_hist.as<int>();
                LMGPU_CUDA(cudaMemsetAsync(hist, 0, size_t(nbuckets) * 4, st));
                k_bd_sort_count<<<g_sort, kBlock, 0, st>>>(items, cnt + 6, mv, nbuckets, hist);
                k_bd_sort_scan<<<1, 32, 0, st>>>(hist, nbuckets);
                k_bd_sort_scatter<<<g_sort, kBlock, 0, st>>>(items, cnt + 6, mv, nbuckets, hist, ws.bd_items_sorted.as<uint2>());
                items = ws.bd_items_sorted.as<uint2>();
            }
            con_k<<<g_con, kBlock, 0, st>>>(s->dev, P, R, items, cnt + 6, sq, cnt + 2, scap, film, cnt + 3);
            mark(-1);
            mark(K_SHADOW);
            sh_k<<<g_sh, kBlock, tsmem, st>>>(bvh, sq, cnt + 2, film, rays + 1, cnt + 3, nullptr, 0, nullptr, f_sh, nullptr, nullptr);
            mark(-1);
            n_sh++;
            LMGPU_CUDA(cudaGetLastError());
            LMGPU_CUDA(cudaMemsetAsync(cnt + 2, 0, 4, st));
        }
        f->accumulated_spp += total;
        const double scale = double(npix) / double(f->accumulated_spp);  // renderer_bdpt.cpp:397-399
        f->scale = scale;
        k_scale<<<1024, 256, 0, st>>>(film, f->out.as<float>(), npix * 3, float(scale));
        LMGPU_CUDA(cudaGetLastError());
        LMGPU_CUDA(cudaEventRecord(e1, st));
        unsigned long long hr[2];
        int herr = 0;
        LMGPU_CUDA(cudaMemcpyAsync(hr, rays, sizeof(hr), cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaMemcpyAsync(&herr, cnt + 3, 4, cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaStreamSynchronize(st));
        float ms = 0.f;
        LMGPU_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        double kms[4] = {0, 0, 0, 0};
        for (size_t i = 0; i + 1 < marks.size(); i++) {
            if (marks[i].first < 0) continue;
            float m = 0.f;
            LMGPU_CUDA(cudaEventElapsedTime(&m, marks[i].second, marks[i + 1].second));
            kms[marks[i].first] += m;
        }
        for (auto& e : marks) cudaEventDestroy(e.second);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (herr & 6) throw Error(LMGPU_ERR_INTERNAL, "connection or strategy queue overflow");
        if (herr) throw Error(LMGPU_ERR_INTERNAL, "traversal consistency check failed");
        if (stats) {
            *stats = lmgpu_render_stats{};
            stats->paths = total;
            stats->extension_rays = int64_t(hr[0]);
            stats->shadow_rays = int64_t(hr[1]);
            stats->rays = int64_t(hr[0] + hr[1]);
            stats->elapsed_ms = ms;
            stats->generate_ms = kms[K_GEN];
            stats->extend_ms = kms[K_EXT];
            stats->shade_ms = kms[K_SHADE];
            stats->shadow_ms = kms[K_SHADOW];
            stats->trace_ms = kms[K_EXT] + kms[K_SHADOW];
            stats->extend_launches = n_ext;
            stats->shadow_launches = n_sh;
        }
    });
}

// ---------------------------------------------------------------------------------------------
// renderer::pt without device allocation (lmgpu_render_pt_noalloc): the wavefront queues live in
// one fixed file-scope device array instead of library-allocated buffers.

}  // extern "C"

namespace lmgpu {
namespace {

// Bytes per in-flight path: two extension queues (origin, direction, throughput, normal: 4 x 16 B,
// ids 8 B), hits 16 B, shadow queue 3 x 16 B.
constexpr size_t kNoallocPerPath = 2 * (4 * 16 + 8) + 16 + 3 * 16;
constexpr size_t kNoallocCounters = 256;
constexpr size_t kNoallocBytes = kNoallocCounters + size_t(LMGPU_NOALLOC_MAX_WAVE) * kNoallocPerPath;

// In host code this name is only a stand-in for the symbol; the device address comes from
// cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {nullptr};

void* noalloc_scratch(int device) {
    if (device < 0 || device >= 64) throw Error(LMGPU_ERR_UNSUPPORTED, "device ordinal above 63");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) {
        void* p = nullptr;
        LMGPU_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        if (!p) throw Error(LMGPU_ERR_CUDA, "cudaGetSymbolAddress returned a null scratch address");
        g_noalloc_ptr[device] = p;
    }
    return g_noalloc_ptr[device];
}

}  // namespace
}  // namespace lmgpu

extern "C" {

int lmgpu_render_pt_noalloc(lmgpu_scene* s, float* d_film, int32_t w, int32_t h, const lmgpu_pt_params* prm, void* stream) {
    return guarded([&] {
        if (!s || !d_film || !prm) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        if (w <= 0 || h <= 0) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "invalid film size");
        if (!s->dev.has_camera) throw Error(LMGPU_ERR_UNSUPPORTED, "Missing camera primitive.");
        if (s->dev.num_lights == 0) throw Error(LMGPU_ERR_UNSUPPORTED, "No light in the scene.");
        if (prm->spp <= 0 || prm->max_verts < 1) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "spp must be > 0 and max_verts >= 1");
        if (prm->max_verts > 255) throw Error(LMGPU_ERR_UNSUPPORTED, "max_verts above 255");
        if (prm->sampling_mode < 0 || prm->sampling_mode > 2 || prm->primary_mode < 0 || prm->primary_mode > 1)
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "unknown sampling mode");
        if (prm->accumulate) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "lmgpu_render_pt_noalloc does not accumulate (accumulate must be 0)");
        if (prm->split_passes) throw Error(LMGPU_ERR_UNSUPPORTED, "lmgpu_render_pt_noalloc does not split passes");
        if (prm->wave_paths < 0 || prm->wave_paths > LMGPU_NOALLOC_MAX_WAVE)
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "wave_paths " + std::to_string(prm->wave_paths) +
                                                        " exceeds LMGPU_NOALLOC_MAX_WAVE (" +
                                                        std::to_string(LMGPU_NOALLOC_MAX_WAVE) + ")");
        int device = 0;
        LMGPU_CUDA(cudaGetDevice(&device));
        char* base = static_cast<char*>(noalloc_scratch(device));
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const int64_t npix = int64_t(w) * h;
        const int64_t total = npix * prm->spp;
        if (total > (int64_t(1) << 32)) throw Error(LMGPU_ERR_UNSUPPORTED, "more than 2^32 paths in one render");
        const int64_t cap = LMGPU_NOALLOC_MAX_WAVE;
        const int64_t wave = std::min(prm->wave_paths > 0 ? prm->wave_paths : cap, total);

        // carve the fixed array: counters, then the per-path queues
        // [0],[1] extension queues, [2] shadow queue, [3] error, [4],[5] extension / shadow ray fetch
        int* cnt = reinterpret_cast<int*>(base);
        const int refill = tuning().trace_refill;
        const Fetch f_ext{cnt + 4, cnt + 5, refill}, f_sh{cnt + 5, cnt + 4, refill};
        unsigned long long* rays = reinterpret_cast<unsigned long long*>(base + 32);
        unsigned long long* sums = reinterpret_cast<unsigned long long*>(base + 64);
        char* p = base + kNoallocCounters;
        auto take = [&](size_t per_path) {
            char* r = p;
            p += per_path * size_t(cap);
            return r;
        };
        ExtQ q[2];
        for (int b = 0; b < 2; b++) {
            q[b].o = reinterpret_cast<float4*>(take(16));
            q[b].d = reinterpret_cast<float4*>(take(16));
            q[b].thr = reinterpret_cast<float4*>(take(16));
            q[b].nrm = reinterpret_cast<float4*>(take(16));
            q[b].ids = reinterpret_cast<uint2*>(take(8));
            q[b].job = nullptr;
        }
        float4* hits = reinterpret_cast<float4*>(take(16));
        ShadowQ sq;
        sq.o = reinterpret_cast<float4*>(take(16));
        sq.d = reinterpret_cast<float4*>(take(16));
        sq.c = reinterpret_cast<float4*>(take(16));
        sq.job = nullptr;
        if (size_t(p - base) > kNoallocBytes) throw Error(LMGPU_ERR_INTERNAL, "scratch layout exceeds the static array");

        PtConst P;
        P.seed = prm->seed;
        P.max_verts = prm->max_verts;
        P.spp = prm->spp;
        P.mode = prm->sampling_mode;
        P.image = prm->primary_mode == LMGPU_PRIMARY_IMAGE;
        P.w = w;
        P.h = h;
        const Bvh8 bvh = s->dev.bvh;
        const size_t tsmem = size_t(2) * 4 * kBlock * size_t(bvh.depth);
        const int g_gen = grid_for(k_pt_generate, kBlock, 0);
        const bool two = s->dev.num_inst > 0;
        auto ext_k = two ? k_pt_extend<false, false, true> : k_pt_extend<false, false, false>;
        auto sh_k = two ? k_pt_shadow<false, false, true> : k_pt_shadow<false, false, false>;
        const int g_ext = grid_for(ext_k, kBlock, tsmem);
        const int g_sh = grid_for(sh_k, kBlock, tsmem);
        auto shade_k = pick_shade(k_pt_shade<2>, k_pt_shade<3>, k_pt_shade<4>, tuning().shade_minblocks);
        const int g_shade = grid_for(shade_k, kBlock, 0);

        LMGPU_CUDA(cudaMemsetAsync(d_film, 0, size_t(npix) * 3 * sizeof(float), st));
        LMGPU_CUDA(cudaMemsetAsync(base, 0, kNoallocCounters, st));
        for (int64_t start = 0; start < total; start += wave) {
            const int64_t n = std::min(wave, total - start);
            int cur = 0;
            LMGPU_CUDA(cudaMemsetAsync(cnt, 0, 12, st));
            LMGPU_CUDA(cudaMemsetAsync(cnt + 4, 0, 8, st));
            k_pt_generate<<<std::min<int64_t>(g_gen, (n + kBlock - 1) / kBlock), kBlock, 0, st>>>(s->dev, P, start, n, q[0],
                                                                                               cnt + 0, sq, cnt + 2);
            if (P.image) {
                sh_k<<<g_sh, kBlock, tsmem, st>>>(bvh, sq, cnt + 2, d_film, rays + 1, cnt + 3, sums, 63, nullptr, f_sh,
                                                  nullptr, nullptr);
                LMGPU_CUDA(cudaMemsetAsync(cnt + 2, 0, 4, st));
            }
            for (int it = 1; it < P.max_verts; it++) {
                ext_k<<<g_ext, kBlock, tsmem, st>>>(bvh, q[cur].o, q[cur].d, cnt + cur, hits, rays, cnt + 3, sums, 63,
                                                    nullptr, f_ext, nullptr, nullptr);
                LMGPU_CUDA(cudaMemsetAsync(cnt + (1 - cur), 0, 4, st));
                LMGPU_CUDA(cudaMemsetAsync(cnt + 2, 0, 4, st));
                shade_k<<<g_shade, kBlock, 0, st>>>(s->dev, P, q[cur], hits, cnt + cur, q[1 - cur], cnt + (1 - cur), sq,
                                                      cnt + 2, d_film);
                sh_k<<<g_sh, kBlock, tsmem, st>>>(bvh, sq, cnt + 2, d_film, rays + 1, cnt + 3, sums, 63, nullptr, f_sh,
                                                  nullptr, nullptr);
                LMGPU_CUDA(cudaGetLastError());
                cur = 1 - cur;
            }
        }
        const double scale = 1.0 / double(prm->spp);  // both primary modes (renderer_pt.cpp:307-312)
        k_scale<<<1024, 256, 0, st>>>(d_film, d_film, npix * 3, float(scale));
        LMGPU_CUDA(cudaGetLastError());
        int herr = 0;
        LMGPU_CUDA(cudaMemcpyAsync(&herr, cnt + 3, sizeof(int), cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaStreamSynchronize(st));
        if (herr) throw Error(LMGPU_ERR_INTERNAL, "traversal consistency check failed");
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Shared wavefront over many jobs (lmgpu_batch_*)

struct lmgpu_batch {
    int64_t cap = 0;
    lmgpu::DevBuf q_o[2], q_d[2], q_thr[2], q_nrm[2], q_ids[2], q_job[2], hits, s_o, s_d, s_c, s_job;
    lmgpu::DevBuf ctl;        // int64: next, total, range[2], remaining, njobs; then int counters, then u64 rays
    lmgpu::DevBuf jobs, pass_done;
    lmgpu::DevBuf job_next, active, alloc;  // planner state: per job, per job, two per job
    size_t jobs_cap = 0, pass_cap = 0, aux_cap = 0;
    size_t jobs_done = 0;                   // job-table entries already on the device
    std::vector<lmgpu::JobDev> host_jobs;
    std::vector<lmgpu_film*> films;
    // per job: samples per pixel submitted (the random-key stride and the most it may run), the
    // current count (lmgpu_batch_job_set_spp), the film's pass count before the job, resolved
    struct JobMeta {
        int32_t spp_budget = 0, spp = 0;
        int64_t film_first = 0;
        bool resolved = false;
    };
    std::vector<JobMeta> meta;
    std::vector<uint32_t> host_pass;      // mirror of pass_done after the last run
    int64_t total = 0;
    uint32_t passes = 0;
    bool table_dirty = false;
    int32_t max_depth = 1;
    // captured chunk of iterations: [0] plain, [1] with event nodes between the kernels
    struct GraphSlot {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        int32_t depth = 0;
        int refill = -1, shade = -1, first_pass = -1, specialize = -1;
        bool two_level = false;
        bool single = false;      // captured for a one-job table
        uint32_t feat = 0;        // that job's scene features (the shade kernel specialised for them)
        lmgpu::Bvh8 bvh{};        // that job's tree and films, passed by value to the trace kernels
        float* film = nullptr;
        float* film_odd = nullptr;
        void clear() {
            if (exec) cudaGraphExecDestroy(exec);
            if (graph) cudaGraphDestroy(graph);
            exec = nullptr;
            graph = nullptr;
        }
    } slot[2];
    int refill = 0, shade_minblocks = 3, first_pass = 1, specialize = 1;
    bool two_level = false;  // some job's scene is instanced
    bool timed = false;      // per-kernel device time (lmgpu_batch_set_timing)
    cudaEvent_t ev[6 * 8] = {};
    double kms[4] = {0, 0, 0, 0};  // extend, shade, shadow, plan + generate
    int64_t chunks_run = 0;
    double elapsed_ms = 0;
    ~lmgpu_batch() {
        slot[0].clear();
        slot[1].clear();
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    }
};

namespace lmgpu {
namespace {

constexpr int kChunkIters = 8;  // even: the queue parity is the same at every chunk boundary

// ctl layout (bytes): 0 next, 8 total, 16 range start, 24 range count, 32 remaining, 40 njobs,
// 48 int counters [0],[1] extension queues, [2] shadow queue, [3] error; 64 u64 rays [2];
// 80 u64 sums [8]; 144 int extension / shadow ray fetch
int64_t* ctl64(lmgpu_batch* b) { return b->ctl.as<int64_t>(); }
int* ctl_cnt(lmgpu_batch* b) { return reinterpret_cast<int*>(b->ctl.as<char>() + 48); }
unsigned long long* ctl_rays(lmgpu_batch* b) { return reinterpret_cast<unsigned long long*>(b->ctl.as<char>() + 64); }
unsigned long long* ctl_sums(lmgpu_batch* b) { return reinterpret_cast<unsigned long long*>(b->ctl.as<char>() + 80); }
int* ctl_fetch(lmgpu_batch* b) { return reinterpret_cast<int*>(b->ctl.as<char>() + 144); }

// Appends v[done, size) to the device copy (all of v after a reallocation); `done` becomes size.
template <typename T>
void grow_upload(DevBuf& buf, size_t& cap, size_t& done, const std::vector<T>& v, cudaStream_t st, bool& realloc) {
    if (v.size() > cap) {
        size_t c = std::max<size_t>(v.size(), 2 * cap);
        if (c < 64) c = 64;
        LMGPU_CUDA(cudaStreamSynchronize(st));
        DevBuf nb;
        nb.alloc(c * sizeof(T));
        std::swap(buf.p, nb.p);
        std::swap(buf.bytes, nb.bytes);
        cap = c;
        realloc = true;
        done = 0;
    }
    if (v.size() > done)
        LMGPU_CUDA(cudaMemcpyAsync(static_cast<T*>(buf.p) + done, v.data() + done, (v.size() - done) * sizeof(T),
                                   cudaMemcpyHostToDevice, st));
    done = v.size();
}

// paths in flight (the queue the next iteration starts from) plus paths not started yet
__global__ void k_wf_left(int64_t* ctl, const int* qcount) { ctl[4] = int64_t(*qcount) + (ctl[1] - ctl[0]); }

__global__ void k_wf_set_total(int64_t* ctl, int64_t total, int64_t njobs) {
    ctl[1] = total;
    ctl[5] = njobs;
}

// The one-job shade kernel specialised for the job scene's features (default register budget).
#ifndef LMGPU_SHADE_SINGLE_MINBLOCKS
#define LMGPU_SHADE_SINGLE_MINBLOCKS 4  // blocks per SM of the specialised kernels (3: 41.0 ms, 5: 39.5 ms, 4: 37.1 ms per frame)
#endif
using WfShadeK = decltype(&k_wf_shade<4, true, kFeatAll>);
WfShadeK wf_shade_single(uint32_t feat) {
    constexpr int mb = LMGPU_SHADE_SINGLE_MINBLOCKS;
    if (feat & (kFeatDelta | kFeatTexture)) return k_wf_shade<mb, true, kFeatAll>;
    switch (feat & 7u) {
    case 0: return k_wf_shade<mb, true, 0u>;
    case 1: return k_wf_shade<mb, true, 1u>;
    case 2: return k_wf_shade<mb, true, 2u>;
    case 3: return k_wf_shade<mb, true, 3u>;
    case 4: return k_wf_shade<mb, true, 4u>;
    case 5: return k_wf_shade<mb, true, 5u>;
    case 6: return k_wf_shade<mb, true, 6u>;
    default: return k_wf_shade<mb, true, 7u>;
    }
}
// feat: the job's features (one job) or the union over the table's jobs. Several jobs: a kernel
// without the textured environment and the mixture when no job has them.
WfShadeK wf_shade_kernel(const lmgpu_batch* b, bool single, uint32_t feat) {
    if (single && b->shade_minblocks >= 4 && b->specialize) return wf_shade_single(feat);
    if (!single && b->shade_minblocks >= 4 && b->specialize && (feat & ~kFeatTwoLevel) == 0u)
        return (feat & kFeatTwoLevel) ? k_wf_shade<4, false, kFeatTwoLevel> : k_wf_shade<4, false, 0u>;
    return single ? pick_shade(k_wf_shade<2, true>, k_wf_shade<3, true>, k_wf_shade<4, true>, b->shade_minblocks)
                  : pick_shade(k_wf_shade<2, false>, k_wf_shade<3, false>, k_wf_shade<4, false>, b->shade_minblocks);
}
uint32_t table_features(const lmgpu_batch* b) {
    uint32_t f = 0u;
    for (const auto& J : b->host_jobs) f |= J.S.feat;
    return f;
}

// Stream-ordered view of one chunk of iterations; captured into a graph.
void enqueue_chunk(lmgpu_batch* b, cudaStream_t st, bool timed) {
    const size_t tsmem = size_t(2) * 4 * kBlock * size_t(b->max_depth);
    Bvh8 bmax{};
    bmax.depth = b->max_depth;
    // one job: the plain trace kernels on its own tree and film (by value: the captured graph is
    // keyed on them), no per-path job ids
    const bool single = b->host_jobs.size() == 1;
    JobDev J0{};
    if (single) J0 = b->host_jobs[0];
    auto ext_k = single ? (b->two_level ? k_pt_extend<false, false, true> : k_pt_extend<false, false, false>)
                        : (b->two_level ? k_pt_extend<false, true, true> : k_pt_extend<false, true, false>);
    auto sh_k = single ? (b->two_level ? k_pt_shadow<false, false, true> : k_pt_shadow<false, false, false>)
                       : (b->two_level ? k_pt_shadow<false, true, true> : k_pt_shadow<false, true, false>);
    const int g_ext = grid_for(ext_k, kBlock, tsmem);
    const int g_sh = grid_for(sh_k, kBlock, tsmem);
    auto shade_k = wf_shade_kernel(b, single, table_features(b));
    const int g_shade = grid_for(shade_k, kBlock, 0);
    const int g_gen = grid_for(k_wf_generate, kBlock, 0);
    Bvh8 tb = bmax;  // stack sized by the deepest tree seen; single job: its own tree
    if (single) {
        tb = J0.S.bvh;
        tb.depth = b->max_depth;
    }
    float* sfilm = single ? J0.film : nullptr;
    int* cnt = ctl_cnt(b);
    const JobDev* jobs = b->jobs.as<JobDev>();
    ExtQ q[2];
    for (int i = 0; i < 2; i++)
        q[i] = ExtQ{b->q_o[i].as<float4>(), b->q_d[i].as<float4>(), b->q_thr[i].as<float4>(), b->q_nrm[i].as<float4>(),
                    b->q_ids[i].as<uint2>(), b->q_job[i].as<uint32_t>()};
    ShadowQ sq{b->s_o.as<float4>(), b->s_d.as<float4>(), b->s_c.as<float4>(), b->s_job.as<uint32_t>()};
    float4* hits = b->hits.as<float4>();
    int* fetch = ctl_fetch(b);
    const Fetch f_ext{fetch, fetch + 1, b->refill}, f_sh{fetch + 1, fetch, b->refill};
    // timed: event record nodes between the kernels, read after each chunk (ev[6*it + k])
    auto mark = [&](int it, int k) {
        if (timed) LMGPU_CUDA(cudaEventRecordWithFlags(b->ev[6 * it + k], st, cudaEventRecordExternal));
    };
    // One bounce iteration: top the queue up with new paths (plan, generate), trace it (extend),
    // shade the hits into the other queue and the shadow queue, trace the shadow rays.
    int cur = 0;
    for (int it = 0; it < kChunkIters; it++) {
        mark(it, 0);
        k_wf_plan<<<1, 32, 0, st>>>(ctl64(b), cnt + cur, b->cap, jobs, b->job_next.as<int64_t>(), b->active.as<ActiveJob>(),
                                    b->alloc.as<AllocEntry>(), b->first_pass);
        k_wf_generate<<<g_gen, kBlock, 0, st>>>(jobs, b->alloc.as<AllocEntry>(), ctl64(b), q[cur], cnt + cur, sq, cnt + 2);
        mark(it, 1);
        ext_k<<<g_ext, kBlock, tsmem, st>>>(tb, q[cur].o, q[cur].d, cnt + cur, hits, ctl_rays(b), cnt + 3, ctl_sums(b), 63,
                                            nullptr, f_ext, single ? nullptr : jobs, single ? nullptr : q[cur].job);
        mark(it, 2);
        LMGPU_CUDA(cudaMemsetAsync(cnt + (1 - cur), 0, sizeof(int), st));
        shade_k<<<g_shade, kBlock, 0, st>>>(jobs, q[cur], hits, cnt + cur, q[1 - cur], cnt + (1 - cur), sq, cnt + 2,
                                            b->pass_done.as<unsigned int>());
        mark(it, 3);
        sh_k<<<g_sh, kBlock, tsmem, st>>>(tb, sq, cnt + 2, sfilm, ctl_rays(b) + 1, cnt + 3, ctl_sums(b), 63, nullptr, f_sh,
                                          single ? nullptr : jobs, single ? J0.film_odd : nullptr);
        mark(it, 4);
        LMGPU_CUDA(cudaMemsetAsync(cnt + 2, 0, sizeof(int), st));
        cur = 1 - cur;
    }
    // exact count of paths in flight or not started, for the host's end-of-chunk check
    k_wf_left<<<1, 1, 0, st>>>(ctl64(b), cnt + cur);
}

// The executable graph for the current tuning, depth and timing; recaptured only when one of
// them changed or a device table moved (realloc).
cudaGraphExec_t ensure_graph(lmgpu_batch* b, bool realloc) {
    b->refill = tuning().trace_refill;
    b->shade_minblocks = tuning().shade_minblocks;
    b->first_pass = tuning().batch_first_pass;
    b->specialize = tuning().shade_specialize;
    if (realloc) {
        b->slot[0].clear();
        b->slot[1].clear();
    }
    auto& g = b->slot[b->timed ? 1 : 0];
    const bool single = b->host_jobs.size() == 1;
    const uint32_t feat = table_features(b);
    const bool same_shape = g.exec && g.depth == b->max_depth && g.refill == b->refill && g.shade == b->shade_minblocks &&
                            g.two_level == b->two_level && g.first_pass == b->first_pass && g.single == single &&
                            g.feat == feat && g.specialize == b->specialize;
    auto same_job = [&] {
        const JobDev& J = b->host_jobs[0];
        return std::memcmp(&g.bvh, &J.S.bvh, sizeof(Bvh8)) == 0 && g.film == J.film && g.film_odd == J.film_odd;
    };
    if (same_shape && (!single || same_job())) return g.exec;
    if (b->timed)
        for (auto& e : b->ev)
            if (!e) LMGPU_CUDA(cudaEventCreate(&e));
    cudaStream_t cs;
    LMGPU_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    // warm-up query of grid sizes outside the capture (occupancy calls are not capturable work)
    const size_t tsmem = size_t(2) * 4 * kBlock * size_t(b->max_depth);
    (void)grid_for(b->two_level ? k_pt_extend<false, true, true> : k_pt_extend<false, true, false>, kBlock, tsmem);
    (void)grid_for(b->two_level ? k_pt_shadow<false, true, true> : k_pt_shadow<false, true, false>, kBlock, tsmem);
    (void)grid_for(b->two_level ? k_pt_extend<false, false, true> : k_pt_extend<false, false, false>, kBlock, tsmem);
    (void)grid_for(b->two_level ? k_pt_shadow<false, false, true> : k_pt_shadow<false, false, false>, kBlock, tsmem);
    (void)grid_for(wf_shade_kernel(b, single, feat), kBlock, 0);
    (void)grid_for(k_wf_generate, kBlock, 0);
    cudaGraph_t ng = nullptr;
    {
        // no other host thread may synchronize the device while the capture is open
        std::unique_lock<std::shared_mutex> capture_lk(capture_mutex());
        cudaError_t began = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (began != cudaSuccess) {
            cudaStreamDestroy(cs);
            LMGPU_CUDA(began);
        }
        try {
            enqueue_chunk(b, cs, b->timed);
        } catch (...) {
            cudaGraph_t gr = nullptr;
            cudaStreamEndCapture(cs, &gr);
            if (gr) cudaGraphDestroy(gr);
            cudaStreamDestroy(cs);
            throw;
        }
        cudaError_t ended = cudaStreamEndCapture(cs, &ng);
        cudaStreamDestroy(cs);
        LMGPU_CUDA(ended);
    }
    // only the job's tree or film changed: the new graph has the same nodes, so update the
    // executable in place
    bool updated = false;
    if (same_shape) {
        cudaGraphExecUpdateResultInfo info;
        updated = cudaGraphExecUpdate(g.exec, ng, &info) == cudaSuccess;
        if (!updated) (void)cudaGetLastError();
    }
    if (updated) {
        if (g.graph) cudaGraphDestroy(g.graph);
        g.graph = ng;
    } else {
        g.clear();
        g.graph = ng;
        LMGPU_CUDA(cudaGraphInstantiate(&g.exec, g.graph, 0));
    }
    g.depth = b->max_depth;
    g.refill = b->refill;
    g.two_level = b->two_level;
    g.first_pass = b->first_pass;
    g.shade = b->shade_minblocks;
    g.specialize = b->specialize;
    g.single = single;
    g.feat = feat;
    if (single) {
        g.bvh = b->host_jobs[0].S.bvh;
        g.film = b->host_jobs[0].film;
        g.film_odd = b->host_jobs[0].film_odd;
    }
    return g.exec;
}

// Adds one timed chunk's kernel times (events of its last launch) to b->kms: [0] extend,
// [1] shade (with the queue-count reset before it), [2] shadow, [3] plan + generate.
void read_chunk_times(lmgpu_batch* b) {
    for (int it = 0; it < kChunkIters; it++) {
        float m[4];
        for (int k = 0; k < 4; k++) LMGPU_CUDA(cudaEventElapsedTime(&m[k], b->ev[6 * it + k], b->ev[6 * it + k + 1]));
        b->kms[3] += m[0];
        b->kms[0] += m[1];
        b->kms[1] += m[2];
        b->kms[2] += m[3];
    }
}

}  // namespace
}  // namespace lmgpu

extern "C" {

int lmgpu_batch_create(lmgpu_batch** out, int64_t queue_paths) {
    return guarded([&] {
        if (!out || queue_paths < 0) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "invalid argument");
        auto b = std::make_unique<lmgpu_batch>();
        b->cap = queue_paths > 0 ? queue_paths : (int64_t(1) << 22);
        if (b->cap > (int64_t(1) << 30)) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "queue_paths above 2^30");
        const size_t c = size_t(b->cap);
        for (int i = 0; i < 2; i++) {
            b->q_o[i].alloc(c * 16); b->q_d[i].alloc(c * 16); b->q_thr[i].alloc(c * 16); b->q_nrm[i].alloc(c * 16);
            b->q_ids[i].alloc(c * 8); b->q_job[i].alloc(c * 4);
        }
        b->hits.alloc(c * 16);
        b->s_o.alloc(2 * c * 16); b->s_d.alloc(2 * c * 16); b->s_c.alloc(2 * c * 16); b->s_job.alloc(2 * c * 4);
        b->ctl.alloc(256);
        LMGPU_CUDA_SYNC(cudaMemset(b->ctl.p, 0, 256));
        *out = b.release();
    });
}

int lmgpu_batch_set_timing(lmgpu_batch* b, int32_t on) {
    return guarded([&] {
        if (!b) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "batch is null");
        b->timed = on != 0;
    });
}

int lmgpu_batch_destroy(lmgpu_batch* b) {
    return guarded([&] { delete b; });
}

int lmgpu_batch_submit(lmgpu_batch* b, lmgpu_scene* s, lmgpu_film* f, const lmgpu_pt_params* prm, int32_t* job_id) {
    return guarded([&] {
        if (!b || !s || !f || !prm) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        if (!s->dev.has_camera) throw Error(LMGPU_ERR_UNSUPPORTED, "Missing camera primitive.");
        if (s->dev.num_lights == 0) throw Error(LMGPU_ERR_UNSUPPORTED, "No light in the scene.");
        if (prm->spp <= 0 || prm->max_verts < 1 || prm->max_verts > 255) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "invalid spp or max_verts");
        if (prm->sampling_mode < 0 || prm->sampling_mode > 2 || prm->primary_mode < 0 || prm->primary_mode > 1)
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "unknown sampling mode");
        const int64_t npix = int64_t(f->w) * f->h;
        if (npix * prm->spp > (int64_t(1) << 32)) throw Error(LMGPU_ERR_UNSUPPORTED, "more than 2^32 paths in one job");
        if (b->host_jobs.size() >= size_t(1) << 30) throw Error(LMGPU_ERR_UNSUPPORTED, "too many jobs");
        if (prm->split_passes && prm->instrument) throw Error(LMGPU_ERR_UNSUPPORTED, "split_passes with instrument");
        ensure_film(f);
        if (!prm->accumulate) {
            LMGPU_CUDA_SYNC(cudaMemset(f->sum.p, 0, size_t(npix) * 3 * 4));
            f->accumulated_spp = 0;
            f->split = prm->split_passes != 0;
            f->passes_even = f->passes_odd = 0;
        } else if (prm->split_passes && !f->split && f->accumulated_spp > 0) {
            throw Error(LMGPU_ERR_UNSUPPORTED, "split_passes on a film that already holds unsplit passes");
        } else if (prm->split_passes) {
            f->split = true;
        }
        if (f->split) {
            if (!f->sum_odd.p || f->accumulated_spp == 0) {
                f->sum_odd.alloc(size_t(npix) * 3 * 4);
                LMGPU_CUDA_SYNC(cudaMemset(f->sum_odd.p, 0, size_t(npix) * 3 * 4));
            }
        }
        lmgpu_batch::JobMeta M;
        M.spp_budget = M.spp = prm->spp;
        M.film_first = f->passes_even + f->passes_odd;
        JobDev J{};
        J.S = s->dev;
        J.P.seed = prm->seed;
        J.P.max_verts = prm->max_verts;
        J.P.spp = prm->spp;
        J.P.mode = prm->sampling_mode;
        J.P.image = prm->primary_mode == LMGPU_PRIMARY_IMAGE;
        J.P.w = f->w;
        J.P.h = f->h;
        J.film = f->sum.as<float>();
        J.film_odd = f->split ? f->sum_odd.as<float>() : nullptr;
        if (f->split) {
            // the film's global pass index decides the accumulator: even -> sum, odd -> sum_odd
            const int64_t first = f->passes_even + f->passes_odd;
            J.parity0 = uint32_t(first & 1);
            f->passes_odd += (prm->spp + (first & 1)) / 2;
            f->passes_even += prm->spp - (prm->spp + (first & 1)) / 2;
        }
        J.path_begin = b->total;
        J.npix = npix;
        J.limit = npix * prm->spp;
        J.pass_off = b->passes;
        b->host_jobs.push_back(J);
        b->films.push_back(f);
        b->meta.push_back(M);
        b->total += npix * prm->spp;
        b->passes += uint32_t(prm->spp);
        b->host_pass.resize(b->passes, 0);
        b->max_depth = std::max(b->max_depth, s->dev.bvh.depth);
        b->two_level = b->two_level || s->dev.num_inst > 0;
        b->table_dirty = true;
        if (job_id) *job_id = int32_t(b->host_jobs.size() - 1);
    });
}

int lmgpu_batch_run(lmgpu_batch* b, int32_t max_chunks, void* stream, int64_t* paths_left) {
    return guarded([&] {
        if (!b) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "batch is null");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        bool realloc = false;
        if (b->table_dirty) {
            grow_upload(b->jobs, b->jobs_cap, b->jobs_done, b->host_jobs, st, realloc);
            // planner state follows the job table's capacity; job_next and active keep their
            // device values, new job_next entries start at zero
            if (b->aux_cap < b->jobs_cap) {
                LMGPU_CUDA(cudaStreamSynchronize(st));
                const size_t c = b->jobs_cap;
                DevBuf nn, na, nal;
                nn.alloc(c * sizeof(int64_t));
                na.alloc(c * sizeof(ActiveJob));
                nal.alloc(2 * c * sizeof(AllocEntry));
                LMGPU_CUDA_SYNC(cudaMemset(nn.p, 0, c * sizeof(int64_t)));
                if (b->aux_cap) {
                    LMGPU_CUDA_SYNC(cudaMemcpy(nn.p, b->job_next.p, b->aux_cap * sizeof(int64_t), cudaMemcpyDeviceToDevice));
                    LMGPU_CUDA_SYNC(cudaMemcpy(na.p, b->active.p, b->aux_cap * sizeof(ActiveJob), cudaMemcpyDeviceToDevice));
                }
                std::swap(b->job_next.p, nn.p); std::swap(b->job_next.bytes, nn.bytes);
                std::swap(b->active.p, na.p); std::swap(b->active.bytes, na.bytes);
                std::swap(b->alloc.p, nal.p); std::swap(b->alloc.bytes, nal.bytes);
                b->aux_cap = c;
                realloc = true;
            }
            // new pass counters start at zero; existing ones keep their device values
            if (b->passes > b->pass_cap) {
                LMGPU_CUDA(cudaStreamSynchronize(st));
                size_t c = std::max<size_t>(size_t(b->passes), 2 * b->pass_cap);
                DevBuf nb;
                nb.alloc(c * 4);
                LMGPU_CUDA_SYNC(cudaMemset(nb.p, 0, c * 4));
                if (b->pass_cap) LMGPU_CUDA_SYNC(cudaMemcpy(nb.p, b->pass_done.p, b->pass_cap * 4, cudaMemcpyDeviceToDevice));
                std::swap(b->pass_done.p, nb.p);
                std::swap(b->pass_done.bytes, nb.bytes);
                b->pass_cap = c;
                realloc = true;
            }
            k_wf_set_total<<<1, 1, 0, st>>>(ctl64(b), b->total, int64_t(b->host_jobs.size()));
            LMGPU_CUDA(cudaGetLastError());
            b->table_dirty = false;
        }
        if (b->host_jobs.empty()) {
            if (paths_left) *paths_left = 0;
            return;
        }
        cudaGraphExec_t exec = ensure_graph(b, realloc);
        cudaEvent_t e0, e1;
        LMGPU_CUDA(cudaEventCreate(&e0));
        LMGPU_CUDA(cudaEventCreate(&e1));
        LMGPU_CUDA(cudaEventRecord(e0, st));
        int64_t left = 0;
        int chunks = 0;
        int herr = 0;
        for (;;) {
            LMGPU_CUDA(cudaGraphLaunch(exec, st));
            chunks++;
            LMGPU_CUDA(cudaMemcpyAsync(&left, ctl64(b) + 4, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
            LMGPU_CUDA(cudaMemcpyAsync(&herr, ctl_cnt(b) + 3, sizeof(int), cudaMemcpyDeviceToHost, st));
            LMGPU_CUDA(cudaStreamSynchronize(st));
            if (b->timed) read_chunk_times(b);
            if (herr) throw Error(LMGPU_ERR_INTERNAL, "traversal consistency check failed");
            if (left == 0 || (max_chunks > 0 && chunks >= max_chunks)) break;
        }
        b->chunks_run += chunks;
        LMGPU_CUDA(cudaEventRecord(e1, st));
        LMGPU_CUDA(cudaMemcpyAsync(b->host_pass.data(), b->pass_done.p, size_t(b->passes) * 4, cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaStreamSynchronize(st));
        float ms = 0.f;
        LMGPU_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        b->elapsed_ms += ms;
        if (paths_left) *paths_left = left;
    });
}

int lmgpu_batch_job_status(const lmgpu_batch* b, int32_t job, int32_t* passes_complete, int32_t* done) {
    return guarded([&] {
        if (!b || job < 0 || size_t(job) >= b->host_jobs.size()) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "unknown job");
        const JobDev& J = b->host_jobs[job];
        const int32_t spp = b->meta[job].spp;
        int32_t k = 0;
        while (k < spp && int64_t(b->host_pass[J.pass_off + k]) >= J.npix) k++;
        if (passes_complete) *passes_complete = k;
        if (done) {
            int32_t all = 1;
            for (int64_t s = 0; s < spp; s++)
                if (int64_t(b->host_pass[J.pass_off + s]) < J.npix) { all = 0; break; }
            *done = all;
        }
    });
}

int lmgpu_batch_job_set_spp(lmgpu_batch* b, int32_t job, int32_t spp, int32_t* spp_out) {
    return guarded([&] {
        if (!b || job < 0 || size_t(job) >= b->host_jobs.size()) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "unknown job");
        JobDev& J = b->host_jobs[job];
        auto& M = b->meta[job];
        lmgpu_film* f = b->films[job];
        if (M.resolved) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "job already resolved");
        if (spp < 1 || spp > M.spp_budget)
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "spp must be in [1, the spp the job was submitted with]");
        if (f->split && f->passes_even + f->passes_odd != M.film_first + M.spp)
            throw Error(LMGPU_ERR_UNSUPPORTED, "a later job accumulates into this job's film");
        const bool on_device = size_t(job) < b->jobs_done;
        int64_t next = 0;
        int64_t ctl[32];
        if (on_device) {
            LMGPU_CUDA_SYNC(cudaMemcpy(ctl, b->ctl.p, sizeof(ctl), cudaMemcpyDeviceToHost));
            LMGPU_CUDA_SYNC(cudaMemcpy(&next, b->job_next.as<int64_t>() + job, sizeof(next), cudaMemcpyDeviceToHost));
        }
        // passes with a started path stay: they complete as they are
        const int32_t started = int32_t((next + J.npix - 1) / J.npix);
        const int32_t nspp = std::max(spp, started);
        if (spp_out) *spp_out = nspp;
        if (nspp == M.spp) return;
        const int64_t delta = int64_t(nspp - M.spp) * J.npix;
        J.limit = int64_t(nspp) * J.npix;
        b->total += delta;
        if (f->split) {
            const int64_t p0 = int64_t(J.parity0);
            f->passes_odd += (nspp + p0) / 2 - (M.spp + p0) / 2;
            f->passes_even += (nspp - (nspp + p0) / 2) - (M.spp - (M.spp + p0) / 2);
        }
        M.spp = nspp;
        if (!on_device) return;  // the next run uploads the job and the total
        char* jobs_dev = static_cast<char*>(b->jobs.p) + size_t(job) * sizeof(JobDev);
        LMGPU_CUDA_SYNC(cudaMemcpy(jobs_dev + offsetof(JobDev, limit), &J.limit, sizeof(int64_t), cudaMemcpyHostToDevice));
        ctl[1] += delta;
        // a job the planner has seen and dropped from its list of jobs with paths left (every path
        // of its old count started) rejoins that list, once
        if (delta > 0 && job < ctl[20]) {
            std::vector<ActiveJob> act(static_cast<size_t>(ctl[21]));
            if (!act.empty())
                LMGPU_CUDA_SYNC(cudaMemcpy(act.data(), b->active.p, act.size() * sizeof(ActiveJob), cudaMemcpyDeviceToHost));
            const bool listed = std::any_of(act.begin(), act.end(), [&](const ActiveJob& A) { return A.job == job; });
            if (!listed) {
                const ActiveJob A{J.npix, J.limit, job, 0};
                LMGPU_CUDA_SYNC(cudaMemcpy(b->active.as<ActiveJob>() + ctl[21], &A, sizeof(A), cudaMemcpyHostToDevice));
                ctl[21] += 1;
            }
        }
        LMGPU_CUDA_SYNC(cudaMemcpy(b->ctl.p, ctl, sizeof(ctl), cudaMemcpyHostToDevice));
    });
}

int lmgpu_batch_resolve(lmgpu_batch* b, int32_t job, void* stream) {
    return guarded([&] {
        if (!b || job < 0 || size_t(job) >= b->host_jobs.size()) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "unknown job");
        const JobDev& J = b->host_jobs[job];
        lmgpu_film* f = b->films[job];
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        auto& M = b->meta[job];
        if (M.resolved) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "job already resolved");
        M.resolved = true;
        f->accumulated_spp += M.spp;
        // renderer_pt.cpp:307-312: 1 / spp in pixel mode; w*h / (w*h*spp paths) in image mode
        const double scale = 1.0 / double(f->accumulated_spp);
        f->scale = scale;
        if (f->split)
            k_scale2<<<256, 256, 0, st>>>(f->sum.as<float>(), f->sum_odd.as<float>(), f->out.as<float>(), J.npix * 3, float(scale));
        else
            k_scale<<<256, 256, 0, st>>>(f->sum.as<float>(), f->out.as<float>(), J.npix * 3, float(scale));
        LMGPU_CUDA(cudaGetLastError());
        LMGPU_CUDA(cudaStreamSynchronize(st));
    });
}

int lmgpu_batch_get_stats(const lmgpu_batch* b, lmgpu_render_stats* out) {
    return guarded([&] {
        if (!b || !out) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        std::memset(out, 0, sizeof(*out));
        unsigned long long r[2];
        LMGPU_CUDA_SYNC(cudaMemcpy(r, reinterpret_cast<const char*>(b->ctl.p) + 64, sizeof(r), cudaMemcpyDeviceToHost));
        out->paths = b->total;
        out->extension_rays = int64_t(r[0]);
        out->shadow_rays = int64_t(r[1]);
        out->rays = int64_t(r[0] + r[1]);
        out->elapsed_ms = b->elapsed_ms;
        out->extend_ms = b->kms[0];
        out->shade_ms = b->kms[1];
        out->shadow_ms = b->kms[2];
        out->generate_ms = b->kms[3];
        out->trace_ms = b->kms[0] + b->kms[2];
        out->extend_launches = b->chunks_run * kChunkIters;
        out->shadow_launches = b->chunks_run * kChunkIters;
    });
}

int lmgpu_batch_reset(lmgpu_batch* b) {
    return guarded([&] {
        if (!b) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "batch is null");
        LMGPU_CUDA_SYNC(cudaDeviceSynchronize());
        b->host_jobs.clear();
        b->films.clear();
        b->meta.clear();
        b->host_pass.clear();
        b->jobs_done = 0;
        b->total = 0;
        b->passes = 0;
        // the captured graphs stay valid: their stack depth and two-level traversal cover any
        // shallower or single-level scene, so max_depth and two_level are kept
        b->elapsed_ms = 0;
        b->chunks_run = 0;
        for (double& k : b->kms) k = 0;
        b->table_dirty = false;
        LMGPU_CUDA_SYNC(cudaMemset(b->ctl.p, 0, 256));
        if (b->pass_cap) LMGPU_CUDA_SYNC(cudaMemset(b->pass_done.p, 0, b->pass_cap * 4));
        if (b->aux_cap) LMGPU_CUDA_SYNC(cudaMemset(b->job_next.p, 0, b->aux_cap * sizeof(int64_t)));
    });
}

}  // extern "C"

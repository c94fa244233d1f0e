// Oracle (test infrastructure only): CPU restatement of Lightmetrica v3's rendering hot path.
//
// Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker for
// the CUDA path; never shipped, never measured as the product. Parity is not pinned to golden
// vectors from the reference: the reference holds none for this path and cannot be built here
// (glm, nlohmann_json, cereal, stb are absent). It is pinned instead by analytic known-answer
// cases (tests/test_oracle_kat.py) and by following these files line by line:
//   src/accel/accel_sahbvh.cpp            -> Accel (build, intersect)
//   src/scene.cpp, include/lm/scene.h     -> Scene (graph, lights, intersect, visible)
//   include/lm/surface.h, include/lm/path.h -> PointGeometry, path:: functions
//   src/mesh/mesh_raw.cpp                 -> Mesh
//   src/camera/camera_pinhole.cpp         -> Camera
//   src/material/material_{diffuse,glossy,glass,mirror}.cpp -> Material
//   src/light/light_{area,envconst,env,point,directional}.cpp, src/texture/texture_bitmap.cpp -> Light
//   src/renderer/renderer_{raycast,pt}.cpp, src/scheduler.cpp, src/parallel/parallel_openmp.cpp
//   src/film/film_bitmap.cpp, include/lm/film.h -> Film
// Templated on Float: double is the faithful mode (the reference's Float), float is the fp32
// parity mode that the GPU is compared with bit-exactly.
#pragma once
#include "lmo_math.hpp"
#include "lmo_philox.hpp"
#include <atomic>
#include <condition_variable>
#include <functional>
#include <memory>
#include <mutex>
#include <numeric>
#include <optional>
#include <queue>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <omp.h>

namespace lmo {

// ------------------------------------------------------------------------------------------------
// include/lm/surface.h:52-196 (PointGeometry)
template <typename F> struct PointGeometry {
    bool degenerated = false;
    bool infinite = false;
    V3<F> p, n, gn, wo;
    V2<F> t;
    V3<F> u, v;
    M3<F> to_world, to_local;

    static PointGeometry make_degenerated(V3<F> p) {
        PointGeometry g; g.degenerated = true; g.infinite = false; g.p = p; return g;
    }
    static PointGeometry make_infinite(V3<F> wo) {
        PointGeometry g; g.degenerated = false; g.infinite = true; g.wo = wo; return g;
    }
    static PointGeometry make_on_surface(V3<F> p, V3<F> n, V3<F> gn, V2<F> t) {
        PointGeometry g;
        g.degenerated = false; g.infinite = false;
        g.p = p; g.n = n; g.gn = gn; g.t = t;
        orthonormal_basis(n, g.u, g.v);
        g.to_world = M3<F>(g.u, g.v, g.n);
        g.to_local = transpose(g.to_world);
        return g;
    }
    static PointGeometry make_on_surface(V3<F> p, V3<F> gn) { return make_on_surface(p, gn, gn, {}); }
    bool opposite(V3<F> w1, V3<F> w2) const { return dot(w1, n) * dot(w2, n) <= F(0); }
    void basis_twosided(V3<F> wi, V3<F>& on, V3<F>& ou, V3<F>& ov) const {
        const bool i = dot(wi, n) > F(0);
        on = i ? n : -n; ou = u; ov = i ? v : -v;
    }
};

// include/lm/surface.h:211-297
enum SIType { SI_None = 0, SI_Camera = 1, SI_Light = 2, SI_Surface = 4 };
template <typename F> struct SceneInteraction {
    int type = SI_None;
    int primitive = -1;
    PointGeometry<F> geom;
    bool is_type(int f) const { return (type & f) > 0; }
    SceneInteraction as_type(int t) const { auto s = *this; s.type = t; return s; }
};

enum class TransDir { LE, EL };

// include/lm/surface.h:329-363
template <typename F> F geometry_term(const PointGeometry<F>& s1, const PointGeometry<F>& s2) {
    if (s1.infinite && s2.infinite) return F(0);
    V3<F> d; F L2;
    if (s1.infinite || s2.infinite) {
        d = s1.infinite ? s1.wo : -s2.wo;
        L2 = F(1);
    } else {
        d = s2.p - s1.p;
        L2 = dot(d, d);
        d = d / std::sqrt(L2);
    }
    const auto cos1 = s1.degenerated || s1.infinite ? F(1) : std::abs(dot(s1.n, d));
    const auto cos2 = s2.degenerated || s2.infinite ? F(1) : std::abs(dot(s2.n, -d));
    return cos1 * cos2 / L2;
}
// include/lm/surface.h:377-390
template <typename F> F convert_pdf_SA_to_projSA(F pdf_SA, const PointGeometry<F>& g, V3<F> d) {
    if (g.degenerated) return pdf_SA;
    const auto J = std::abs(dot(g.n, d));
    if (J == F(0)) return F(0);
    return pdf_SA / J;
}
// include/lm/surface.h:424-438
template <typename F> F shading_normal_correction(const PointGeometry<F>& g, V3<F> wi, V3<F> wo, TransDir td) {
    const auto local_wi = g.to_local * wi;
    const auto local_wo = g.to_local * wo;
    const auto wi_dot_ng = dot(wi, g.gn);
    const auto wo_dot_ng = dot(wo, g.gn);
    const auto wi_dot_ns = local_wi.z;
    const auto wo_dot_ns = local_wo.z;
    if (wi_dot_ng * wi_dot_ns <= F(0) || wo_dot_ng * wo_dot_ns <= F(0)) return F(0);
    if (td == TransDir::LE) return wi_dot_ns * wo_dot_ng / (wo_dot_ns * wi_dot_ng);
    return F(1);
}

// ------------------------------------------------------------------------------------------------
// src/mesh/mesh_raw.cpp:37-104
template <typename F> struct Mesh {
    struct FI { int p, t, n; };
    std::vector<V3<F>> ps, ns;
    std::vector<V2<F>> ts;
    std::vector<FI> fs;
    struct Point { V3<F> p, n; V2<F> t; };
    struct Tri { Point p1, p2, p3; };
    struct InterpolatedPoint { V3<F> p, n, gn; V2<F> t; };
    int num_triangles() const { return int(fs.size()) / 3; }
    // A face whose first corner has no normal index (n < 0) takes the geometric normal as its
    // shading normal, as an OBJ model's mesh does (model_wavefrontobj.cpp:285-321).
    V3<F> normal_at(int n) const { return n < 0 ? V3<F>() : ns[n]; }
    Tri triangle_at(int face) const {
        const auto f1 = fs[3 * face], f2 = fs[3 * face + 1], f3 = fs[3 * face + 2];
        return {{ps[f1.p], normal_at(f1.n), ts[f1.t]}, {ps[f2.p], normal_at(f2.n), ts[f2.t]},
                {ps[f3.p], normal_at(f3.n), ts[f3.t]}};
    }
    InterpolatedPoint surface_point(int face, V2<F> uv) const {
        const auto i1 = fs[3 * face], i2 = fs[3 * face + 1], i3 = fs[3 * face + 2];
        const auto gn = geometry_normal(ps[i1.p], ps[i2.p], ps[i3.p]);
        return {mix_barycentric(ps[i1.p], ps[i2.p], ps[i3.p], uv),
                i1.n < 0 ? gn : normalize(mix_barycentric(ns[i1.n], ns[i2.n], ns[i3.n], uv)),
                gn,
                mix_barycentric2(ts[i1.t], ts[i2.t], ts[i3.t], uv)};
    }
};

// ------------------------------------------------------------------------------------------------
// src/camera/camera_pinhole.cpp:48-238
template <typename F> struct Camera {
    V3<F> position, center, up, u, v, w;
    F vfov = 0, tf = 0, aspect = 1;
    void construct(V3<F> pos, V3<F> ctr, V3<F> up_, F vfov_, F aspect_) {
        position = pos; center = ctr; up = up_;
        w = normalize(position - center);
        u = normalize(cross(up, w));
        v = cross(w, u);
        vfov = vfov_;
        tf = std::tan(vfov * C<F>::Pi / F(180) * F(.5));
        aspect = aspect_;
    }
    F J(V3<F> wo) const {
        const auto V = transpose(M3<F>(u, v, w));
        const auto wo_eye = V * wo;
        const F cos_theta = -wo_eye.z;
        const F inv_cos_theta = F(1) / cos_theta;
        const F A = tf * tf * aspect * F(4);
        return inv_cos_theta * inv_cos_theta * inv_cos_theta / A;
    }
    Ray<F> primary_ray(V2<F> rp) const {
        rp = V2<F>(F(2) * rp.x - F(1), F(2) * rp.y - F(1));
        const auto d = normalize(V3<F>(aspect * tf * rp.x, tf * rp.y, F(-1)));
        return {position, u * d.x + v * d.y + w * d.z};
    }
    std::optional<V2<F>> raster_position(V3<F> wo) const {
        const auto to_eye = transpose(M3<F>(u, v, w));
        const auto wo_eye = to_eye * wo;
        if (wo_eye.z >= 0) return {};
        const auto rp = V2<F>(-wo_eye.x / wo_eye.z / tf / aspect, -wo_eye.y / wo_eye.z / tf) * F(.5);
        const auto rq = V2<F>(rp.x + F(.5), rp.y + F(.5));
        if (rq.x < F(0) || rq.x > F(1) || rq.y < F(0) || rq.y > F(1)) return {};
        return rq;
    }
    F pdf_direction(V3<F> wo) const {
        if (!raster_position(wo)) return F(0);
        return J(wo);
    }
    V3<F> eval(V3<F> wo) const {
        if (!raster_position(wo)) return V3<F>(F(0));
        return V3<F>(J(wo));
    }
    // camera_pinhole.cpp:178-203: the connection from a scene point to the camera: the camera
    // point, wo from it toward the scene point, weight J(wo) / (1 / G)
    struct DirectSample { PointGeometry<F> geom; V3<F> wo; V3<F> weight; };
    F pdf_direct(const PointGeometry<F>& g, const PointGeometry<F>& gE) const {
        if (g.infinite) return F(0);
        const F G = geometry_term(g, gE);
        return G == F(0) ? F(0) : F(1) / G;
    }
    std::optional<DirectSample> sample_direct(const PointGeometry<F>& g) const {
        if (g.infinite) return {};
        const auto gE = PointGeometry<F>::make_degenerated(position);
        const auto wo = normalize(g.p - position);
        const auto We = V3<F>(J(wo));
        const auto p = pdf_direct(g, gE);
        if (p == F(0)) return {};
        return DirectSample{gE, wo, We / p};
    }
};

// ------------------------------------------------------------------------------------------------
// Materials: src/material/material_{diffuse,glossy,glass,mirror}.cpp, and
// material::mixture_wavefrontobj (src/model/model_wavefrontobj.cpp:361-517) without a texture
// alpha mask: diffuse (Kd) + GGX glossy (Ks, ax, ay) summed, one lobe sampled
enum MatType { MAT_DIFFUSE = 0, MAT_GLOSSY = 1, MAT_GLASS = 2, MAT_MIRROR = 3, MAT_MIXTURE = 4 };

// src/texture/texture_bitmap.cpp:68-85: nearest texel of the wrapped texture coordinate, row 0 at
// the bottom (stbi's vertical flip on load); texels stored row-major with c channels (3 or 4).
template <typename F> struct Texture {
    int w = 0, h = 0, c = 3;
    std::vector<float> data;
    int index(V2<F> t) const {
        const auto u = t.x - std::floor(t.x);
        const auto v = t.y - std::floor(t.y);
        const int x = std::clamp(int(u * F(w)), 0, w - 1);
        const int y = std::clamp(int(v * F(h)), 0, h - 1);
        return w * y + x;
    }
    V3<F> eval(V2<F> t) const {
        const int i = index(t);
        return V3<F>(F(data[c * i]), F(data[c * i + 1]), F(data[c * i + 2]));
    }
    F eval_alpha(V2<F> t) const { return F(data[c * index(t) + 3]); }
    bool has_alpha() const { return c == 4; }
};

template <typename F> struct DirectionSample { V3<F> wo; V3<F> weight; };
template <typename F> struct ComponentSample { int comp; F weight; };

template <typename F> struct Material {
    int type = MAT_DIFFUSE;
    V3<F> Kd = V3<F>(F(1)), Ks;
    F ax = 0, ay = 0, Ni = 1;
    // material_diffuse.cpp:36-40 (mapKd has priority over Kd); model_wavefrontobj.cpp:403-410 (the
    // mixture's alpha mask: its mapKd texture when that has an alpha channel)
    std::shared_ptr<const Texture<F>> mapKd, mask;

    V3<F> kd_at(const PointGeometry<F>& g) const { return mapKd ? mapKd->eval(g.t) : Kd; }
    F alpha_at(const PointGeometry<F>& g) const { return mask ? mask->eval_alpha(g.t) : F(1); }

    // material_glossy.cpp:43-59
    F normal_dist(V3<F> wh, V3<F> u, V3<F> v, V3<F> n) const {
        return F(1) / (C<F>::Pi * ax * ay * sq(sq(dot(wh, u) / ax) + sq(dot(wh, v) / ay) + sq(dot(wh, n))));
    }
    F shadowG(V3<F> wi, V3<F> wo, V3<F> u, V3<F> v, V3<F> n) const {
        auto G1 = [&](V3<F> w) {
            const auto c = dot(w, n);
            const auto s = std::max(C<F>::Eps, safe_sqrt(F(1) - c * c));
            const auto cp = dot(w, u) / s;
            const auto cs = dot(w, v) / s;
            const auto a2 = sq(cp * ax) + sq(cs * ay);
            return c == F(0) ? F(0) : F(2) / (F(1) + safe_sqrt(F(1) + a2 * sq(s / c)));
        };
        return G1(wi) * G1(wo);
    }
    // material_glass.cpp:84-98
    F fresnel(V3<F> wi, V3<F> wt, const PointGeometry<F>& g) const {
        const bool in = dot(wi, g.n) > F(0);
        const auto cos = in ? dot(wi, g.n) : dot(wt, g.n);
        const auto r = (F(1) - Ni) / (F(1) + Ni);
        const auto r2 = r * r;
        return r2 + (F(1) - r2) * std::pow(F(1) - cos, F(5));
    }
    void glass_refr(const PointGeometry<F>& g, V3<F> wi, V3<F>& wt, bool& total, F& eta, F& Fr) const {
        const bool in = dot(wi, g.n) > F(0);
        const auto n = in ? g.n : -g.n;
        eta = in ? F(1) / Ni : Ni;
        const auto rr = refraction(wi, n, eta);
        wt = rr.wt; total = rr.total;
        Fr = total ? F(1) : fresnel(wi, wt, g);
    }

    // the mixture's component 1 is the alpha mask's pass-through (model_wavefrontobj.cpp:513-515)
    bool is_specular_component(int comp) const {
        return type == MAT_GLASS || type == MAT_MIRROR || (type == MAT_MIXTURE && comp != 0);
    }

    // material_glass.cpp:143-158 (component sampling on); model_wavefrontobj.cpp:422-425 (alpha);
    // a single component elsewhere
    F pdf_component(int comp, const PointGeometry<F>& g, V3<F> wi) const {
        if (type == MAT_MIXTURE) {
            const F a = alpha_at(g);
            return comp == 0 ? a : F(1) - a;
        }
        if (type != MAT_GLASS) return F(1);
        V3<F> wt; bool total; F eta, Fr;
        glass_refr(g, wi, wt, total, eta, Fr);
        return comp == 0 ? Fr : F(1) - Fr;
    }

    ComponentSample<F> sample_component(V2<F> uc, const PointGeometry<F>& g, V3<F> wi) const {
        if (type == MAT_GLASS) {  // material_glass.cpp:123-143 (component sampling on)
            V3<F> wt; bool total; F eta, Fr;
            glass_refr(g, wi, wt, total, eta, Fr);
            const int comp = uc.x < Fr ? 0 : 1;
            const auto pdf = comp == 0 ? Fr : F(1) - Fr;
            return {comp, F(1) / pdf};
        }
        if (type == MAT_MIXTURE) {  // model_wavefrontobj.cpp:413-420
            const F a = alpha_at(g);
            if (uc.x < a) return {0, F(1) / a};
            return {1, F(1) / (F(1) - a)};
        }
        return {0, F(1)};
    }

    // model_wavefrontobj.cpp:427-435: probability of sampling the diffuse lobe (the diffuse lobe's
    // reflectance is its texel where it has a texture)
    F diffuse_selection_prob(const PointGeometry<F>& g) const {
        const auto kd = kd_at(g);
        const F wd = std::max(kd.x, std::max(kd.y, kd.z)), wg = std::max(Ks.x, std::max(Ks.y, Ks.z));
        if (wd == F(0) && wg == F(0)) return F(1);
        return wd / (wd + wg);
    }
    // material_diffuse.cpp:63-71 / material_glossy.cpp:70-86, direction only
    V3<F> diffuse_dir(V2<F> ud, const PointGeometry<F>& g, V3<F> wi) const {
        V3<F> n, u, v; g.basis_twosided(wi, n, u, v);
        const auto d = sample_cosine_weighted(ud);
        return u * d.x + v * d.y + n * d.z;
    }
    std::optional<V3<F>> glossy_dir(V2<F> ud, const PointGeometry<F>& g, V3<F> wi) const {
        V3<F> n, u, v; g.basis_twosided(wi, n, u, v);
        const auto u1 = ud.x * F(2) * C<F>::Pi;
        const auto u2 = ud.y;
        const auto wh = normalize(safe_sqrt(u2 / (F(1) - u2)) * (ax * std::cos(u1) * u + ay * std::sin(u1) * v) + n);
        const auto wo = reflection(wi, wh);
        if (g.opposite(wi, wo)) return {};
        return wo;
    }
    V3<F> glossy_eval(const PointGeometry<F>& g, V3<F> wi, V3<F> wo) const {
        if (g.opposite(wi, wo)) return V3<F>();
        const auto wh = normalize(wi + wo);
        V3<F> n, u, v; g.basis_twosided(wi, n, u, v);
        const auto one_m = V3<F>(F(1)) - Ks;
        const auto Fr = Ks + one_m * std::pow(F(1) - dot(wo, wh), F(5));
        return Ks * Fr * (normal_dist(wh, u, v, n) * shadowG(wi, wo, u, v, n) / (F(4) * dot(wi, n) * dot(wo, n)));
    }
    F glossy_pdf(const PointGeometry<F>& g, V3<F> wi, V3<F> wo) const {
        if (g.opposite(wi, wo)) return F(0);
        const auto wh = normalize(wi + wo);
        V3<F> n, u, v; g.basis_twosided(wi, n, u, v);
        return normal_dist(wh, u, v, n) * dot(wh, n) / (F(4) * dot(wo, wh) * dot(wo, n));
    }

    std::optional<DirectionSample<F>> sample_direction(V2<F> ud, V2<F> udc, const PointGeometry<F>& g, V3<F> wi, int comp, TransDir td) const {
        switch (type) {
        case MAT_DIFFUSE:  // material_diffuse.cpp:63-71
            return DirectionSample<F>{diffuse_dir(ud, g, wi), kd_at(g)};
        case MAT_GLOSSY: {  // material_glossy.cpp:70-86
            const auto wo = glossy_dir(ud, g, wi);
            if (!wo) return {};
            const auto f = eval(g, wi, *wo, 0, td, false);
            const auto p = pdf_direction(g, wi, *wo, 0, false);
            return DirectionSample<F>{*wo, f / p};
        }
        case MAT_MIXTURE: {  // model_wavefrontobj.cpp:437-471
            if (comp != 0) {
                // the alpha mask's pass-through: the reference returns weight 1 (its f / p, computed
                // beside it, is unused), so the path carries the component weight 1 / (1 - alpha)
                return DirectionSample<F>{-wi, V3<F>(F(1))};
            }
            V3<F> wo;
            if (udc.x < diffuse_selection_prob(g)) {
                wo = diffuse_dir(ud, g, wi);
            } else {
                const auto w = glossy_dir(ud, g, wi);
                if (!w) return {};
                wo = *w;
            }
            const auto f = eval(g, wi, wo, comp, td, false);
            const auto p = pdf_direction(g, wi, wo, comp, false);
            return DirectionSample<F>{wo, f / p};
        }
        case MAT_GLASS: {  // material_glass.cpp:163-188
            if (comp == 0) {
                const auto wo = reflection(wi, g.n);
                const auto f = eval(g, wi, wo, comp, td, false);
                const auto p = pdf_direction(g, wi, wo, comp, false);
                return DirectionSample<F>{wo, f / p};
            } else {
                V3<F> wt; bool total; F eta, Fr;
                glass_refr(g, wi, wt, total, eta, Fr);
                const auto wo = wt;
                const auto f = eval(g, wi, wo, comp, td, false);
                const auto p = pdf_direction(g, wi, wo, comp, false);
                return DirectionSample<F>{wo, f / p};
            }
        }
        case MAT_MIRROR:  // material_mirror.cpp:40-45
            return DirectionSample<F>{reflection(wi, g.n), V3<F>(F(1))};
        }
        return {};
    }

    F pdf_direction(const PointGeometry<F>& g, V3<F> wi, V3<F> wo, int comp, bool eval_delta) const {
        switch (type) {
        case MAT_DIFFUSE: return g.opposite(wi, wo) ? F(0) : F(1) / C<F>::Pi;
        case MAT_GLOSSY: return glossy_pdf(g, wi, wo);
        case MAT_MIXTURE: {  // model_wavefrontobj.cpp:484-494
            if (comp != 0) return eval_delta ? F(0) : F(1);
            const F w = diffuse_selection_prob(g);
            const F pd = g.opposite(wi, wo) ? F(0) : F(1) / C<F>::Pi;
            return w * pd + (F(1) - w) * glossy_pdf(g, wi, wo);
        }
        case MAT_GLASS: return eval_delta ? F(0) : F(1);
        case MAT_MIRROR: return eval_delta ? F(0) : F(1);
        }
        return F(0);
    }

    V3<F> eval(const PointGeometry<F>& g, V3<F> wi, V3<F> wo, int comp, TransDir td, bool eval_delta) const {
        switch (type) {
        case MAT_DIFFUSE:
            if (g.opposite(wi, wo)) return V3<F>();
            return kd_at(g) / C<F>::Pi;
        case MAT_GLOSSY: return glossy_eval(g, wi, wo);
        case MAT_MIXTURE: {  // model_wavefrontobj.cpp:496-507
            const F a = alpha_at(g);
            if (comp != 0) return eval_delta ? V3<F>(F(0)) : V3<F>(F(1) - a);
            const V3<F> fd = g.opposite(wi, wo) ? V3<F>() : kd_at(g) / C<F>::Pi;
            return (fd + glossy_eval(g, wi, wo)) * a;
        }
        case MAT_GLASS: {
            if (eval_delta) return V3<F>(F(0));
            V3<F> wt; bool total; F eta, Fr;
            glass_refr(g, wi, wt, total, eta, Fr);
            if (comp == 0) return V3<F>(Fr);
            const auto refr_corr = td == TransDir::EL ? eta * eta : F(1);
            return V3<F>((F(1) - Fr) * refr_corr);
        }
        case MAT_MIRROR:
            return eval_delta ? V3<F>(F(0)) : V3<F>(F(1));
        }
        return V3<F>();
    }

    std::optional<V3<F>> reflectance(const PointGeometry<F>& g) const {
        switch (type) {
        case MAT_DIFFUSE: return kd_at(g);
        case MAT_GLOSSY: return Ks;
        case MAT_MIXTURE: return kd_at(g);
        default: return V3<F>(F(0));
        }
    }
};

// ------------------------------------------------------------------------------------------------
// Lights: src/light/light_area.cpp, light_envconst.cpp, light_env.cpp, light_point.cpp,
// light_directional.cpp
enum LightType { LIGHT_AREA = 0, LIGHT_ENVCONST = 1, LIGHT_ENV = 2, LIGHT_POINT = 3, LIGHT_DIRECTIONAL = 4 };

template <typename F> struct LightSample { PointGeometry<F> geom; V3<F> wo; V3<F> weight; };

template <typename F> struct Light {
    int type = LIGHT_AREA;
    V3<F> Ke;            // area: Ke; envconst, point, directional: Le
    V3<F> pos;           // point: its world position; directional: its normalized direction
    int mesh = -1;       // area
    Dist<F> dist;        // area: triangle-area CDF
    F invA = 0;          // area
    // env
    int tw = 0, th = 0, tc = 3;
    std::vector<float> texels;
    F rot = 0, scale = 1;
    Dist2<F> dist2;

    bool is_env() const { return type == LIGHT_ENVCONST || type == LIGHT_ENV; }
    bool is_infinite() const { return is_env() || type == LIGHT_DIRECTIONAL; }
    // light_directional.cpp:131-133 (the others: false)
    bool is_specular() const { return type == LIGHT_DIRECTIONAL; }
    bool is_delta() const { return type == LIGHT_POINT || type == LIGHT_DIRECTIONAL; }

    // texture_bitmap.cpp:68-75
    V3<F> tex_eval(V2<F> t) const {
        const auto u = t.x - std::floor(t.x);
        const auto v = t.y - std::floor(t.y);
        const int x = std::clamp(int(u * tw), 0, tw - 1);
        const int y = std::clamp(int(v * th), 0, th - 1);
        const int i = tw * y + x;
        return V3<F>(F(texels[tc * i]), F(texels[tc * i + 1]), F(texels[tc * i + 2]));
    }
    // light_env.cpp:55-72
    void init_env() {
        std::vector<F> ls(size_t(tw) * th);
        for (int i = 0; i < tw * th; i++) {
            const int x = i % tw, y = i / tw;
            const int k = tw * y + x;
            const auto v = V3<F>(F(texels[tc * k]), F(texels[tc * k + 1]), F(texels[tc * k + 2])) * scale;
            ls[i] = comp_max(v) * std::sin(C<F>::Pi * (F(i) / tw + F(.5)) / th);
        }
        dist2.init(ls, tw, th);
    }

    V3<F> eval(const PointGeometry<F>& g, V3<F> wo) const {
        switch (type) {
        case LIGHT_AREA: return dot(wo, g.n) <= F(0) ? V3<F>(F(0)) : Ke;
        case LIGHT_ENVCONST: return Ke;
        case LIGHT_POINT: return Ke;        // light_point.cpp:117-119
        case LIGHT_DIRECTIONAL: return Ke;  // light_directional.cpp:143-145 without eval_delta
        case LIGHT_ENV: {
            const auto d = -g.wo;
            auto at = std::atan2(d.x, d.z);
            at = at < F(0) ? at + F(2) * C<F>::Pi : at;
            const auto t = (at - rot) * F(.5) / C<F>::Pi;
            return tex_eval(V2<F>(t - std::floor(t), std::acos(d.y) / C<F>::Pi)) * scale;
        }
        }
        return V3<F>();
    }

    F pdf_direct(const PointGeometry<F>& g, const PointGeometry<F>& gL, const Transform<F>& tr, V3<F> wo) const {
        switch (type) {
        case LIGHT_AREA: {  // light_area.cpp:163-169
            if (dot(wo, gL.n) <= F(0)) return F(0);
            const auto G = geometry_term(g, gL);
            return G == F(0) ? F(0) : (invA / tr.J) / G;
        }
        case LIGHT_ENVCONST: {  // light_envconst.cpp:109-112
            const auto d = -gL.wo;
            return convert_pdf_SA_to_projSA(pdf_uniform_sphere<F>(), g, d);
        }
        case LIGHT_ENV: {  // light_env.cpp:165-181
            const auto d = -gL.wo;
            auto at = std::atan2(d.x, d.z);
            at = at < F(0) ? at + F(2) * C<F>::Pi : at;
            const auto t = (at - rot) * F(.5) / C<F>::Pi;
            const auto u = t - std::floor(t);
            const auto v = std::acos(d.y) / C<F>::Pi;
            const auto st = safe_sqrt(F(1) - d.y * d.y);
            if (st == F(0)) return F(0);
            const auto pdfSA = dist2.pdf(u, v) / (F(2) * C<F>::Pi * C<F>::Pi * st);
            return convert_pdf_SA_to_projSA(pdfSA, g, d);
        }
        case LIGHT_POINT: {  // light_point.cpp:97-100
            const auto G = geometry_term(g, gL);
            return G == F(0) ? F(0) : F(1) / G;
        }
        case LIGHT_DIRECTIONAL:  // light_directional.cpp:121-124 without eval_delta
            return convert_pdf_SA_to_projSA(F(1), g, -gL.wo);
        }
        return F(0);
    }
};

// ------------------------------------------------------------------------------------------------
// include/lm/scenenode.h
template <typename F> struct SceneNode {
    bool is_primitive = false;
    int index = 0;
    int mesh = -1, material = -1, light = -1, camera = -1;
    std::vector<int> children;
    bool instanced = false;
    std::optional<M4<F>> local;
};

template <typename F> struct Hit {
    F t; V2<F> uv; int flattened_node; int primitive; int face; int global_tri;
};

// ------------------------------------------------------------------------------------------------
// src/accel/accel_sahbvh.cpp:26-300
template <typename F> struct Tri {
    V3<F> p1, e1, e2;
    Bound<F> b;
    V3<F> c;
    int flattened_node = 0, face = 0;
    Tri() {}
    Tri(V3<F> p1_, V3<F> p2, V3<F> p3, int fn, int f) : p1(p1_), flattened_node(fn), face(f) {
        e1 = p2 - p1; e2 = p3 - p1;
        b = merge(b, p1); b = merge(b, p2); b = merge(b, p3);
        c = b.center();
    }
    struct TriHit { F t, u, v; };
    // Moller & Trumbore 1997, as accel_sahbvh.cpp:58-75
    std::optional<TriHit> intersect(const Ray<F>& r, F tl, F th) const {
        const auto p = cross(r.d, e2);
        const auto tv = r.o - p1;
        const auto q = cross(tv, e1);
        const auto d = dot(e1, p);
        const auto ad = std::abs(d);
        const auto s = std::copysign(F(1), d);
        const auto u = dot(tv, p) * s;
        const auto v = dot(r.d, q) * s;
        if (ad < F(1e-8) || u < F(0) || v < F(0) || u + v > ad) return {};
        const auto t = dot(e2, q) / d;
        if (t < tl || th < t) return {};
        return TriHit{t, u / ad, v / ad};
    }
};

// The hit distance the GPU's accel API reports for an accepted fp32 hit: the formula of
// accel_sahbvh.cpp:58-75 (p = d x e2, tv = o - p1, q = tv x e1, t = (e2 . q) / (e1 . p)) evaluated
// in double on the same fp32 ray and triangle (p1, e1, e2), rounded once to float. Which triangle
// is hit is still decided by the fp32 test.
inline float refine_hit_t(const V3<float>& o, const V3<float>& d, const Tri<float>& tr) {
    auto D = [](const V3<float>& v) { return V3<double>(double(v.x), double(v.y), double(v.z)); };
    const auto p = cross(D(d), D(tr.e2));
    const auto tv = D(o) - D(tr.p1);
    const auto q = cross(tv, D(tr.e1));
    return float(dot(D(tr.e2), q) / dot(D(tr.e1), p));
}

template <typename F> struct Accel {
    struct Node { Bound<F> b; bool leaf = false; int s = 0, e = 0, c1 = 0, c2 = 0; };
    struct Flat { Transform<F> tr; int primitive; };
    std::vector<Node> nodes;
    std::vector<Tri<F>> trs;
    std::vector<int> indices;
    std::vector<Flat> flat;
    bool robust = false;  // fp32 parity mode only (see Bound::isect)

    template <typename TraverseFn>
    void build(TraverseFn traverse_tris, int nthreads) {
        trs.clear(); flat.clear();
        traverse_tris(trs, flat);
        const int nt = int(trs.size());
        if (nt == 0) { nodes.clear(); indices.clear(); return; }
        struct Entry { int index, start, end; };
        std::queue<Entry> q;
        q.push({0, 0, nt});
        nodes.assign(size_t(2) * nt - 1, {});
        indices.assign(nt, 0);
        std::iota(indices.begin(), indices.end(), 0);
        std::mutex mu;
        std::condition_variable cv;
        std::atomic<int> pr{0};
        std::atomic<int> nn{1};
        bool done = false;
        auto process = [&]() {
            std::vector<F> l(nt + 1), r(nt + 1);
            while (true) {
                Entry en;
                {
                    std::unique_lock<std::mutex> lk(mu);
                    cv.wait(lk, [&]() { return done || !q.empty(); });
                    if (done) break;
                    en = q.front(); q.pop();
                }
                const int ni = en.index, s = en.start, e = en.end;
                Node& n = nodes[ni];
                for (int i = s; i < e; i++) n.b = merge(n.b, trs[indices[i]].b);
                auto st = [&](int ax) {
                    std::sort(&indices[s], &indices[e - 1] + 1, [&](int i1, int i2) { return trs[i1].c[ax] < trs[i2].c[ax]; });
                };
                auto make_leaf = [&]() {
                    n.leaf = true; n.s = s; n.e = e;
                    pr += e - s;
                    if (pr == nt) {
                        std::unique_lock<std::mutex> lk(mu);
                        done = true;
                        cv.notify_all();
                    }
                };
                if (e - s < 2) { make_leaf(); continue; }
                F b = C<F>::Inf;
                int bi = -1, ba = -1;
                for (int a = 0; a < 3; a++) {
                    st(a);
                    Bound<F> bl, br;
                    for (int i = 0; i <= e - s; i++) {
                        const int j = e - s - i;
                        l[i] = bl.surface_area() * F(i);
                        r[j] = br.surface_area() * F(i);
                        bl = i < e - s ? merge(bl, trs[indices[s + i]].b) : bl;
                        br = j > 0 ? merge(br, trs[indices[s + j - 1]].b) : br;
                    }
                    for (int i = 1; i < e - s; i++) {
                        const auto c = F(1) + (l[i] + r[i]) / n.b.surface_area();
                        if (c < b) { b = c; bi = i; ba = a; }
                    }
                }
                if (b > F(e - s)) { make_leaf(); continue; }
                st(ba);
                const int m = s + bi;
                std::unique_lock<std::mutex> lk(mu);
                q.push({n.c1 = nn++, s, m});
                q.push({n.c2 = nn++, m, e});
                cv.notify_one();
            }
        };
        std::vector<std::thread> ths(std::max(1, nthreads));
        for (auto& th : ths) th = std::thread(process);
        for (auto& th : ths) th.join();
    }

    std::optional<Hit<F>> intersect(const Ray<F>& ray, F tmin, F tmax) const {
        if (nodes.empty()) return {};
        std::optional<typename Tri<F>::TriHit> mh, h;
        int mi = -1;
        int s[99]{};
        int si = 0;
        while (si >= 0) {
            const auto& n = nodes.at(s[si--]);
            if (!n.b.isect(ray, tmin, tmax, robust)) continue;
            if (!n.leaf) {
                s[++si] = n.c1;
                s[++si] = n.c2;
                continue;
            }
            for (int i = n.s; i < n.e; i++) {
                if ((h = trs[indices[i]].intersect(ray, tmin, tmax))) {
                    mh = h; tmax = h->t; mi = i;
                }
            }
        }
        if (!mh) return {};
        const int gi = indices.at(mi);
        const auto& tr = trs.at(gi);
        const auto& fn = flat.at(tr.flattened_node);
        return Hit<F>{tmax, V2<F>(mh->u, mh->v), tr.flattened_node, fn.primitive, tr.face, gi};
    }

    // Exhaustive closest hit (tests only): the smallest t over every triangle the Moller-Trumbore
    // test accepts in [tmin, tmax], ties to the smallest flattened triangle index.
    std::optional<Hit<F>> intersect_brute(const Ray<F>& ray, F tmin, F tmax) const {
        int best = -1; typename Tri<F>::TriHit bh{};
        for (int i = 0; i < int(trs.size()); i++) {
            const auto h = trs[i].intersect(ray, tmin, tmax);
            if (h && (best < 0 || h->t < bh.t)) { best = i; bh = *h; }
        }
        if (best < 0) return {};
        const auto& tr = trs[best];
        return Hit<F>{bh.t, V2<F>(bh.u, bh.v), tr.flattened_node, flat[tr.flattened_node].primitive, tr.face, best};
    }
};

// ------------------------------------------------------------------------------------------------
// src/scene.cpp:20-400 + include/lm/scene.h:343-364
template <typename F> struct Scene {
    using Float = F;
    std::vector<SceneNode<F>> nodes;
    std::vector<Mesh<F>> meshes;
    std::vector<Material<F>> materials;
    std::vector<std::shared_ptr<const Texture<F>>> textures;
    std::vector<Light<F>> lights_assets;
    std::vector<Camera<F>> cameras;
    std::optional<int> camera_;
    struct LightPrimitiveIndex { Transform<F> tr; int index; };
    std::vector<LightPrimitiveIndex> lights_;
    std::unordered_map<int, int> light_indices_map_;
    std::optional<int> env_light_;
    Accel<F> accel;
    bool built = false;
    V3<F> sphere_center;   // the lights' scene bound (SphereBound, math.h:184-195)
    F sphere_radius = 0;

    Scene() { reset(); }
    void reset() {
        nodes.clear(); camera_ = {}; lights_.clear(); light_indices_map_.clear(); env_light_ = {};
        SceneNode<F> root; root.index = 0; nodes.push_back(root);
        built = false;
    }
    int create_primitive_node(int mesh, int material, int light, int camera) {
        if (mesh < 0 && material < 0 && light < 0 && camera < 0) throw std::invalid_argument("Invalid primitive node. Given assets are invalid.");
        if (camera >= 0 && light >= 0) throw std::invalid_argument("Primitive cannot be both camera and light.");
        if ((mesh < 0 && material >= 0) || (mesh >= 0 && material < 0)) throw std::invalid_argument("You must specify both mesh and material.");
        const int index = int(nodes.size());
        if (camera >= 0) camera_ = index;
        if (light >= 0 && lights_assets.at(light).is_env()) {
            if (env_light_) throw std::invalid_argument("Environment light is already registered.");
            env_light_ = index;
        }
        SceneNode<F> n; n.is_primitive = true; n.index = index;
        n.mesh = mesh; n.material = material; n.light = light; n.camera = camera;
        nodes.push_back(n);
        return index;
    }
    int create_group_node(const M4<F>& m) {
        SceneNode<F> n; n.index = int(nodes.size()); n.local = m; nodes.push_back(n); return n.index;
    }
    int create_instance_group_node() {
        SceneNode<F> n; n.index = int(nodes.size()); n.instanced = true; nodes.push_back(n); return n.index;
    }
    void add_child(int parent, int child) {
        if (parent < 0 || parent >= int(nodes.size())) return;
        auto& node = nodes.at(parent);
        if (node.is_primitive) return;
        node.children.push_back(child);
    }
    void traverse_primitive_nodes(const std::function<void(const SceneNode<F>&, const M4<F>&)>& fn) const {
        std::function<void(int, M4<F>)> visit = [&](int index, M4<F> gm) {
            const auto& node = nodes.at(index);
            fn(node, gm);
            if (!node.is_primitive) {
                const auto M = node.local ? gm * *node.local : gm;
                for (int c : node.children) visit(c, M);
            }
        };
        visit(0, M4<F>());
    }
    static V3<F> xform_point(const M4<F>& m, V3<F> p) {
        const auto r = m * V4<F>(p, F(1));
        return {r.x, r.y, r.z};
    }

    void build(int nthreads, bool robust) {
        light_indices_map_.clear();
        lights_.clear();
        traverse_primitive_nodes([&](const SceneNode<F>& node, const M4<F>& gm) {
            if (node.is_primitive && node.light >= 0) {
                light_indices_map_[node.index] = int(lights_.size());
                lights_.push_back({Transform<F>(gm), node.index});
            }
        });
        // scene.cpp:288-311: the bound of every mesh primitive's transformed triangles, handed to
        // the lights as a bounding sphere (light_envconst.cpp:38-43)
        Bound<F> bound;
        traverse_primitive_nodes([&](const SceneNode<F>& node, const M4<F>& gm) {
            if (!node.is_primitive || node.mesh < 0) return;
            const auto& mesh = meshes.at(node.mesh);
            for (int f = 0; f < mesh.num_triangles(); f++) {
                const auto tri = mesh.triangle_at(f);
                bound = merge(bound, xform_point(gm, tri.p1.p));
                bound = merge(bound, xform_point(gm, tri.p2.p));
                bound = merge(bound, xform_point(gm, tri.p3.p));
            }
        });
        sphere_center = (bound.max + bound.min) * F(.5);
        sphere_radius = length(bound.max - sphere_center) * F(1.01);
        accel.robust = robust;
        accel.build([&](std::vector<Tri<F>>& trs, std::vector<typename Accel<F>::Flat>& flat) {
            traverse_primitive_nodes([&](const SceneNode<F>& node, const M4<F>& gm) {
                if (!node.is_primitive || node.mesh < 0) return;
                const int fi = int(flat.size());
                flat.push_back({Transform<F>(gm), node.index});
                const auto& mesh = meshes.at(node.mesh);
                for (int f = 0; f < mesh.num_triangles(); f++) {
                    const auto tri = mesh.triangle_at(f);
                    trs.emplace_back(xform_point(gm, tri.p1.p), xform_point(gm, tri.p2.p), xform_point(gm, tri.p3.p), fi, f);
                }
            });
        }, nthreads);
        built = true;
    }

    SceneInteraction<F> surface_from_hit(const Hit<F>& h) const {
        const auto& prim = nodes.at(h.primitive);
        const auto p = meshes.at(prim.mesh).surface_point(h.face, h.uv);
        const auto& tr = accel.flat.at(h.flattened_node).tr;
        SceneInteraction<F> si;
        si.type = SI_Surface;
        si.primitive = h.primitive;
        si.geom = PointGeometry<F>::make_on_surface(xform_point(tr.M, p.p), normalize(tr.normal_M * p.n), normalize(tr.normal_M * p.gn), p.t);
        return si;
    }

    std::optional<SceneInteraction<F>> intersect(const Ray<F>& ray, F tmin = C<F>::Eps, F tmax = C<F>::Inf) const {
        const auto hit = accel.intersect(ray, tmin, tmax);
        if (!hit) {
            if (tmax < C<F>::Inf) return {};
            if (!env_light_) return {};
            SceneInteraction<F> si;
            si.type = SI_Light; si.primitive = *env_light_;
            si.geom = PointGeometry<F>::make_infinite(-ray.d);
            return si;
        }
        return surface_from_hit(*hit);
    }
    bool visible(const SceneInteraction<F>& a, const SceneInteraction<F>& b) const {
        auto vis = [&](const SceneInteraction<F>& s1, const SceneInteraction<F>& s2) {
            const auto wo = s2.geom.infinite ? -s2.geom.wo : normalize(s2.geom.p - s1.geom.p);
            const auto tmax = s2.geom.infinite ? C<F>::Inf - F(1) : distance(s1.geom.p, s2.geom.p) * (F(1) - C<F>::Eps);
            return !intersect(Ray<F>{s1.geom.p, wo}, C<F>::Eps, tmax);
        };
        return a.geom.infinite ? vis(b, a) : vis(a, b);
    }
    bool is_light(const SceneInteraction<F>& sp) const { return nodes.at(sp.primitive).light >= 0; }
    int num_lights() const { return int(lights_.size()); }
    std::pair<int, F> sample_light_selection(F u) const {
        const int n = int(lights_.size());
        const int i = std::clamp(int(u * n), 0, n - 1);
        return {i, F(1) / n};
    }
    F pdf_light_selection() const { return F(1) / int(lights_.size()); }
    const Camera<F>& camera() const { return cameras.at(nodes.at(*camera_).camera); }
    const Light<F>& light_of(int node) const { return lights_assets.at(nodes.at(node).light); }
    const Material<F>& material_of(int node) const { return materials.at(nodes.at(node).material); }

    // light_area.cpp:48-60 (position sampling on the light's mesh, transformed)
    PointGeometry<F> sample_position_on_triangle_mesh(const Light<F>& L, V2<F> up, F upc, const Transform<F>& tr) const {
        const int i = L.dist.sample(upc);
        const auto s = safe_sqrt(up.x);
        const auto tri = meshes.at(L.mesh).triangle_at(i);
        const auto a = tri.p1.p, b = tri.p2.p, c = tri.p3.p;
        const auto p = mix_barycentric(a, b, c, V2<F>(F(1) - s, up.y * s));
        const auto gn = geometry_normal(a, b, c);
        const auto p_trans = xform_point(tr.M, p);
        const auto gn_trans = normalize(tr.normal_M * gn);
        return PointGeometry<F>::make_on_surface(p_trans, gn_trans);
    }

    // path.h:493-530 sample_direct(LE) with RaySampleU u = {up, upc, ud, udc}
    std::optional<LightSample<F>> sample_direct_light(const double* u8, const SceneInteraction<F>& sp, int& light_node) const {
        const V2<F> up{F(u8[0]), F(u8[1])}, upc{F(u8[2]), F(u8[3])}, ud{F(u8[4]), F(u8[5])};
        const auto [li, p_sel] = sample_light_selection(upc.x);
        const auto& lpi = lights_.at(li);
        light_node = lpi.index;
        const auto& L = light_of(lpi.index);
        const auto& g = sp.geom;
        std::optional<LightSample<F>> s;
        switch (L.type) {
        case LIGHT_AREA: {  // light_area.cpp:148-161
            const auto gL = sample_position_on_triangle_mesh(L, up, upc.y, lpi.tr);
            const auto wo = normalize(g.p - gL.p);
            const auto pL = L.pdf_direct(g, gL, lpi.tr, wo);
            if (pL == F(0)) return {};
            const auto Le = L.eval(gL, wo);
            s = LightSample<F>{gL, wo, Le / pL};
            break;
        }
        case LIGHT_ENVCONST: {  // light_envconst.cpp:94-107
            const auto wo = sample_uniform_sphere(ud);
            const auto gL = PointGeometry<F>::make_infinite(wo);
            const auto Le = L.eval(gL, wo);
            const auto pL = L.pdf_direct(g, gL, lpi.tr, wo);
            if (pL == F(0)) return {};
            s = LightSample<F>{gL, wo, Le / pL};
            break;
        }
        case LIGHT_ENV: {  // light_env.cpp:146-163
            const auto uu = L.dist2.sample(ud.x, ud.y, up.x, up.y);
            const auto t = C<F>::Pi * uu.y;
            const auto st = std::sin(t);
            const auto p = F(2) * C<F>::Pi * uu.x + L.rot;
            const auto wo = -V3<F>(st * std::sin(p), std::cos(t), st * std::cos(p));
            const auto gL = PointGeometry<F>::make_infinite(wo);
            const auto pL = L.pdf_direct(g, gL, lpi.tr, wo);
            if (pL == F(0)) return {};
            const auto Le = L.eval(gL, wo);
            s = LightSample<F>{gL, wo, Le / pL};
            break;
        }
        case LIGHT_POINT: {  // light_point.cpp:84-95
            const auto wo = normalize(g.p - L.pos);
            const auto gL = PointGeometry<F>::make_degenerated(L.pos);
            const auto pL = L.pdf_direct(g, gL, lpi.tr, wo);
            if (pL == F(0)) return {};
            s = LightSample<F>{gL, wo, L.Ke / pL};
            break;
        }
        case LIGHT_DIRECTIONAL: {  // light_directional.cpp:109-119
            const auto gL = PointGeometry<F>::make_infinite(L.pos);
            const auto pL = L.pdf_direct(g, gL, lpi.tr, L.pos);
            if (pL == F(0)) return {};
            s = LightSample<F>{gL, L.pos, L.Ke / pL};
            break;
        }
        }
        if (s) s->weight = s->weight / p_sel;
        return s;
    }
    // path.h:101-118 sample_primary_ray(LE) with u = {up, upc, ud, udc}: a light by upc.x, then its
    // sample_ray (light_area.cpp:78-100, light_envconst.cpp:47-68, light_env.cpp:86-107); the
    // weight is divided by the selection probability. LightSample::wo is the ray direction.
    std::optional<LightSample<F>> sample_primary_ray_light(const double* u8) const {
        const V2<F> up{F(u8[0]), F(u8[1])}, upc{F(u8[2]), F(u8[3])}, ud{F(u8[4]), F(u8[5])};
        const auto [li, p_sel] = sample_light_selection(upc.x);
        const auto& lpi = lights_.at(li);
        const auto& L = light_of(lpi.index);
        LightSample<F> s;
        if (L.type == LIGHT_AREA) {
            const auto gL = sample_position_on_triangle_mesh(L, up, upc.y, lpi.tr);
            const auto pA = L.invA / lpi.tr.J;
            const auto wl = sample_cosine_weighted(ud);
            V3<F> u, v;
            orthonormal_basis(gL.n, u, v);
            const auto wo = u * wl.x + v * wl.y + gL.n * wl.z;
            const auto Le = L.eval(gL, wo);
            const auto p = pA * (F(1) / C<F>::Pi);
            s = LightSample<F>{gL, wo, Le / p};
        } else if (L.type == LIGHT_POINT) {
            // light_point.cpp:39-49: a uniform direction from the light's position
            const auto d = sample_uniform_sphere(ud);
            s = LightSample<F>{PointGeometry<F>::make_degenerated(L.pos), d, L.Ke / pdf_uniform_sphere<F>()};
        } else if (L.type == LIGHT_DIRECTIONAL) {
            // light_directional.cpp:49-70: the light's direction from a point on the disk of the
            // scene's bounding sphere facing it
            const auto d = L.pos;
            const auto pl = sample_uniform_disk(up) * sphere_radius;
            V3<F> u, v;
            orthonormal_basis(d, u, v);
            auto gL = PointGeometry<F>::make_infinite(d);
            gL.p = sphere_center + sphere_radius * (-d) + (u * pl.x + v * pl.y);
            const auto p = F(1) / (C<F>::Pi * sphere_radius * sphere_radius);
            s = LightSample<F>{gL, d, L.eval(gL, d) / p};
        } else {
            // a uniform direction, then a point on the disk of the scene's bounding sphere facing it
            const auto d = sample_uniform_sphere(ud);
            const auto pl = sample_uniform_disk(up) * sphere_radius;
            V3<F> u, v;
            orthonormal_basis(d, u, v);
            auto gL = PointGeometry<F>::make_infinite(d);
            gL.p = sphere_center + sphere_radius * (-d) + (u * pl.x + v * pl.y);
            const auto Le = L.eval(gL, d);
            const auto p = pdf_uniform_sphere<F>() * (F(1) / (C<F>::Pi * sphere_radius * sphere_radius));
            s = LightSample<F>{gL, d, Le / p};
        }
        s.weight = s.weight / p_sel;
        return s;
    }
    // path.h:563-583 pdf_direct for a light endpoint
    F pdf_direct_light(const SceneInteraction<F>& sp, const SceneInteraction<F>& spL, V3<F> wo) const {
        const int li = light_indices_map_.at(spL.primitive);
        const auto& lpi = lights_.at(li);
        return pdf_light_selection() * light_of(spL.primitive).pdf_direct(sp.geom, spL.geom, lpi.tr, wo);
    }
};

// ------------------------------------------------------------------------------------------------
// Random numbers. RngMT restates include/lm/math.h:204-271 (std::mt19937 with
// uniform_real_distribution<double>; the float variant rounds the double toward -inf).
// RngPhilox is the counter-based stream the GPU uses: path-keyed, fixed slots per vertex, so a
// GPU path and an oracle path consume identical numbers.
struct RngMT {
    std::mt19937 eng;
    std::uniform_real_distribution<double> dist;
    bool as_float = false;
    explicit RngMT(unsigned int seed, bool f) : as_float(f) { eng.seed(seed); }
    double u() {
        const double rd = dist(eng);
        if (!as_float) return rd;
        float rf = float(rd);
        if (double(rf) > rd) rf = std::nextafter(rf, -std::numeric_limits<float>::infinity());
        return double(rf);
    }
};

struct PathRng {
    // mode 0: sequential mt19937 (the reference's consumption order); mode 1: philox slots
    int mode = 0;
    RngMT* mt = nullptr;
    uint32_t seed = 0;
    uint64_t path = 0;
    double seq() { return mt->u(); }
    // slot in [0,16) of vertex nv
    double slot(int nv, int s) { return double(philox_uniform(seed, path, uint32_t(nv), uint32_t(s))); }
};

// ------------------------------------------------------------------------------------------------
// src/film/film_bitmap.cpp (splat via CAS, rescale) with double accumulators.
struct Film {
    int w = 0, h = 0;
    struct Px { double r, g, b; };
    std::vector<std::atomic<Px>> data;
    std::vector<std::atomic<Px>> m2;
    bool with_m2 = false;
    Film(int w_, int h_, bool m2_) : w(w_), h(h_), data(size_t(w_) * h_), m2(m2_ ? size_t(w_) * h_ : 0), with_m2(m2_) {
        for (auto& v : data) v.store(Px{0, 0, 0});
        for (auto& v : m2) v.store(Px{0, 0, 0});
    }
    static void add(std::atomic<Px>& a, Px v) {
        Px e = a.load();
        while (!a.compare_exchange_weak(e, Px{e.r + v.r, e.g + v.g, e.b + v.b})) {}
    }
    template <typename F> void raster_to_pixel(V2<F> rp, int& x, int& y) const {
        x = std::clamp(int(rp.x * F(w)), 0, w - 1);
        y = std::clamp(int(rp.y * F(h)), 0, h - 1);
    }
    template <typename F> void splat(V2<F> rp, V3<F> c) {
        int x, y; raster_to_pixel(rp, x, y);
        add(data[size_t(y) * w + x], Px{double(c.x), double(c.y), double(c.z)});
    }
    // a path's total contribution c, squared into the second moment (the per-sample variance)
    template <typename F> void add_m2(V2<F> rp, V3<F> c) {
        if (!with_m2) return;
        int x, y; raster_to_pixel(rp, x, y);
        add(m2[size_t(y) * w + x], Px{double(c.x) * double(c.x), double(c.y) * double(c.y), double(c.z) * double(c.z)});
    }
};

// ------------------------------------------------------------------------------------------------
// src/renderer/renderer_raycast.cpp:62-101
template <typename F>
void render_raycast(const Scene<F>& scene, int w, int h, V3<F> bg, bool use_constant_color, bool visualize_normal,
                    const V3<F>* color, double* out, int nthreads) {
    const auto& cam = scene.camera();
    const long long n = (long long)w * h;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (long long index = 0; index < n; index++) {
        const int x = int(index % w), y = int(index / w);
        const auto ray = cam.primary_ray(V2<F>((F(x) + F(.5)) / F(w), (F(y) + F(.5)) / F(h)));
        const auto sp = scene.intersect(ray);
        V3<F> c;
        if (!sp) c = bg;
        else if (visualize_normal) c = vabs(sp->geom.n);
        else if (sp->geom.infinite) c = scene.light_of(sp->primitive).eval(sp->geom, sp->geom.wo);
        else {
            const auto R = color ? std::optional<V3<F>>(*color) : scene.material_of(sp->primitive).reflectance(sp->geom);
            c = R ? *R : V3<F>();
            if (!use_constant_color) c *= F(.2) + F(.8) * std::abs(dot(sp->geom.n, -ray.d));
        }
        out[3 * index] = double(c.x); out[3 * index + 1] = double(c.y); out[3 * index + 2] = double(c.z);
    }
}

// ------------------------------------------------------------------------------------------------
// src/renderer/renderer_pt.cpp:80-315
struct PTParams {
    int w, h;
    long long spp;
    int max_verts;
    unsigned int seed;
    int sampling_mode;    // 0 naive, 1 nee, 2 mis
    int primary_mode;     // 0 pixel, 1 image
    int rng_mode;         // 0 mt19937 per thread (reference), 1 philox per path
    int with_m2;
};

template <typename F>
void render_pt(const Scene<F>& scene, const PTParams& P, double* out, double* out_m2, long long* rays_out, int nthreads) {
    using V3F = V3<F>;
    if (scene.nodes.size() <= 1) throw std::runtime_error("Missing primitives.");
    if (!scene.camera_) throw std::runtime_error("Missing camera primitive.");
    if (scene.num_lights() == 0) throw std::runtime_error("No light in the scene.");
    Film film(P.w, P.h, P.with_m2 && P.primary_mode == 0);
    const auto& cam = scene.camera();
    const bool pixel_mode = P.primary_mode == 0;
    const long long num_pixels = (long long)P.w * P.h;
    const long long total = num_pixels * P.spp;
    const int nth = std::max(1, nthreads);
    std::vector<RngMT*> rngs(nth, nullptr);
    for (int i = 0; i < nth; i++) rngs[i] = new RngMT(P.seed + i, std::is_same<F, float>::value);
    std::vector<long long> rays(nth, 0);

#pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
    for (long long index = 0; index < total; index++) {
        const int tid = omp_get_thread_num();
        const long long pixel_index = index / P.spp;
        PathRng rng; rng.mode = P.rng_mode; rng.mt = rngs[tid]; rng.seed = P.seed; rng.path = (uint64_t)index;
        auto U = [&](int nv, int s) -> double { return rng.mode == 0 ? rng.seq() : rng.slot(nv, s); };
        // two numbers in stream order (the order of a constructor's arguments is unspecified)
        auto U2 = [&](int nv, int s) { const double a = U(nv, s); const double b = U(nv, s + 1); return V2<F>(F(a), F(b)); };
        long long& nrays = rays[tid];

        F wx, wy, ww, wh;
        if (pixel_mode) {
            const int x = int(pixel_index % P.w), y = int(pixel_index / P.w);
            const F dx = F(1) / F(P.w), dy = F(1) / F(P.h);
            wx = dx * F(x); wy = dy * F(y); ww = dx; wh = dy;
        } else { wx = 0; wy = 0; ww = 1; wh = 1; }

        // sample_position(EL) + sample_component(camera): PositionSampleU (4) + ComponentSampleU (2)
        if (rng.mode == 0) { for (int k = 0; k < 6; k++) rng.seq(); }
        SceneInteraction<F> sp;
        sp.type = SI_Camera; sp.primitive = *scene.camera_;
        sp.geom = PointGeometry<F>::make_degenerated(cam.position);
        int comp = 0;
        V3F throughput(F(1));
        V3F wi{};
        V2<F> raster_pos{};
        V3F L(F(0));  // the path's total (pixel mode: every splat of a path lands on raster_pos), for m2
        bool have_rp = false;

        for (int nv = 1; nv < P.max_verts; nv++) {
            const bool is_specular = sp.type == SI_Surface && scene.material_of(sp.primitive).is_specular_component(comp);
            const bool samplable_by_nee = P.sampling_mode != 0 && (pixel_mode ? (nv > 1 && !is_specular) : !is_specular);

            if (samplable_by_nee) [&] {
                double u8[8];
                for (int k = 0; k < 8; k++) u8[k] = U(nv, k);
                int light_node = -1;
                const auto sL = scene.sample_direct_light(u8, sp, light_node);
                if (!sL) return;
                SceneInteraction<F> spL; spL.type = SI_Light; spL.primitive = light_node; spL.geom = sL->geom;
                nrays++;
                if (!scene.visible(sp, spL)) return;
                V2<F> rp = raster_pos;
                if (nv == 1) {
                    const auto rp_ = cam.raster_position(-sL->wo);
                    if (!rp_) return;
                    rp = *rp_;
                }
                const auto wo = -sL->wo;
                V3F fs;
                if (sp.type == SI_Camera) fs = cam.eval(wo);
                else fs = scene.material_of(sp.primitive).eval(sp.geom, wi, wo, comp, TransDir::EL, true) *
                          shading_normal_correction(sp.geom, wi, wo, TransDir::EL);
                if (is_zero(fs)) return;
                F mis_w = F(1);
                // renderer_pt.cpp:166-180: a light that BSDF sampling cannot reach (a specular
                // light, or a degenerate light position) keeps weight 1
                const bool samplable_by_bsdf = !scene.light_of(light_node).is_specular() && !sL->geom.degenerated;
                if (P.sampling_mode == 2 && samplable_by_bsdf) {
                    const F p_light = scene.pdf_direct_light(sp, spL, sL->wo);
                    const F p_bsdf = sp.type == SI_Camera ? cam.pdf_direction(wo)
                                                          : scene.material_of(sp.primitive).pdf_direction(sp.geom, wi, wo, comp, true);
                    mis_w = balance_heuristic(p_light, p_bsdf);
                }
                const auto Cc = throughput * fs * sL->weight * mis_w;
                film.splat(rp, Cc);  // each contribution as it comes, as renderer_pt.cpp:190-191 does
                L += Cc;
            }();

            // Direction sampling
            std::optional<DirectionSample<F>> s;
            if (nv == 1) {
                // camera_pinhole.cpp:143-148 with the pixel-window jitter of renderer_pt.cpp:199-201.
                // `Vec2(x+w*rng.u(), y+h*rng.u())` leaves the order of its two draws to the compiler;
                // GCC (and MSVC) evaluate the arguments right to left, so y takes the first number.
                const double j1 = U(nv, 9);
                const double j0 = U(nv, 8);
                const V2<F> ud(wx + ww * F(j0), wy + wh * F(j1));
                U(nv, 10); U(nv, 11);
                s = DirectionSample<F>{cam.primary_ray(ud).d, V3F(F(1))};
            } else {
                const V2<F> ud = U2(nv, 8);
                const V2<F> udc = U2(nv, 10);
                const auto& mat = scene.material_of(sp.primitive);
                const auto ms = mat.sample_direction(ud, udc, sp.geom, wi, comp, TransDir::EL);
                if (ms) s = DirectionSample<F>{ms->wo, ms->weight * shading_normal_correction(sp.geom, wi, ms->wo, TransDir::EL)};
            }
            if (!s) break;

            if (nv == 1) {
                const auto rp = cam.raster_position(s->wo);
                raster_pos = rp ? *rp : V2<F>();
                have_rp = true;
            }

            nrays++;
            const auto hit = scene.intersect(Ray<F>{sp.geom.p, s->wo});
            if (!hit) break;

            throughput *= s->weight;

            const bool samplable_by_direct_hit = P.sampling_mode == 1 ? !samplable_by_nee : true;
            if (samplable_by_direct_hit && scene.is_light(*hit)) [&] {
                const auto spL = hit->as_type(SI_Light);
                const auto woL = -s->wo;
                const auto fs = scene.light_of(spL.primitive).eval(spL.geom, woL);
                F mis_w = F(1);
                if (P.sampling_mode != 0 && samplable_by_nee) {
                    const F pdf_bsdf = sp.type == SI_Camera ? cam.pdf_direction(s->wo)
                                                            : scene.material_of(sp.primitive).pdf_direction(sp.geom, wi, s->wo, comp, true);
                    const F pdf_light = scene.pdf_direct_light(sp, spL, woL);
                    mis_w = balance_heuristic(pdf_bsdf, pdf_light);
                }
                const auto Cc = throughput * fs * mis_w;
                film.splat(raster_pos, Cc);
                L += Cc;
            }();

            if (hit->geom.infinite) break;

            if (nv > 5) {
                const F q = std::max(F(.2), F(1) - comp_max(throughput));
                if (F(U(nv, 12)) < q) break;
                throughput /= F(1) - q;
            }

            ComponentSample<F> sc{0, F(1)};
            {
                const V2<F> uc = U2(nv, 13);
                if (hit->type == SI_Surface) sc = scene.material_of(hit->primitive).sample_component(uc, hit->geom, -s->wo);
            }
            throughput *= sc.weight;

            wi = -s->wo;
            sp = *hit;
            comp = sc.comp;
        }
        if (pixel_mode && have_rp) film.add_m2(raster_pos, L);
    }

    for (auto* r : rngs) delete r;
    // renderer_pt.cpp:307-312 (rescale)
    // pixel mode: 1 / spp (scheduler::spp); image mode: w*h / (paths processed) with the
    // w*h*spp paths this loop takes (scheduler::spi), also 1 / spp
    const double scale = 1.0 / double(P.spp);
    for (long long i = 0; i < num_pixels; i++) {
        const auto v = film.data[i].load();
        out[3 * i] = v.r * scale; out[3 * i + 1] = v.g * scale; out[3 * i + 2] = v.b * scale;
        if (out_m2 && film.with_m2) {
            const auto m = film.m2[i].load();
            out_m2[3 * i] = m.r; out_m2[3 * i + 1] = m.g; out_m2[3 * i + 2] = m.b;
        }
    }
    if (rays_out) {
        long long t = 0;
        for (auto r : rays) t += r;
        *rays_out = t;
    }
}

// ------------------------------------------------------------------------------------------------
// src/renderer/renderer_lt.cpp:50-160 (light tracing with NEE to the camera), scheduled as
// scheduler::spi::sample (src/scheduler.cpp:114-138): light paths [first_path, first_path +
// num_samples). Philox slots: vertex 1 slots 0-7 the primary ray (up, upc, ud, udc), then as
// render_pt: the ray that left vertex nv takes its roulette from slot 12 and the component of
// the vertex it hits from slots 13-14 of vertex nv; vertex nv's camera connection slots 0-7
// (unused by the pinhole camera) and its direction slots 8-11.
struct LTParams {
    int w, h;
    long long num_samples;
    long long first_path;
    int max_verts;
    unsigned int seed;
    int rng_mode;
};

template <typename F>
void render_lt(const Scene<F>& scene, const LTParams& P, double* out, long long* rays_out, int nthreads) {
    using V3F = V3<F>;
    if (scene.nodes.size() <= 1) throw std::runtime_error("Missing primitives.");
    if (!scene.camera_) throw std::runtime_error("Missing camera primitive.");
    if (scene.num_lights() == 0) throw std::runtime_error("No light in the scene.");
    Film film(P.w, P.h, false);
    const auto& cam = scene.camera();
    const int nth = std::max(1, nthreads);
    std::vector<RngMT*> rngs(nth, nullptr);
    for (int i = 0; i < nth; i++) rngs[i] = new RngMT(P.seed + i, std::is_same<F, float>::value);
    std::vector<long long> rays(nth, 0);

#pragma omp parallel for schedule(dynamic, 64) num_threads(nth)
    for (long long index = 0; index < P.num_samples; index++) {
        const int tid = omp_get_thread_num();
        PathRng rng; rng.mode = P.rng_mode; rng.mt = rngs[tid]; rng.seed = P.seed; rng.path = (uint64_t)(P.first_path + index);
        auto U = [&](int nv, int s) -> double { return rng.mode == 0 ? rng.seq() : rng.slot(nv, s); };
        // two numbers in stream order (the order of a constructor's arguments is unspecified)
        auto U2 = [&](int nv, int s) { const double a = U(nv, s); const double b = U(nv, s + 1); return V2<F>(F(a), F(b)); };
        long long& nrays = rays[tid];

        double u8[8];
        for (int k = 0; k < 8; k++) u8[k] = U(1, k);
        const auto s0 = scene.sample_primary_ray_light(u8);
        if (!s0) continue;
        nrays++;
        const auto hit0 = scene.intersect(Ray<F>{s0->geom.p, s0->wo});
        if (!hit0 || hit0->geom.infinite) continue;
        V3F throughput = s0->weight;
        auto sample_comp = [&](int nv, const SceneInteraction<F>& sp, V3<F> wi) {
            const V2<F> uc = U2(nv, 13);
            return sp.type == SI_Surface ? scene.material_of(sp.primitive).sample_component(uc, sp.geom, wi) : ComponentSample<F>{0, F(1)};
        };
        const auto sc0 = sample_comp(1, *hit0, -s0->wo);
        throughput *= sc0.weight;
        SceneInteraction<F> sp = *hit0;
        V3F wi = -s0->wo;
        int comp = sc0.comp;

        for (int nv = 2; nv < P.max_verts; nv++) {
            // camera_pinhole.cpp:178-203 sample_direct: the camera point, wo from it toward sp,
            // weight J(wo) / (1 / G)
            [&] {
                for (int k = 0; k < 8; k++) U(nv, k);
                const auto sE = cam.sample_direct(sp.geom);
                if (!sE) return;
                const auto gE = sE->geom;
                const auto wE = sE->wo;
                const auto weightE = sE->weight;
                SceneInteraction<F> spE; spE.type = SI_Camera; spE.primitive = *scene.camera_; spE.geom = gE;
                nrays++;
                if (!scene.visible(sp, spE)) return;
                const auto rp = cam.raster_position(wE);
                if (!rp) return;
                const auto wo = -wE;
                const auto fs = scene.material_of(sp.primitive).eval(sp.geom, wi, wo, comp, TransDir::LE, true) *
                                shading_normal_correction(sp.geom, wi, wo, TransDir::LE);
                film.splat(*rp, throughput * fs * weightE);
            }();

            const V2<F> ud = U2(nv, 8);
            const V2<F> udc = U2(nv, 10);
            const auto ms = scene.material_of(sp.primitive).sample_direction(ud, udc, sp.geom, wi, comp, TransDir::LE);
            if (!ms) break;
            const auto w = ms->weight * shading_normal_correction(sp.geom, wi, ms->wo, TransDir::LE);
            nrays++;
            const auto hit = scene.intersect(Ray<F>{sp.geom.p, ms->wo});
            if (!hit) break;
            throughput *= w;
            if (hit->geom.infinite) break;
            if (nv > 5) {
                const F q = std::max(F(.2), F(1) - comp_max(throughput));
                if (F(U(nv, 12)) < q) break;
                throughput /= F(1) - q;
            }
            const auto sc = sample_comp(nv, *hit, -ms->wo);
            throughput *= sc.weight;
            wi = -ms->wo;
            sp = *hit;
            comp = sc.comp;
        }
    }

    for (auto* r : rngs) delete r;
    // renderer_lt.cpp:157 (rescale by the pixel count over the light paths)
    const long long num_pixels = (long long)P.w * P.h;
    const double scale = double(num_pixels) / double(P.num_samples);
    for (long long i = 0; i < num_pixels; i++) {
        const auto v = film.data[i].load();
        out[3 * i] = v.r * scale; out[3 * i + 1] = v.g * scale; out[3 * i + 2] = v.b * scale;
    }
    if (rays_out) {
        long long t = 0;
        for (auto r : rays) t += r;
        *rays_out = t;
    }
}

// ------------------------------------------------------------------------------------------------
// Bidirectional path tracing: src/renderer/renderer_bdpt.cpp:297-413 (renderer::bdpt) over the
// path structure of include/lm/bidir.h. Every function below restates one of bidir.h's in the
// same order of operations; the vertex and endpoint queries are path.h's dispatch by interaction
// type. Philox slots: the eye subpath's vertex i draws from "vertex" kBdEye + i and the light
// subpath's from kBdLight + i: slots 0-7 the primary ray (RaySampleU; the camera uses ud = slots
// 4-5), slots 8-11 the direction sampled at vertex i, slots 13-14 the component of the vertex hit
// by the ray that leaves vertex i.
constexpr int kBdEye = 1;
constexpr int kBdLight = 129;

template <typename F> struct BdVert {
    SceneInteraction<F> sp;
    int comp = 0;
};

template <typename F> struct Bidir {
    using V3F = V3<F>;
    const Scene<F>& scene;
    explicit Bidir(const Scene<F>& s) : scene(s) {}

    const Camera<F>& cam() const { return scene.camera(); }
    const Light<F>& light(const SceneInteraction<F>& sp) const { return scene.light_of(sp.primitive); }
    const Transform<F>& light_tr(const SceneInteraction<F>& sp) const {
        return scene.lights_.at(scene.light_indices_map_.at(sp.primitive)).tr;
    }

    // path.h:695-725
    bool is_specular(const SceneInteraction<F>& sp, int comp) const {
        if (sp.type == SI_Surface) return scene.material_of(sp.primitive).is_specular_component(comp);
        if (sp.type == SI_Light) return light(sp).is_specular();  // light::directional
        return false;  // the pinhole camera is not specular
    }
    bool is_connectable(const SceneInteraction<F>& sp) const {
        if (sp.type == SI_Camera) return true;                   // camera_pinhole.cpp:228-230
        // light_area.cpp:181, light_point.cpp:113; light_env*.cpp and light_directional.cpp: false
        return light(sp).type == LIGHT_AREA || light(sp).type == LIGHT_POINT;
    }
    // path.h:761-775 (eval_contrb_direction)
    V3F eval_dir(const SceneInteraction<F>& sp, V3F wi, V3F wo, int comp, TransDir td, bool eval_delta) const {
        if (sp.type == SI_Camera) return cam().eval(wo);
        if (sp.type == SI_Light) return light(sp).eval(sp.geom, wo);
        return scene.material_of(sp.primitive).eval(sp.geom, wi, wo, comp, td, eval_delta) *
               shading_normal_correction(sp.geom, wi, wo, td);
    }
    // path.h:457-470 (eval_delta false); light_area.cpp:124-129
    F pdf_dir(const SceneInteraction<F>& sp, V3F wi, V3F wo, int comp) const {
        if (sp.type == SI_Camera) return cam().pdf_direction(wo);
        if (sp.type == SI_Light) {
            if (light(sp).type == LIGHT_POINT) return pdf_uniform_sphere<F>();  // light_point.cpp:64-66
            if (light(sp).type != LIGHT_AREA) throw std::runtime_error("pdf_direction of an infinite light");
            return dot(wo, sp.geom.n) <= F(0) ? F(0) : F(1) / C<F>::Pi;
        }
        return scene.material_of(sp.primitive).pdf_direction(sp.geom, wi, wo, comp, false);
    }
    // path.h:228-234
    F pdf_comp(const SceneInteraction<F>& sp, V3F wi, int comp) const {
        return sp.type == SI_Surface ? scene.material_of(sp.primitive).pdf_component(comp, sp.geom, wi) : F(1);
    }
    // path.h:327-344 with camera_pinhole.cpp:172 and light_area.cpp:142
    F pdf_position(const SceneInteraction<F>& sp) const {
        if (sp.type == SI_Camera) return F(1);
        const auto& L = light(sp);
        if (L.type == LIGHT_POINT) return scene.pdf_light_selection();  // light_point.cpp:78-80
        if (L.type != LIGHT_AREA) throw std::runtime_error("pdf_position of an infinite light");
        return scene.pdf_light_selection() * (L.invA / light_tr(sp).J);
    }
    // path.h:149-162 with camera_pinhole.cpp:142-146, light_area.cpp:102-106,
    // light_envconst.cpp:70-74, light_env.cpp:109-113, light_point.cpp:51-53 and
    // light_directional.cpp:72-75 (eval_delta false)
    F pdf_primary_ray(const SceneInteraction<F>& sp, V3F wo) const {
        if (sp.type == SI_Camera) return cam().pdf_direction(wo) * F(1);
        const auto& L = light(sp);
        F p;
        if (L.type == LIGHT_AREA) {
            p = (L.invA / light_tr(sp).J) * (dot(wo, sp.geom.n) <= F(0) ? F(0) : F(1) / C<F>::Pi);
        } else if (L.type == LIGHT_POINT) {
            p = pdf_uniform_sphere<F>();  // light_point.cpp:51-53
        } else if (L.type == LIGHT_DIRECTIONAL) {
            p = F(1) / (C<F>::Pi * scene.sphere_radius * scene.sphere_radius);  // light_directional.cpp:72-75
        } else {
            p = pdf_uniform_sphere<F>() * (F(1) / (C<F>::Pi * scene.sphere_radius * scene.sphere_radius));
        }
        return scene.pdf_light_selection() * p;
    }

    // bidir.h:140-155
    static V3F direction(const BdVert<F>* a, const BdVert<F>* b) {
        if (!a || !b) return V3F();
        if (a->sp.geom.infinite) return a->sp.geom.wo;
        if (b->sp.geom.infinite) return -b->sp.geom.wo;
        return normalize(b->sp.geom.p - a->sp.geom.p);
    }

    // bidir.h:507-591 (sample_subpath_from_endpoint); U(vertex, slot) draws a number
    template <typename Ufn>
    std::vector<BdVert<F>> sample_subpath(Ufn&& U, int base, int max_verts, TransDir td, long long& nrays) const {
        std::vector<BdVert<F>> vs;
        auto U2 = [&](int nv, int k) { const double a = U(nv, k); const double b = U(nv, k + 1); return V2<F>(F(a), F(b)); };
        if (max_verts == 0) return vs;
        while (int(vs.size()) < max_verts) {
            Ray<F> ray;
            if (vs.empty()) {
                double u8[8];
                for (int k = 0; k < 8; k++) u8[k] = U(base, k);
                SceneInteraction<F> sp;
                V3F wo;
                if (td == TransDir::EL) {
                    sp.type = SI_Camera; sp.primitive = *scene.camera_;
                    sp.geom = PointGeometry<F>::make_degenerated(cam().position);
                    wo = cam().primary_ray(V2<F>(F(u8[4]), F(u8[5]))).d;
                } else {
                    const auto s = scene.sample_primary_ray_light(u8);
                    if (!s) break;
                    // the light chosen by u8[2] (path.h:102-104)
                    const int li = scene.sample_light_selection(F(u8[2])).first;
                    sp.type = SI_Light; sp.primitive = scene.lights_.at(li).index;
                    sp.geom = s->geom;
                    wo = s->wo;
                }
                vs.push_back({sp, 0});
                ray = Ray<F>{sp.geom.p, wo};
            } else {
                const int i = int(vs.size()) - 1;
                const auto& v = vs[i];
                const auto wi = direction(&v, i > 0 ? &vs[i - 1] : nullptr);
                const auto ud = U2(base + i, 8);
                const auto udc = U2(base + i, 10);
                const auto ms = scene.material_of(v.sp.primitive).sample_direction(ud, udc, v.sp.geom, wi, v.comp, td);
                if (!ms) break;
                ray = Ray<F>{v.sp.geom.p, ms->wo};
            }
            nrays++;
            const auto hit = scene.intersect(ray);
            if (!hit) break;
            const auto uc = U2(base + int(vs.size()) - 1, 13);
            const auto sc = hit->type == SI_Surface ? scene.material_of(hit->primitive).sample_component(uc, hit->geom, -ray.d)
                                                    : ComponentSample<F>{0, F(1)};
            vs.push_back({*hit, sc.comp});
            if (hit->geom.infinite) break;
        }
        return vs;
    }

    // A full path x_0 (light endpoint) .. x_{n-1} (camera endpoint) with its accessors (bidir.h:79-111)
    struct FullPath {
        std::vector<BdVert<F>> vs;
        int n() const { return int(vs.size()); }
        const BdVert<F>* at(int i, TransDir td) const {
            if (i < 0 || i >= n()) return nullptr;
            return &vs[td == TransDir::LE ? i : n() - 1 - i];
        }
    };

    // bidir.h:593-643 (connect_subpaths); `visible` counts the connection ray
    std::optional<FullPath> connect(const std::vector<BdVert<F>>& L, const std::vector<BdVert<F>>& E, int s, int t,
                                    long long& nrays) const {
        FullPath P;
        if (s == 0) {
            if (E[t - 1].sp.geom.degenerated) return {};
            for (int i = t - 1; i >= 0; i--) P.vs.push_back(E[i]);
        } else if (t == 0) {
            if (L[s - 1].sp.geom.degenerated) return {};
            for (int i = 0; i < s; i++) P.vs.push_back(L[i]);
        } else {
            const auto& vL = L[s - 1];
            const auto& vE = E[t - 1];
            if (vL.sp.geom.infinite || vE.sp.geom.infinite) return {};
            nrays++;
            if (!scene.visible(vL.sp, vE.sp)) return {};
            for (int i = 0; i < s; i++) P.vs.push_back(L[i]);
            for (int i = t - 1; i >= 0; i--) P.vs.push_back(E[i]);
        }
        if (!scene.is_light(P.vs.front().sp)) return {};
        if (P.vs.back().sp.type != SI_Camera) return {};
        P.vs.front().sp = P.vs.front().sp.as_type(SI_Light);
        return P;
    }

    // bidir.h:185-224
    bool samplable(const FullPath& P, int s) const {
        const int t = P.n() - s;
        if (s == 0) {
            const auto* v = P.at(0, TransDir::LE);
            return !v->sp.geom.degenerated && !is_specular(v->sp, v->comp);
        }
        if (t == 0) {
            const auto* v = P.at(0, TransDir::EL);
            return !v->sp.geom.degenerated && !is_specular(v->sp, v->comp);
        }
        const auto* vL = P.at(s - 1, TransDir::LE);
        const auto* vE = P.at(t - 1, TransDir::EL);
        if (s == 1 && !is_connectable(vL->sp)) return false;
        if (t == 1 && !is_connectable(vE->sp)) return false;
        return !is_specular(vL->sp, vL->comp) && !is_specular(vE->sp, vE->comp);
    }

    // bidir.h:233-275 (eval_subpath_sampling_weight)
    V3F alpha(const FullPath& P, int l, TransDir td) const {
        if (l == 0) return V3F(F(1));
        int i = 0;
        V3F a(F(0));
        const auto* v0 = P.at(0, td);
        if (is_connectable(v0->sp)) {
            a = V3F(F(1)) / (pdf_position(v0->sp) * pdf_comp(v0->sp, V3F(), v0->comp));
        } else {
            const auto* v1 = P.at(1, td);
            const auto d01 = direction(v0, v1);
            const auto f = eval_dir(v0->sp, V3F(), d01, v0->comp, td, false);
            if (is_zero(f)) return V3F(F(0));
            a = f / (pdf_primary_ray(v0->sp, d01) * pdf_comp(v0->sp, V3F(), v0->comp) * pdf_comp(v1->sp, -d01, v1->comp));
            i++;
        }
        for (; i < l - 1; i++) {
            const auto* v = P.at(i, td);
            const auto* vn = P.at(i + 1, td);
            const auto wi = direction(v, P.at(i - 1, td));
            const auto wo = direction(v, vn);
            const auto f = eval_dir(v->sp, wi, wo, v->comp, td, false);
            if (is_zero(f)) return V3F(F(0));
            a *= f / pdf_dir(v->sp, wi, wo, v->comp) / pdf_comp(vn->sp, -wo, vn->comp);
        }
        return a;
    }

    // bidir.h:288-313 (eval_connection_term)
    V3F connection(const FullPath& P, int s) const {
        const int t = P.n() - s;
        if (s == 0 && t > 0) {
            const auto* v = P.at(0, TransDir::LE);
            return eval_dir(v->sp, V3F(), direction(v, P.at(1, TransDir::LE)), v->comp, TransDir::LE, true);
        }
        if (s > 0 && t == 0) {
            const auto* v = P.at(0, TransDir::EL);
            return eval_dir(v->sp, V3F(), direction(v, P.at(1, TransDir::EL)), v->comp, TransDir::EL, true);
        }
        const auto* vL = P.at(s - 1, TransDir::LE);
        const auto* vE = P.at(t - 1, TransDir::EL);
        const auto fL = eval_dir(vL->sp, direction(vL, P.at(s - 2, TransDir::LE)), direction(vL, vE), vL->comp, TransDir::LE, true);
        const auto fE = eval_dir(vE->sp, direction(vE, P.at(t - 2, TransDir::EL)), direction(vE, vL), vE->comp, TransDir::EL, true);
        return fL * geometry_term(vL->sp.geom, vE->sp.geom) * fE;
    }

    // bidir.h:325-343 (eval_sampling_weight_bidir)
    V3F weight(const FullPath& P, int s) const {
        const auto aL = alpha(P, s, TransDir::LE);
        if (is_zero(aL)) return V3F(F(0));
        const auto aE = alpha(P, P.n() - s, TransDir::EL);
        if (is_zero(aE)) return V3F(F(0));
        return aL * connection(P, s) * aE;
    }

    // bidir.h:397-449 (pdf_bidir). with_comp = false leaves out the component pdfs, as the
    // cached pdfs of renderer::bdptopt do (renderer_bdptopt.cpp:145-215).
    F pdf(const FullPath& P, int s, bool with_comp = true) const {
        auto pcomp = [&](const SceneInteraction<F>& sp, V3F wi, int comp) { return with_comp ? pdf_comp(sp, wi, comp) : F(1); };
        if (!samplable(P, s)) return F(0);
        auto sub = [&](int l, TransDir td) -> F {
            if (l == 0) return F(1);
            int i = 0;
            F p = F(0);
            const auto* v0 = P.at(0, td);
            if (is_connectable(v0->sp)) {
                p = pdf_position(v0->sp) * pcomp(v0->sp, V3F(), v0->comp);
            } else {
                const auto* v1 = P.at(1, td);
                const auto d01 = direction(v0, v1);
                p = pdf_primary_ray(v0->sp, d01) * geometry_term(v0->sp.geom, v1->sp.geom) * pcomp(v0->sp, V3F(), v0->comp) *
                    pcomp(v1->sp, -d01, v1->comp);
                i++;
            }
            for (; i < l - 1; i++) {
                const auto* v = P.at(i, td);
                const auto* vn = P.at(i + 1, td);
                const auto wi = direction(v, P.at(i - 1, td));
                const auto wo = direction(v, vn);
                p *= pcomp(vn->sp, -wo, vn->comp) * (pdf_dir(v->sp, wi, wo, v->comp) * geometry_term(v->sp.geom, vn->sp.geom));
            }
            return p;
        };
        return sub(s, TransDir::LE) * sub(P.n() - s, TransDir::EL);
    }

    // bidir.h:460-479 (power heuristic over every strategy of the path). The reference asserts a
    // nonzero pdf of the strategy that sampled the path; a zero one contributes nothing here.
    // balance: renderer_bdptopt.cpp:315-400, the balance heuristic over pdfs without component
    // pdfs (the same ratios as its cached forward / reverse pdfs).
    F mis(const FullPath& P, int s, bool balance = false) const {
        const F ps = pdf(P, s, !balance);
        if (ps == F(0)) return F(0);
        F inv = F(0);
        for (int s2 = 0; s2 <= P.n(); s2++) {
            const F pi = pdf(P, s2, !balance);
            if (pi == F(0)) continue;
            const F r = pi / ps;
            inv += balance ? r : r * r;
        }
        return F(1) / inv;
    }
};

// mode: 0 renderer::bdpt, 1 renderer::pt_naive_path, 2 renderer::pt_nee_path,
// 3 renderer::lt_nee_path, 4 renderer::bdptopt
enum BdMode { BD_ALL = 0, BD_PT_NAIVE = 1, BD_PT_NEE = 2, BD_LT_NEE = 3, BD_OPT = 4 };
struct BDPTParams {
    int w, h;
    long long num_samples;
    long long first_path;
    int min_verts, max_verts;
    unsigned int seed;
    int rng_mode;
    int mode;
};

template <typename F>
void render_bdpt(const Scene<F>& scene, const BDPTParams& P, double* out, long long* rays_out, int nthreads) {
    using V3F = V3<F>;
    if (scene.nodes.size() <= 1) throw std::runtime_error("Missing primitives.");
    if (!scene.camera_) throw std::runtime_error("Missing camera primitive.");
    if (scene.num_lights() == 0) throw std::runtime_error("No light in the scene.");
    Film film(P.w, P.h, false);
    const Bidir<F> B(scene);
    const int nth = std::max(1, nthreads);
    std::vector<RngMT*> rngs(nth, nullptr);
    for (int i = 0; i < nth; i++) rngs[i] = new RngMT(P.seed + i, std::is_same<F, float>::value);
    std::vector<long long> rays(nth, 0);

#pragma omp parallel for schedule(dynamic, 16) num_threads(nth)
    for (long long index = 0; index < P.num_samples; index++) {
        const int tid = omp_get_thread_num();
        PathRng rng; rng.mode = P.rng_mode; rng.mt = rngs[tid]; rng.seed = P.seed; rng.path = (uint64_t)(P.first_path + index);
        auto U = [&](int nv, int s) -> double { return rng.mode == 0 ? rng.seq() : rng.slot(nv, s); };
        long long& nrays = rays[tid];
        // subpath lengths: renderer_bdpt.cpp:72, 143-144, 219-220; renderer_bdptopt.cpp:487-488
        const int maxE = P.mode == BD_LT_NEE ? 1 : P.max_verts;
        const int maxL = P.mode == BD_PT_NEE ? 1 : P.max_verts;
        const auto E = B.sample_subpath(U, kBdEye, maxE, TransDir::EL, nrays);
        const auto L = P.mode == BD_PT_NAIVE ? std::vector<BdVert<F>>() : B.sample_subpath(U, kBdLight, maxL, TransDir::LE, nrays);
        const int nE = int(E.size()), nL = int(L.size());
        auto contribute = [&](int s, int t, bool weighted) {
            const auto path = B.connect(L, E, s, t, nrays);
            if (!path) return;
            auto Cu = B.weight(*path, s);
            if (P.mode == BD_OPT && s == 0 && path->vs.front().sp.type == SI_Light && E[t - 1].sp.type == SI_Surface) {
                // bdptopt's eye alpha keeps the last vertex's component weight (renderer_bdptopt.cpp:265-270)
                const auto& v = E[t - 1];
                Cu = Cu / B.pdf_comp(v.sp, Bidir<F>::direction(&v, &E[t - 2]), v.comp);
            }
            if (is_zero(Cu)) return;
            const F w = weighted ? B.mis(*path, s, P.mode == BD_OPT) : F(1);
            // bidir.h:167-171: the raster position of the camera's first edge
            const auto* vE = path->at(0, TransDir::EL);
            const auto rp = scene.camera().raster_position(Bidir<F>::direction(vE, path->at(1, TransDir::EL)));
            if (!rp) return;  // the reference dereferences it unchecked; only rounding reaches here
            film.splat(*rp, w * Cu);
        };
        if (P.mode == BD_ALL || P.mode == BD_OPT) {
            for (int s = 0; s <= nL; s++) {
                for (int t = 0; t <= nE; t++) {
                    const int k = s + t;
                    if (k < P.min_verts || P.max_verts < k) continue;
                    contribute(s, t, true);
                }
            }
        } else if (P.mode == BD_PT_NAIVE) {  // renderer_bdpt.cpp:77-105
            for (int t = 2; t <= nE; t++) {
                if (t < P.min_verts || P.max_verts < t) continue;
                contribute(0, t, false);
            }
        } else {  // renderer_bdpt.cpp:149-186 (pt_nee_path) and 228-278 (lt_nee_path)
            for (int k = 2; k <= nL + nE; k++) {
                if (k < P.min_verts || P.max_verts < k) continue;
                int s = P.mode == BD_PT_NEE ? 1 : k - 1;
                int t = k - s;
                if (s > nL || t > nE) continue;
                if (P.mode == BD_PT_NEE && B.is_specular(E[t - 1].sp, E[t - 1].comp)) {
                    s = 0;
                    t = k;
                    if (s > nL || t > nE) continue;
                }
                contribute(s, t, false);
            }
        }
    }

    for (auto* r : rngs) delete r;
    // renderer_bdpt.cpp:397-399
    const long long num_pixels = (long long)P.w * P.h;
    const double scale = double(num_pixels) / double(P.num_samples);
    for (long long i = 0; i < num_pixels; i++) {
        const auto v = film.data[i].load();
        out[3 * i] = v.r * scale; out[3 * i + 1] = v.g * scale; out[3 * i + 2] = v.b * scale;
    }
    if (rays_out) {
        long long t = 0;
        for (auto r : rays) t += r;
        *rays_out = t;
    }
}

}  // namespace lmo

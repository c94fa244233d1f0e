// Oracle (test infrastructure only): C entry points over the CPU restatement in lmo.hpp, loaded
// with ctypes by tests/ and by bench.py's CPU-baseline leg. One handle holds a scene in either
// precision (double = the reference's Float, float = the fp32 parity mode).
#include "lmo.hpp"
#include <chrono>
#include <cstring>
#include <memory>
#include <type_traits>

using namespace lmo;

namespace {

thread_local std::string g_err;

struct Handle {
    bool dbl;
    std::unique_ptr<Scene<double>> sd;
    std::unique_ptr<Scene<float>> sf;
};

template <typename Fn>
int dispatch(Handle* h, Fn&& fn) {
    try {
        return h->dbl ? fn(*h->sd) : fn(*h->sf);
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

int fail(const char* msg) {
    g_err = msg;
    return -1;
}

}  // namespace

extern "C" {

const char* lmo_last_error() { return g_err.c_str(); }

void* lmo_create(int use_double) {
    auto* h = new Handle();
    h->dbl = use_double != 0;
    if (h->dbl) h->sd.reset(new Scene<double>());
    else h->sf.reset(new Scene<float>());
    return h;
}

void lmo_destroy(void* p) { delete static_cast<Handle*>(p); }

// mesh::raw (src/mesh/mesh_raw.cpp:50-68): ps/ns flat xyz, ts flat uv, per-corner indices.
int lmo_add_mesh(void* p, const float* ps, int nps, const float* ns, int nns, const float* ts, int nts,
                 const int* fp, const int* ft, const int* fn, int ncorners) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        Mesh<F> m;
        for (int i = 0; i < nps; i++) m.ps.push_back(V3<F>(F(ps[3 * i]), F(ps[3 * i + 1]), F(ps[3 * i + 2])));
        for (int i = 0; i < nns; i++) m.ns.push_back(V3<F>(F(ns[3 * i]), F(ns[3 * i + 1]), F(ns[3 * i + 2])));
        for (int i = 0; i < nts; i++) m.ts.push_back(V2<F>(F(ts[2 * i]), F(ts[2 * i + 1])));
        if (m.ts.empty()) m.ts.push_back(V2<F>());
        for (int i = 0; i < ncorners; i++) {
            const int t = ft && nts > 0 ? ft[i] : 0;
            if (t < 0 || t >= int(m.ts.size())) return fail("texture coordinate index out of range");
            if (fn[i] >= nns || (fn[i] < 0 && fn[i - i % 3] >= 0)) return fail("normal index out of range");
            m.fs.push_back({fp[i], t, fn[i]});
        }
        S.meshes.push_back(std::move(m));
        return int(S.meshes.size()) - 1;
    });
}

// type: 0 diffuse (Kd), 1 glossy (Ks, ax, ay), 2 glass (Ni), 3 mirror. params: 5 doubles.
int lmo_add_material(void* p, int type, const double* prm) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        Material<F> m;
        m.type = type;
        if (type == MAT_DIFFUSE) m.Kd = V3<F>(F(prm[0]), F(prm[1]), F(prm[2]));
        if (type == MAT_GLOSSY) { m.Ks = V3<F>(F(prm[0]), F(prm[1]), F(prm[2])); m.ax = F(prm[3]); m.ay = F(prm[4]); }
        if (type == MAT_GLASS) m.Ni = F(prm[0]);
        if (type == MAT_MIXTURE) {
            m.Kd = V3<F>(F(prm[0]), F(prm[1]), F(prm[2]));
            m.Ks = V3<F>(F(prm[3]), F(prm[4]), F(prm[5]));
            m.ax = F(prm[6]);
            m.ay = F(prm[7]);
        }
        S.materials.push_back(m);
        return int(S.materials.size()) - 1;
    });
}

// texture::bitmap (texture_bitmap.cpp:40-85): w x h texels of c (3 or 4) floats, row 0 at the bottom.
int lmo_add_texture(void* p, const float* data, int w, int hgt, int c) {
    auto* h = static_cast<Handle*>(p);
    if (!data || w <= 0 || hgt <= 0 || (c != 3 && c != 4)) return fail("texture: invalid size or channel count");
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        auto t = std::make_shared<Texture<F>>();
        t->w = w; t->h = hgt; t->c = c;
        t->data.assign(data, data + size_t(w) * hgt * c);
        S.textures.push_back(t);
        return int(S.textures.size()) - 1;
    });
}

// material::diffuse's mapKd (and the mixture's diffuse lobe), and the mixture's alpha mask: texture
// indices or -1.
int lmo_set_material_textures(void* p, int mat, int mapKd, int mask) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        if (mat < 0 || mat >= int(S.materials.size())) return fail("material index out of range");
        const int nt = int(S.textures.size());
        if (mapKd >= nt || mask >= nt) return fail("texture index out of range");
        if (mask >= 0 && !S.textures[mask]->has_alpha()) return fail("alpha mask texture without an alpha channel");
        S.materials[mat].mapKd = mapKd >= 0 ? S.textures[mapKd] : nullptr;
        S.materials[mat].mask = mask >= 0 ? S.textures[mask] : nullptr;
        return 0;
    });
}

// light::area (src/light/light_area.cpp:68-80): the triangle-area CDF is built on the untransformed mesh.
int lmo_add_light_area(void* p, const double* Ke, int mesh) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        Light<F> L;
        L.type = LIGHT_AREA;
        L.Ke = V3<F>(F(Ke[0]), F(Ke[1]), F(Ke[2]));
        L.mesh = mesh;
        const auto& m = S.meshes.at(mesh);
        for (int f = 0; f < m.num_triangles(); f++) {
            const auto tri = m.triangle_at(f);
            const auto cr = cross(tri.p2.p - tri.p1.p, tri.p3.p - tri.p1.p);
            L.dist.add(safe_sqrt(dot(cr, cr)) * F(.5));
        }
        L.invA = F(1) / L.dist.c.back();
        L.dist.norm();
        S.lights_assets.push_back(std::move(L));
        return int(S.lights_assets.size()) - 1;
    });
}

int lmo_add_light_envconst(void* p, const double* Le) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        Light<F> L;
        L.type = LIGHT_ENVCONST;
        L.Ke = V3<F>(F(Le[0]), F(Le[1]), F(Le[2]));
        S.lights_assets.push_back(std::move(L));
        return int(S.lights_assets.size()) - 1;
    });
}

// light::point (src/light/light_point.cpp:34-37): Le and a world-space position.
int lmo_add_light_point(void* p, const double* Le, const double* position) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        Light<F> L;
        L.type = LIGHT_POINT;
        L.Ke = V3<F>(F(Le[0]), F(Le[1]), F(Le[2]));
        L.pos = V3<F>(F(position[0]), F(position[1]), F(position[2]));
        S.lights_assets.push_back(std::move(L));
        return int(S.lights_assets.size()) - 1;
    });
}

// light::directional (src/light/light_directional.cpp:34-37): Le and the normalized direction.
int lmo_add_light_directional(void* p, const double* Le, const double* direction) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        Light<F> L;
        L.type = LIGHT_DIRECTIONAL;
        L.Ke = V3<F>(F(Le[0]), F(Le[1]), F(Le[2]));
        L.pos = normalize(V3<F>(F(direction[0]), F(direction[1]), F(direction[2])));
        S.lights_assets.push_back(std::move(L));
        return int(S.lights_assets.size()) - 1;
    });
}

// light::env with an in-memory texture (row 0 = first row of `texels`, c channels, fp32).
int lmo_add_light_env(void* p, const float* texels, int w, int hgt, int c, double rot_deg, double scale) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        Light<F> L;
        L.type = LIGHT_ENV;
        L.tw = w; L.th = hgt; L.tc = c;
        L.texels.assign(texels, texels + size_t(w) * hgt * c);
        L.rot = F(rot_deg) * C<F>::Pi / F(180);
        L.scale = F(scale);
        L.init_env();
        S.lights_assets.push_back(std::move(L));
        return int(S.lights_assets.size()) - 1;
    });
}

int lmo_add_camera(void* p, const double* pos, const double* center, const double* up, double vfov, double aspect) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        Camera<F> c;
        c.construct(V3<F>(F(pos[0]), F(pos[1]), F(pos[2])), V3<F>(F(center[0]), F(center[1]), F(center[2])),
                    V3<F>(F(up[0]), F(up[1]), F(up[2])), F(vfov), F(aspect));
        S.cameras.push_back(c);
        return int(S.cameras.size()) - 1;
    });
}

int lmo_create_primitive_node(void* p, int mesh, int material, int light, int camera) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float; return S.create_primitive_node(mesh, material, light, camera); });
}

int lmo_create_group_node(void* p, const double* m16) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float; return S.create_group_node(M4<F>::from_colmajor(m16)); });
}

int lmo_create_instance_group_node(void* p) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float; return S.create_instance_group_node(); });
}

int lmo_add_child(void* p, int parent, int child) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float; S.add_child(parent, child); return 0; });
}

int lmo_root_node(void*) { return 0; }

// Scene::build (src/scene.cpp:274-317) with the accel::sahbvh build; returns seconds via *secs.
int lmo_build(void* p, int nthreads, int robust, double* secs) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        const auto t0 = std::chrono::steady_clock::now();
        S.build(nthreads > 0 ? nthreads : int(std::thread::hardware_concurrency()), robust != 0);
        if (secs) *secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return 0;
    });
}

int lmo_num_triangles(void* p) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float; return int(S.accel.trs.size()); });
}

// Flattened triangles as the accel stores them (accel_sahbvh.cpp:41-49): p1, e1 = p2 - p1,
// e2 = p3 - p1, each rounded in the scene's precision.
int lmo_get_triangles(void* p, float* out9) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        for (size_t i = 0; i < S.accel.trs.size(); i++) {
            const auto& t = S.accel.trs[i];
            const F v[9] = {t.p1.x, t.p1.y, t.p1.z, t.e1.x, t.e1.y, t.e1.z, t.e2.x, t.e2.y, t.e2.z};
            for (int k = 0; k < 9; k++) out9[9 * i + k] = float(v[k]);
        }
        return 0;
    });
}

// Accel::intersect over a batch of rays. rays: n x 8 floats (ox,oy,oz,tmin,dx,dy,dz,tmax).
// Outputs: t (float64), u, v (float64), global triangle index (-1 = miss). brute != 0 uses the
// exhaustive test instead of the BVH. Returns the elapsed seconds in *secs.
int lmo_intersect(void* p, const float* rays, long long n, double* t_out, double* uv_out, int* tri_out,
                  int nthreads, int brute, int refine_t, double* secs) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        const auto t0 = std::chrono::steady_clock::now();
        const int nth = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(nth)
        for (long long i = 0; i < n; i++) {
            const float* r = rays + 8 * i;
            Ray<F> ray{V3<F>(F(r[0]), F(r[1]), F(r[2])), V3<F>(F(r[4]), F(r[5]), F(r[6]))};
            const auto hit = brute ? S.accel.intersect_brute(ray, F(r[3]), F(r[7])) : S.accel.intersect(ray, F(r[3]), F(r[7]));
            if (hit) {
                t_out[i] = double(hit->t); uv_out[2 * i] = double(hit->uv.x); uv_out[2 * i + 1] = double(hit->uv.y);
                if constexpr (std::is_same_v<F, float>)
                    if (refine_t) t_out[i] = double(refine_hit_t(ray.o, ray.d, S.accel.trs.at(hit->global_tri)));
                tri_out[i] = hit->global_tri;
            } else {
                t_out[i] = 0; uv_out[2 * i] = 0; uv_out[2 * i + 1] = 0; tri_out[i] = -1;
            }
        }
        if (secs) *secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return 0;
    });
}

int lmo_render_raycast(void* p, int w, int hgt, const double* bg, int use_constant_color, int visualize_normal,
                       const double* color, double* out, int nthreads, double* secs) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        const auto t0 = std::chrono::steady_clock::now();
        V3<F> bgc{F(bg[0]), F(bg[1]), F(bg[2])};
        V3<F> col;
        if (color) col = V3<F>(F(color[0]), F(color[1]), F(color[2]));
        render_raycast<F>(S, w, hgt, bgc, use_constant_color != 0, visualize_normal != 0, color ? &col : nullptr, out,
                          nthreads > 0 ? nthreads : omp_get_max_threads());
        if (secs) *secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return 0;
    });
}

int lmo_render_pt(void* p, int w, int hgt, long long spp, int max_verts, unsigned int seed, int sampling_mode,
                  int primary_mode, int rng_mode, double* out, double* out_m2, long long* rays, int nthreads, double* secs) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        const auto t0 = std::chrono::steady_clock::now();
        PTParams P{w, hgt, spp, max_verts, seed, sampling_mode, primary_mode, rng_mode, out_m2 != nullptr};
        render_pt<F>(S, P, out, out_m2, rays, nthreads > 0 ? nthreads : omp_get_max_threads());
        if (secs) *secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return 0;
    });
}

int lmo_render_lt(void* p, int w, int hgt, long long num_samples, long long first_path, int max_verts, unsigned int seed,
                  int rng_mode, double* out, long long* rays, int nthreads, double* secs) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        const auto t0 = std::chrono::steady_clock::now();
        LTParams P{w, hgt, num_samples, first_path, max_verts, seed, rng_mode};
        render_lt<F>(S, P, out, rays, nthreads > 0 ? nthreads : omp_get_max_threads());
        if (secs) *secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return 0;
    });
}

int lmo_render_bdpt(void* p, int w, int hgt, long long num_samples, long long first_path, int min_verts, int max_verts,
                    unsigned int seed, int rng_mode, int mode, double* out, long long* rays, int nthreads, double* secs) {
    auto* h = static_cast<Handle*>(p);
    return dispatch(h, [&](auto& S) -> int {
        using F = typename std::decay_t<decltype(S)>::Float;
        const auto t0 = std::chrono::steady_clock::now();
        BDPTParams P{w, hgt, num_samples, first_path, min_verts, max_verts, seed, rng_mode, mode};
        render_bdpt<F>(S, P, out, rays, nthreads > 0 ? nthreads : omp_get_max_threads());
        if (secs) *secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return 0;
    });
}

float lmo_philox_uniform(unsigned int seed, unsigned long long path, unsigned int vertex, unsigned int slot) {
    return philox_uniform(seed, path, vertex, slot);
}

int lmo_max_threads() { return omp_get_max_threads(); }

// The restated math.h helpers in double precision over n records, with the same record layout as
// the reference library's lmref_math_eval, so that tests can compare the two bit for bit.
int lmo_math_eval(const char* fn, const double* in, long long n, double* out) {
    using V = V3<double>;
    auto v3 = [](const double* p) { return V(p[0], p[1], p[2]); };
    auto put3 = [](double* o, V v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; };
    const std::string f(fn);
    for (long long i = 0; i < n; i++) {
        if (f == "reflection") {
            const double* a = in + 6 * i;
            put3(out + 3 * i, reflection(v3(a), v3(a + 3)));
        } else if (f == "refraction") {
            const double* a = in + 7 * i;
            const auto r = refraction(v3(a), v3(a + 3), a[6]);
            put3(out + 4 * i, r.wt);
            out[4 * i + 3] = r.total ? 1 : 0;
        } else if (f == "orthonormal_basis") {
            V u, v;
            orthonormal_basis(v3(in + 3 * i), u, v);
            put3(out + 6 * i, u);
            put3(out + 6 * i + 3, v);
        } else if (f == "geometry_normal") {
            const double* a = in + 9 * i;
            put3(out + 3 * i, geometry_normal(v3(a), v3(a + 3), v3(a + 6)));
        } else if (f == "sample_uniform_disk") {
            const auto d = sample_uniform_disk(V2<double>(in[2 * i], in[2 * i + 1]));
            out[2 * i] = d.x; out[2 * i + 1] = d.y;
        } else if (f == "sample_cosine_weighted") {
            put3(out + 3 * i, sample_cosine_weighted(V2<double>(in[2 * i], in[2 * i + 1])));
        } else if (f == "sample_uniform_sphere") {
            put3(out + 3 * i, sample_uniform_sphere(V2<double>(in[2 * i], in[2 * i + 1])));
        } else if (f == "balance_heuristic") {
            out[i] = balance_heuristic(in[2 * i], in[2 * i + 1]);
        } else if (f == "safe_sqrt") {
            out[i] = safe_sqrt(in[i]);
        } else if (f == "transform_J") {
            out[i] = Transform<double>(M4<double>::from_colmajor(in + 16 * i)).J;
        } else if (f == "bound_isect") {
            const double* a = in + 14 * i;
            Bound<double> b;
            b.min = v3(a);
            b.max = v3(a + 3);
            const Ray<double> r{v3(a + 6), v3(a + 9)};
            // Bound::isect with the range it narrowed (math.h:143-158 isect_range)
            double tmin = a[12], tmax = a[13];
            bool hit = true;
            for (int k = 0; k < 3 && hit; k++) {
                const double vd = 1.0 / r.d[k];
                double t1 = (b.min[k] - r.o[k]) * vd, t2 = (b.max[k] - r.o[k]) * vd;
                if (vd < 0) std::swap(t1, t2);
                tmin = t1 < tmin ? tmin : t1;
                tmax = tmax < t2 ? tmax : t2;
                if (tmax < tmin) hit = false;
            }
            if (hit != b.isect(r, a[12], a[13], false)) return fail("isect and isect_range disagree");
            out[3 * i] = hit ? 1 : 0; out[3 * i + 1] = tmin; out[3 * i + 2] = tmax;
        } else {
            return fail("unknown function");
        }
    }
    return 0;
}

int lmo_dist2_eval(const double* v, int cols, int rows, long long n, const double* uvq, const double* u4,
                   double* pdf_out, double* sample_out) {
    Dist2<double> d;
    d.init(std::vector<double>(v, v + size_t(cols) * rows), cols, rows);
    for (long long i = 0; i < n; i++) {
        pdf_out[i] = d.pdf(uvq[2 * i], uvq[2 * i + 1]);
        const auto s = d.sample(u4[4 * i], u4[4 * i + 1], u4[4 * i + 2], u4[4 * i + 3]);
        sample_out[2 * i] = s.x; sample_out[2 * i + 1] = s.y;
    }
    return 0;
}

namespace {
// Every Material query of m over n records with the layout of the reference library's
// lmref_material_query.
void material_records(const Material<double>& m, const double* rec, long long n, double* out) {
    using V = V3<double>;
    auto v3 = [](const double* p) { return V(p[0], p[1], p[2]); };
    auto put3 = [](double* o, V v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; };
    for (long long i = 0; i < n; i++) {
        const double* r = rec + 26 * i;
        double* o = out + 18 * i;
        const auto g = PointGeometry<double>::make_on_surface(v3(r), v3(r + 3), v3(r + 6), V2<double>(r[9], r[10]));
        const V wi = v3(r + 11), wo = v3(r + 14);
        const int comp = int(r[17]);
        const auto td = r[18] != 0 ? TransDir::EL : TransDir::LE;
        const bool ed = r[19] != 0;
        put3(o, m.eval(g, wi, wo, comp, td, ed));
        o[3] = m.pdf_direction(g, wi, wo, comp, ed);
        const auto s = m.sample_direction(V2<double>(r[20], r[21]), V2<double>(r[22], r[23]), g, wi, comp, td);
        o[4] = s ? 1 : 0;
        put3(o + 5, s ? s->wo : V());
        put3(o + 8, s ? s->weight : V());
        const auto cs = m.sample_component(V2<double>(r[24], r[25]), g, wi);
        o[11] = cs.comp;
        o[12] = cs.weight;
        o[13] = m.pdf_component(comp, g, wi);
        put3(o + 14, m.reflectance(g).value_or(V()));
        o[17] = m.is_specular_component(comp) ? 1 : 0;
    }
}
}  // namespace

// Every Material query of the restated material `type` (parameters as lmo_add_material) in double,
// over n records with the layout of the reference library's lmref_material_query.
int lmo_material_query(int type, const double* prm, const double* rec, long long n, double* out) {
    using V = V3<double>;
    auto v3 = [](const double* p) { return V(p[0], p[1], p[2]); };
    Material<double> m;
    m.type = type;
    if (type == MAT_DIFFUSE) m.Kd = v3(prm);
    if (type == MAT_GLOSSY) { m.Ks = v3(prm); m.ax = prm[3]; m.ay = prm[4]; }
    if (type == MAT_GLASS) m.Ni = prm[0];
    material_records(m, rec, n, out);
    return 0;
}

// The same queries on material `mat` of a double-precision scene, with the textures bound to it.
int lmo_scene_material_query(void* p, int mat, const double* rec, long long n, double* out) {
    auto* h = static_cast<Handle*>(p);
    if (!h->dbl) return fail("material queries need a double-precision scene");
    if (mat < 0 || mat >= int(h->sd->materials.size())) return fail("material index out of range");
    material_records(h->sd->materials[size_t(mat)], rec, n, out);
    return 0;
}

// Texture `tex` of a double-precision scene at n texture coordinates (uv[2] each). Out, 5 per
// point: eval[3], eval_alpha (0 without alpha), has_alpha.
int lmo_texture_query(void* p, int tex, const double* uv, long long n, double* out) {
    auto* h = static_cast<Handle*>(p);
    if (!h->dbl) return fail("texture queries need a double-precision scene");
    if (tex < 0 || tex >= int(h->sd->textures.size())) return fail("texture index out of range");
    const auto& t = *h->sd->textures[size_t(tex)];
    const bool a = t.has_alpha();
    for (long long i = 0; i < n; i++) {
        const V2<double> q(uv[2 * i], uv[2 * i + 1]);
        const auto v = t.eval(q);
        out[5 * i] = v.x; out[5 * i + 1] = v.y; out[5 * i + 2] = v.z;
        out[5 * i + 3] = a ? t.eval_alpha(q) : 0;
        out[5 * i + 4] = a ? 1 : 0;
    }
    return 0;
}

// Light queries of a built double-precision scene that holds exactly one light, over records with
// the layout of the reference library's lmref_light_query: direct sampling toward a shading point
// (with its pdf and the emitted radiance) and emission sampling, as path.h's sample_direct and
// sample_primary_ray call them for that light.
int lmo_light_query(void* p, const double* rec, long long n, double* out) {
    auto* h = static_cast<Handle*>(p);
    if (!h->dbl) return fail("light queries need a double-precision scene");
    auto& S = *h->sd;
    if (!S.built || S.num_lights() != 1) return fail("light queries need a built scene with one light");
    using V = V3<double>;
    auto v3 = [](const double* q) { return V(q[0], q[1], q[2]); };
    auto put3 = [](double* o, V v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; };
    const auto& lpi = S.lights_.at(0);
    const auto& L = S.light_of(lpi.index);
    try {
        for (long long i = 0; i < n; i++) {
            const double* r = rec + 14 * i;
            double* o = out + 33 * i;
            std::fill(o, o + 33, 0.0);
            SceneInteraction<double> sp;
            sp.type = SI_Surface;
            sp.geom = PointGeometry<double>::make_on_surface(v3(r), v3(r + 3), v3(r + 6), V2<double>());
            const double u8[8] = {r[9], r[10], 0.0, r[11], r[12], r[13], 0.0, 0.0};
            int node = -1;
            if (const auto sd = S.sample_direct_light(u8, sp, node)) {
                o[0] = 1;
                put3(o + 1, sd->geom.p); put3(o + 4, sd->geom.n); put3(o + 7, sd->geom.wo);
                put3(o + 10, sd->wo); put3(o + 13, sd->weight);
                o[16] = L.pdf_direct(sp.geom, sd->geom, lpi.tr, sd->wo);
                put3(o + 17, L.eval(sd->geom, sd->wo));
            }
            if (const auto sr = S.sample_primary_ray_light(u8)) {
                o[20] = 1;
                put3(o + 21, sr->geom.p); put3(o + 24, sr->geom.n); put3(o + 27, sr->wo); put3(o + 30, sr->weight);
            }
        }
    } catch (const std::exception& e) {
        return fail(e.what());
    }
    return 0;
}

// The restated camera::pinhole in double over records with the layout of the reference library's
// lmref_camera_query.
int lmo_camera_query(const double* prm, const double* rec, long long n, double* out) {
    using V = V3<double>;
    auto v3 = [](const double* q) { return V(q[0], q[1], q[2]); };
    auto put3 = [](double* o, V v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; };
    Camera<double> cam;
    cam.construct(v3(prm), v3(prm + 3), v3(prm + 6), prm[9], prm[10]);
    for (long long i = 0; i < n; i++) {
        const double* r = rec + 11 * i;
        double* o = out + 21 * i;
        std::fill(o, o + 21, 0.0);
        const auto ray = cam.primary_ray(V2<double>(r[0], r[1]));
        put3(o, ray.o);
        put3(o + 3, ray.d);
        const V wo = v3(r + 2);
        if (const auto rp = cam.raster_position(wo)) {
            o[6] = 1; o[7] = rp->x; o[8] = rp->y;
        }
        o[9] = cam.pdf_direction(wo);
        put3(o + 10, cam.eval(wo));
        const auto g = PointGeometry<double>::make_on_surface(v3(r + 5), v3(r + 8));
        if (const auto sd = cam.sample_direct(g)) {
            o[13] = 1;
            put3(o + 14, sd->wo);
            put3(o + 17, sd->weight);
            o[20] = cam.pdf_direct(g, sd->geom);
        }
    }
    return 0;
}

// n uniforms of the restated reference Rng (RngMT), double or float flavour.
int lmo_rng_mt(unsigned int seed, int as_float, long long n, double* out) {
    RngMT r(seed, as_float != 0);
    for (long long i = 0; i < n; i++) out[i] = r.u();
    return 0;
}

}  // extern "C"

extern "C" void lmo_philox4x32(unsigned int c0, unsigned int c1, unsigned int c2, unsigned int c3, unsigned int k0,
                               unsigned int k1, unsigned int* out4) {
    const Philox4 r = philox4x32_10(c0, c1, c2, c3, k0, k1);
    for (int i = 0; i < 4; i++) out4[i] = r.v[i];
}

// Oracle (test infrastructure only): C entry points into the reference's own code, compiled from
// its sources (src/accel/accel_sahbvh.cpp, src/material/material_{diffuse,glossy,glass,mirror}.cpp,
// src/light/light_{area,envconst,point,directional}.cpp, src/camera/camera_pinhole.cpp,
// include/lm/math.h and
// include/lm/surface.h, unmodified) into
// oracle/_ref/liblmref.so by oracle/Makefile's `ref` target. Tests call them through ctypes to
// check the CPU restatement (liblmoracle.so) against the reference itself, and
// tests/golden/make_ref_fixtures.py records reference hits that the GPU tests compare with.
//
// The scene here is the part of the reference's Scene_ that an accel's build sees: a node graph
// whose node 0 is the root group, group nodes with optional local transforms, and primitive nodes
// holding a mesh::raw-style indexed triangle mesh. Traversal follows src/scene.cpp:216-230
// (depth first, children in insertion order, global = parent global * local).
#include <pch.h>
#include <lm/core.h>
#include <lm/accel.h>
#include <lm/scene.h>
#include <lm/mesh.h>
#include <lm/material.h>
#include <lm/light.h>
#include <lm/camera.h>

#include <chrono>
#include <cstring>
#include <omp.h>

using namespace lm;

namespace {

thread_local std::string g_err;

// src/mesh/mesh_raw.cpp:70-85: triangles are three indexed positions per face.
class RawMesh final : public Mesh {
public:
    std::vector<Vec3> ps;
    std::vector<int> fs;
    void foreach_triangle(const ProcessTriangleFunc& f) const override {
        for (int fi = 0; fi < int(fs.size()) / 3; fi++) f(fi, triangle_at(fi));
    }
    Tri triangle_at(int face) const override {
        Tri t;
        t.p1.p = ps.at(fs.at(3 * face));
        t.p2.p = ps.at(fs.at(3 * face + 1));
        t.p3.p = ps.at(fs.at(3 * face + 2));
        return t;
    }
    int num_triangles() const override { return int(fs.size()) / 3; }
};

class GraphScene final : public Scene {
public:
    std::vector<SceneNode> nodes;
    std::vector<std::unique_ptr<RawMesh>> meshes;
    std::vector<int> parents;  // each node is attached at most once
    std::unique_ptr<Accel> accel;
    std::vector<long long> tri_offset;  // per node: first flattened triangle, -1 for non-meshes

    GraphScene() {
        SceneNode root{};
        root.type = SceneNodeType::Group;
        root.index = 0;
        nodes.push_back(root);
        parents.push_back(-1);
    }
    void traverse_primitive_nodes(const NodeTraverseFunc& traverse_func) const override {
        std::function<void(int, Mat4)> visit = [&](int index, Mat4 global_transform) {
            const auto& node = nodes.at(index);
            traverse_func(node, global_transform);
            if (node.type == SceneNodeType::Group) {
                const auto M = node.group.local_transform ? global_transform * *node.group.local_transform
                                                          : global_transform;
                for (int child : node.group.children) visit(child, M);
            }
        };
        visit(0, Mat4(1_f));
    }
};

GraphScene* S(void* p) { return static_cast<GraphScene*>(p); }

template <typename Fn> int guarded(Fn&& fn) {
    try {
        return fn();
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

Vec3 v3(const double* p) { return Vec3(p[0], p[1], p[2]); }
void put3(double* o, Vec3 v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }

}  // namespace

extern "C" {

const char* lmref_last_error() { return g_err.c_str(); }

void* lmref_scene_create() { return new GraphScene(); }
void lmref_scene_destroy(void* p) { delete S(p); }

// Mesh from float positions (nps x 3) and position indices (nf x 3); returns its id.
int lmref_scene_add_mesh(void* p, const float* ps, int nps, const int* fp, int nf) {
    return guarded([&] {
        auto m = std::make_unique<RawMesh>();
        m->ps.reserve(nps);
        for (int i = 0; i < nps; i++) m->ps.emplace_back(Float(ps[3 * i]), Float(ps[3 * i + 1]), Float(ps[3 * i + 2]));
        m->fs.assign(fp, fp + 3 * size_t(nf));
        for (int i : m->fs)
            if (i < 0 || i >= nps) throw std::out_of_range("face index out of range");
        S(p)->meshes.push_back(std::move(m));
        return int(S(p)->meshes.size()) - 1;
    });
}

int lmref_scene_primitive(void* p, int mesh) {
    return guarded([&] {
        auto* s = S(p);
        SceneNode n{};
        n.type = SceneNodeType::Primitive;
        n.index = int(s->nodes.size());
        n.primitive.mesh = mesh >= 0 ? s->meshes.at(mesh).get() : nullptr;
        s->nodes.push_back(n);
        s->parents.push_back(-1);
        return n.index;
    });
}

// Group node; m16 (column-major) or null for a group without a local transform.
int lmref_scene_group(void* p, const double* m16) {
    return guarded([&] {
        auto* s = S(p);
        SceneNode n{};
        n.type = SceneNodeType::Group;
        n.index = int(s->nodes.size());
        if (m16) {
            Mat4 M;
            for (int c = 0; c < 4; c++) M[c] = Vec4(m16[4 * c], m16[4 * c + 1], m16[4 * c + 2], m16[4 * c + 3]);
            n.group.local_transform = M;
        }
        s->nodes.push_back(n);
        s->parents.push_back(-1);
        return n.index;
    });
}

int lmref_scene_add_child(void* p, int parent, int child) {
    return guarded([&] {
        auto* s = S(p);
        if (s->nodes.at(parent).type != SceneNodeType::Group) throw std::invalid_argument("parent is not a group");
        if (child <= 0 || s->parents.at(child) >= 0) throw std::invalid_argument("node already attached");
        s->parents[child] = parent;
        s->nodes[parent].group.children.push_back(child);
        return 0;
    });
}

// Builds the accel registered under `key` (e.g. "accel::sahbvh") over the scene.
int lmref_accel_build(void* p, const char* key, double* secs) {
    return guarded([&] {
        auto* s = S(p);
        std::unique_ptr<Component> c(refshim::create(key));
        auto* a = dynamic_cast<Accel*>(c.get());
        if (!a) throw std::invalid_argument(std::string("no accel registered as ") + key);
        c.release();
        s->accel.reset(a);
        s->tri_offset.assign(s->nodes.size(), -1);
        long long off = 0;
        s->traverse_primitive_nodes([&](const SceneNode& n, Mat4) {
            if (n.type != SceneNodeType::Primitive || !n.primitive.mesh) return;
            s->tri_offset[n.index] = off;
            off += n.primitive.mesh->num_triangles();
        });
        const auto t0 = std::chrono::steady_clock::now();
        s->accel->build(*s);
        if (secs) *secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return 0;
    });
}

// Accel::intersect over n rays (n x 8 floats: ox oy oz tmin dx dy dz tmax). Outputs per ray: t, u,
// v, the primitive node, the face and the flattened triangle index (traversal order; -1 = miss).
int lmref_accel_intersect(void* p, const float* rays, long long n, double* t, double* uv, int* prim, int* face,
                          long long* tri, int nthreads) {
    auto* s = S(p);
    if (!s->accel) { g_err = "accel not built"; return -1; }
    int rc = 0;
    const int nth = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nth)
    for (long long i = 0; i < n; i++) {
        const float* r = rays + 8 * i;
        const Ray ray{Vec3(r[0], r[1], r[2]), Vec3(r[4], r[5], r[6])};
        try {
            const auto h = s->accel->intersect(ray, Float(r[3]), Float(r[7]));
            if (h) {
                t[i] = h->t; uv[2 * i] = h->uv.x; uv[2 * i + 1] = h->uv.y;
                prim[i] = h->primitive; face[i] = h->face;
                tri[i] = s->tri_offset.at(h->primitive) + h->face;
            } else {
                t[i] = 0; uv[2 * i] = 0; uv[2 * i + 1] = 0; prim[i] = -1; face[i] = -1; tri[i] = -1;
            }
        } catch (const std::exception& e) {
#pragma omp critical
            { g_err = e.what(); rc = -1; }
        }
    }
    return rc;
}

// math.h helpers over n records of fixed width (see the table in tests/test_oracle_ref_pin.py).
int lmref_math_eval(const char* fn, const double* in, long long n, double* out) {
    return guarded([&] {
        const std::string f(fn);
        for (long long i = 0; i < n; i++) {
            if (f == "reflection") {
                const double* a = in + 6 * i;
                put3(out + 3 * i, math::reflection(v3(a), v3(a + 3)));
            } else if (f == "refraction") {
                const double* a = in + 7 * i;
                const auto r = math::refraction(v3(a), v3(a + 3), a[6]);
                put3(out + 4 * i, r.wt);
                out[4 * i + 3] = r.total ? 1 : 0;
            } else if (f == "orthonormal_basis") {
                const auto [u, v] = math::orthonormal_basis(v3(in + 3 * i));
                put3(out + 6 * i, u);
                put3(out + 6 * i + 3, v);
            } else if (f == "geometry_normal") {
                const double* a = in + 9 * i;
                put3(out + 3 * i, math::geometry_normal(v3(a), v3(a + 3), v3(a + 6)));
            } else if (f == "sample_uniform_disk") {
                const auto d = math::sample_uniform_disk(Vec2(in[2 * i], in[2 * i + 1]));
                out[2 * i] = d.x; out[2 * i + 1] = d.y;
            } else if (f == "sample_cosine_weighted") {
                put3(out + 3 * i, math::sample_cosine_weighted(Vec2(in[2 * i], in[2 * i + 1])));
            } else if (f == "sample_uniform_sphere") {
                put3(out + 3 * i, math::sample_uniform_sphere(Vec2(in[2 * i], in[2 * i + 1])));
            } else if (f == "balance_heuristic") {
                out[i] = math::balance_heuristic(in[2 * i], in[2 * i + 1]);
            } else if (f == "safe_sqrt") {
                out[i] = math::safe_sqrt(in[i]);
            } else if (f == "transform_J") {
                Mat4 M;
                for (int c = 0; c < 4; c++)
                    M[c] = Vec4(in[16 * i + 4 * c], in[16 * i + 4 * c + 1], in[16 * i + 4 * c + 2], in[16 * i + 4 * c + 3]);
                out[i] = Transform(M).J;
            } else if (f == "bound_isect") {
                // min3 max3 o3 d3 tmin tmax -> hit, tmin', tmax' (Bound::isect_range)
                const double* a = in + 14 * i;
                Bound b;
                b.min = v3(a);
                b.max = v3(a + 3);
                Float tmin = a[12], tmax = a[13];
                const bool hit = b.isect_range(Ray{v3(a + 6), v3(a + 9)}, tmin, tmax);
                out[3 * i] = hit ? 1 : 0; out[3 * i + 1] = tmin; out[3 * i + 2] = tmax;
            } else {
                throw std::invalid_argument("unknown function " + f);
            }
        }
        return 0;
    });
}

// A material component created under its key with its properties: diffuse Kd[3]; glossy Ks[3],
// ax, ay; glass Ni; mirror none. Returns a handle for lmref_material_query.
void* lmref_material_create(const char* key, const double* prm) {
    try {
        const std::string k(key);
        Json j;
        if (k == "material::diffuse") j.set("Kd", {prm[0], prm[1], prm[2]});
        else if (k == "material::glossy") { j.set("Ks", {prm[0], prm[1], prm[2]}); j.set("ax", {prm[3]}); j.set("ay", {prm[4]}); }
        else if (k == "material::glass") j.set("Ni", {prm[0]});
        std::unique_ptr<Component> c(refshim::create(k));
        if (!dynamic_cast<Material*>(c.get())) throw std::invalid_argument("no material registered as " + k);
        c->construct(j);
        return c.release();
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}
void lmref_material_destroy(void* m) { delete static_cast<Component*>(m); }

// Every Material query over n records of 26 doubles: p[3] n[3] gn[3] t[2] wi[3] wo[3] comp
// trans_dir(0 = LE, 1 = EL) eval_delta ud[2] udc[2] uc[2]. Out, 18 per record: eval[3]
// pdf_direction, sample_direction (valid, wo[3], weight[3]), sample_component (comp, weight),
// pdf_component, reflectance[3], is_specular_component.
int lmref_material_query(void* mp, const double* rec, long long n, double* out) {
    return guarded([&] {
        const auto* m = dynamic_cast<const Material*>(static_cast<Component*>(mp));
        if (!m) throw std::invalid_argument("not a material");
        for (long long i = 0; i < n; i++) {
            const double* r = rec + 26 * i;
            double* o = out + 18 * i;
            const auto g = PointGeometry::make_on_surface(v3(r), v3(r + 3), v3(r + 6), Vec2(r[9], r[10]));
            const Vec3 wi = v3(r + 11), wo = v3(r + 14);
            const int comp = int(r[17]);
            const auto td = r[18] != 0 ? Material::TransDir::EL : Material::TransDir::LE;
            const bool ed = r[19] != 0;
            put3(o, m->eval(g, wi, wo, comp, td, ed));
            o[3] = m->pdf_direction(g, wi, wo, comp, ed);
            const auto s = m->sample_direction({Vec2(r[20], r[21]), Vec2(r[22], r[23])}, g, wi, comp, td);
            o[4] = s ? 1 : 0;
            put3(o + 5, s ? s->wo : Vec3());
            put3(o + 8, s ? s->weight : Vec3());
            const auto cs = m->sample_component({Vec2(r[24], r[25])}, g, wi);
            o[11] = cs.comp;
            o[12] = cs.weight;
            o[13] = m->pdf_component(comp, g, wi);
            put3(o + 14, m->reflectance(g));
            o[17] = m->is_specular_component(comp) ? 1 : 0;
        }
        return 0;
    });
}

// A light component under its key: area Ke[3] over mesh `mesh` of the scene; envconst Le[3];
// point Le[3], position[3]; directional Le[3], direction[3]. Its scene bound is the bound of the
// scene's transformed triangles (src/scene.cpp:288-311).
void* lmref_light_create(void* scene, const char* key, const double* prm, int mesh) {
    try {
        auto* s = S(scene);
        const std::string k(key);
        Json j;
        if (k == "light::area") {
            j.set("Ke", {prm[0], prm[1], prm[2]});
            refshim::add_named("lmref_light_mesh", s->meshes.at(mesh).get());
            j.set_str("mesh", "lmref_light_mesh");
        } else {
            j.set("Le", {prm[0], prm[1], prm[2]});
            if (k == "light::point") j.set("position", {prm[3], prm[4], prm[5]});
            if (k == "light::directional") j.set("direction", {prm[3], prm[4], prm[5]});
        }
        std::unique_ptr<Component> c(refshim::create(k));
        auto* L = dynamic_cast<Light*>(c.get());
        if (!L) throw std::invalid_argument("no light registered as " + k);
        c->construct(j);
        Bound bound;
        s->traverse_primitive_nodes([&](const SceneNode& node, Mat4 global_transform) {
            if (node.type != SceneNodeType::Primitive || !node.primitive.mesh) return;
            node.primitive.mesh->foreach_triangle([&](int, const Mesh::Tri& tri) {
                bound = merge(bound, Vec3(global_transform * Vec4(tri.p1.p, 1_f)));
                bound = merge(bound, Vec3(global_transform * Vec4(tri.p2.p, 1_f)));
                bound = merge(bound, Vec3(global_transform * Vec4(tri.p3.p, 1_f)));
            });
        });
        L->set_scene_bound(bound);
        return c.release();
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}
void lmref_light_destroy(void* l) { delete static_cast<Component*>(l); }

// Light queries under the transform m16 (column-major) over n records of 14 doubles: the shading
// point p[3] n[3] gn[3], then up[2] upc ud[2]. Out, 33 per record: sample_direct (valid, geomL.p[3],
// geomL.n[3], geomL.wo[3], wo[3], weight[3]), pdf_direct at that sample, eval(geomL, wo), and
// sample_ray (valid, geomL.p[3], geomL.n[3], wo[3], weight[3]).
int lmref_light_query(void* lp, const double* m16, const double* rec, long long n, double* out) {
    return guarded([&] {
        const auto* L = dynamic_cast<const Light*>(static_cast<Component*>(lp));
        if (!L) throw std::invalid_argument("not a light");
        Mat4 M;
        for (int c = 0; c < 4; c++) M[c] = Vec4(m16[4 * c], m16[4 * c + 1], m16[4 * c + 2], m16[4 * c + 3]);
        const Transform tr(M);
        for (long long i = 0; i < n; i++) {
            const double* r = rec + 14 * i;
            double* o = out + 33 * i;
            std::fill(o, o + 33, 0.0);
            const auto g = PointGeometry::make_on_surface(v3(r), v3(r + 3), v3(r + 6));
            const Light::RaySampleU u{Vec2(r[9], r[10]), r[11], Vec2(r[12], r[13])};
            if (const auto sd = L->sample_direct(u, g, tr)) {
                o[0] = 1;
                put3(o + 1, sd->geom.p); put3(o + 4, sd->geom.n); put3(o + 7, sd->geom.wo);
                put3(o + 10, sd->wo); put3(o + 13, sd->weight);
                o[16] = L->pdf_direct(g, sd->geom, tr, sd->wo, false);
                put3(o + 17, L->eval(sd->geom, sd->wo, false));
            }
            if (const auto sr = L->sample_ray(u, tr)) {
                o[20] = 1;
                put3(o + 21, sr->geom.p); put3(o + 24, sr->geom.n); put3(o + 27, sr->wo); put3(o + 30, sr->weight);
            }
        }
        return 0;
    });
}

// camera::pinhole from position[3], center[3], up[3], vfov, aspect, over n records of 11 doubles:
// a raster position rp[2], a direction wo[3], a scene point p[3] n[3]. Out, 21 per record:
// primary_ray(rp) (o[3], d[3]); raster_position(wo) (valid, rp[2]); pdf_direction(wo); eval(wo)[3];
// sample_direct toward the point (valid, wo[3], weight[3]) and its pdf_direct.
int lmref_camera_query(const double* prm, const double* rec, long long n, double* out) {
    return guarded([&] {
        Json j;
        j.set("position", {prm[0], prm[1], prm[2]});
        j.set("center", {prm[3], prm[4], prm[5]});
        j.set("up", {prm[6], prm[7], prm[8]});
        j.set("vfov", {prm[9]});
        j.set("aspect", {prm[10]});
        std::unique_ptr<Component> c(refshim::create("camera::pinhole"));
        auto* cam = dynamic_cast<Camera*>(c.get());
        if (!cam) throw std::invalid_argument("no camera::pinhole registered");
        c->construct(j);
        for (long long i = 0; i < n; i++) {
            const double* r = rec + 11 * i;
            double* o = out + 21 * i;
            std::fill(o, o + 21, 0.0);
            const auto ray = cam->primary_ray(Vec2(r[0], r[1]));
            put3(o, ray.o);
            put3(o + 3, ray.d);
            const Vec3 wo = v3(r + 2);
            if (const auto rp = cam->raster_position(wo)) {
                o[6] = 1; o[7] = rp->x; o[8] = rp->y;
            }
            const auto g0 = PointGeometry::make_degenerated(Vec3());
            o[9] = cam->pdf_direction(g0, wo);
            put3(o + 10, cam->eval(wo));
            const auto g = PointGeometry::make_on_surface(v3(r + 5), v3(r + 8));
            if (const auto sd = cam->sample_direct({Vec2()}, g)) {
                o[13] = 1;
                put3(o + 14, sd->wo);
                put3(o + 17, sd->weight);
                o[20] = cam->pdf_direct(g, sd->geom, sd->wo);
            }
        }
        return 0;
    });
}

// Dist2 (math.h:378-432) over a cols x rows table: pdf at n (u, v) points and n samples from
// n 4-tuples of uniforms.
int lmref_dist2_eval(const double* v, int cols, int rows, long long n, const double* uvq, const double* u4,
                     double* pdf_out, double* sample_out) {
    return guarded([&] {
        Dist2 d;
        d.init(std::vector<Float>(v, v + size_t(cols) * rows), cols, rows);
        for (long long i = 0; i < n; i++) {
            pdf_out[i] = d.pdf(uvq[2 * i], uvq[2 * i + 1]);
            const auto s = d.sample(Vec4(u4[4 * i], u4[4 * i + 1], u4[4 * i + 2], u4[4 * i + 3]));
            sample_out[2 * i] = s.x; sample_out[2 * i + 1] = s.y;
        }
        return 0;
    });
}

// The reference's Rng (math.h:204-271): n uniforms from Rng(seed), double or float flavour.
int lmref_rng(int seed, int as_float, long long n, double* out) {
    return guarded([&] {
        if (as_float) {
            detail::RngImpl<float> r(seed);
            for (long long i = 0; i < n; i++) out[i] = double(r.u());
        } else {
            detail::RngImpl<double> r(seed);
            for (long long i = 0; i < n; i++) out[i] = r.u();
        }
        return 0;
    });
}

}  // extern "C"

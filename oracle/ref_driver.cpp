// Oracle (test infrastructure only): C entry points into the reference's own code, compiled from
// its sources, unmodified, into oracle/_ref/liblmref.so by oracle/Makefile's `ref` target:
// src/scene.cpp, src/accel/accel_sahbvh.cpp, src/mesh/mesh_raw.cpp,
// src/material/material_{diffuse,glossy,glass,mirror}.cpp,
// src/light/light_{area,envconst,point,directional}.cpp, src/camera/camera_pinhole.cpp,
// src/film/film_bitmap.cpp, src/scheduler.cpp, src/renderer/renderer_{pt,lt,bdpt}.cpp, and the
// headers they include (math.h, surface.h, scene.h, path.h, bidir.h, ...). Tests call them through
// ctypes (oracle/ref.py) to check the CPU restatement (liblmoracle.so) against the reference
// itself, and tests/golden/make_ref_fixtures.py records reference outputs that the GPU tests
// compare with.
//
// A handle owns one reference scene (scene::default over accel::sahbvh) and the assets its nodes
// refer to, created through the component factories under locators "$.h<handle>.<name>", as the
// reference's user API does. The parallel loop the schedulers and the film call is the
// reference's OpenMP loop with one thread: indices in order, thread id 0.
#include <pch.h>
#include <lm/core.h>
#include <lm/accel.h>
#include <lm/scene.h>
#include <lm/mesh.h>
#include <lm/material.h>
#include <lm/light.h>
#include <lm/camera.h>
#include <lm/film.h>
#include <lm/renderer.h>
#include <lm/texture.h>
#include <lm/model.h>
#include <lm/objloader.h>
#include <stb/stb_image.h>
#include <lm/parallel.h>
#include <lm/progress.h>
#include <lm/debug.h>

#include <chrono>
#include <cstring>
#include <omp.h>

using namespace lm;

// ------------------------------------------------------------------------------------------------
// The reference's parallel, progress and debug entry points (src/parallel.cpp, src/progress.cpp
// and src/debug.cpp dispatch to configurable backends): a sequential loop with thread id 0, no
// progress reports, no debug polling.

LM_NAMESPACE_BEGIN(LM_NAMESPACE)
LM_NAMESPACE_BEGIN(parallel)
void init(const std::string&, const Json&) {}
void shutdown() {}
int num_threads() { return 1; }
bool main_thread() { return true; }
void foreach(long long num_samples, const ParallelProcessFunc& process_func, const ProgressUpdateFunc& progress_func) {
    for (long long i = 0; i < num_samples; i++) process_func(i, 0);
    if (progress_func) progress_func(num_samples);
}
LM_NAMESPACE_END(parallel)
LM_NAMESPACE_BEGIN(debug)
void poll(const Json&) {}
LM_NAMESPACE_END(debug)
LM_NAMESPACE_BEGIN(progress)
void init(const std::string&, const Json&) {}
void shutdown() {}
void start(ProgressMode, long long, double) {}
void end() {}
void update(long long) {}
void update_time(Float) {}
LM_NAMESPACE_END(progress)
LM_NAMESPACE_END(LM_NAMESPACE)

namespace {

thread_local std::string g_err;

// An indexed triangle mesh for scenes too large for a JSON property list (the accel's build reads
// triangles only): the triangle iteration of src/mesh/mesh_raw.cpp:70-85.
class RawMesh final : public Mesh {
public:
    std::vector<Vec3> ps;
    std::vector<int> fs;
    void foreach_triangle(const ProcessTriangleFunc& f) const override {
        for (int fi = 0; fi < int(fs.size()) / 3; fi++) f(fi, triangle_at(fi));
    }
    Tri triangle_at(int face) const override {
        Tri t{};
        t.p1.p = ps.at(fs.at(3 * face));
        t.p2.p = ps.at(fs.at(3 * face + 1));
        t.p3.p = ps.at(fs.at(3 * face + 2));
        return t;
    }
    InterpolatedPoint surface_point(int, Vec2) const override {
        throw std::runtime_error("RawMesh holds positions only; render with mesh::raw meshes");
    }
    int num_triangles() const override { return int(fs.size()) / 3; }
};

struct Handle {
    int id = 0;
    std::vector<std::unique_ptr<Component>> assets;  // owned; registered by locator
    std::vector<std::string> locs;
    std::vector<int> mesh_assets;                    // mesh id -> asset index
    Scene* scene = nullptr;
    Accel* accel = nullptr;
    int scene_asset = -1;
    std::string default_material;
    std::vector<long long> tri_offset;               // per node: first flattened triangle

    ~Handle() {
        for (const auto& l : locs) refshim::remove_named(l);
    }
    std::string loc(const std::string& name) const { return "$.h" + std::to_string(id) + "." + name; }
    int add(const std::string& name, std::unique_ptr<Component> c) {
        if (!c) throw std::invalid_argument("no component registered for " + name);
        const auto l = loc(name);
        refshim::add_named(l, c.get());
        locs.push_back(l);
        assets.push_back(std::move(c));
        return int(assets.size()) - 1;
    }
    // Registered by locator before construct(), as assetgroup.cpp:62-86 does: a model's
    // construct() hands its own locator's children (meshes, textures) to the lights and
    // materials it creates.
    template <typename T> int create(const std::string& key, const std::string& name, const Json& prop) {
        std::unique_ptr<Component> c(refshim::make(key));
        if (!c || !dynamic_cast<T*>(c.get())) throw std::invalid_argument("cannot create " + key);
        c->lmref_set_ids(key, loc(name));
        const int id = add(name, std::move(c));
        try {
            assets.back()->construct(prop);
        } catch (...) {
            refshim::remove_named(locs.back());
            locs.pop_back();
            assets.pop_back();
            throw;
        }
        return id;
    }
    std::string next_name() const { return "asset" + std::to_string(assets.size()); }
    const std::string& asset_loc(int i) const { return locs.at(size_t(i)); }
};

int g_next_handle = 0;

// objloader::init (objloader.cpp:13-15) runs once, as lm::init does (user.cpp:59).
bool& objloader_ready() {
    static bool r = false;
    return r;
}

Handle* H(void* p) { return static_cast<Handle*>(p); }

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
Json arr(const float* v, long long n) {
    Json j = Json::array();
    for (long long i = 0; i < n; i++) j.push_back(Json(double(v[i])));
    return j;
}
Json arr(const int* v, long long n) {
    Json j = Json::array();
    for (long long i = 0; i < n; i++) j.push_back(Json(v[i]));
    return j;
}
Mat4 mat4(const double* m16) {
    Mat4 M;
    for (int c = 0; c < 4; c++) M[c] = Vec4(m16[4 * c], m16[4 * c + 1], m16[4 * c + 2], m16[4 * c + 3]);
    return M;
}
Json camera_prop(const double* prm) {
    return Json{{"position", v3(prm)}, {"center", v3(prm + 3)}, {"up", v3(prm + 6)}, {"vfov", prm[9]}, {"aspect", prm[10]}};
}

void material_records(const Material* m, const double* rec, long long n, double* out) {
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
}

}  // namespace

extern "C" {

const char* lmref_last_error() { return g_err.c_str(); }

// ------------------------------------------------------------------------------------------------
// Scene and assets

void* lmref_scene_create() {
    try {
        auto h = std::make_unique<Handle>();
        h->id = g_next_handle++;
        const int a = h->create<Accel>("accel::sahbvh", "accel", Json::object());
        h->accel = dynamic_cast<Accel*>(h->assets[a].get());
        h->scene_asset = h->create<Scene>("scene::default", "scene", Json{{"accel", h->asset_loc(a)}});
        h->scene = dynamic_cast<Scene*>(h->assets[h->scene_asset].get());
        const int m = h->create<Material>("material::diffuse", "default_material", Json{{"Kd", Vec3(1_f)}});
        h->default_material = h->asset_loc(m);
        return h.release();
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}
void lmref_scene_destroy(void* p) { delete H(p); }

// Mesh from float positions (nps x 3) and position indices (nf x 3), for the accel only.
int lmref_scene_add_mesh(void* p, const float* ps, int nps, const int* fp, int nf) {
    return guarded([&] {
        auto* h = H(p);
        auto m = std::make_unique<RawMesh>();
        m->ps.reserve(size_t(nps));
        for (int i = 0; i < nps; i++) m->ps.emplace_back(Float(ps[3 * i]), Float(ps[3 * i + 1]), Float(ps[3 * i + 2]));
        m->fs.assign(fp, fp + 3 * size_t(nf));
        for (int i : m->fs)
            if (i < 0 || i >= nps) throw std::out_of_range("face index out of range");
        const int id = int(h->mesh_assets.size());
        const auto name = "mesh" + std::to_string(id);
        m->lmref_set_ids("mesh::positions", h->loc(name));
        h->mesh_assets.push_back(h->add(name, std::move(m)));
        return id;
    });
}

// mesh::raw (src/mesh/mesh_raw.cpp) from its properties: ps, ns, ts and per-corner indices.
int lmref_scene_add_mesh_raw(void* p, const float* ps, int nps, const float* ns, int nns, const float* ts, int nts,
                             const int* fp, const int* ft, const int* fn, int ncorners) {
    return guarded([&] {
        auto* h = H(p);
        Json fs = Json::object();
        fs["p"] = arr(fp, ncorners);
        fs["t"] = arr(ft, ncorners);
        fs["n"] = arr(fn, ncorners);
        Json prop = Json::object();
        prop["ps"] = arr(ps, 3LL * nps);
        prop["ns"] = arr(ns, 3LL * nns);
        prop["ts"] = arr(ts, 2LL * nts);
        prop["fs"] = fs;
        const int id = int(h->mesh_assets.size());
        h->mesh_assets.push_back(h->create<Mesh>("mesh::raw", "mesh" + std::to_string(id), prop));
        return id;
    });
}

// Materials: diffuse Kd[3]; glossy Ks[3], ax, ay; glass Ni; mirror none. Returns an asset id.
int lmref_scene_add_material(void* p, const char* key, const double* prm) {
    return guarded([&] {
        auto* h = H(p);
        const std::string k(key);
        Json j = Json::object();
        if (k == "material::diffuse") j["Kd"] = Vec3(prm[0], prm[1], prm[2]);
        else if (k == "material::glossy") { j["Ks"] = Vec3(prm[0], prm[1], prm[2]); j["ax"] = prm[3]; j["ay"] = prm[4]; }
        else if (k == "material::glass") j["Ni"] = prm[0];
        return h->create<Material>(k, h->next_name(), j);
    });
}

// Lights: area Ke[3] over mesh `mesh`; envconst Le[3]; point Le[3], position[3]; directional
// Le[3], direction[3]. Returns an asset id.
int lmref_scene_add_light(void* p, const char* key, const double* prm, int mesh) {
    return guarded([&] {
        auto* h = H(p);
        const std::string k(key);
        Json j = Json::object();
        if (k == "light::area") {
            j["Ke"] = Vec3(prm[0], prm[1], prm[2]);
            j["mesh"] = h->asset_loc(h->mesh_assets.at(size_t(mesh)));
        } else {
            j["Le"] = Vec3(prm[0], prm[1], prm[2]);
            if (k == "light::point") j["position"] = Vec3(prm[3], prm[4], prm[5]);
            if (k == "light::directional") j["direction"] = Vec3(prm[3], prm[4], prm[5]);
        }
        return h->create<Light>(k, h->next_name(), j);
    });
}

// camera::pinhole: position[3], center[3], up[3], vfov, aspect. Returns an asset id.
int lmref_scene_add_camera(void* p, const double* prm) {
    return guarded([&] { return H(p)->create<Camera>("camera::pinhole", H(p)->next_name(), camera_prop(prm)); });
}

// film::bitmap of w x h. Returns an asset id.
int lmref_scene_add_film(void* p, int w, int hgt) {
    return guarded([&] { return H(p)->create<Film>("film::bitmap", H(p)->next_name(), Json{{"w", w}, {"h", hgt}}); });
}

// An image for texture::bitmap under `path` (the stand-in stb_image's registry): h rows of w x c
// floats, top row first, as decoded from a file.
int lmref_register_image(const char* path, int w, int hgt, int c, const float* texels) {
    return guarded([&] {
        if (w <= 0 || hgt <= 0 || c < 3 || c > 4) throw std::invalid_argument("image shape");
        auto& im = lmref_stb::images()[lmref_stb::key(path)];
        im.w = w;
        im.h = hgt;
        im.c = c;
        im.texels.assign(texels, texels + size_t(w) * size_t(hgt) * size_t(c));
        return 0;
    });
}

// texture::bitmap (src/texture/texture_bitmap.cpp) of a registered image. Returns an asset id.
int lmref_scene_add_texture(void* p, const char* path, int flip) {
    return guarded([&] {
        return H(p)->create<Texture>("texture::bitmap", H(p)->next_name(), Json{{"path", path}, {"flip", flip != 0}});
    });
}

// A material whose texture is an asset of the scene (-1 = none): material::diffuse Kd[3] with
// mapKd; material::mixture_wavefrontobj (model_wavefrontobj.cpp:339-513) Kd[3], Ks[3], ax, ay,
// no_alpha_mask with mapKd. Returns an asset id.
int lmref_scene_add_material_tex(void* p, const char* key, const double* prm, int map_kd) {
    return guarded([&] {
        auto* h = H(p);
        const std::string k(key);
        const std::string tex = map_kd >= 0 ? h->asset_loc(map_kd) : std::string();
        Json j = Json::object();
        if (k == "material::diffuse") {
            j["Kd"] = v3(prm);
            if (map_kd >= 0) j["mapKd"] = tex;
        } else if (k == "material::mixture_wavefrontobj") {
            j["Kd"] = v3(prm);
            j["Ks"] = v3(prm + 3);
            j["ax"] = prm[6];
            j["ay"] = prm[7];
            j["no_alpha_mask"] = prm[8] != 0;
            j["mapKd"] = tex;
        } else {
            throw std::invalid_argument("no textured form of " + k);
        }
        return h->create<Material>(k, h->next_name(), j);
    });
}

// light::env (src/light/light_env.cpp) over a registered image `path` (loaded flipped, as
// texture::bitmap does by default), rot in degrees, scale. Returns an asset id.
int lmref_scene_add_light_env(void* p, const char* path, double rot, double scale) {
    return guarded([&] {
        return H(p)->create<Light>("light::env", H(p)->next_name(),
                                   Json{{"path", path}, {"rot", rot}, {"scale", scale}});
    });
}

// model::wavefrontobj (src/model/model_wavefrontobj.cpp) of an OBJ file, read by the reference's
// objloader::simple (src/objloader/objloader_simple.cpp); its textures come from the image
// registry under the paths the model makes of the MTL's map_Kd. skip_specular_mat as the model's
// property; base_material an asset id or -1. Returns an asset id.
int lmref_scene_add_model(void* p, const char* path, int skip_specular_mat, int base_material) {
    return guarded([&] {
        auto* h = H(p);
        if (!objloader_ready()) {
            objloader::init();
            objloader_ready() = true;
        }
        Json j{{"path", path}, {"skip_specular_mat", skip_specular_mat != 0}};
        if (base_material >= 0) j["base_material"] = h->asset_loc(base_material);
        return h->create<Model>("model::wavefrontobj", h->next_name(), j);
    });
}

// Scene::add_child_from_model (scene.cpp:158-180): one primitive node per group of the model
// under node `parent`.
int lmref_scene_add_child_from_model(void* p, int parent, int model) {
    return guarded([&] {
        auto* h = H(p);
        const int before = h->scene->num_nodes();
        h->scene->add_child_from_model(parent, h->asset_loc(model));
        return h->scene->num_nodes() - before;
    });
}

// Texture asset `tex` at n texture coordinates (uv[2] each). Out, 5 per point: eval[3],
// eval_alpha (0 without alpha), has_alpha.
int lmref_texture_query(void* p, int tex, const double* uv, long long n, double* out) {
    return guarded([&] {
        const auto* t = dynamic_cast<const Texture*>(H(p)->assets.at(size_t(tex)).get());
        if (!t) throw std::invalid_argument("not a texture");
        const bool a = t->has_alpha();
        for (long long i = 0; i < n; i++) {
            const Vec2 q(uv[2 * i], uv[2 * i + 1]);
            put3(out + 5 * i, t->eval(q));
            out[5 * i + 3] = a ? t->eval_alpha(q) : 0;
            out[5 * i + 4] = a ? 1 : 0;
        }
        return 0;
    });
}

// Primitive node (Scene::create_primitive_node, scene.cpp:71-126) over a mesh id and material,
// light and camera asset ids (-1 = none). A mesh without a material gets a white diffuse one; a
// node with nothing gets a camera (the node a scene's camera primitive takes).
int lmref_scene_primitive_ex(void* p, int mesh, int material, int light, int camera) {
    return guarded([&] {
        auto* h = H(p);
        Json j = Json::object();
        if (mesh >= 0) {
            j["mesh"] = h->asset_loc(h->mesh_assets.at(size_t(mesh)));
            j["material"] = material >= 0 ? h->asset_loc(material) : h->default_material;
        } else if (material >= 0) {
            j["material"] = h->asset_loc(material);
        }
        if (light >= 0) j["light"] = h->asset_loc(light);
        if (camera >= 0) j["camera"] = h->asset_loc(camera);
        if (mesh < 0 && material < 0 && light < 0 && camera < 0) {
            static const double cam[11] = {0, 0, 1, 0, 0, 0, 0, 1, 0, 30, 1};
            j["camera"] = h->asset_loc(h->create<Camera>("camera::pinhole", h->next_name(), camera_prop(cam)));
        }
        return h->scene->create_primitive_node(j);
    });
}
int lmref_scene_primitive(void* p, int mesh) { return lmref_scene_primitive_ex(p, mesh, -1, -1, -1); }

// Group node; m16 (column-major) or null for an identity transform.
int lmref_scene_group(void* p, const double* m16) {
    return guarded([&] { return H(p)->scene->create_group_node(m16 ? mat4(m16) : Mat4(1_f)); });
}

int lmref_scene_add_child(void* p, int parent, int child) {
    return guarded([&] {
        auto* h = H(p);
        if (parent < 0 || parent >= h->scene->num_nodes() || child <= 0 || child >= h->scene->num_nodes())
            throw std::out_of_range("node index out of range");
        h->scene->add_child(parent, child);
        return 0;
    });
}

// Scene::build (scene.cpp:274-316): light transforms, the scene bound handed to the lights, the
// accel's build. Records each mesh node's first flattened triangle (traversal order).
int lmref_scene_build(void* p, double* secs) {
    return guarded([&] {
        auto* h = H(p);
        h->tri_offset.assign(size_t(h->scene->num_nodes()), -1);
        long long off = 0;
        h->scene->traverse_primitive_nodes([&](const SceneNode& n, Mat4) {
            if (n.type != SceneNodeType::Primitive || !n.primitive.mesh) return;
            h->tri_offset[size_t(n.index)] = off;
            off += n.primitive.mesh->num_triangles();
        });
        const auto t0 = std::chrono::steady_clock::now();
        h->scene->build();
        if (secs) *secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return 0;
    });
}

// Accel::intersect over n rays (n x 8 floats: ox oy oz tmin dx dy dz tmax). Outputs per ray: t, u,
// v, the primitive node, the face and the flattened triangle index (traversal order; -1 = miss).
int lmref_accel_intersect(void* p, const float* rays, long long n, double* t, double* uv, int* prim, int* face,
                          long long* tri, int nthreads) {
    auto* h = H(p);
    int rc = 0;
    const int nth = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nth)
    for (long long i = 0; i < n; i++) {
        const float* r = rays + 8 * i;
        const Ray ray{Vec3(r[0], r[1], r[2]), Vec3(r[4], r[5], r[6])};
        try {
            const auto hit = h->accel->intersect(ray, Float(r[3]), Float(r[7]));
            if (hit) {
                t[i] = hit->t; uv[2 * i] = hit->uv.x; uv[2 * i + 1] = hit->uv.y;
                prim[i] = hit->primitive; face[i] = hit->face;
                tri[i] = h->tri_offset.at(size_t(hit->primitive)) + hit->face;
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

// renderer::pt (src/renderer/renderer_pt.cpp) over the scene into film asset `film`: max_verts,
// seed, sampling_mode (0 naive, 1 nee, 2 mis), primary mode (0 pixel with `samples` spp, 1 image
// with `samples` samples), scheduler::{spp,spi}::sample. The render runs on a new thread, so the
// renderer's per-thread Rng starts from seed + 0. out: the film's h x w x 3 after its rescale.
int lmref_render_pt(void* p, int film, long long samples, int max_verts, unsigned int seed, int sampling_mode,
                    int primary_mode, double* out) {
    return guarded([&] {
        auto* h = H(p);
        static const char* modes[] = {"naive", "nee", "mis"};
        if (sampling_mode < 0 || sampling_mode > 2) throw std::invalid_argument("sampling mode");
        Json prop = Json::object();
        prop["scene"] = h->asset_loc(h->scene_asset);
        prop["output"] = h->asset_loc(film);
        prop["max_verts"] = max_verts;
        prop["seed"] = seed;
        prop["sampling_mode"] = modes[sampling_mode];
        prop["scheduler"] = "sample";
        prop["primary_ray_sampling_mode"] = primary_mode == 0 ? "pixel" : "image";
        if (primary_mode == 0) prop["spp"] = samples;
        else prop["num_samples"] = samples;
        auto r = comp::create<Renderer>("renderer::pt", h->loc("renderer"), prop);
        if (!r) throw std::invalid_argument("cannot create renderer::pt");
        std::string err;
        std::thread th([&] {
            try {
                r->render();
            } catch (const std::exception& e) {
                err = e.what();
            }
        });
        th.join();
        if (!err.empty()) throw std::runtime_error(err);
        auto* f = dynamic_cast<Film*>(h->assets.at(size_t(film)).get());
        const auto b = f->buffer();
        std::memcpy(out, b.data, sizeof(double) * 3 * size_t(b.w) * size_t(b.h));
        return 0;
    });
}

// renderer::raycast (src/renderer/renderer_raycast.cpp) over the scene into film asset `film`:
// background bg[3], use_constant_color, visualize_normal, and a constant color[3] when has_color.
// out: the film's h x w x 3.
int lmref_render_raycast(void* p, int film, const double* bg, int use_constant_color, int visualize_normal, int has_color,
                         const double* color, double* out) {
    return guarded([&] {
        auto* h = H(p);
        Json prop = Json::object();
        prop["scene"] = h->asset_loc(h->scene_asset);
        prop["output"] = h->asset_loc(film);
        prop["bg_color"] = v3(bg);
        prop["use_constant_color"] = use_constant_color != 0;
        prop["visualize_normal"] = visualize_normal != 0;
        if (has_color) prop["color"] = v3(color);
        auto r = comp::create<Renderer>("renderer::raycast", h->loc("renderer_raycast"), prop);
        if (!r) throw std::invalid_argument("cannot create renderer::raycast");
        r->render();
        auto* f = dynamic_cast<Film*>(h->assets.at(size_t(film)).get());
        const auto b = f->buffer();
        std::memcpy(out, b.data, sizeof(double) * 3 * size_t(b.w) * size_t(b.h));
        return 0;
    });
}

// A light-tracing renderer of the reference over the scene into film asset `film`, scheduled by
// scheduler::spi::sample over `num_samples` light paths: key "renderer::lt", "renderer::bdpt"
// (min_verts, max_verts) or one of bdpt's strategy renderers ("renderer::pt_naive_path",
// "renderer::pt_nee_path", "renderer::lt_nee_path"). One thread, Rng seeded `seed`, as
// lmref_render_pt. out: the film's h x w x 3 after its rescale.
int lmref_render_spi(void* p, const char* key, int film, long long num_samples, int min_verts, int max_verts,
                     unsigned int seed, double* out) {
    return guarded([&] {
        auto* h = H(p);
        Json prop = Json::object();
        prop["scene"] = h->asset_loc(h->scene_asset);
        prop["output"] = h->asset_loc(film);
        prop["min_verts"] = min_verts;
        prop["max_verts"] = max_verts;
        prop["seed"] = seed;
        prop["scheduler"] = "sample";
        prop["num_samples"] = num_samples;
        auto r = comp::create<Renderer>(key, h->loc("renderer"), prop);
        if (!r) throw std::invalid_argument(std::string("cannot create ") + key);
        std::string err;
        std::thread th([&] {
            try {
                r->render();
            } catch (const std::exception& e) {
                err = e.what();
            }
        });
        th.join();
        if (!err.empty()) throw std::runtime_error(err);
        auto* f = dynamic_cast<Film*>(h->assets.at(size_t(film)).get());
        const auto b = f->buffer();
        std::memcpy(out, b.data, sizeof(double) * 3 * size_t(b.w) * size_t(b.h));
        return 0;
    });
}

// ------------------------------------------------------------------------------------------------
// Components on their own

// A material component created under its key with its properties: diffuse Kd[3]; glossy Ks[3],
// ax, ay; glass Ni; mirror none. Returns a handle for lmref_material_query.
void* lmref_material_create(const char* key, const double* prm) {
    try {
        const std::string k(key);
        Json j = Json::object();
        if (k == "material::diffuse") j["Kd"] = Vec3(prm[0], prm[1], prm[2]);
        else if (k == "material::glossy") { j["Ks"] = Vec3(prm[0], prm[1], prm[2]); j["ax"] = prm[3]; j["ay"] = prm[4]; }
        else if (k == "material::glass") j["Ni"] = prm[0];
        auto c = comp::create<Material>(k, "$.lmref_material", j);
        if (!c) throw std::invalid_argument("no material registered as " + k);
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
        material_records(m, rec, n, out);
        return 0;
    });
}

// The same queries on material asset `mat` of a scene (a textured one among them).
int lmref_scene_material_query(void* p, int mat, const double* rec, long long n, double* out) {
    return guarded([&] {
        const auto* m = dynamic_cast<const Material*>(H(p)->assets.at(size_t(mat)).get());
        if (!m) throw std::invalid_argument("not a material");
        material_records(m, rec, n, out);
        return 0;
    });
}

// Light asset `light` of the scene, after lmref_scene_build handed it the scene bound. Queries
// under the transform m16 (column-major) over n records of 14 doubles: the shading point p[3]
// n[3] gn[3], then up[2] upc ud[2]. Out, 33 per record: sample_direct (valid, geomL.p[3],
// geomL.n[3], geomL.wo[3], wo[3], weight[3]), pdf_direct at that sample, eval(geomL, wo), and
// sample_ray (valid, geomL.p[3], geomL.n[3], wo[3], weight[3]).
int lmref_light_query(void* p, int light, const double* m16, const double* rec, long long n, double* out) {
    return guarded([&] {
        const auto* L = dynamic_cast<const Light*>(H(p)->assets.at(size_t(light)).get());
        if (!L) throw std::invalid_argument("not a light");
        const Transform tr(mat4(m16));
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
        auto cam = comp::create<Camera>("camera::pinhole", "$.lmref_camera", camera_prop(prm));
        if (!cam) throw std::invalid_argument("no camera::pinhole registered");
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

// math.h helpers over n records of fixed width (record layouts as lmo_math_eval's).
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
                out[i] = Transform(mat4(in + 16 * i)).J;
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

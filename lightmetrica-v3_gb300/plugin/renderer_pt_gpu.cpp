// renderer::pt_gpu -- the reference's renderer::pt (src/renderer/renderer_pt.cpp:51-315) on liblmgpu.
//
// A plugin for the reference (loaded with lm.comp.load_plugin, src/component.cpp:219-249); same
// props as renderer::pt (scene, output, max_verts, seed, sampling_mode,
// primary_ray_sampling_mode, spp). It uses only the reference's public headers and
// include/lmgpu.h, and links against liblmgpu.so. It cannot be compiled in this repository: the
// reference's dependencies (glm, nlohmann_json, cereal) are not available here.
//
// render() flattens the scene graph into an lmgpu_scene_desc: per triangle the world-space
// positions (as accel_sahbvh.cpp:132-151 flattens them), normals transformed by normal_M, the
// geometric normal and its primitive row; per primitive its material and light rows; the lights in
// traversal order (scene.cpp:279-286); the camera. Material and light parameters come from
// Component::underlying_value("gpu"), which the reference's material and light plugins answer
// with their construction props once the one-function patch listed in INTEGRATION.md is applied
// (their fields are private). The estimate lands in the device film and is copied into the
// reference's film::bitmap with Film::set_pixel.
#include <lm/core.h>
#include <lm/renderer.h>
#include <lm/scene.h>
#include <lm/mesh.h>
#include <lm/material.h>
#include <lm/light.h>
#include <lm/camera.h>
#include <lm/film.h>
#include <lm/texture.h>

#include <map>
#include <vector>

#include "lmgpu.h"

LM_NAMESPACE_BEGIN(LM_NAMESPACE)

namespace {

void check(int rc) {
    if (rc != LMGPU_OK) LM_THROW_EXCEPTION(Error::FailedToRender, lmgpu_last_error());
}

void put3(float* d, Vec3 v) { d[0] = float(v.x); d[1] = float(v.y); d[2] = float(v.z); }

// A material row from the material's "gpu" value: {"type": "diffuse" | "glossy" | "glass" |
// "mirror" | "mixture_wavefrontobj", "Kd", "Ks", "ax", "ay", "Ni"}.
lmgpu_material material_row(const Material* m) {
    const Json v = m->underlying_value("gpu");
    if (v.is_null()) LM_THROW_EXCEPTION(Error::Unsupported, "material has no GPU description: " + m->key());
    const std::string type = v["type"];
    lmgpu_material r{};
    r.map_kd = r.mask = -1;
    if (type == "diffuse") {
        r.type = LMGPU_MAT_DIFFUSE;
        put3(r.color, v["Kd"].get<Vec3>());
    } else if (type == "glossy") {
        r.type = LMGPU_MAT_GLOSSY;
        put3(r.color, v["Ks"].get<Vec3>());
        r.ax = float(v["ax"].get<Float>());
        r.ay = float(v["ay"].get<Float>());
    } else if (type == "glass") {
        r.type = LMGPU_MAT_GLASS;
        r.ni = float(v["Ni"].get<Float>());
    } else if (type == "mirror") {
        r.type = LMGPU_MAT_MIRROR;
    } else if (type == "mixture_wavefrontobj") {
        r.type = LMGPU_MAT_MIXTURE;
        put3(r.color, v["Kd"].get<Vec3>());
        put3(r.ks, v["Ks"].get<Vec3>());
        r.ax = float(v["ax"].get<Float>());
        r.ay = float(v["ay"].get<Float>());
    } else {
        LM_THROW_EXCEPTION(Error::Unsupported, "material type not on the GPU path: " + type);
    }
    return r;
}

}  // namespace

class Renderer_PT_GPU final : public Renderer {
private:
    Scene* scene_;
    Film* film_;
    int max_verts_;
    unsigned seed_;
    long long spp_;
    int sampling_mode_, primary_mode_;
    mutable lmgpu_accel* accel_ = nullptr;
    mutable lmgpu_scene* gscene_ = nullptr;
    mutable lmgpu_film* gfilm_ = nullptr;

public:
    ~Renderer_PT_GPU() {
        if (gscene_) lmgpu_scene_destroy(gscene_);
        if (accel_) lmgpu_accel_destroy(accel_);
        if (gfilm_) lmgpu_film_destroy(gfilm_);
    }

    virtual void construct(const Json& prop) override {
        scene_ = json::comp_ref<Scene>(prop, "scene");
        film_ = json::comp_ref<Film>(prop, "output");
        max_verts_ = json::value<int>(prop, "max_verts");
        seed_ = json::value<unsigned>(prop, "seed", 0);
        spp_ = json::value<long long>(prop, "spp");
        const auto s = json::value<std::string>(prop, "sampling_mode", "mis");
        sampling_mode_ = s == "naive" ? LMGPU_SAMPLING_NAIVE : s == "nee" ? LMGPU_SAMPLING_NEE : LMGPU_SAMPLING_MIS;
        primary_mode_ = json::value<std::string>(prop, "primary_ray_sampling_mode", "pixel") == "image"
                            ? LMGPU_PRIMARY_IMAGE
                            : LMGPU_PRIMARY_PIXEL;
    }

    // Scene::build's flattening, into device tables (once; rebuilt when the renderer is re-made).
    void upload() const {
        std::vector<float> pos, nrm, gns, ltp, ltg, lta, env;
        std::vector<int32_t> tri_prim, prim_mat, prim_light;
        std::vector<lmgpu_material> mats;
        std::vector<lmgpu_light> lights;
        std::map<const Material*, int> mat_index;
        lmgpu_scene_desc d{};

        // lights in traversal order first (the primitive table refers to them)
        std::map<int, int> light_of_node;
        scene_->traverse_primitive_nodes([&](const SceneNode& node, Mat4 M) {
            if (node.type != SceneNodeType::Primitive || !node.primitive.light) return;
            const Json v = node.primitive.light->underlying_value("gpu");
            if (v.is_null()) LM_THROW_EXCEPTION(Error::Unsupported, "light has no GPU description");
            const std::string type = v["type"];
            lmgpu_light L{};
            if (type == "area") {  // light_area.cpp:68-80: CDF over mesh-local areas, J = |det M3|
                L.type = LMGPU_LIGHT_AREA;
                put3(L.ke, v["Ke"].get<Vec3>());
                L.tri_offset = int64_t(lta.size());
                L.transform_j = float(std::abs(glm::determinant(Mat3(M))));
                node.primitive.mesh->foreach_triangle([&](int, const Mesh::Tri& t) {
                    const Vec3 c = glm::cross(t.p2.p - t.p1.p, t.p3.p - t.p1.p);
                    lta.push_back(float(glm::length(c) * .5_f));
                    const Vec3 gw = glm::normalize(Transform(M).normal_M * glm::normalize(c));
                    for (const Vec3& p : {t.p1.p, t.p2.p, t.p3.p}) {
                        const Vec3 w = Vec3(M * Vec4(p, 1_f));
                        ltp.insert(ltp.end(), {float(w.x), float(w.y), float(w.z)});
                    }
                    ltg.insert(ltg.end(), {float(gw.x), float(gw.y), float(gw.z)});
                });
                L.tri_count = int64_t(lta.size()) - L.tri_offset;
            } else if (type == "envconst") {
                L.type = LMGPU_LIGHT_ENVCONST;
                put3(L.ke, v["Le"].get<Vec3>());
            } else if (type == "env") {  // light_env.cpp: the lat-long texels through Texture::buffer
                L.type = LMGPU_LIGHT_ENV;
                auto* tex = dynamic_cast<Texture*>(node.primitive.light->underlying("envmap"));
                const TextureBuffer b = tex->buffer();
                L.env_w = b.w;
                L.env_h = b.h;
                L.env_offset = int64_t(env.size());
                for (int i = 0; i < b.w * b.h; i++)
                    for (int k = 0; k < 3; k++) env.push_back(b.data[b.c * i + std::min(k, b.c - 1)]);
                L.rot_deg = float(v["rot"].get<Float>());
                L.scale = float(v.value("scale", 1_f));
            } else if (type == "point") {
                L.type = LMGPU_LIGHT_POINT;
                put3(L.ke, v["Le"].get<Vec3>());
                put3(L.vec, v["position"].get<Vec3>());
            } else if (type == "directional") {
                L.type = LMGPU_LIGHT_DIRECTIONAL;
                put3(L.ke, v["Le"].get<Vec3>());
                put3(L.vec, v["direction"].get<Vec3>());
            } else {
                LM_THROW_EXCEPTION(Error::Unsupported, "light type not on the GPU path: " + type);
            }
            light_of_node[node.index] = int(lights.size());
            lights.push_back(L);
        });

        // geometry in traversal order: the accel's flattening order
        scene_->traverse_primitive_nodes([&](const SceneNode& node, Mat4 M) {
            if (node.type != SceneNodeType::Primitive || !node.primitive.mesh) return;
            const Material* m = node.primitive.material;
            auto it = mat_index.find(m);
            if (it == mat_index.end()) {
                it = mat_index.emplace(m, int(mats.size())).first;
                mats.push_back(material_row(m));
            }
            const int prim = int(prim_mat.size());
            prim_mat.push_back(it->second);
            const auto li = light_of_node.find(node.index);
            prim_light.push_back(li == light_of_node.end() ? -1 : li->second);
            const Transform T(M);
            node.primitive.mesh->foreach_triangle([&](int, const Mesh::Tri& t) {
                for (const auto* c : {&t.p1, &t.p2, &t.p3}) {
                    const Vec3 w = Vec3(M * Vec4(c->p, 1_f));
                    pos.insert(pos.end(), {float(w.x), float(w.y), float(w.z)});
                    const Vec3 n = T.normal_M * c->n;
                    nrm.insert(nrm.end(), {float(n.x), float(n.y), float(n.z)});
                }
                const Vec3 g = glm::normalize(T.normal_M * math::geometry_normal(t.p1.p, t.p2.p, t.p3.p));
                gns.insert(gns.end(), {float(g.x), float(g.y), float(g.z)});
                tri_prim.push_back(prim);
            });
        });

        if (!accel_) check(lmgpu_accel_create(&accel_));
        check(lmgpu_accel_build(accel_, pos.data(), int64_t(pos.size() / 9)));
        d.num_tris = int64_t(pos.size() / 9);
        d.positions = pos.data();
        d.normals = nrm.data();
        d.geo_normals = gns.data();
        d.tri_prim = tri_prim.data();
        d.num_prims = int32_t(prim_mat.size());
        d.prim_material = prim_mat.data();
        d.prim_light = prim_light.data();
        d.num_materials = int32_t(mats.size());
        d.materials = mats.data();
        d.num_lights = int32_t(lights.size());
        d.lights = lights.data();
        d.num_light_tris = int64_t(lta.size());
        d.light_tri_p = ltp.data();
        d.light_tri_gn = ltg.data();
        d.light_tri_area = lta.data();
        d.num_env_texels = int64_t(env.size());
        d.env_texels = env.data();
        // the camera (camera_pinhole.cpp:66-74 answers these)
        const auto* cam = scene_->node_at(scene_->camera_node()).primitive.camera;
        const Json c = cam->underlying_value();
        d.has_camera = 1;
        put3(d.camera.position, c["eye"].get<Vec3>());
        put3(d.camera.center, c["center"].get<Vec3>());
        put3(d.camera.up, c["up"].get<Vec3>());
        d.camera.vfov = float(c["vfov"].get<Float>());
        d.camera.aspect = float(c["aspect"].get<Float>());
        check(lmgpu_scene_create(&gscene_, accel_, &d));
        const auto size = film_->size();
        check(lmgpu_film_create(&gfilm_, size.w, size.h));
    }

    virtual Json render() const override {
        scene_->require_renderable();
        if (!gscene_) upload();
        lmgpu_pt_params p{};
        p.spp = spp_;
        p.max_verts = max_verts_;
        p.seed = seed_;
        p.sampling_mode = sampling_mode_;
        p.primary_mode = primary_mode_;
        lmgpu_render_stats st{};
        check(lmgpu_render_pt(gscene_, gfilm_, &p, nullptr, &st));
        const auto size = film_->size();
        std::vector<float> rgb(size_t(size.w) * size.h * 3);
        check(lmgpu_film_read(gfilm_, rgb.data()));
        film_->clear();
        for (int y = 0; y < size.h; y++)
            for (int x = 0; x < size.w; x++) {
                const float* c = &rgb[3 * (size_t(y) * size.w + x)];
                film_->set_pixel(x, y, Vec3(c[0], c[1], c[2]));
            }
        return {{"processed", spp_}, {"elapsed", st.elapsed_ms / 1e3}, {"rays", st.rays}};
    }
};

LM_COMP_REG_IMPL(Renderer_PT_GPU, "renderer::pt_gpu");

LM_NAMESPACE_END(LM_NAMESPACE)

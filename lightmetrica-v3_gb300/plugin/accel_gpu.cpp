// accel::gpu -- the reference's Accel slot (include/lm/accel.h:26-71) bound to liblmgpu.
//
// A plugin for the reference (loaded with lm.comp.load_plugin, src/component.cpp:219-249). It uses
// only the reference's public headers and include/lmgpu.h, and links against liblmgpu.so. It
// cannot be compiled in this repository: the reference's dependencies (glm, nlohmann_json,
// cereal) are not available here.
//
// build() flattens the scene graph as accel_sahbvh.cpp:132-151 does (world-space triangles in
// traversal order) and builds the 8-wide tree; intersect() is the scalar form of the batched
// lmgpu_accel_intersect and maps the flattened triangle index back to (primitive, face) as
// accel_sahbvh.cpp:296-298 does. Renderers should batch (renderer::pt_gpu does).
#include <lm/core.h>
#include <lm/accel.h>
#include <lm/scene.h>
#include <lm/mesh.h>

#include <algorithm>
#include <vector>

#include "lmgpu.h"

LM_NAMESPACE_BEGIN(LM_NAMESPACE)

class Accel_GPU final : public Accel {
private:
    lmgpu_accel* h_ = nullptr;
    int builder_ = LMGPU_BUILDER_HOST_SAH;
    struct Flat {
        Transform tr;
        int primitive;
        int first_face;  // flattened index of the primitive's first triangle
    };
    std::vector<Flat> flat_;

    static void check(int rc) {
        if (rc != LMGPU_OK) LM_THROW_EXCEPTION(Error::FailedToRender, lmgpu_last_error());
    }

public:
    ~Accel_GPU() {
        if (h_) lmgpu_accel_destroy(h_);
    }

    // Props: builder ("sah" on the host threads, the default, or "ploc" on the GPU).
    virtual void construct(const Json& prop) override {
        builder_ = json::value<std::string>(prop, "builder", "sah") == "ploc" ? LMGPU_BUILDER_GPU_PLOC
                                                                               : LMGPU_BUILDER_HOST_SAH;
    }

    virtual void build(const Scene& scene) override {
        std::vector<float> tri;
        flat_.clear();
        int faces = 0;
        scene.traverse_primitive_nodes([&](const SceneNode& node, Mat4 M) {
            if (node.type != SceneNodeType::Primitive || !node.primitive.mesh) return;
            flat_.push_back({Transform(M), node.index, faces});
            node.primitive.mesh->foreach_triangle([&](int, const Mesh::Tri& t) {
                for (const Vec3& p : {t.p1.p, t.p2.p, t.p3.p}) {
                    const Vec3 w = Vec3(M * Vec4(p, 1_f));
                    tri.insert(tri.end(), {float(w.x), float(w.y), float(w.z)});
                }
                faces++;
            });
        });
        if (!h_) check(lmgpu_accel_create(&h_));
        check(lmgpu_accel_build_ex(h_, tri.data(), int64_t(tri.size() / 9), builder_));
    }

    virtual std::optional<Hit> intersect(Ray ray, Float tmin, Float tmax) const override {
        const float r[8] = {float(ray.o.x), float(ray.o.y), float(ray.o.z), float(tmin),
                            float(ray.d.x), float(ray.d.y), float(ray.d.z), float(tmax)};
        lmgpu_hit h;
        check(lmgpu_accel_intersect(h_, r, 1, &h));
        if (h.prim < 0) return {};
        const auto it = std::upper_bound(flat_.begin(), flat_.end(), h.prim,
                                         [](int v, const Flat& f) { return v < f.first_face; }) - 1;
        return Hit{Float(h.t), Vec2(h.u, h.v), it->tr, it->primitive, h.prim - it->first_face};
    }

    // The device handle, for renderer::pt_gpu (which renders on the same tree).
    virtual void* underlying_raw_pointer(const std::string&) const override { return h_; }
};

LM_COMP_REG_IMPL(Accel_GPU, "accel::gpu");

LM_NAMESPACE_END(LM_NAMESPACE)

// Oracle (test infrastructure only): the reference's Accel interface (include/lm/accel.h:26-71),
// restated so that src/accel/accel_sahbvh.cpp compiles against it: build from a scene, and the
// closest hit with its distance, barycentric coordinates, global transform, primitive node and
// face.
#pragma once
#include <lm/core.h>

LM_NAMESPACE_BEGIN(LM_NAMESPACE)

class Accel : public Component {
public:
    virtual void build(const Scene& scene) = 0;
    struct Hit {
        Float t;
        Vec2 uv;
        Transform global_transform;
        int primitive;
        int face;
    };
    virtual std::optional<Hit> intersect(Ray ray, Float tmin, Float tmax) const = 0;
};

LM_NAMESPACE_END(LM_NAMESPACE)

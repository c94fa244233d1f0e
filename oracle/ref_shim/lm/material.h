// Oracle (test infrastructure only): the reference's Material interface (include/lm/material.h),
// restated with the same types and virtual signatures so that the reference's material sources
// compile against it unmodified.
#pragma once
#include <lm/core.h>
#include <lm/surface.h>

LM_NAMESPACE_BEGIN(LM_NAMESPACE)

class Material : public Component {
public:
    enum class TransDir {
        LE,
        EL
    };
    struct ComponentSample {
        int comp;
        Float weight;
    };
    struct ComponentSampleU {
        Vec2 uc;
    };
    virtual ComponentSample sample_component(const ComponentSampleU& u, const PointGeometry& geom, Vec3 wi) const = 0;
    virtual Float pdf_component(int comp, const PointGeometry& geom, Vec3 wi) const = 0;
    struct DirectionSample {
        Vec3 wo;
        Vec3 weight;
    };
    struct DirectionSampleU {
        Vec2 ud;
        Vec2 udc;
    };
    virtual std::optional<DirectionSample> sample_direction(const DirectionSampleU& u, const PointGeometry& geom, Vec3 wi, int comp, TransDir trans_dir) const = 0;
    virtual Float pdf_direction(const PointGeometry& geom, Vec3 wi, Vec3 wo, int comp, bool eval_delta) const = 0;
    virtual Vec3 eval(const PointGeometry& geom, Vec3 wi, Vec3 wo, int comp, TransDir trans_dir, bool eval_delta) const = 0;
    virtual bool is_specular_component(int comp) const = 0;
    virtual Vec3 reflectance(const PointGeometry& geom) const = 0;
};

LM_NAMESPACE_END(LM_NAMESPACE)

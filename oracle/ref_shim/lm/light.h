// Oracle (test infrastructure only): the reference's Light interface (include/lm/light.h),
// restated with the same types and virtual signatures so that the reference's light sources
// compile against it unmodified.
#pragma once
#include <lm/core.h>
#include <lm/surface.h>

LM_NAMESPACE_BEGIN(LM_NAMESPACE)

class Light : public Component {
public:
    virtual void set_scene_bound(const Bound& bound) { (void)bound; }
    struct RaySample {
        PointGeometry geom;
        Vec3 wo;
        Vec3 weight;
    };
    struct RaySampleU {
        Vec2 up;
        Float upc;
        Vec2 ud;
    };
    virtual std::optional<RaySample> sample_ray(const RaySampleU& u, const Transform& transform) const = 0;
    virtual Float pdf_ray(const PointGeometry& geom, Vec3 wo, const Transform& transform, bool eval_delta) const = 0;
    struct DirectionSample {
        Vec3 wo;
        Vec3 weight;
    };
    struct DirectionSampleU {
        Vec2 ud;
    };
    virtual std::optional<DirectionSample> sample_direction(const DirectionSampleU& u, const PointGeometry& geom) const = 0;
    virtual Float pdf_direction(const PointGeometry& geom, Vec3 wo) const = 0;
    struct PositionSample {
        PointGeometry geom;
        Vec3 weight;
    };
    struct PositionSampleU {
        Vec2 up;
        Float upc;
    };
    virtual std::optional<PositionSample> sample_position(const PositionSampleU& u, const Transform& transform) const = 0;
    virtual Float pdf_position(const PointGeometry& geom, const Transform& transform) const = 0;
    virtual std::optional<RaySample> sample_direct(const RaySampleU& u, const PointGeometry& geom, const Transform& transform) const = 0;
    virtual Float pdf_direct(const PointGeometry& geom, const PointGeometry& geomL, const Transform& transform, Vec3 wo, bool eval_delta) const = 0;
    virtual bool is_specular() const = 0;
    virtual bool is_infinite() const = 0;
    virtual bool is_env() const { return false; }
    virtual bool is_connectable(const PointGeometry& geom) const = 0;
    virtual Vec3 eval(const PointGeometry& geom, Vec3 wo, bool eval_delta) const = 0;
};

LM_NAMESPACE_END(LM_NAMESPACE)

// Oracle (test infrastructure only): the reference's Camera interface (include/lm/camera.h),
// restated with the same types and virtual signatures so that the reference's camera source
// compiles against it unmodified.
#pragma once
#include <lm/core.h>
#include <lm/surface.h>

LM_NAMESPACE_BEGIN(LM_NAMESPACE)

class Camera : public Component {
public:
    virtual void set_aspect_ratio(Float aspect) = 0;
    virtual Mat4 view_matrix() const = 0;
    virtual Mat4 projection_matrix() const = 0;
    virtual Ray primary_ray(Vec2 rp) const = 0;
    struct RaySample {
        PointGeometry geom;
        Vec3 wo;
        Vec3 weight;
    };
    struct RaySampleU {
        Vec2 ud;
    };
    virtual std::optional<RaySample> sample_ray(const RaySampleU& u) const = 0;
    virtual Float pdf_ray(const PointGeometry& geom, Vec3 wo) const = 0;
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
        Vec2 udp;
    };
    virtual std::optional<PositionSample> sample_position(const PositionSampleU& u) const = 0;
    virtual Float pdf_position(const PointGeometry& geom) const = 0;
    virtual std::optional<RaySample> sample_direct(const RaySampleU& u, const PointGeometry& geom) const = 0;
    virtual Float pdf_direct(const PointGeometry& geom, const PointGeometry& geomE, Vec3 wo) const = 0;
    virtual std::optional<Vec2> raster_position(Vec3 wo) const = 0;
    virtual bool is_connectable(const PointGeometry& geom) const = 0;
    virtual Vec3 eval(Vec3 wo) const = 0;
};

LM_NAMESPACE_END(LM_NAMESPACE)

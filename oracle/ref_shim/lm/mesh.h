// Oracle (test infrastructure only): the reference's Mesh interface (include/lm/mesh.h:20-80),
// restated without its component and serialization machinery: the vertex and triangle records and
// the triangle iteration the accel's build uses.
#pragma once
#include <lm/core.h>

LM_NAMESPACE_BEGIN(LM_NAMESPACE)

class Mesh : public Component {
public:
    struct Point {
        Vec3 p;  // position
        Vec3 n;  // normal
        Vec2 t;  // texture coordinates
    };
    struct Tri {
        Point p1, p2, p3;
    };
    using ProcessTriangleFunc = std::function<void(int face, const Tri& tri)>;
    virtual void foreach_triangle(const ProcessTriangleFunc& process_triangle) const = 0;
    virtual Tri triangle_at(int face) const = 0;
    virtual int num_triangles() const = 0;
};

LM_NAMESPACE_END(LM_NAMESPACE)

// Oracle (test infrastructure only): the part of the reference's Scene interface that an accel's
// build calls (include/lm/scene.h:163-177, include/lm/scenenode.h:18-80): the scene node record
// and the traversal of primitive nodes with their global transforms.
#pragma once
#include <lm/core.h>
#include <lm/mesh.h>

LM_NAMESPACE_BEGIN(LM_NAMESPACE)

enum class SceneNodeType {
    Primitive,
    Group,
};

struct SceneNode {
    SceneNodeType type;
    int index;
    struct Primitive {
        Mesh* mesh = nullptr;
    } primitive;
    struct Group {
        std::vector<int> children;
        std::optional<Mat4> local_transform;
    } group;
};

class Scene {
public:
    virtual ~Scene() = default;
    using NodeTraverseFunc = std::function<void(const SceneNode& node, Mat4 global_transform)>;
    virtual void traverse_primitive_nodes(const NodeTraverseFunc& traverse_func) const = 0;
};

LM_NAMESPACE_END(LM_NAMESPACE)

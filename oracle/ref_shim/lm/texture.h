// Oracle (test infrastructure only): the reference's Texture interface (include/lm/texture.h),
// restated so that sources holding a texture reference compile; no texture implementation is
// compiled into oracle/_ref.
#pragma once
#include <lm/core.h>

LM_NAMESPACE_BEGIN(LM_NAMESPACE)

class Texture : public Component {
public:
    virtual Vec3 eval(Vec2 t) const = 0;
    virtual Vec3 eval_by_pixel_coords(int x, int y) const = 0;
    virtual Float eval_alpha(Vec2 t) const { (void)t; return 0_f; }
    virtual bool has_alpha() const { return false; }
};

LM_NAMESPACE_END(LM_NAMESPACE)

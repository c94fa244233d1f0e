// Oracle (test infrastructure only): stand-in for stb_image, a third-party single-header image
// decoder that the reference includes from its build environment (it is not among the
// reference's sources). src/texture/texture_bitmap.cpp:55-66 calls
// stbi_set_flip_vertically_on_load, stbi_loadf, stbi_failure_reason and stbi_image_free.
//
// Decoding image files is not on the path under test, so images come from an in-memory registry
// that the checker fills with decoded float texels, top row first as an image file stores them
// (lmref_register_image). stbi_loadf returns a malloc'd copy with the rows reversed when flipping
// is on, which is what stb_image's vertical flip does; req_comp must be 0 (the only value
// texture_bitmap.cpp passes), so the image keeps its own channel count.
#pragma once
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <map>
#include <string>
#include <vector>

namespace lmref_stb {
struct Image {
    int w = 0, h = 0, c = 0;
    std::vector<float> texels;  // h rows of w x c floats, top row first
};
inline std::map<std::string, Image>& images() {
    static std::map<std::string, Image> r;
    return r;
}
// Registry key of a path: separators and dot segments normalised, so "a/b/../t.png" and
// "a/t.png" name the same image.
inline std::string key(const std::string& path) {
    return std::filesystem::path(path).lexically_normal().generic_string();
}
inline bool& flip() {
    static bool f = false;
    return f;
}
inline std::string& failure() {
    static std::string s;
    return s;
}
}  // namespace lmref_stb

inline void stbi_set_flip_vertically_on_load(int flag) { lmref_stb::flip() = flag != 0; }

inline float* stbi_loadf(const char* filename, int* x, int* y, int* comp, int req_comp) {
    const auto it = lmref_stb::images().find(lmref_stb::key(filename));
    if (it == lmref_stb::images().end()) {
        lmref_stb::failure() = "can't fopen";
        return nullptr;
    }
    if (req_comp != 0) {
        lmref_stb::failure() = "unsupported req_comp";
        return nullptr;
    }
    const auto& im = it->second;
    const size_t row = size_t(im.w) * size_t(im.c);
    auto* out = static_cast<float*>(std::malloc(sizeof(float) * row * size_t(im.h)));
    if (!out) {
        lmref_stb::failure() = "outofmem";
        return nullptr;
    }
    for (int r = 0; r < im.h; r++) {
        const int src = lmref_stb::flip() ? im.h - 1 - r : r;
        std::memcpy(out + size_t(r) * row, im.texels.data() + size_t(src) * row, sizeof(float) * row);
    }
    *x = im.w;
    *y = im.h;
    *comp = im.c;
    return out;
}

inline const char* stbi_failure_reason() { return lmref_stb::failure().c_str(); }

inline void stbi_image_free(void* p) { std::free(p); }

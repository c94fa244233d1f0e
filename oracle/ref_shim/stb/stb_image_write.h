// Oracle (test infrastructure only): declarations the reference's film source calls to save
// images. Saving is not used by the checker; each call reports failure.
#pragma once
inline int stbi_write_png(const char*, int, int, int, const void*, int) { return 0; }
inline int stbi_write_jpg(const char*, int, int, int, const void*, int) { return 0; }
inline int stbi_write_hdr(const char*, int, int, int, const float*) { return 0; }

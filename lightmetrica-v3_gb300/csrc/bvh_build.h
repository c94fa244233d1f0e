// Host-side builder for the 8-wide quantized BVH that the trace kernels walk.
//
// The reference builds a binary SAH BVH with a full sort per node (accel_sahbvh.cpp:127-267) and
// walks it with a depth-first stack. Here a binned SAH binary tree is built on the host threads,
// then collapsed into 8-wide nodes whose child boxes are quantized to 8 bits per plane relative to
// the node frame and rounded outward with a margin of at least one quantum on every side, so each
// dequantized box strictly contains the exact child box (the slab test relies on the margin).
//
// Node layout (80 bytes, five 16-byte words, read with vectorized loads):
//   w0: px, py, pz (float bits)      | ex | ey<<8 | ez<<16 | imask<<24
//   w1: child_base | tri_base | meta[0..3] | meta[4..7]
//   w2: qlo_x[0..3] | qlo_x[4..7] | qlo_y[0..3] | qlo_y[4..7]
//   w3: qlo_z[0..3] | qlo_z[4..7] | qhi_x[0..3] | qhi_x[4..7]
//   w4: qhi_y[0..3] | qhi_y[4..7] | qhi_z[0..3] | qhi_z[4..7]
// Child slot i spans plane value p + q * 2^(e-127) on each axis. imask bit i marks an internal
// child (meta 0x80); its node index is child_base + popcount(imask & ((1<<i)-1)). meta[i] = 0
// marks an empty slot; a leaf child has meta = (count << 5) | offset with its `count` (1..3)
// triangles at tri_base + offset. Slots are assigned so that visiting slot (k XOR octant) for k = 0..7 goes
// roughly front to back for rays whose direction-sign octant is `octant`.
//
// Triangle layout (48 bytes, three 16-byte words), in leaf order:
//   (p1.x, p1.y, p1.z, e1.x) (e1.y, e1.z, e2.x, e2.y) (e2.z, id bits, 0, 0)
// with e1 = p2 - p1 and e2 = p3 - p1 rounded once in fp32, as Tri's constructor does
// (accel_sahbvh.cpp:41-49), and id the flattened triangle index.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace lmgpu {

struct Bvh8Host {
    std::vector<uint32_t> nodes;  // 20 words per node
    std::vector<float> tris;      // 12 floats per triangle
    int32_t max_depth = 0;
    double sah_cost = 0;
};

// Top-level (instance) trees: every leaf holds exactly one primitive and is written as a child
// pseudo-node instead of triangle records, marked by an exponent byte ex = 0xFF (no real node
// uses it) and carrying the primitive index in child_base (w1.x). The traversal enters the
// instance there.
constexpr uint32_t kInstanceMarker = 0xFFu;

struct BuildOptions {
    bool leaf_nodes = false;  // top-level mode (see above); tris stays empty
    // children per node the collapse may use (2..8): the node layout keeps 8 slots, a narrower
    // tree leaves the rest empty (the autotuner compares widths)
    int max_width = 8;
};

// tri_p: n x 9 floats (p1, p2, p3); in top-level mode each "triangle" is (lo, hi, lo) of one
// instance's world box. Returns false with `err` set on invalid input.
bool build_bvh8(const float* tri_p, int64_t n, Bvh8Host& out, std::string* err, const BuildOptions& opt = {});

// Decoded view of one node, for tests and debugging.
struct Bvh8NodeView {
    float origin[3];
    float scale[3];
    uint8_t imask;
    uint32_t child_base, tri_base;
    uint8_t meta[8];
    uint8_t qlo[3][8], qhi[3][8];
};
Bvh8NodeView decode_node(const uint32_t* words);

}  // namespace lmgpu

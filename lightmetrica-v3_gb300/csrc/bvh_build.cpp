// Host-side binned-SAH build and collapse to the 8-wide quantized layout (see bvh_build.h).
// Compiled by the host compiler with OpenMP; the binary build recurses as OpenMP tasks.
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <omp.h>

namespace lmgpu {

namespace {

constexpr int kMaxLeaf = 3;     // triangles per leaf child (3 bits of meta hold the count)
constexpr int kBins = 32;
constexpr int kTaskGrain = 8192;
constexpr int kMedianDepth = 64;  // below this depth a degenerate split falls back to the median

struct AABB {
    float lo[3], hi[3];
    void reset() {
        for (int a = 0; a < 3; a++) { lo[a] = std::numeric_limits<float>::infinity(); hi[a] = -std::numeric_limits<float>::infinity(); }
    }
    void grow(const AABB& b) {
        for (int a = 0; a < 3; a++) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); }
    }
    void grow(const float* p) {
        for (int a = 0; a < 3; a++) { lo[a] = std::min(lo[a], p[a]); hi[a] = std::max(hi[a], p[a]); }
    }
    double area() const {
        if (!(hi[0] >= lo[0])) return 0.0;
        const double dx = double(hi[0]) - lo[0], dy = double(hi[1]) - lo[1], dz = double(hi[2]) - lo[2];
        return 2.0 * (dx * dy + dy * dz + dz * dx);
    }
};

struct BinNode {
    AABB box;
    int32_t left = -1, right = -1;
    int32_t start = 0, count = 0;
};

struct Builder {
    const float* P = nullptr;
    int64_t n = 0;
    std::vector<AABB> tb;
    std::vector<float> cen;  // 3 per triangle
    std::vector<int32_t> idx;
    std::vector<BinNode> nodes;
    std::atomic<int32_t> next{1};

    void split_median(int start, int count, int axis, int& mid) {
        mid = start + count / 2;
        std::nth_element(idx.begin() + start, idx.begin() + mid, idx.begin() + start + count,
                         [&](int32_t a, int32_t b) { return cen[3 * a + axis] < cen[3 * b + axis]; });
    }

    void build(int32_t ni, int start, int count, int depth) {
        BinNode& node = nodes[ni];
        node.start = start;
        node.count = count;
        AABB box, cb;
        box.reset(); cb.reset();
        for (int i = start; i < start + count; i++) {
            box.grow(tb[idx[i]]);
            cb.grow(&cen[3 * idx[i]]);
        }
        node.box = box;
        if (count == 1) return;

        // Binned SAH over centroid bounds (C_trav = 1, C_tri = 1, costs relative to node area).
        int best_axis = -1, best_split = -1;
        double best_cost = std::numeric_limits<double>::infinity();
        const double parea = box.area();
        for (int a = 0; a < 3; a++) {
            const float ext = cb.hi[a] - cb.lo[a];
            if (!(ext > 0.f)) continue;
            AABB bb[kBins];
            int bc[kBins] = {0};
            for (int b = 0; b < kBins; b++) bb[b].reset();
            const float k = float(kBins) / ext;
            for (int i = start; i < start + count; i++) {
                const int t = idx[i];
                int b = int((cen[3 * t + a] - cb.lo[a]) * k);
                b = std::min(std::max(b, 0), kBins - 1);
                bb[b].grow(tb[t]);
                bc[b]++;
            }
            double ra[kBins];
            int rc[kBins];
            AABB acc; acc.reset();
            int c = 0;
            for (int b = kBins - 1; b > 0; b--) {
                acc.grow(bb[b]); c += bc[b];
                ra[b] = acc.area(); rc[b] = c;
            }
            acc.reset(); c = 0;
            for (int b = 0; b < kBins - 1; b++) {
                acc.grow(bb[b]); c += bc[b];
                if (c == 0 || rc[b + 1] == 0) continue;
                const double cost = acc.area() * c + ra[b + 1] * rc[b + 1];
                if (cost < best_cost) { best_cost = cost; best_axis = a; best_split = b; }
            }
        }
        const double split_cost = parea > 0 ? 1.0 + best_cost / parea : std::numeric_limits<double>::infinity();
        (void)split_cost;  // the binary tree splits down to single triangles; the collapse picks leaves

        int mid = -1;
        if (best_axis >= 0 && depth < kMedianDepth) {
            const float ext = cb.hi[best_axis] - cb.lo[best_axis];
            const float k = float(kBins) / ext;
            auto it = std::partition(idx.begin() + start, idx.begin() + start + count, [&](int32_t t) {
                int b = int((cen[3 * t + best_axis] - cb.lo[best_axis]) * k);
                b = std::min(std::max(b, 0), kBins - 1);
                return b <= best_split;
            });
            mid = int(it - idx.begin());
        }
        if (mid <= start || mid >= start + count) {
            int axis = 0;
            for (int a = 1; a < 3; a++)
                if (cb.hi[a] - cb.lo[a] > cb.hi[axis] - cb.lo[axis]) axis = a;
            split_median(start, count, axis, mid);
        }
        const int32_t l = next.fetch_add(2);
        node.left = l;
        node.right = l + 1;
        const int lc = mid - start, rcnt = start + count - mid;
        if (count > kTaskGrain) {
#pragma omp task default(shared) firstprivate(l, start, lc, depth)
            build(l, start, lc, depth + 1);
#pragma omp task default(shared) firstprivate(l, mid, rcnt, depth)
            build(l + 1, mid, rcnt, depth + 1);
        } else {
            build(l, start, lc, depth + 1);
            build(l + 1, mid, rcnt, depth + 1);
        }
    }
};

inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// Quantizes child boxes into the node frame. Per axis the frame is origin p and quantum
// s = 2^(eb-127); plane q lies at the exact real value p + q*s. Every child gets a margin of at
// least one quantum outside its exact box on both sides (qlo <= (lo - p)/s - 1, qhi >= (hi - p)/s
// + 1), which the traversal's one-FMA slab test needs to stay conservative. The origin sits two
// quanta below the node box so that the margins always fit in [0, 255].
int exponent_for(double v) {  // smallest biased exponent eb with 2^(eb-127) >= v
    if (!(v > 0)) return 1;
    int e2;
    const double m = std::frexp(v, &e2);  // v = m * 2^e2, m in [0.5, 1)
    int eb = (m == 0.5 ? e2 - 1 : e2) + 127;
    return std::min(254, std::max(1, eb));
}

bool quantize_axis(float lo, float hi, const AABB* cbox, const bool* valid, int a, int eb, float& origin,
                   uint8_t* qlo, uint8_t* qhi) {
    const double s = std::ldexp(1.0, eb - 127);
    double pd = double(lo) - 2.0 * s;
    float p = float(pd);
    if (double(p) > pd) p = std::nextafter(p, -std::numeric_limits<float>::infinity());
    if (!(double(p) < double(lo) - s)) return false;  // quantum below float resolution at lo
    for (int k = 0; k < 8; k++) {
        if (!valid[k]) { qlo[k] = 255; qhi[k] = 0; continue; }  // inverted: no ray enters
        const double l = (double(cbox[k].lo[a]) - double(p)) / s;
        const double h = (double(cbox[k].hi[a]) - double(p)) / s;
        const double ql = std::floor(l) - 1.0, qh = std::ceil(h) + 1.0;
        if (ql < 0.0 || qh > 255.0) return false;
        // margins re-checked in long double: plane + s stays at or below lo, plane - s at or above hi
        const long double pl = (long double)p + (long double)ql * s, ph = (long double)p + (long double)qh * s;
        if (pl + s > (long double)cbox[k].lo[a] || ph - s < (long double)cbox[k].hi[a]) return false;
        qlo[k] = uint8_t(ql);
        qhi[k] = uint8_t(qh);
    }
    origin = p;
    return true;
}

bool quantize(const AABB& nb, const AABB* cbox, const bool* valid, int eb_out[3], float origin[3], uint8_t qlo[3][8],
              uint8_t qhi[3][8]) {
    for (int a = 0; a < 3; a++) {
        const double ext = double(nb.hi[a]) - double(nb.lo[a]);
        const double mag = std::max(std::fabs(double(nb.lo[a])), std::fabs(double(nb.hi[a])));
        int eb = std::max(exponent_for(ext / 251.0), exponent_for(mag * 1.2e-7));
        bool ok = false;
        for (; eb <= 254 && !ok; eb++) {
            ok = quantize_axis(nb.lo[a], nb.hi[a], cbox, valid, a, eb, origin[a], qlo[a], qhi[a]);
            if (ok) eb_out[a] = eb;
        }
        if (!ok) return false;
    }
    return true;
}

}  // namespace

bool build_bvh8(const float* tri_p, int64_t n, Bvh8Host& out, std::string* err, const BuildOptions& opt) {
    out = Bvh8Host();
    if (n <= 0) {
        if (err) *err = "accel build: no triangles";
        return false;
    }
    if (n > (int64_t(1) << 31) - 1) {
        if (err) *err = "accel build: more than 2^31-1 triangles";
        return false;
    }
    Builder B;
    B.P = tri_p;
    B.n = n;
    B.tb.resize(n);
    B.cen.resize(3 * n);
    B.idx.resize(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        AABB b; b.reset();
        for (int k = 0; k < 3; k++) b.grow(tri_p + 9 * i + 3 * k);
        for (int a = 0; a < 3; a++) {
            if (!std::isfinite(b.lo[a]) || !std::isfinite(b.hi[a])) { b.lo[a] = 0; b.hi[a] = 0; }
            B.cen[3 * i + a] = 0.5f * (b.lo[a] + b.hi[a]);
        }
        B.tb[i] = b;
        B.idx[i] = int32_t(i);
    }
    for (int64_t i = 0; i < n; i++)
        for (int k = 0; k < 9; k++)
            if (!std::isfinite(tri_p[9 * i + k])) {
                if (err) *err = "accel build: non-finite vertex coordinate";
                return false;
            }
    B.nodes.resize(size_t(2) * n);
#pragma omp parallel
#pragma omp single
    B.build(0, 0, int(n), 0);
    const int32_t nb = B.next.load();
    B.nodes.resize(nb);

    // ---- SAH-optimal collapse to 8-wide nodes (Ylitie, Karras & Laine, HPG 2017) ----------------
    // cost[n][i-1]: cheapest way to represent binary subtree n with at most i slots of its parent:
    //   i = 1: a leaf (at most kMaxLeaf triangles, cost A * c_prim * count) or a wide node
    //          (A * c_node + the best split of its two children over 8 slots);
    //   i > 1: the i-1 option, or the subtree's two children placed directly with k and i-k slots.
    constexpr float kCNode = 1.0f, kCPrim = 0.3f;
    const int W = opt.leaf_nodes ? 8 : std::min(8, std::max(2, opt.max_width));
    const float inf = std::numeric_limits<float>::infinity();
    std::vector<float> cost(size_t(nb) * 8);
    std::vector<int8_t> dec(size_t(nb) * 8);  // i=1: 0 leaf / 1 node; i>1: 0 = as i-1, k = split
    std::vector<int8_t> dnode(size_t(nb), 0);  // k of the node's own 8-slot split
    for (int32_t ni = nb - 1; ni >= 0; ni--) {
        const BinNode& b = B.nodes[ni];
        const float A = float(b.box.area());
        float* c = &cost[size_t(ni) * 8];
        int8_t* d = &dec[size_t(ni) * 8];
        const int max_leaf = opt.leaf_nodes ? 1 : kMaxLeaf;
        const float cleaf = b.count <= max_leaf ? A * kCPrim * float(b.count) : inf;
        if (b.left < 0) {
            for (int i = 0; i < 8; i++) { c[i] = cleaf; d[i] = 0; }
            continue;
        }
        const float* cl = &cost[size_t(b.left) * 8];
        const float* cr = &cost[size_t(b.right) * 8];
        float dist[9];
        int8_t dk[9];
        for (int j = 2; j <= 8; j++) {
            dist[j] = inf;
            dk[j] = 1;
            for (int k = 1; k < j; k++) {
                const float v = cl[k - 1] + cr[j - k - 1];
                if (v < dist[j]) { dist[j] = v; dk[j] = int8_t(k); }
            }
        }
        const float cnode = A * kCNode + dist[W];
        c[0] = std::min(cleaf, cnode);
        d[0] = cleaf <= cnode ? 0 : 1;
        dnode[ni] = dk[W];
        for (int i = 2; i <= 8; i++) {
            if (c[i - 2] <= dist[i]) { c[i - 1] = c[i - 2]; d[i - 1] = 0; }
            else { c[i - 1] = dist[i]; d[i - 1] = dk[i]; }
        }
    }
    {
        const float ra = float(B.nodes[0].box.area());
        out.sah_cost = ra > 0 ? double(cost[0]) / ra : 0.0;
    }
    struct Child { int32_t bin; bool leaf; };
    // children of binary subtree m given i slots, appended to `out`
    std::function<void(int32_t, int, std::vector<Child>&)> emit = [&](int32_t m, int i, std::vector<Child>& v) {
        while (i > 1 && dec[size_t(m) * 8 + i - 1] == 0) i--;
        if (i == 1) {
            v.push_back({m, B.nodes[m].left < 0 || dec[size_t(m) * 8] == 0});
            return;
        }
        const int k = dec[size_t(m) * 8 + i - 1];
        emit(B.nodes[m].left, k, v);
        emit(B.nodes[m].right, i - k, v);
    };

    struct Pending { int32_t bin; int32_t wide; int32_t depth; };
    std::vector<Pending> queue;
    queue.push_back({0, 0, 1});
    out.nodes.assign(20, 0);
    if (!opt.leaf_nodes) out.tris.reserve(size_t(12) * n);
    size_t qi = 0;
    int32_t max_depth = 1;
    std::vector<Child> kids;
    kids.reserve(8);
    while (qi < queue.size()) {
        const Pending pd = queue[qi++];
        max_depth = std::max(max_depth, pd.depth);
        // children of this wide node, as binary node indices
        kids.clear();
        const BinNode& root = B.nodes[pd.bin];
        if (root.left < 0 || (pd.bin == 0 && dec[0] == 0)) {
            kids.push_back({pd.bin, true});  // the whole tree is one leaf
        } else {
            emit(root.left, dnode[pd.bin], kids);
            emit(root.right, W - dnode[pd.bin], kids);
        }
        const int nch = int(kids.size());
        if (nch < 1 || nch > 8) {
            if (err) *err = "accel build: internal error (child count)";
            return false;
        }
        int32_t ch[8];
        bool is_leaf[8];
        for (int i = 0; i < nch; i++) { ch[i] = kids[i].bin; is_leaf[i] = kids[i].leaf; }
        // octant-ordered slot assignment (greedy on dot(centroid - center, octant direction))
        AABB nbox; nbox.reset();
        for (int i = 0; i < nch; i++) nbox.grow(B.nodes[ch[i]].box);
        float ctr[3];
        for (int a = 0; a < 3; a++) ctr[a] = 0.5f * (nbox.lo[a] + nbox.hi[a]);
        double cost[8][8];
        for (int i = 0; i < nch; i++) {
            const AABB& b = B.nodes[ch[i]].box;
            for (int s = 0; s < 8; s++) {
                double c = 0;
                for (int a = 0; a < 3; a++) {
                    const double d = 0.5 * (double(b.lo[a]) + b.hi[a]) - ctr[a];
                    c += ((s >> a) & 1) ? -d : d;
                }
                cost[i][s] = c;
            }
        }
        int slot_of[8];
        int child_in[8];
        for (int s = 0; s < 8; s++) child_in[s] = -1;
        bool used[8] = {false};
        for (int k = 0; k < nch; k++) {
            int bi = -1, bs = -1;
            double bc = std::numeric_limits<double>::infinity();
            for (int i = 0; i < nch; i++) {
                if (used[i]) continue;
                for (int s = 0; s < 8; s++) {
                    if (child_in[s] >= 0) continue;
                    if (cost[i][s] < bc) { bc = cost[i][s]; bi = i; bs = s; }
                }
            }
            used[bi] = true;
            child_in[bs] = bi;
            slot_of[bi] = bs;
        }
        (void)slot_of;
        // allocate internal children (slot order) and leaf triangles (slot order)
        uint8_t imask = 0, meta[8] = {0};
        AABB cbox[8];
        bool valid[8] = {false};
        const uint32_t child_base = uint32_t(out.nodes.size() / 20);
        const uint32_t tri_base = uint32_t(out.tris.size() / 12);
        for (int s = 0; s < 8; s++) {
            const int i = child_in[s];
            if (i < 0) continue;
            const BinNode& c = B.nodes[ch[i]];
            valid[s] = true;
            cbox[s] = c.box;
            if (!is_leaf[i]) {
                imask |= uint8_t(1u << s);
                meta[s] = 0x80;  // any nonzero value marks the slot as used
                const int32_t wi = int32_t(out.nodes.size() / 20);
                out.nodes.resize(out.nodes.size() + 20, 0);
                queue.push_back({ch[i], wi, pd.depth + 1});
            } else if (opt.leaf_nodes) {
                if (c.count != 1) {
                    if (err) *err = "accel build: internal error (top-level leaf size)";
                    return false;
                }
                imask |= uint8_t(1u << s);
                meta[s] = 0x80;
                const size_t wi = out.nodes.size();
                out.nodes.resize(out.nodes.size() + 20, 0);
                out.nodes[wi + 3] = kInstanceMarker;
                out.nodes[wi + 4] = uint32_t(B.idx[c.start]);
            }
        }
        for (int s = 0; s < 8; s++) {
            const int i = child_in[s];
            if (i < 0 || (imask >> s) & 1) continue;  // empty, internal or an instance pseudo-node
            const BinNode& c = B.nodes[ch[i]];
            const uint32_t off = uint32_t(out.tris.size() / 12) - tri_base;
            if (c.count < 1 || c.count > kMaxLeaf || off > 31) {
                if (err) *err = "accel build: internal error (leaf layout)";
                return false;
            }
            meta[s] = uint8_t((c.count << 5) | off);
            for (int k = c.start; k < c.start + c.count; k++) {
                const int32_t t = B.idx[k];
                const float* p = tri_p + 9 * int64_t(t);
                const float p1[3] = {p[0], p[1], p[2]};
                const float e1[3] = {p[3] - p[0], p[4] - p[1], p[5] - p[2]};
                const float e2[3] = {p[6] - p[0], p[7] - p[1], p[8] - p[2]};
                const float rec[12] = {p1[0], p1[1], p1[2], e1[0], e1[1], e1[2], e2[0], e2[1], e2[2], bitsf(uint32_t(t)), 0.f, 0.f};
                out.tris.insert(out.tris.end(), rec, rec + 12);
            }
        }
        // quantize
        int eb[3];
        float origin[3];
        uint8_t qlo[3][8], qhi[3][8];
        if (!quantize(nbox, cbox, valid, eb, origin, qlo, qhi)) {
            if (err) *err = "accel build: box quantization failed";
            return false;
        }
        uint32_t* w = &out.nodes[size_t(pd.wide) * 20];
        w[0] = fbits(origin[0]); w[1] = fbits(origin[1]); w[2] = fbits(origin[2]);
        w[3] = uint32_t(eb[0]) | (uint32_t(eb[1]) << 8) | (uint32_t(eb[2]) << 16) | (uint32_t(imask) << 24);
        w[4] = child_base;
        w[5] = tri_base;
        auto pack4 = [](const uint8_t* b) {
            return uint32_t(b[0]) | (uint32_t(b[1]) << 8) | (uint32_t(b[2]) << 16) | (uint32_t(b[3]) << 24);
        };
        w[6] = pack4(meta); w[7] = pack4(meta + 4);
        w[8] = pack4(qlo[0]); w[9] = pack4(qlo[0] + 4); w[10] = pack4(qlo[1]); w[11] = pack4(qlo[1] + 4);
        w[12] = pack4(qlo[2]); w[13] = pack4(qlo[2] + 4); w[14] = pack4(qhi[0]); w[15] = pack4(qhi[0] + 4);
        w[16] = pack4(qhi[1]); w[17] = pack4(qhi[1] + 4); w[18] = pack4(qhi[2]); w[19] = pack4(qhi[2] + 4);
    }
    out.max_depth = max_depth;
    if (!opt.leaf_nodes && int64_t(out.tris.size() / 12) != n) {
        if (err) *err = "accel build: internal error (triangle count)";
        return false;
    }
    return true;
}

Bvh8NodeView decode_node(const uint32_t* w) {
    Bvh8NodeView v;
    for (int a = 0; a < 3; a++) {
        v.origin[a] = bitsf(w[a]);
        v.scale[a] = bitsf(((w[3] >> (8 * a)) & 0xffu) << 23);
    }
    v.imask = uint8_t(w[3] >> 24);
    v.child_base = w[4];
    v.tri_base = w[5];
    for (int s = 0; s < 8; s++) {
        v.meta[s] = uint8_t(w[6 + s / 4] >> (8 * (s % 4)));
        for (int a = 0; a < 3; a++) {
            v.qlo[a][s] = uint8_t(w[8 + 2 * a + s / 4] >> (8 * (s % 4)));
            v.qhi[a][s] = uint8_t(w[14 + 2 * a + s / 4] >> (8 * (s % 4)));
        }
    }
    return v;
}

}  // namespace lmgpu

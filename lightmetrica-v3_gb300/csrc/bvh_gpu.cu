// GPU build of the 8-wide quantized BVH (the node and triangle layout of bvh_build.h), the device
// counterpart of build_bvh8:
//
//   1. triangle boxes and centroid bounds; 30-bit Morton codes of the centroids;
//   2. a radix sort of (code, triangle) pairs (CUB);
//   3. PLOC clustering (Meister & Bittner, "Parallel Locally-Ordered Clustering for Bounding
//      Volume Hierarchy Construction", TVCG 2018): every cluster finds the neighbour within
//      kRadius places of the sorted order whose merged box has the smallest surface area; mutual
//      nearest neighbours merge into a new binary node; compaction by prefix sums; repeat until
//      one cluster is left. Node ids come from the prefix sums, so the tree is deterministic;
//   4. the SAH-optimal 8-wide collapse cost of every binary node (Ylitie, Karras & Laine, HPG
//      2017; the same recurrence and constants as the host builder), computed when the node is
//      created, since its children are final by then;
//   5. top-down emission, one launch per level: each wide node gathers its children from the
//      collapse decisions, orders them by octant, takes contiguous slots for its internal children
//      and its leaf triangles (atomics), writes the triangle records (p1, e1 = p2 - p1, e2 = p3 - p1
//      rounded once in fp32, as Tri's constructor) and quantizes the child boxes exactly as the
//      host builder does (outward rounding plus one quantum of margin, checked in double: the
//      planes p + q * 2^e are exact in double for the exponents chosen).
//
// The reference builds its binary SAH tree with full sorts on the host (accel_sahbvh.cpp:127-267).
// Closest hits do not depend on the tree (the traversal's tie rule is the smaller triangle index),
// so any of these builders gives the same hits.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "bvh_build.h"
#include "runtime.h"

namespace lmgpu {
namespace gpubuild {

constexpr int kMaxLeaf = 3;      // triangles per leaf child (3 bits of meta hold the count)
// PLOC neighbourhood: kRadius clusters on either side. Trace speed of the resulting trees on
// the 3.8M-triangle headline scene (64 spp, Mrays/s; the host SAH builder's tree: 2,680):
// radius 4 -> 2,594, 6 -> 2,684, 8 -> 2,636, 16 -> 2,497, 32 -> 2,540. On random-triangle soups of
// 1.5k-160k triangles every radius from 4 to 8 stays within 1-7 % of the host builder's trees.
constexpr int kRadius = 6;
constexpr int kBlock = 256;
constexpr float kCNode = 1.0f, kCPrim = 0.3f;

// error bits
constexpr int kErrNonFinite = 1, kErrQuantize = 2, kErrLayout = 4;

struct Nodes {
    float4* lo;       // binary node boxes (w unused)
    float4* hi;
    int32_t* left;    // -1 for a leaf
    int32_t* right;   // leaf: its triangle
    int32_t* count;   // triangles below
    float* cost;      // 8 per node: collapse cost with at most i slots of the parent
    int8_t* dec;      // 8 per node: i = 1: 0 leaf / 1 wide node; i > 1: 0 = as i - 1, k = split k | i - k
    int8_t* dnode;    // the node's own split of 8 slots between its children
};

__device__ inline float box_area(float4 lo, float4 hi) {
    if (!(hi.x >= lo.x)) return 0.f;
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return 2.f * (dx * dy + dy * dz + dz * dx);
}

// float -> uint32 with the same order (atomicMin / atomicMax on floats)
__device__ inline uint32_t ordered(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ inline float unordered(uint32_t u) {
    const uint32_t b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

// Triangle boxes, centroids, centroid bounds (cb: 3 ordered minima then 3 ordered maxima).
__global__ void k_prep(const float* __restrict__ P, int64_t n, float4* __restrict__ tlo, float4* __restrict__ thi,
                       float4* __restrict__ cen, uint32_t* cb, int* err) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        float v[9];
        bool finite = true;
        for (int k = 0; k < 9; k++) {
            v[k] = P[9 * i + k];
            finite = finite && isfinite(v[k]);
        }
        if (!finite) atomicOr(err, kErrNonFinite);
        float lo[3], hi[3], c[3];
        for (int a = 0; a < 3; a++) {
            lo[a] = fminf(fminf(v[a], v[3 + a]), v[6 + a]);
            hi[a] = fmaxf(fmaxf(v[a], v[3 + a]), v[6 + a]);
            if (!isfinite(lo[a]) || !isfinite(hi[a])) lo[a] = hi[a] = 0.f;
            c[a] = 0.5f * (lo[a] + hi[a]);
            mn[a] = fminf(mn[a], c[a]);
            mx[a] = fmaxf(mx[a], c[a]);
        }
        tlo[i] = make_float4(lo[0], lo[1], lo[2], 0.f);
        thi[i] = make_float4(hi[0], hi[1], hi[2], 0.f);
        cen[i] = make_float4(c[0], c[1], c[2], 0.f);
    }
    for (int a = 0; a < 3; a++) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
    }
    if ((threadIdx.x & 31) == 0 && mn[0] <= mx[0]) {
        for (int a = 0; a < 3; a++) {
            atomicMin(cb + a, ordered(mn[a]));
            atomicMax(cb + 3 + a, ordered(mx[a]));
        }
    }
}

__device__ inline uint32_t spread10(uint32_t x) {  // 10 bits -> every third bit
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

__global__ void k_morton(const float4* __restrict__ cen, int64_t n, const uint32_t* __restrict__ cb,
                         uint32_t* __restrict__ keys, int32_t* __restrict__ vals) {
    float lo[3], inv[3];
    for (int a = 0; a < 3; a++) {
        lo[a] = unordered(cb[a]);
        const float ext = unordered(cb[3 + a]) - lo[a];
        inv[a] = ext > 0.f ? 1024.f / ext : 0.f;
    }
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const float4 c = cen[i];
        const float cc[3] = {c.x, c.y, c.z};
        uint32_t q[3];
        for (int a = 0; a < 3; a++) q[a] = uint32_t(fminf(fmaxf((cc[a] - lo[a]) * inv[a], 0.f), 1023.f));
        keys[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
        vals[i] = int32_t(i);
    }
}

// Collapse cost of node `id` from its children's (their costs are final).
__device__ void collapse_cost(const Nodes& N, int32_t id, int32_t l, int32_t r, float4 lo, float4 hi, int32_t count,
                              int W) {
    const float A = box_area(lo, hi);
    const float cleaf = count <= kMaxLeaf ? A * kCPrim * float(count) : INFINITY;
    float* c = N.cost + size_t(id) * 8;
    int8_t* d = N.dec + size_t(id) * 8;
    if (l < 0) {
        for (int i = 0; i < 8; i++) { c[i] = cleaf; d[i] = 0; }
        N.dnode[id] = 1;
        return;
    }
    float cl[8], cr[8];
    for (int i = 0; i < 8; i++) { cl[i] = N.cost[size_t(l) * 8 + i]; cr[i] = N.cost[size_t(r) * 8 + i]; }
    float dist[9];
    int8_t dk[9];
    for (int j = 2; j <= 8; j++) {
        dist[j] = INFINITY;
        dk[j] = 1;
        for (int k = 1; k < j; k++) {
            const float v = cl[k - 1] + cr[j - k - 1];
            if (v < dist[j]) { dist[j] = v; dk[j] = int8_t(k); }
        }
    }
    const float cnode = A * kCNode + dist[W];
    float c0 = fminf(cleaf, cnode);
    c[0] = c0;
    d[0] = cleaf <= cnode ? 0 : 1;
    N.dnode[id] = dk[W];
    float prev = c0;
    for (int i = 2; i <= 8; i++) {
        if (prev <= dist[i]) { c[i - 1] = prev; d[i - 1] = 0; }
        else { c[i - 1] = dist[i]; d[i - 1] = dk[i]; prev = dist[i]; }
    }
}

// Leaves in Morton order: leaf k holds triangle vals[k]; every leaf starts as its own cluster.
__global__ void k_leaves(const int32_t* __restrict__ vals, int64_t n, const float4* __restrict__ tlo,
                         const float4* __restrict__ thi, Nodes N, int32_t* __restrict__ clusters) {
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += int64_t(gridDim.x) * blockDim.x) {
        const int32_t t = vals[k];
        const float4 lo = tlo[t], hi = thi[t];
        N.lo[k] = lo;
        N.hi[k] = hi;
        N.left[k] = -1;
        N.right[k] = t;
        N.count[k] = 1;
        collapse_cost(N, int32_t(k), -1, -1, lo, hi, 1, 8);
        clusters[k] = int32_t(k);
    }
}

// Nearest neighbour of every cluster within kRadius places: the smallest merged surface area, ties
// to the smaller position (a total order, so the closest pair is always mutual). Boxes of the block's
// window are staged in shared memory.
__global__ void __launch_bounds__(kBlock) k_nearest(const int32_t* __restrict__ clusters, int32_t m,
                                                    const float4* __restrict__ nlo, const float4* __restrict__ nhi,
                                                    int32_t* __restrict__ nn) {
    __shared__ float4 slo[kBlock + 2 * kRadius], shi[kBlock + 2 * kRadius];
    const int32_t base = int32_t(blockIdx.x) * kBlock - kRadius;
    for (int k = threadIdx.x; k < kBlock + 2 * kRadius; k += kBlock) {
        const int32_t p = base + k;
        if (p >= 0 && p < m) {
            const int32_t c = clusters[p];
            slo[k] = nlo[c];
            shi[k] = nhi[c];
        }
    }
    __syncthreads();
    const int32_t i = int32_t(blockIdx.x) * kBlock + threadIdx.x;
    if (i >= m) return;
    const int li = threadIdx.x + kRadius;
    const float4 alo = slo[li], ahi = shi[li];
    unsigned long long best = ~0ull;
    const int32_t j0 = max(0, i - kRadius), j1 = min(m - 1, i + kRadius);
    for (int32_t j = j0; j <= j1; j++) {
        if (j == i) continue;
        const int lj = j - base;
        const float4 blo = slo[lj], bhi = shi[lj];
        const float4 ulo = make_float4(fminf(alo.x, blo.x), fminf(alo.y, blo.y), fminf(alo.z, blo.z), 0.f);
        const float4 uhi = make_float4(fmaxf(ahi.x, bhi.x), fmaxf(ahi.y, bhi.y), fmaxf(ahi.z, bhi.z), 0.f);
        const unsigned long long key = (static_cast<unsigned long long>(__float_as_uint(box_area(ulo, uhi))) << 32) |
                                       uint32_t(j);
        best = key < best ? key : best;
    }
    nn[i] = m > 1 ? int32_t(best & 0xffffffffu) : i;
}

// flags[i]: bit 32 = i starts a merge (mutual pair, i the smaller position); bit 0 = i stays a
// cluster (no merge, or the merge's first position).
__global__ void k_merge_flags(const int32_t* __restrict__ nn, int32_t m, unsigned long long* __restrict__ flags) {
    const int32_t i = int32_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int32_t j = nn[i];
    const bool mutual = j != i && nn[j] == i;
    const bool lead = mutual && i < j;
    flags[i] = (static_cast<unsigned long long>(lead) << 32) | ((!mutual || lead) ? 1ull : 0ull);
}

__global__ void k_merge(const int32_t* __restrict__ cin, int32_t m, const int32_t* __restrict__ nn,
                        const unsigned long long* __restrict__ flags, const unsigned long long* __restrict__ scan,
                        int32_t next_id, Nodes N, int32_t* __restrict__ cout, unsigned long long* totals, int W) {
    const int32_t i = int32_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const unsigned long long f = flags[i], s = scan[i];
    if (i == m - 1) *totals = s + f;
    if (!(f & 1ull)) return;
    const int32_t slot = int32_t(s & 0xffffffffu);
    if (f >> 32) {
        const int32_t id = next_id + int32_t(s >> 32);
        const int32_t a = cin[i], b = cin[nn[i]];
        const float4 alo = N.lo[a], ahi = N.hi[a], blo = N.lo[b], bhi = N.hi[b];
        const float4 lo = make_float4(fminf(alo.x, blo.x), fminf(alo.y, blo.y), fminf(alo.z, blo.z), 0.f);
        const float4 hi = make_float4(fmaxf(ahi.x, bhi.x), fmaxf(ahi.y, bhi.y), fmaxf(ahi.z, bhi.z), 0.f);
        const int32_t cnt = N.count[a] + N.count[b];
        N.lo[id] = lo;
        N.hi[id] = hi;
        N.left[id] = a;
        N.right[id] = b;
        N.count[id] = cnt;
        collapse_cost(N, id, a, b, lo, hi, cnt, W);
        cout[slot] = id;
    } else {
        cout[slot] = cin[i];
    }
}

// ---- emission ------------------------------------------------------------------------------

struct Emit {
    Nodes N;
    const float* P;          // input triangles (p1, p2, p3)
    uint32_t* nodes;         // 20 words per wide node
    float4* tris;            // 3 float4 per triangle record
    int32_t* tri_slot;       // flattened triangle index -> record
    int32_t* q_bin;          // wide node -> its binary node
    int32_t* wide_count;
    int32_t* tri_count;
    int32_t root;
    int32_t wide_cap;
    int* err;
    int width;               // children per node (2..8)
};

__device__ inline uint32_t fbits(float f) { return __float_as_uint(f); }

// smallest biased exponent eb with 2^(eb-127) >= v (bvh_build.cpp exponent_for)
__device__ int exponent_for(double v) {
    if (!(v > 0)) return 1;
    int e2;
    const double mm = frexp(v, &e2);
    int eb = (mm == 0.5 ? e2 - 1 : e2) + 127;
    return min(254, max(1, eb));
}

// bvh_build.cpp quantize_axis, with the margin check in double: lo, hi, p are floats and
// q * 2^(eb-127) a multiple of the quantum, which the exponent choice keeps within 2^-45 of |p|,
// so p + q * s is exact in double.
__device__ bool quantize_axis(float lo, const float4* clo, const float4* chi, const bool* valid, int a, int eb,
                              float& origin, uint8_t* qlo, uint8_t* qhi) {
    const double s = ldexp(1.0, eb - 127);
    const double pd = double(lo) - 2.0 * s;
    float p = __double2float_rn(pd);
    if (double(p) > pd) p = nextafterf(p, -INFINITY);
    if (!(double(p) < double(lo) - s)) return false;
    for (int k = 0; k < 8; k++) {
        if (!valid[k]) { qlo[k] = 255; qhi[k] = 0; continue; }
        const float bl = a == 0 ? clo[k].x : (a == 1 ? clo[k].y : clo[k].z);
        const float bh = a == 0 ? chi[k].x : (a == 1 ? chi[k].y : chi[k].z);
        const double l = (double(bl) - double(p)) / s;
        const double h = (double(bh) - double(p)) / s;
        const double ql = floor(l) - 1.0, qh = ceil(h) + 1.0;
        if (ql < 0.0 || qh > 255.0) return false;
        const double pl = double(p) + ql * s, ph = double(p) + qh * s;
        if (pl + s > double(bl) || ph - s < double(bh)) return false;
        qlo[k] = uint8_t(ql);
        qhi[k] = uint8_t(qh);
    }
    origin = p;
    return true;
}

__global__ void k_emit(Emit E, int32_t w0, int32_t w1) {
    const int32_t w = w0 + int32_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (w >= w1) return;
    const Nodes& N = E.N;
    const int32_t bin = E.q_bin[w];
    // children of this wide node (binary node ids) and whether each is a leaf
    int32_t ch[8];
    bool leaf[8];
    int nch = 0;
    if (N.left[bin] < 0 || (bin == E.root && N.dec[size_t(bin) * 8] == 0)) {
        ch[0] = bin;
        leaf[0] = true;
        nch = 1;
    } else {
        // depth-first over (binary node, slots), left before right
        int32_t sm[16];
        int si[16];
        int sp = 0;
        const int k0 = N.dnode[bin];
        sm[sp] = N.right[bin]; si[sp++] = E.width - k0;
        sm[sp] = N.left[bin]; si[sp++] = k0;
        while (sp > 0) {
            const int32_t m = sm[--sp];
            int i = si[sp];
            while (i > 1 && N.dec[size_t(m) * 8 + i - 1] == 0) i--;
            if (i == 1) {
                if (nch >= 8) { atomicOr(E.err, kErrLayout); return; }
                ch[nch] = m;
                leaf[nch] = N.left[m] < 0 || N.dec[size_t(m) * 8] == 0;
                nch++;
                continue;
            }
            const int k = N.dec[size_t(m) * 8 + i - 1];
            if (sp + 2 > 16) { atomicOr(E.err, kErrLayout); return; }
            sm[sp] = N.right[m]; si[sp++] = i - k;
            sm[sp] = N.left[m]; si[sp++] = k;
        }
    }
    // octant-ordered slots (bvh_build.cpp: greedy on dot(centroid - center, octant direction))
    float4 nlo = make_float4(INFINITY, INFINITY, INFINITY, 0.f), nhi = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
    for (int i = 0; i < nch; i++) {
        const float4 a = N.lo[ch[i]], b = N.hi[ch[i]];
        nlo = make_float4(fminf(nlo.x, a.x), fminf(nlo.y, a.y), fminf(nlo.z, a.z), 0.f);
        nhi = make_float4(fmaxf(nhi.x, b.x), fmaxf(nhi.y, b.y), fmaxf(nhi.z, b.z), 0.f);
    }
    const float ctr[3] = {0.5f * (nlo.x + nhi.x), 0.5f * (nlo.y + nhi.y), 0.5f * (nlo.z + nhi.z)};
    int child_in[8];
    bool used[8];
    for (int s = 0; s < 8; s++) { child_in[s] = -1; used[s] = false; }
    for (int k = 0; k < nch; k++) {
        int bi = -1, bs = -1;
        double bc = INFINITY;
        for (int i = 0; i < nch; i++) {
            if (used[i]) continue;
            const float4 a = N.lo[ch[i]], b = N.hi[ch[i]];
            const double dc[3] = {0.5 * (double(a.x) + b.x) - ctr[0], 0.5 * (double(a.y) + b.y) - ctr[1],
                                  0.5 * (double(a.z) + b.z) - ctr[2]};
            for (int s = 0; s < 8; s++) {
                if (child_in[s] >= 0) continue;
                double c = 0;
                for (int ax = 0; ax < 3; ax++) c += ((s >> ax) & 1) ? -dc[ax] : dc[ax];
                if (c < bc) { bc = c; bi = i; bs = s; }
            }
        }
        used[bi] = true;
        child_in[bs] = bi;
    }
    // slots for internal children (contiguous wide nodes) and leaf triangles (contiguous records)
    int nint = 0, ntri = 0;
    for (int i = 0; i < nch; i++) {
        if (leaf[i]) ntri += N.count[ch[i]];
        else nint++;
    }
    const int32_t child_base = nint ? atomicAdd(E.wide_count, nint) : 0;
    const int32_t tri_base = ntri ? atomicAdd(E.tri_count, ntri) : 0;
    if (child_base + nint > E.wide_cap) { atomicOr(E.err, kErrLayout); return; }
    uint8_t imask = 0, meta[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    float4 clo[8], chi[8];
    bool valid[8];
    int ki = 0, off = 0;
    for (int s = 0; s < 8; s++) {
        valid[s] = false;
        const int i = child_in[s];
        if (i < 0) continue;
        valid[s] = true;
        clo[s] = N.lo[ch[i]];
        chi[s] = N.hi[ch[i]];
        if (!leaf[i]) {
            imask |= uint8_t(1u << s);
            meta[s] = 0x80;
            E.q_bin[child_base + ki] = ch[i];
            ki++;
            continue;
        }
        const int cnt = N.count[ch[i]];
        if (cnt < 1 || cnt > kMaxLeaf || off > 31) { atomicOr(E.err, kErrLayout); return; }
        meta[s] = uint8_t((cnt << 5) | off);
        // the leaf's triangles, left to right
        int32_t st[8];
        int sp = 0;
        st[sp++] = ch[i];
        while (sp > 0) {
            const int32_t m = st[--sp];
            if (N.left[m] < 0) {
                const int32_t t = N.right[m];
                const float* p = E.P + 9 * int64_t(t);
                const float p1x = p[0], p1y = p[1], p1z = p[2];
                const float4 a = make_float4(p1x, p1y, p1z, __fsub_rn(p[3], p1x));
                const float4 b = make_float4(__fsub_rn(p[4], p1y), __fsub_rn(p[5], p1z), __fsub_rn(p[6], p1x),
                                             __fsub_rn(p[7], p1y));
                const float4 c = make_float4(__fsub_rn(p[8], p1z), __uint_as_float(uint32_t(t)), 0.f, 0.f);
                const int32_t rec = tri_base + off;
                E.tris[size_t(rec) * 3] = a;
                E.tris[size_t(rec) * 3 + 1] = b;
                E.tris[size_t(rec) * 3 + 2] = c;
                E.tri_slot[t] = rec;
                off++;
                continue;
            }
            if (sp + 2 > 8) { atomicOr(E.err, kErrLayout); return; }
            st[sp++] = N.right[m];
            st[sp++] = N.left[m];
        }
    }
    // quantize (bvh_build.cpp quantize)
    int eb[3];
    float origin[3];
    uint8_t qlo[3][8], qhi[3][8];
    const float nl[3] = {nlo.x, nlo.y, nlo.z}, nh[3] = {nhi.x, nhi.y, nhi.z};
    for (int a = 0; a < 3; a++) {
        const double ext = double(nh[a]) - double(nl[a]);
        const double mag = fmax(fabs(double(nl[a])), fabs(double(nh[a])));
        int e = max(exponent_for(ext / 251.0), exponent_for(mag * 1.2e-7));
        bool ok = false;
        for (; e <= 254 && !ok; e++) {
            ok = quantize_axis(nl[a], clo, chi, valid, a, e, origin[a], qlo[a], qhi[a]);
            if (ok) eb[a] = e;
        }
        if (!ok) { atomicOr(E.err, kErrQuantize); return; }
    }
    uint32_t* o = E.nodes + size_t(w) * 20;
    auto pack4 = [](const uint8_t* b) {
        return uint32_t(b[0]) | (uint32_t(b[1]) << 8) | (uint32_t(b[2]) << 16) | (uint32_t(b[3]) << 24);
    };
    o[0] = fbits(origin[0]); o[1] = fbits(origin[1]); o[2] = fbits(origin[2]);
    o[3] = uint32_t(eb[0]) | (uint32_t(eb[1]) << 8) | (uint32_t(eb[2]) << 16) | (uint32_t(imask) << 24);
    o[4] = uint32_t(child_base);
    o[5] = uint32_t(tri_base);
    o[6] = pack4(meta); o[7] = pack4(meta + 4);
    o[8] = pack4(qlo[0]); o[9] = pack4(qlo[0] + 4); o[10] = pack4(qlo[1]); o[11] = pack4(qlo[1] + 4);
    o[12] = pack4(qlo[2]); o[13] = pack4(qlo[2] + 4); o[14] = pack4(qhi[0]); o[15] = pack4(qhi[0] + 4);
    o[16] = pack4(qhi[1]); o[17] = pack4(qhi[1] + 4); o[18] = pack4(qhi[2]); o[19] = pack4(qhi[2] + 4);
}

int grid_of(int64_t n) { return int(std::min<int64_t>((n + kBlock - 1) / kBlock, int64_t(1) << 20)); }

}  // namespace gpubuild

// Builds into device buffers: `nodes` (20 words per wide node), `tris` (12 floats per record),
// `tri_slot` (flattened index -> record). Synchronous on `st`.
void build_bvh8_gpu(const float* tri_p, int64_t n, DevBuf& nodes, DevBuf& tris, DevBuf& tri_slot, int64_t& num_nodes,
                    int32_t& depth, double& sah_cost, cudaStream_t st) {
    using namespace gpubuild;
    if (n <= 0) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "accel build: no triangles");
    if (n > (int64_t(1) << 30)) throw Error(LMGPU_ERR_UNSUPPORTED, "accel build: more than 2^30 triangles on the GPU builder");
    const size_t nn = size_t(2) * size_t(n);
    const int width = std::min(8, std::max(2, tuning().node_width));
    DevBuf P, tlo, thi, cen, cb, err, keys[2], vals[2], blo, bhi, bl, br, bc, cost, dec, dnode, cl[2], nnb, flags, scan,
        totals, q, wide_count, tri_count, tmp;
    P.alloc(size_t(n) * 36);
    LMGPU_CUDA(cudaMemcpyAsync(P.p, tri_p, size_t(n) * 36, cudaMemcpyHostToDevice, st));
    tlo.alloc(size_t(n) * 16); thi.alloc(size_t(n) * 16); cen.alloc(size_t(n) * 16);
    cb.alloc(6 * 4); err.alloc(4);
    const uint32_t cb0[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    LMGPU_CUDA(cudaMemcpyAsync(cb.p, cb0, sizeof(cb0), cudaMemcpyHostToDevice, st));
    LMGPU_CUDA(cudaMemsetAsync(err.p, 0, 4, st));
    const int g = grid_of(n);
    k_prep<<<g, kBlock, 0, st>>>(P.as<float>(), n, tlo.as<float4>(), thi.as<float4>(), cen.as<float4>(), cb.as<uint32_t>(),
                                 err.as<int>());
    for (int b = 0; b < 2; b++) { keys[b].alloc(size_t(n) * 4); vals[b].alloc(size_t(n) * 4); }
    k_morton<<<g, kBlock, 0, st>>>(cen.as<float4>(), n, cb.as<uint32_t>(), keys[0].as<uint32_t>(), vals[0].as<int32_t>());
    LMGPU_CUDA(cudaGetLastError());
    {
        cub::DoubleBuffer<uint32_t> dk(keys[0].as<uint32_t>(), keys[1].as<uint32_t>());
        cub::DoubleBuffer<int32_t> dv(vals[0].as<int32_t>(), vals[1].as<int32_t>());
        size_t tb = 0;
        LMGPU_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, dk, dv, int(n), 0, 30, st));
        tmp.alloc(tb);
        LMGPU_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, dk, dv, int(n), 0, 30, st));
        if (dv.Current() != vals[0].as<int32_t>()) {
            LMGPU_CUDA(cudaMemcpyAsync(vals[0].p, dv.Current(), size_t(n) * 4, cudaMemcpyDeviceToDevice, st));
        }
    }
    blo.alloc(nn * 16); bhi.alloc(nn * 16); bl.alloc(nn * 4); br.alloc(nn * 4); bc.alloc(nn * 4);
    cost.alloc(nn * 8 * 4); dec.alloc(nn * 8); dnode.alloc(nn);
    Nodes N{blo.as<float4>(), bhi.as<float4>(), bl.as<int32_t>(), br.as<int32_t>(), bc.as<int32_t>(), cost.as<float>(),
            dec.as<int8_t>(), dnode.as<int8_t>()};
    cl[0].alloc(size_t(n) * 4); cl[1].alloc(size_t(n) * 4);
    k_leaves<<<g, kBlock, 0, st>>>(vals[0].as<int32_t>(), n, tlo.as<float4>(), thi.as<float4>(), N, cl[0].as<int32_t>());
    LMGPU_CUDA(cudaGetLastError());
    int hbits = 0;
    LMGPU_CUDA(cudaMemcpyAsync(&hbits, err.p, 4, cudaMemcpyDeviceToHost, st));
    LMGPU_CUDA(cudaStreamSynchronize(st));
    if (hbits & kErrNonFinite) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "accel build: non-finite vertex coordinate");

    // PLOC
    nnb.alloc(size_t(n) * 4); flags.alloc(size_t(n) * 8); scan.alloc(size_t(n) * 8); totals.alloc(8);
    size_t sb = 0;
    LMGPU_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, sb, flags.as<unsigned long long>(), scan.as<unsigned long long>(),
                                             int(n), st));
    tmp.alloc(sb);
    int32_t m = int32_t(n), next_id = int32_t(n);
    int cur = 0, iters = 0;
    while (m > 1) {
        const int gm = int((m + kBlock - 1) / kBlock);
        k_nearest<<<gm, kBlock, 0, st>>>(cl[cur].as<int32_t>(), m, N.lo, N.hi, nnb.as<int32_t>());
        k_merge_flags<<<gm, kBlock, 0, st>>>(nnb.as<int32_t>(), m, flags.as<unsigned long long>());
        LMGPU_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, sb, flags.as<unsigned long long>(), scan.as<unsigned long long>(),
                                                 m, st));
        k_merge<<<gm, kBlock, 0, st>>>(cl[cur].as<int32_t>(), m, nnb.as<int32_t>(), flags.as<unsigned long long>(),
                                       scan.as<unsigned long long>(), next_id, N, cl[1 - cur].as<int32_t>(),
                                       totals.as<unsigned long long>(), width);
        LMGPU_CUDA(cudaGetLastError());
        unsigned long long tot = 0;
        LMGPU_CUDA(cudaMemcpyAsync(&tot, totals.p, 8, cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaStreamSynchronize(st));
        const int32_t merges = int32_t(tot >> 32), keep = int32_t(tot & 0xffffffffu);
        if (merges < 1 || keep != m - merges) throw Error(LMGPU_ERR_INTERNAL, "accel build: clustering made no progress");
        next_id += merges;
        m = keep;
        cur = 1 - cur;
        if (++iters > 100000) throw Error(LMGPU_ERR_INTERNAL, "accel build: clustering did not converge");
    }
    int32_t root = 0;
    LMGPU_CUDA(cudaMemcpyAsync(&root, cl[cur].p, 4, cudaMemcpyDeviceToHost, st));
    float rc = 0.f;
    float4 rlo, rhi;
    LMGPU_CUDA(cudaMemcpyAsync(&rc, N.cost + size_t(root) * 8, 4, cudaMemcpyDeviceToHost, st));
    LMGPU_CUDA(cudaMemcpyAsync(&rlo, N.lo + root, 16, cudaMemcpyDeviceToHost, st));
    LMGPU_CUDA(cudaMemcpyAsync(&rhi, N.hi + root, 16, cudaMemcpyDeviceToHost, st));
    LMGPU_CUDA(cudaStreamSynchronize(st));
    {
        const double dx = double(rhi.x) - rlo.x, dy = double(rhi.y) - rlo.y, dz = double(rhi.z) - rlo.z;
        const double ra = 2.0 * (dx * dy + dy * dz + dz * dx);
        sah_cost = ra > 0 ? double(rc) / ra : 0.0;
    }

    // emission, level by level
    const int32_t cap = int32_t(std::max<int64_t>(n, 1));  // wide nodes never exceed the triangles
    nodes.alloc(size_t(cap) * 80);
    tris.alloc(size_t(n) * 48);
    tri_slot.alloc(size_t(n) * 4);
    q.alloc(size_t(cap) * 4);
    wide_count.alloc(4);
    tri_count.alloc(4);
    const int32_t one = 1;
    LMGPU_CUDA(cudaMemcpyAsync(q.p, &root, 4, cudaMemcpyHostToDevice, st));
    LMGPU_CUDA(cudaMemcpyAsync(wide_count.p, &one, 4, cudaMemcpyHostToDevice, st));
    LMGPU_CUDA(cudaMemsetAsync(tri_count.p, 0, 4, st));
    Emit E{N, P.as<float>(), nodes.as<uint32_t>(), tris.as<float4>(), tri_slot.as<int32_t>(), q.as<int32_t>(),
           wide_count.as<int32_t>(), tri_count.as<int32_t>(), root, cap, err.as<int>(), width};
    int32_t w0 = 0, w1 = 1, levels = 0;
    while (w0 < w1) {
        k_emit<<<int((w1 - w0 + 127) / 128), 128, 0, st>>>(E, w0, w1);
        LMGPU_CUDA(cudaGetLastError());
        int32_t nw = 0;
        LMGPU_CUDA(cudaMemcpyAsync(&nw, wide_count.p, 4, cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaMemcpyAsync(&hbits, err.p, 4, cudaMemcpyDeviceToHost, st));
        LMGPU_CUDA(cudaStreamSynchronize(st));
        if (hbits & kErrQuantize) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "accel build: box quantization failed");
        if (hbits) throw Error(LMGPU_ERR_INTERNAL, "accel build: internal error (wide node layout)");
        levels++;
        w0 = w1;
        w1 = nw;
    }
    int32_t nt = 0;
    LMGPU_CUDA(cudaMemcpyAsync(&nt, tri_count.p, 4, cudaMemcpyDeviceToHost, st));
    LMGPU_CUDA(cudaStreamSynchronize(st));
    if (int64_t(nt) != n) throw Error(LMGPU_ERR_INTERNAL, "accel build: internal error (triangle count)");
    num_nodes = w1;
    depth = levels;
}

}  // namespace lmgpu

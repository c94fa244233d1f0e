// Host check of lightmetrica-v3_gb300/csrc/hit_t.h: whenever the double-float evaluation decides
// (hit_t_fast returns true), its float must equal the fp64 chain's float bit for bit. Prints, per
// case family, the cases, the decided ones and the disagreements. Build with -ffp-contract=off.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "hit_t.h"

using lmgpu_ht::hit_t_fast;
using lmgpu_ht::hit_t_fp64;

namespace {

struct Stats {
    long long cases = 0, decided = 0, bad = 0;
};

// One ray aimed at the point p1 + b1 e1 + b2 e2 of a triangle from origin o (all float).
void run_case(Stats& st, const float o[3], const float tgt[3], const float p1[3], const float e1[3], const float e2[3]) {
    float d[3] = {tgt[0] - o[0], tgt[1] - o[1], tgt[2] - o[2]};
    const float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    if (!(len > 0.f)) return;
    for (float& x : d) x /= len;
    st.cases++;
    float fast = 0.f;
    if (!hit_t_fast(o, d, p1, e1, e2, fast)) return;
    st.decided++;
    const float ref = hit_t_fp64(o, d, p1, e1, e2);
    uint32_t a, b;
    std::memcpy(&a, &fast, 4);
    std::memcpy(&b, &ref, 4);
    if (a != b) {
        if (st.bad < 5)
            std::printf("MISMATCH fast %.9g fp64 %.9g o %a %a %a d %a %a %a p1 %a %a %a e1 %a %a %a e2 %a %a %a\n", fast, ref,
                        o[0], o[1], o[2], d[0], d[1], d[2], p1[0], p1[1], p1[2], e1[0], e1[1], e1[2], e2[0], e2[1], e2[2]);
        st.bad++;
    }
}

}  // namespace

int main(int argc, char** argv) {
    const long long n = argc > 1 ? std::atoll(argv[1]) : 200000;
    const unsigned seed = argc > 2 ? unsigned(std::atoi(argv[2])) : 1u;
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<float> U(-1.f, 1.f), U01(0.f, 1.f);
    const char* names[] = {"random", "grazing", "far_small", "large_coords", "small_coords", "axis_aligned", "vertex_edge",
                           "quantized"};
    long long total_bad = 0;
    for (int fam = 0; fam < 8; fam++) {
        Stats st;
        for (long long i = 0; i < n; i++) {
            float scale = 10.f, tri = 2.f, dist = 20.f;
            if (fam == 2) { tri = 1e-3f; dist = 1e3f; }
            if (fam == 3) { scale = 1e4f; tri = 5e2f; dist = 2e4f; }
            if (fam == 4) { scale = 1e-3f; tri = 1e-4f; dist = 2e-3f; }
            float p1[3], e1[3], e2[3], o[3], tgt[3];
            for (int k = 0; k < 3; k++) {
                p1[k] = U(rng) * scale;
                e1[k] = U(rng) * tri;
                e2[k] = U(rng) * tri;
            }
            if (fam == 5) {  // an axis-aligned triangle: one coordinate shared, zeros in the edges
                const int ax = int(rng() % 3);
                e1[ax] = 0.f;
                e2[ax] = 0.f;
            }
            if (fam == 7) {  // coordinates on a 1/64 grid, as modelled scenes often are
                for (int k = 0; k < 3; k++) {
                    p1[k] = std::round(p1[k] * 64.f) / 64.f;
                    e1[k] = std::round(e1[k] * 64.f) / 64.f;
                    e2[k] = std::round(e2[k] * 64.f) / 64.f;
                }
            }
            float b1 = U01(rng), b2 = U01(rng);
            if (b1 + b2 > 1.f) { b1 = 1.f - b1; b2 = 1.f - b2; }
            if (fam == 6) {  // vertices and edge midpoints
                const int w = int(rng() % 6);
                const float bb[6][2] = {{0, 0}, {1, 0}, {0, 1}, {.5f, 0}, {0, .5f}, {.5f, .5f}};
                b1 = bb[w][0];
                b2 = bb[w][1];
            }
            for (int k = 0; k < 3; k++) tgt[k] = p1[k] + b1 * e1[k] + b2 * e2[k];
            if (fam == 1) {  // origin near the triangle's plane: the ray grazes it
                float nrm[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
                const float nl = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
                if (!(nl > 0.f)) continue;
                // an in-plane offset of up to `dist` and a plane offset of 1e-1 .. 1e-7 of it
                const float a1 = U(rng) * dist, a2 = U(rng) * dist;
                const float h = dist * std::pow(10.f, -1.f - 6.f * U01(rng)) * (U(rng) < 0 ? -1.f : 1.f);
                for (int k = 0; k < 3; k++) o[k] = tgt[k] + a1 * e1[k] / tri + a2 * e2[k] / tri + nrm[k] / nl * h;
            } else {
                for (int k = 0; k < 3; k++) o[k] = tgt[k] + U(rng) * dist;
            }
            run_case(st, o, tgt, p1, e1, e2);
        }
        std::printf("%s cases %lld decided %lld bad %lld\n", names[fam], st.cases, st.decided, st.bad);
        total_bad += st.bad;
    }
    return total_bad == 0 ? 0 : 1;
}

// Accel C-ABI (include/lmgpu.h): build the 8-wide BVH on the host, keep it resident on the
// device, and trace batches of rays with one thread per ray.
#include <algorithm>
#include <array>
#include <cmath>
#include <chrono>
#include <cstring>
#include <mutex>
#include <vector>

#include "hit_t.h"
#include "lmgpu_dev.cuh"
#include "runtime.h"

namespace lmgpu {

namespace {
thread_local std::string g_last_error;
}

void set_last_error(const std::string& msg) { g_last_error = msg; }

DeviceInfo& current_device() {
    thread_local DeviceInfo info;
    thread_local bool init = false;
    if (!init) {
        LMGPU_CUDA(cudaGetDevice(&info.device));
        LMGPU_CUDA(cudaDeviceGetAttribute(&info.num_sms, cudaDevAttrMultiProcessorCount, info.device));
        init = true;
    }
    return info;
}

Tuning& tuning() {
    static Tuning t;
    return t;
}

// The builders' options from the process-wide tuning (node width).
BuildOptions tuned_build_options() {
    BuildOptions o;
    o.max_width = tuning().node_width;
    return o;
}

std::shared_mutex& capture_mutex() {
    static std::shared_mutex m;
    return m;
}

constexpr int kTraceBlock = 128;

// Hit distance of an accepted hit: the reference's fp64 distance (accel_sahbvh.cpp:58-75) from the
// same fp32 ray and triangle record (p1, e1, e2), rounded once to float (hit_t.h: a double-float
// evaluation that falls back to the fp64 chain when it cannot decide the float). The fp32 test
// still decides which triangle is hit and where the traversal stops; this only makes the reported
// t agree with the reference's fp64 value to fp32 rounding (an fp32 t of a grazing hit can be
// 2e-5 off relative).
__device__ inline float refine_hit_t(const float4 ra, const float4 rb, const float4 a, const float4 b, const float4 c) {
    const float o[3] = {ra.x, ra.y, ra.z}, d[3] = {rb.x, rb.y, rb.z}, p1[3] = {a.x, a.y, a.z};
    const float e1[3] = {a.w, b.x, b.y}, e2[3] = {b.z, b.w, c.x};
    return lmgpu_ht::hit_t(o, d, p1, e1, e2);
}

// rays: 2 float4 per ray (o, tmin) (d, tmax). refill > 0: block b of G takes the groups of 32
// consecutive rays b, b + G, b + 2G, ... and its warps fetch from them dynamically through a
// shared-memory counter (no state outside the launch, so calls on several streams may overlap).
// Interleaving the groups gives every block a sample of the whole batch: with one contiguous
// chunk per block, rays in caller order (camera rays, bounces sorted by origin or direction) left
// some blocks all the expensive rays, and a batch of diffuse bounces in pixel order traced 11 %
// slower than the same rays shuffled. refill == 0: one ray per thread, grid-stride.
template <bool kAnyHit, bool kTwoLevel>
__global__ void __launch_bounds__(kTraceBlock) k_trace_batch(Bvh8 bvh, const float4* __restrict__ rays, int64_t n,
                                                            lmgpu_hit* __restrict__ hits, uint8_t* __restrict__ occluded,
                                                            int* __restrict__ err, int refill) {
    extern __shared__ uint32_t smem[];
    __shared__ int s_fetch;
    const int stride = blockDim.x;
    uint32_t* sb = smem + threadIdx.x;
    uint32_t* sbits = smem + stride * bvh.depth + threadIdx.x;
    int lerr = 0;
    auto store = [&](int64_t i, const TraceHit& h) {
        if (kAnyHit) {
            occluded[i] = h.id >= 0 ? 1 : 0;
        } else {
            lmgpu_hit r;
            r.t = h.id >= 0 ? h.t : 0.f;
            r.u = h.u;
            r.v = h.v;
            r.prim = h.id;
            hits[i] = r;
        }
    };
    if (refill > 0) {
        const int64_t G = gridDim.x, blk = blockIdx.x;
        const int64_t ngroups = (n + 31) / 32;
        const int64_t mine = blk < ngroups ? (ngroups - 1 - blk) / G + 1 : 0;
        // only the batch's last group can be short, and it is this block's last one if it is ours
        int64_t count = mine * 32;
        if (mine > 0 && blk + (mine - 1) * G == ngroups - 1) count -= ngroups * 32 - n;
        auto ray_of = [&](int k) { return (blk + int64_t(k >> 5) * G) * 32 + (k & 31); };
        if (threadIdx.x == 0) s_fetch = 0;
        __syncthreads();
        fetch_loop<kAnyHit, false, kTwoLevel>(
            int(count), Fetch{&s_fetch, nullptr, refill}, bvh, sb, sbits, stride, &lerr,
            [&](int k, Trav& s, Bvh8&) {
                const int64_t i = ray_of(k);
                const float4 a = rays[2 * i], b = rays[2 * i + 1];
                trav_init(s, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, b.w);
            },
            [&](int k, const Trav& s) { store(ray_of(k), s.best); });
    } else {
        for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
            const float4 a = rays[2 * i], b = rays[2 * i + 1];
            store(i, trace_bvh8<kAnyHit, false, kTwoLevel>(bvh, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, b.w, sb, sbits, stride,
                                                nullptr, nullptr, &lerr));
        }
    }
    if (lerr) atomicOr(err, lerr);
}

// The fp64 hit distance of every closest hit (refine_hit_t), as a pass of its own after the
// trace: inside the persistent traversal loop the lanes whose ray ends would run its long chain
// of double ops while the warp's other lanes wait.
__global__ void __launch_bounds__(256) k_refine_hits(const float4* __restrict__ rays, lmgpu_hit* __restrict__ hits,
                                                     int64_t n, const float4* __restrict__ tris,
                                                     const int32_t* __restrict__ tri_slot) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const int32_t id = hits[i].prim;
        if (id < 0) continue;
        const float4* tp = tris + size_t(__ldg(tri_slot + id)) * 3;
        hits[i].t = refine_hit_t(rays[2 * i], rays[2 * i + 1], __ldg(tp), __ldg(tp + 1), __ldg(tp + 2));
    }
}

// Instrumented pass: node visits and triangle tests summed over every `sample`-th ray.
template <bool kAnyHit, bool kTwoLevel>
__global__ void __launch_bounds__(kTraceBlock) k_trace_count(Bvh8 bvh, const float4* __restrict__ rays, int64_t n,
                                                            int sample, unsigned long long* sums, int* err) {
    extern __shared__ uint32_t smem[];
    const int stride = blockDim.x;
    uint32_t* sb = smem + threadIdx.x;
    uint32_t* sbits = smem + stride * bvh.depth + threadIdx.x;
    int lerr = 0;
    uint32_t nodes = 0, tris = 0, cnt = 0;
    for (int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; j * sample < n; j += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i = j * sample;
        const float4 a = rays[2 * i], b = rays[2 * i + 1];
        trace_bvh8<kAnyHit, true, kTwoLevel>(bvh, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, b.w, sb, sbits, stride, &nodes, &tris,
                                  &lerr);
        cnt++;
    }
    atomicAdd(&sums[0], (unsigned long long)nodes);
    atomicAdd(&sums[1], (unsigned long long)tris);
    atomicAdd(&sums[2], (unsigned long long)cnt);
    if (lerr) atomicOr(err, lerr);
}

template <typename K>
int trace_grid(K kernel, size_t smem, int64_t n) {
    if (smem > 48 * 1024) LMGPU_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = 0;
    LMGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTraceBlock, smem));
    per_sm = per_sm < 1 ? 1 : per_sm;
    const int64_t need = (n + kTraceBlock - 1) / kTraceBlock;
    int64_t g = int64_t(per_sm) * current_device().num_sms;
    if (need < g) g = need;
    return int(g < 1 ? 1 : g);
}

Bvh8 device_view(const lmgpu_accel* a) {
    Bvh8 b;
    b.nodes = a->nodes.as<const uint4>();
    b.tris = a->tris.as<const float4>();
    b.depth = a->depth;
    b.num_nodes = uint32_t(a->num_nodes);
    b.inst = a->num_instances > 0 ? a->inst.as<const float4>() : nullptr;
    b.max_visits = a->max_visits ? a->max_visits : uint32_t(a->num_nodes);
    return b;
}

size_t trace_smem(const lmgpu_accel* a) { return size_t(2) * 4 * kTraceBlock * size_t(a->depth); }

void check_built(const lmgpu_accel* a) {
    if (!a) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "accel is null");
    if (a->num_nodes == 0) throw Error(LMGPU_ERR_UNINITIALIZED, "accel is not built (call lmgpu_accel_build)");
    if (a->depth > 96) throw Error(LMGPU_ERR_UNSUPPORTED, "BVH deeper than the traversal stack supports");
}

void launch_trace(const lmgpu_accel* a, const void* d_rays, int64_t n, void* d_hits, uint8_t* d_occ, cudaStream_t st,
                  int* d_err) {
    if (n <= 0) return;
    if ((reinterpret_cast<uintptr_t>(d_rays) & 15u) != 0)
        throw Error(LMGPU_ERR_INVALID_ARGUMENT, "ray buffer must be 16-byte aligned");
    const Bvh8 b = device_view(a);
    const size_t smem = trace_smem(a);
    auto run = [&](auto kernel) {
        const int g = trace_grid(kernel, smem, n);
        kernel<<<g, kTraceBlock, smem, st>>>(b, static_cast<const float4*>(d_rays), n, static_cast<lmgpu_hit*>(d_hits), d_occ,
                                             d_err, tuning().trace_refill);
    };
    const bool two = a->num_instances > 0;
    if (d_occ) two ? run(k_trace_batch<true, true>) : run(k_trace_batch<true, false>);
    else two ? run(k_trace_batch<false, true>) : run(k_trace_batch<false, false>);
    LMGPU_CUDA(cudaGetLastError());
    if (!d_occ && !two && a->tri_slot.p && n > 0) {
        const int g = int(std::min<int64_t>((n + 255) / 256, int64_t(current_device().num_sms) * 8));
        k_refine_hits<<<g, 256, 0, st>>>(static_cast<const float4*>(d_rays), static_cast<lmgpu_hit*>(d_hits), n,
                                         a->tris.as<const float4>(), a->tri_slot.as<const int32_t>());
        LMGPU_CUDA(cudaGetLastError());
    }
}

}  // namespace lmgpu

using namespace lmgpu;

extern "C" {

const char* lmgpu_last_error(void) { return g_last_error.c_str(); }

int lmgpu_version(void) { return 1; }

int lmgpu_tune_set(const char* key, int64_t value) {
    return guarded([&] {
        if (!key) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "key is null");
        const std::string k(key);
        if (k == "trace_refill") {
            if (value < 0 || value > 32) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "trace_refill must be in [0, 32]");
            tuning().trace_refill = int(value);
        } else if (k == "batch_first_pass") {
            if (value != 0 && value != 1) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "batch_first_pass must be 0 or 1");
            tuning().batch_first_pass = int(value);
        } else if (k == "shade_minblocks") {
            if (value < 2 || value > 4) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "shade_minblocks must be 2, 3 or 4");
            tuning().shade_minblocks = int(value);
        } else if (k == "node_width") {
            if (value < 2 || value > 8) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "node_width must be in [2, 8]");
            tuning().node_width = int(value);
        } else if (k == "shade_specialize") {
            if (value != 0 && value != 1) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "shade_specialize must be 0 or 1");
            tuning().shade_specialize = int(value);
        } else {
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "unknown tuning key: " + k);
        }
    });
}

int lmgpu_tune_get(const char* key, int64_t* value) {
    return guarded([&] {
        if (!key || !value) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        const std::string k(key);
        if (k == "trace_refill") *value = tuning().trace_refill;
        else if (k == "shade_minblocks") *value = tuning().shade_minblocks;
        else if (k == "batch_first_pass") *value = tuning().batch_first_pass;
        else if (k == "node_width") *value = tuning().node_width;
        else if (k == "shade_specialize") *value = tuning().shade_specialize;
        else throw Error(LMGPU_ERR_INVALID_ARGUMENT, "unknown tuning key: " + k);
    });
}

int lmgpu_set_device(int device) {
    return guarded([&] {
        LMGPU_CUDA(cudaSetDevice(device));
        DeviceInfo& d = current_device();
        d.device = device;
        LMGPU_CUDA(cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, device));
    });
}

int lmgpu_accel_create(lmgpu_accel** out) {
    return guarded([&] {
        if (!out) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "out is null");
        *out = new lmgpu_accel();  // device memory is allocated by lmgpu_accel_build
    });
}

int lmgpu_accel_destroy(lmgpu_accel* accel) {
    return guarded([&] { delete accel; });
}

int lmgpu_accel_build(lmgpu_accel* accel, const float* tri_p, int64_t num_tris) {
    return lmgpu_accel_build_ex(accel, tri_p, num_tris, LMGPU_BUILDER_HOST_SAH);
}

int lmgpu_accel_build_ex(lmgpu_accel* accel, const float* tri_p, int64_t num_tris, int32_t builder) {
    return guarded([&] {
        if (!accel || (!tri_p && num_tris > 0)) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "accel or triangles null");
        if (builder != LMGPU_BUILDER_HOST_SAH && builder != LMGPU_BUILDER_GPU_PLOC)
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "unknown builder");
        const auto t0 = std::chrono::steady_clock::now();
        if (builder == LMGPU_BUILDER_GPU_PLOC) {
            cudaStream_t st;
            LMGPU_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            int64_t nn = 0;
            int32_t depth = 0;
            double sah = 0;
            try {
                build_bvh8_gpu(tri_p, num_tris, accel->nodes, accel->tris, accel->tri_slot, nn, depth, sah, st);
            } catch (...) {
                cudaStreamDestroy(st);
                throw;
            }
            cudaStreamDestroy(st);
            accel->num_nodes = nn;
            accel->depth = depth;
            accel->sah_cost = sah;
        } else {
        Bvh8Host h;
        std::string err;
        if (!build_bvh8(tri_p, num_tris, h, &err, tuned_build_options())) throw Error(LMGPU_ERR_INVALID_ARGUMENT, err);
        accel->nodes.upload(h.nodes.data(), h.nodes.size());
        accel->tris.upload(h.tris.data(), h.tris.size());
        {
            // flattened triangle index -> leaf-order record, for the fp64 hit distance
            std::vector<int32_t> slot(size_t(num_tris), -1);
            for (int64_t k = 0; k < num_tris; k++) {
                uint32_t id;
                std::memcpy(&id, &h.tris[size_t(12) * k + 9], sizeof(id));
                if (int64_t(id) >= num_tris || slot[id] != -1) throw Error(LMGPU_ERR_INTERNAL, "triangle records are not a permutation");
                slot[id] = int32_t(k);
            }
            accel->tri_slot.upload(slot.data(), slot.size());
        }
        accel->num_nodes = int64_t(h.nodes.size() / 20);
        accel->depth = h.max_depth;
        accel->sah_cost = h.sah_cost;
        }
        accel->err.alloc(sizeof(int));
        LMGPU_CUDA_SYNC(cudaMemset(accel->err.p, 0, sizeof(int)));
        accel->num_tris = num_tris;
        accel->builder = builder;
        accel->inst.release();
        accel->num_instances = 0;
        accel->max_visits = 0;
        accel->inst_blas.clear();
        accel->inst_xform.clear();
        accel->inst_id_base.clear();
        accel->blas_offsets.clear();
        LMGPU_CUDA_SYNC(cudaDeviceSynchronize());
        accel->build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    });
}

int lmgpu_accel_build_instanced(lmgpu_accel* accel, const float* tri_p, const int64_t* blas_offsets, int32_t num_blas,
                                const lmgpu_instance* instances, int32_t num_instances) {
    return lmgpu_accel_build_instanced_ex(accel, tri_p, blas_offsets, num_blas, instances, num_instances,
                                          LMGPU_BUILDER_HOST_SAH);
}

int lmgpu_accel_build_instanced_ex(lmgpu_accel* accel, const float* tri_p, const int64_t* blas_offsets, int32_t num_blas,
                                   const lmgpu_instance* instances, int32_t num_instances, int32_t builder) {
    return guarded([&] {
        if (builder != LMGPU_BUILDER_HOST_SAH && builder != LMGPU_BUILDER_GPU_PLOC)
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "unknown builder");
        if (!accel || !tri_p || !blas_offsets || !instances) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        if (num_blas < 1 || num_instances < 1) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "need at least one BLAS and one instance");
        if (blas_offsets[0] != 0) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "blas_offsets[0] must be 0");
        for (int32_t b = 0; b < num_blas; b++)
            if (blas_offsets[b + 1] <= blas_offsets[b]) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "every BLAS needs a triangle");
        const auto t0 = std::chrono::steady_clock::now();
        // bottom level: one 8-wide tree per triangle set, hit indices local to the set
        std::vector<Bvh8Host> bl(static_cast<size_t>(num_blas));
        std::vector<std::array<double, 6>> lbox(static_cast<size_t>(num_blas));
        for (int32_t b = 0; b < num_blas; b++) {
            const int64_t off = blas_offsets[b], cnt = blas_offsets[b + 1] - off;
            if (builder == LMGPU_BUILDER_GPU_PLOC) {
                // the BLAS built on the GPU, brought back for the merge into one node array
                DevBuf dn, dt, ds;
                int64_t nn = 0;
                int32_t depth = 0;
                double sah = 0;
                cudaStream_t st;
                LMGPU_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
                try {
                    build_bvh8_gpu(tri_p + 9 * off, cnt, dn, dt, ds, nn, depth, sah, st);
                } catch (...) {
                    cudaStreamDestroy(st);
                    throw;
                }
                cudaStreamDestroy(st);
                bl[b].nodes.resize(size_t(nn) * 20);
                bl[b].tris.resize(size_t(cnt) * 12);
                LMGPU_CUDA_SYNC(cudaMemcpy(bl[b].nodes.data(), dn.p, size_t(nn) * 80, cudaMemcpyDeviceToHost));
                LMGPU_CUDA_SYNC(cudaMemcpy(bl[b].tris.data(), dt.p, size_t(cnt) * 48, cudaMemcpyDeviceToHost));
                bl[b].max_depth = depth;
                bl[b].sah_cost = sah;
            } else {
                std::string err;
                if (!build_bvh8(tri_p + 9 * off, cnt, bl[b], &err, tuned_build_options()))
                    throw Error(LMGPU_ERR_INVALID_ARGUMENT, err);
            }
            std::array<double, 6> bx{1e300, 1e300, 1e300, -1e300, -1e300, -1e300};
            for (int64_t i = 9 * off; i < 9 * (off + cnt); i += 3)
                for (int a = 0; a < 3; a++) {
                    bx[a] = std::min(bx[a], double(tri_p[i + a]));
                    bx[3 + a] = std::max(bx[3 + a], double(tri_p[i + a]));
                }
            lbox[b] = bx;
        }
        // instances: inverse transforms, world boxes (the 8 transformed corners of the BLAS box,
        // rounded outward to fp32), first hit indices
        std::vector<float> tl(size_t(9) * num_instances);
        std::vector<float4> rec(size_t(4) * num_instances);
        std::vector<int64_t> id_base(static_cast<size_t>(num_instances));
        std::vector<double> xf(size_t(12) * num_instances);
        int64_t total = 0;
        for (int32_t i = 0; i < num_instances; i++) {
            const lmgpu_instance& in = instances[i];
            if (in.blas < 0 || in.blas >= num_blas) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "instance refers to a missing BLAS");
            double M[12];
            for (int k = 0; k < 12; k++) {
                M[k] = double(in.transform[k]);
                if (!std::isfinite(M[k])) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "non-finite instance transform");
                xf[size_t(12) * i + k] = M[k];
            }
            const double a00 = M[0], a01 = M[1], a02 = M[2], a10 = M[4], a11 = M[5], a12 = M[6], a20 = M[8], a21 = M[9], a22 = M[10];
            const double det = a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) + a02 * (a10 * a21 - a11 * a20);
            if (!(std::fabs(det) > 1e-30)) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "singular instance transform");
            const double inv[9] = {(a11 * a22 - a12 * a21) / det, (a02 * a21 - a01 * a22) / det, (a01 * a12 - a02 * a11) / det,
                                   (a12 * a20 - a10 * a22) / det, (a00 * a22 - a02 * a20) / det, (a02 * a10 - a00 * a12) / det,
                                   (a10 * a21 - a11 * a20) / det, (a01 * a20 - a00 * a21) / det, (a00 * a11 - a01 * a10) / det};
            const double t[3] = {M[3], M[7], M[11]};
            for (int r = 0; r < 3; r++) {
                const double tr = -(inv[3 * r] * t[0] + inv[3 * r + 1] * t[1] + inv[3 * r + 2] * t[2]);
                rec[4 * size_t(i) + r] = make_float4(float(inv[3 * r]), float(inv[3 * r + 1]), float(inv[3 * r + 2]), float(tr));
            }
            const auto& bx = lbox[in.blas];
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            for (int c = 0; c < 8; c++) {
                const double p[3] = {bx[(c & 1) ? 3 : 0], bx[(c & 2) ? 4 : 1], bx[(c & 4) ? 5 : 2]};
                for (int r = 0; r < 3; r++) {
                    const double w = M[4 * r] * p[0] + M[4 * r + 1] * p[1] + M[4 * r + 2] * p[2] + M[4 * r + 3];
                    lo[r] = std::min(lo[r], w);
                    hi[r] = std::max(hi[r], w);
                }
            }
            for (int r = 0; r < 3; r++) {
                // pad by a relative 2^-20 for the fp32 rounding of the ray transform, then round outward
                const double pad = 1e-6 * std::max({std::fabs(lo[r]), std::fabs(hi[r]), hi[r] - lo[r], 1e-30});
                float l = float(lo[r] - pad), h = float(hi[r] + pad);
                if (double(l) > lo[r] - pad) l = std::nextafter(l, -INFINITY);
                if (double(h) < hi[r] + pad) h = std::nextafter(h, INFINITY);
                tl[9 * size_t(i) + r] = l;
                tl[9 * size_t(i) + 3 + r] = h;
                tl[9 * size_t(i) + 6 + r] = l;
            }
            id_base[i] = total;
            total += blas_offsets[in.blas + 1] - blas_offsets[in.blas];
        }
        if (total > (int64_t(1) << 31) - 1) throw Error(LMGPU_ERR_UNSUPPORTED, "more than 2^31-1 instanced triangles");
        // top level over the instance boxes; its leaves are instance pseudo-nodes
        Bvh8Host top;
        std::string err;
        BuildOptions opt;
        opt.leaf_nodes = true;
        if (!build_bvh8(tl.data(), num_instances, top, &err, opt)) throw Error(LMGPU_ERR_INVALID_ARGUMENT, err);
        // one node array: top level first, then every BLAS with its child and triangle bases moved
        std::vector<uint32_t> nodes = top.nodes;
        std::vector<float> tris;
        std::vector<uint32_t> root(static_cast<size_t>(num_blas));
        std::vector<uint64_t> bnodes(static_cast<size_t>(num_blas));
        int32_t bdepth = 0;
        for (int32_t b = 0; b < num_blas; b++) {
            const uint32_t noff = uint32_t(nodes.size() / 20), toff = uint32_t(tris.size() / 12);
            root[b] = noff;
            bnodes[b] = bl[b].nodes.size() / 20;
            for (size_t k = 0; k < bl[b].nodes.size(); k += 20) {
                uint32_t w[20];
                std::memcpy(w, &bl[b].nodes[k], sizeof(w));
                w[4] += noff;
                w[5] += toff;
                nodes.insert(nodes.end(), w, w + 20);
            }
            tris.insert(tris.end(), bl[b].tris.begin(), bl[b].tris.end());
            bdepth = std::max(bdepth, bl[b].max_depth);
        }
        if (nodes.size() / 20 > size_t(UINT32_MAX)) throw Error(LMGPU_ERR_UNSUPPORTED, "too many BVH nodes");
        uint64_t visits = top.nodes.size() / 20;
        for (int32_t i = 0; i < num_instances; i++) {
            visits += bnodes[instances[i].blas];
            const uint32_t rb[4] = {root[instances[i].blas], uint32_t(id_base[i]), 0u, 0u};
            std::memcpy(&rec[4 * size_t(i) + 3], rb, sizeof(rb));
        }
        accel->nodes.upload(nodes.data(), nodes.size());
        accel->tris.upload(tris.data(), tris.size());
        accel->tri_slot.release();  // two-level hits keep the fp32 distance of the instance-frame ray
        accel->inst.upload(rec.data(), rec.size());
        accel->err.alloc(sizeof(int));
        LMGPU_CUDA_SYNC(cudaMemset(accel->err.p, 0, sizeof(int)));
        accel->num_tris = total;
        accel->num_nodes = int64_t(nodes.size() / 20);
        accel->depth = top.max_depth + bdepth;
        accel->sah_cost = top.sah_cost;
        accel->num_instances = num_instances;
        accel->max_visits = uint32_t(std::min<uint64_t>(visits, UINT32_MAX));
        accel->inst_blas.resize(size_t(num_instances));
        for (int32_t i = 0; i < num_instances; i++) accel->inst_blas[i] = instances[i].blas;
        accel->inst_xform = xf;
        accel->inst_id_base = id_base;
        accel->blas_offsets.assign(blas_offsets, blas_offsets + num_blas + 1);
        LMGPU_CUDA_SYNC(cudaDeviceSynchronize());
        accel->build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    });
}

int lmgpu_accel_intersect(lmgpu_accel* accel, const float* rays, int64_t n, lmgpu_hit* hits) {
    return guarded([&] {
        check_built(accel);
        if (n < 0 || (n > 0 && (!rays || !hits))) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "rays or hits null");
        if (n == 0) return;
        accel->scratch_rays.alloc(size_t(n) * 32);
        accel->scratch_hits.alloc(size_t(n) * sizeof(lmgpu_hit));
        // With page-locked host buffers the batch goes in chunks of 2^21 rays through three streams:
        // one copies every chunk in back to back, one traces each chunk once its rays are in, one
        // copies each chunk's hits out once traced, so the copy engines and the trace run side by
        // side (two streams that each copied in, traced and copied out their own chunks kept the
        // next copy-in waiting behind a copy-out: 2,914 Mrays/s against 4,178 on the device).
        // Pageable buffers go in one copy each way (chunked copies from pageable memory measured
        // slower: 1,102 -> 775 Mrays/s).
        constexpr int64_t kChunk = int64_t(1) << 21;
        auto page_locked = [](const void* p) {
            cudaPointerAttributes a{};
            if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
                cudaGetLastError();  // clear the (non-sticky) error an unknown pointer may leave
                return false;
            }
            return a.type == cudaMemoryTypeHost;
        };
        if (n <= kChunk || !page_locked(rays) || !page_locked(hits)) {
            LMGPU_CUDA_SYNC(cudaMemset(accel->err.p, 0, sizeof(int)));
            LMGPU_CUDA_SYNC(cudaMemcpy(accel->scratch_rays.p, rays, size_t(n) * 32, cudaMemcpyHostToDevice));
            launch_trace(accel, accel->scratch_rays.p, n, accel->scratch_hits.p, nullptr, 0, accel->err.as<int>());
            LMGPU_CUDA_SYNC(cudaMemcpy(hits, accel->scratch_hits.p, size_t(n) * sizeof(lmgpu_hit), cudaMemcpyDeviceToHost));
        } else {
            std::shared_lock<std::shared_mutex> lk(capture_mutex());
            const int64_t nchunks = (n + kChunk - 1) / kChunk;
            cudaStream_t sts[3] = {nullptr, nullptr, nullptr};  // copy in, trace, copy out
            std::vector<cudaEvent_t> evs(size_t(2 * nchunks), nullptr);
            auto release = [&] {
                for (auto st : sts)
                    if (st) {
                        cudaStreamSynchronize(st);
                        cudaStreamDestroy(st);
                    }
                for (auto e : evs)
                    if (e) cudaEventDestroy(e);
            };
            cudaError_t first_err = cudaSuccess;
            try {
                for (auto& st : sts) LMGPU_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
                for (auto& e : evs) LMGPU_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
                char* d_r = static_cast<char*>(accel->scratch_rays.p);
                char* d_h = static_cast<char*>(accel->scratch_hits.p);
                // the error flag is cleared on the trace stream before its first trace
                LMGPU_CUDA(cudaMemsetAsync(accel->err.p, 0, sizeof(int), sts[1]));
                for (int64_t c = 0; c < nchunks; c++) {
                    const int64_t off = c * kChunk, m = std::min(kChunk, n - off);
                    LMGPU_CUDA(cudaMemcpyAsync(d_r + off * 32, rays + off * 8, size_t(m) * 32, cudaMemcpyHostToDevice, sts[0]));
                    LMGPU_CUDA(cudaEventRecord(evs[size_t(2 * c)], sts[0]));
                }
                for (int64_t c = 0; c < nchunks; c++) {
                    const int64_t off = c * kChunk, m = std::min(kChunk, n - off);
                    LMGPU_CUDA(cudaStreamWaitEvent(sts[1], evs[size_t(2 * c)], 0));
                    launch_trace(accel, d_r + off * 32, m, d_h + off * int64_t(sizeof(lmgpu_hit)), nullptr, sts[1],
                                 accel->err.as<int>());
                    LMGPU_CUDA(cudaEventRecord(evs[size_t(2 * c + 1)], sts[1]));
                }
                for (int64_t c = 0; c < nchunks; c++) {
                    const int64_t off = c * kChunk, m = std::min(kChunk, n - off);
                    LMGPU_CUDA(cudaStreamWaitEvent(sts[2], evs[size_t(2 * c + 1)], 0));
                    LMGPU_CUDA(cudaMemcpyAsync(hits + off, d_h + off * int64_t(sizeof(lmgpu_hit)), size_t(m) * sizeof(lmgpu_hit),
                                               cudaMemcpyDeviceToHost, sts[2]));
                }
                for (auto st : sts) {
                    const cudaError_t e = cudaStreamSynchronize(st);
                    if (first_err == cudaSuccess) first_err = e;
                }
            } catch (...) {
                release();
                throw;
            }
            release();
            LMGPU_CUDA(first_err);
        }
        int herr = 0;
        LMGPU_CUDA_SYNC(cudaMemcpy(&herr, accel->err.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (herr) throw Error(LMGPU_ERR_INTERNAL, "traversal consistency check failed (code " + std::to_string(herr) + ")");
    });
}

int lmgpu_accel_intersect_device(lmgpu_accel* accel, const void* d_rays, int64_t n, void* d_hits, void* stream) {
    return guarded([&] {
        check_built(accel);
        if (n < 0 || (n > 0 && (!d_rays || !d_hits))) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "rays or hits null");
        launch_trace(accel, d_rays, n, d_hits, nullptr, static_cast<cudaStream_t>(stream), accel->err.as<int>());
    });
}

int lmgpu_accel_occluded_device(lmgpu_accel* accel, const void* d_rays, int64_t n, uint8_t* d_occluded, void* stream) {
    return guarded([&] {
        check_built(accel);
        if (n < 0 || (n > 0 && (!d_rays || !d_occluded))) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "rays or output null");
        launch_trace(accel, d_rays, n, nullptr, d_occluded, static_cast<cudaStream_t>(stream), accel->err.as<int>());
    });
}

int lmgpu_accel_get_stats(const lmgpu_accel* accel, lmgpu_accel_stats* out) {
    return guarded([&] {
        if (!accel || !out) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        std::memset(out, 0, sizeof(*out));
        out->num_tris = accel->num_tris;
        out->num_nodes = accel->num_nodes;
        out->max_depth = accel->depth;
        out->build_seconds = accel->build_seconds;
        out->sah_cost = accel->sah_cost;
        out->device_bytes = int64_t(accel->nodes.bytes + accel->tris.bytes + accel->inst.bytes);
        out->num_instances = accel->num_instances;
    });
}

int lmgpu_bvh8_build_host(const float* tri_p, int64_t num_tris, uint32_t* nodes, float* tris, int64_t* num_nodes,
                          int32_t* max_depth) {
    return guarded([&] {
        if (!tri_p || !nodes || !tris || !num_nodes || !max_depth) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        Bvh8Host h;
        std::string err;
        if (!build_bvh8(tri_p, num_tris, h, &err, tuned_build_options())) throw Error(LMGPU_ERR_INVALID_ARGUMENT, err);
        if (h.nodes.size() > size_t(20) * size_t(num_tris > 0 ? num_tris : 1))
            throw Error(LMGPU_ERR_INTERNAL, "node count above the documented bound");
        std::memcpy(nodes, h.nodes.data(), h.nodes.size() * 4);
        std::memcpy(tris, h.tris.data(), h.tris.size() * 4);
        *num_nodes = int64_t(h.nodes.size() / 20);
        *max_depth = h.max_depth;
    });
}

int lmgpu_bvh8_build_gpu(const float* tri_p, int64_t num_tris, uint32_t* nodes, float* tris, int64_t* num_nodes,
                         int32_t* max_depth) {
    return guarded([&] {
        if (!tri_p || !nodes || !tris || !num_nodes || !max_depth) throw Error(LMGPU_ERR_INVALID_ARGUMENT, "null argument");
        DevBuf dn, dt, ds;
        int64_t nn = 0;
        int32_t depth = 0;
        double sah = 0;
        cudaStream_t st;
        LMGPU_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        try {
            build_bvh8_gpu(tri_p, num_tris, dn, dt, ds, nn, depth, sah, st);
        } catch (...) {
            cudaStreamDestroy(st);
            throw;
        }
        cudaStreamDestroy(st);
        if (nn > (num_tris > 0 ? num_tris : 1)) throw Error(LMGPU_ERR_INTERNAL, "node count above the documented bound");
        LMGPU_CUDA_SYNC(cudaMemcpy(nodes, dn.p, size_t(nn) * 80, cudaMemcpyDeviceToHost));
        LMGPU_CUDA_SYNC(cudaMemcpy(tris, dt.p, size_t(num_tris) * 48, cudaMemcpyDeviceToHost));
        *num_nodes = nn;
        *max_depth = depth;
    });
}

int lmgpu_accel_trace_counts(lmgpu_accel* accel, const void* d_rays, int64_t n, int32_t any_hit, int32_t sample,
                             double* mean_nodes, double* mean_tris) {
    return guarded([&] {
        check_built(accel);
        if (!d_rays || n <= 0 || sample <= 0 || !mean_nodes || !mean_tris)
            throw Error(LMGPU_ERR_INVALID_ARGUMENT, "invalid argument");
        DevBuf sums;
        sums.alloc(3 * sizeof(unsigned long long));
        LMGPU_CUDA_SYNC(cudaMemset(sums.p, 0, 3 * sizeof(unsigned long long)));
        LMGPU_CUDA_SYNC(cudaMemset(accel->err.p, 0, sizeof(int)));
        const Bvh8 b = device_view(accel);
        const size_t smem = trace_smem(accel);
        const int64_t m = (n + sample - 1) / sample;
        auto run = [&](auto kernel) {
            const int g = trace_grid(kernel, smem, m);
            kernel<<<g, kTraceBlock, smem>>>(b, static_cast<const float4*>(d_rays), n, sample, sums.as<unsigned long long>(),
                                             accel->err.as<int>());
        };
        const bool two = accel->num_instances > 0;
        if (any_hit) two ? run(k_trace_count<true, true>) : run(k_trace_count<true, false>);
        else two ? run(k_trace_count<false, true>) : run(k_trace_count<false, false>);
        LMGPU_CUDA(cudaGetLastError());
        unsigned long long h[3];
        LMGPU_CUDA_SYNC(cudaMemcpy(h, sums.p, sizeof(h), cudaMemcpyDeviceToHost));
        const double c = h[2] ? double(h[2]) : 1.0;
        *mean_nodes = double(h[0]) / c;
        *mean_tris = double(h[1]) / c;
    });
}

}  // extern "C"

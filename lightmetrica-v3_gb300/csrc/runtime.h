// Host-side runtime shared by the C-ABI translation units: status codes, error text, device
// buffers and the opaque handle types declared in include/lmgpu.h.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <shared_mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/lmgpu.h"
#include "bvh_build.h"

namespace lmgpu {

// An error carrying an LMGPU_ERR_* code; C entry points catch it and return the code.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

#define LMGPU_CUDA(call)                                                                         \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            throw ::lmgpu::Error(e_ == cudaErrorMemoryAllocation ? LMGPU_ERR_OUT_OF_MEMORY : LMGPU_ERR_CUDA, \
                                 std::string(#call) + ": " + cudaGetErrorString(e_));           \
    } while (0)

// Stream capture (the shared wavefront's CUDA graphs) against calls that may synchronize the
// device implicitly: cudaMalloc, cudaFree, synchronous copies and memsets, cudaDeviceSynchronize.
// Such a call made by another host thread while a capture is open (a scene built on a worker
// thread while the serving loop captures its chunk) invalidates the capture. The capture holds
// this mutex exclusively; those calls hold it shared, so they wait only while a capture is open
// (microseconds) and never wait on each other.
std::shared_mutex& capture_mutex();

#define LMGPU_CUDA_SYNC(call)                                                                    \
    do {                                                                                          \
        std::shared_lock<std::shared_mutex> lk_(::lmgpu::capture_mutex());                         \
        LMGPU_CUDA(call);                                                                         \
    } while (0)

// Runs `fn` and converts any failure into a status code plus lmgpu_last_error() text.
template <typename Fn>
int guarded(Fn&& fn) {
    try {
        fn();
        return LMGPU_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return LMGPU_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return LMGPU_ERR_INTERNAL;
    }
}

// Owning device allocation.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) {
            std::shared_lock<std::shared_mutex> lk(capture_mutex());
            cudaFree(p);
        }
        p = nullptr;
        bytes = 0;
    }
    void alloc(size_t n) {
        if (n <= bytes && p) return;
        release();
        if (n == 0) return;
        LMGPU_CUDA_SYNC(cudaMalloc(&p, n));
        bytes = n;
    }
    template <typename T>
    void upload(const T* src, size_t count) {
        alloc(count * sizeof(T));
        if (count) LMGPU_CUDA(cudaMemcpy(p, src, count * sizeof(T), cudaMemcpyHostToDevice));
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

// GPU builder of the 8-wide tree (bvh_gpu.cu): device buffers in the layout of bvh_build.h, plus
// the flattened-index -> record map. Synchronous on `st`.
void build_bvh8_gpu(const float* tri_p, int64_t n, DevBuf& nodes, DevBuf& tris, DevBuf& tri_slot, int64_t& num_nodes,
                    int32_t& depth, double& sah_cost, cudaStream_t st);

struct DeviceInfo {
    int device = 0;
    int num_sms = 0;
};
DeviceInfo& current_device();

// Launch-shape parameters that change speed but never results (set through lmgpu_tune_set).
struct Tuning {
    // Persistent trace kernels: idle lanes of a warp fetch new rays once fewer than this many
    // lanes still trace (1..32); 0 runs one ray per thread, grid-stride, without refills.
    int trace_refill = 24;
    // Shade kernels: resident blocks per SM their register budget allows (2, 3 or 4).
    int shade_minblocks = 4;
    // Shared wavefront: start every job's sample-0 paths before other paths (1) or start paths
    // strictly in submission order (0).
    int batch_first_pass = 1;
    // BVH builds: children per node the 8-wide collapse may use (2..8; the layout keeps 8 slots)
    int node_width = 8;
    // Shade kernels: 1 = the kernel specialised for the scene's features, 0 = the full-feature one
    int shade_specialize = 1;
};
Tuning& tuning();

}  // namespace lmgpu

struct lmgpu_accel {
    int device = 0;
    int64_t num_tris = 0;    // triangles a ray can hit (instanced: counted once per instance)
    int64_t num_nodes = 0;   // node records (instanced: top-level + instance pseudo-nodes + every BLAS)
    int32_t depth = 0;       // traversal stack bound (instanced: top-level depth + deepest BLAS)
    double build_seconds = 0;
    double sah_cost = 0;
    lmgpu::DevBuf nodes, tris;
    lmgpu::DevBuf tri_slot;  // single-level builds: flattened triangle index -> leaf-order record
    int32_t builder = 0;     // LMGPU_BUILDER_* of the last build
    lmgpu::DevBuf scratch_rays, scratch_hits, err;
    // two-level builds only
    lmgpu::DevBuf inst;                      // per instance: inverse transform rows (3 float4), {root, id_base}
    int32_t num_instances = 0;
    uint32_t max_visits = 0;                 // node visits one ray can make (0: num_nodes)
    std::vector<int32_t> inst_blas;          // per instance: its BLAS
    std::vector<double> inst_xform;          // per instance: world-from-local, 12 doubles (row-major 3x4)
    std::vector<int64_t> inst_id_base;       // per instance: first hit index
    std::vector<int64_t> blas_offsets;       // BLAS b owns triangles [blas_offsets[b], blas_offsets[b+1])
};

/*
 * lmgpu -- GB300-native ray traversal and path tracing behind Lightmetrica v3's Accel and
 * Renderer interfaces. C ABI: plain pointers, sizes and status codes; no C++ or torch types.
 *
 * Every entry point returns LMGPU_OK (0) or an LMGPU_ERR_* code; the message of the last failure
 * on the calling thread is lmgpu_last_error(). No exception crosses this boundary.
 *
 * Conventions shared with the reference (include/lm/math.h:54-56): Inf = 1e10, Eps = 1e-3 (an
 * absolute ray offset). Ray tests follow src/accel/accel_sahbvh.cpp:58-75 (Moller-Trumbore with
 * the reference's operation order) in fp32 with IEEE rounding and no fused multiply-add.
 */
#ifndef LMGPU_H
#define LMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LMGPU_OK 0
#define LMGPU_ERR_INVALID_ARGUMENT 1 /* lm::Error::InvalidArgument (include/lm/exception.h) */
#define LMGPU_ERR_UNSUPPORTED 2      /* lm::Error::Unsupported */
#define LMGPU_ERR_UNINITIALIZED 3    /* lm::Error::Uninitialized: e.g. render before build */
#define LMGPU_ERR_CUDA 4             /* a CUDA runtime call failed */
#define LMGPU_ERR_OUT_OF_MEMORY 5    /* device allocation failed or the HBM budget is exceeded */
#define LMGPU_ERR_TIMEOUT 6          /* a bounded device-side wait gave up */
#define LMGPU_ERR_INTERNAL 7         /* a device-side consistency check failed */

typedef struct lmgpu_accel lmgpu_accel;
typedef struct lmgpu_scene lmgpu_scene;
typedef struct lmgpu_film lmgpu_film;

/* Closest-hit record. Replaces Accel::Hit (include/lm/accel.h:49-55): `prim` is the flattened
 * triangle index (the order in which Accel::build visits primitives and faces), which the caller
 * maps to (primitive node, face) exactly as accel_sahbvh.cpp:296-298 maps indices_[mi].
 * prim == -1 means no hit. t is the ray parameter, (u, v) the barycentrics of p2 and p3. */
typedef struct lmgpu_hit {
    float t, u, v;
    int32_t prim;
} lmgpu_hit;

/* Accel statistics for reports (not part of the reference interface). */
typedef struct lmgpu_accel_stats {
    int64_t num_tris;
    int64_t num_nodes;       /* 8-wide nodes, 80 bytes each */
    int32_t max_depth;       /* 8-wide levels, root = 1 (two-level: top + deepest BLAS) */
    int32_t num_instances;   /* 0 for a single-level build */
    double build_seconds;    /* host SAH build + collapse + upload */
    double sah_cost;         /* SAH cost of the binary tree before collapsing */
    int64_t device_bytes;    /* nodes + triangles resident on the device */
} lmgpu_accel_stats;

/* ---------------------------------------------------------------------------------------------
 * Library
 */
const char* lmgpu_last_error(void);
int lmgpu_version(void);
/* Launch-shape tuning (no reference counterpart). Keys:
 *   "trace_refill"  persistent trace kernels of the path tracers: a warp's idle lanes fetch new
 *                   rays once fewer than this many lanes still trace (1..32; default 24); 0 runs
 *                   one ray per thread without refills.
 *   "shade_minblocks" shade kernels: 256-thread blocks per SM their register budget must allow
 *                   (2: up to 128 registers; 3: up to 80; 4: up to 64, the default).
 *   "batch_first_pass" shared wavefront: start the sample-0 paths of every job before any other
 *                   path (1, the default: a newly admitted job's first image does not wait behind
 *                   older jobs' later samples) or start paths in submission order (0).
 *   "node_width"     BVH builds (both builders): children per node the collapse may use (2..8,
 *                   default 8; the 80-byte node keeps 8 slots, a narrower tree leaves some empty).
 *   "shade_specialize" path-tracing shade kernels: 1 (default) runs the kernel specialised for the
 *                   scene's features, 0 the full-feature kernel.
 * Tuning changes speed only, never results. Process-wide; set it between renders. */
int lmgpu_tune_set(const char* key, int64_t value);
int lmgpu_tune_get(const char* key, int64_t* value);

/* Selects the CUDA device used by every later call on this thread's handles (default 0). */
int lmgpu_set_device(int device);

/* ---------------------------------------------------------------------------------------------
 * Accel. Replaces the accel::sahbvh / accel::nanort / accel::embree slot.
 */

/* Accel construction. The accel's Json props (embree_params.h:105-115 for accel::embree) have no
 * counterpart; the builder is chosen per build (lmgpu_accel_build_ex). */
int lmgpu_accel_create(lmgpu_accel** out);
int lmgpu_accel_destroy(lmgpu_accel* accel);

/* Accel::build(const Scene&) (include/lm/accel.h:38; accel_sahbvh.cpp:127-151 flattens the scene
 * graph first). The caller passes the flattened triangles: tri_p holds num_tris x 9 floats, the
 * world-space p1, p2, p3 of each triangle in flattening order. The data is copied. */
int lmgpu_accel_build(lmgpu_accel* accel, const float* tri_p, int64_t num_tris);

/* Builders of the 8-wide tree (the reference's accel_sahbvh.cpp:127-267 sorts fully per node on
 * the host). Closest hits do not depend on the builder: the traversal's tie rule (the smaller
 * triangle index) makes them independent of the tree.
 *  LMGPU_BUILDER_HOST_SAH -- binned SAH binary tree on the host threads, SAH-optimal 8-wide
 *                            collapse (lmgpu_accel_build's builder);
 *  LMGPU_BUILDER_GPU_PLOC -- on the GPU: Morton order, PLOC clustering into a binary tree, the same
 *                            SAH-optimal collapse and quantization. */
#define LMGPU_BUILDER_HOST_SAH 0
#define LMGPU_BUILDER_GPU_PLOC 1
int lmgpu_accel_build_ex(lmgpu_accel* accel, const float* tri_p, int64_t num_tris, int32_t builder);

/* One instance of a bottom-level triangle set: `transform` is its world-from-local matrix, the top
 * three rows of the 4x4 (row-major; the last row is 0 0 0 1). */
typedef struct lmgpu_instance {
    int32_t blas;
    int32_t reserved;
    float transform[12];
} lmgpu_instance;

/* Two-level build, the accel::embreeinstanced form of Accel::build (accel_embree_instanced.cpp:
 * 84-230: one level of instancing; an instance group's subtree is flattened once in its own frame
 * and shared by all its instances). tri_p holds the triangles of every bottom-level set (BLAS)
 * back to back, each set in its own frame; BLAS b owns triangles [blas_offsets[b],
 * blas_offsets[b + 1]). The top level is an 8-wide tree over the instances' world boxes. Hit
 * indices count the instances' triangles in instance order: instance i's local triangle j is
 * index id_base(i) + j with id_base(i) the sum of the earlier instances' BLAS sizes, the order in
 * which a flattening of the same scene graph would list them. Triangle tests run in the
 * instance's frame (ray moved by the fp32 inverse transform), so t, u, v agree with a flattened
 * build up to that rounding. The data is copied. */
int lmgpu_accel_build_instanced(lmgpu_accel* accel, const float* tri_p, const int64_t* blas_offsets, int32_t num_blas,
                                const lmgpu_instance* instances, int32_t num_instances);
/* The same with the bottom-level trees built by `builder` (LMGPU_BUILDER_*); the top level over the
 * instance boxes is always built on the host (one leaf per instance). */
int lmgpu_accel_build_instanced_ex(lmgpu_accel* accel, const float* tri_p, const int64_t* blas_offsets, int32_t num_blas,
                                   const lmgpu_instance* instances, int32_t num_instances, int32_t builder);

/* Accel::intersect(Ray, tmin, tmax) (include/lm/accel.h:70; accel_sahbvh.cpp:269-299) over a
 * batch. Host buffers: rays is n x 8 floats (ox, oy, oz, tmin, dx, dy, dz, tmax); hits receives n
 * records. Copies in, traces, copies out, and returns when the hits are in `hits`. With page-locked
 * (pinned) host buffers, batches larger than 2^21 rays go in chunks through three streams (copy in,
 * trace, copy out), so that the copies run beside the trace. */
int lmgpu_accel_intersect(lmgpu_accel* accel, const float* rays, int64_t n, lmgpu_hit* hits);

/* Same, device-resident: d_rays (n x 8 floats, 16-byte aligned) and d_hits (n records) are
 * device pointers; the trace is enqueued on `stream` (a cudaStream_t, 0 = legacy default stream)
 * and the call returns without synchronizing. */
int lmgpu_accel_intersect_device(lmgpu_accel* accel, const void* d_rays, int64_t n, void* d_hits, void* stream);

/* Scene::visible (include/lm/scene.h:343-364) is a closest-hit query whose result is only tested
 * for existence; this any-hit form returns the same boolean per ray: d_occluded[i] = 1 if any
 * triangle is hit in [tmin, tmax]. Device pointers, enqueued on `stream`. */
int lmgpu_accel_occluded_device(lmgpu_accel* accel, const void* d_rays, int64_t n, uint8_t* d_occluded, void* stream);

int lmgpu_accel_get_stats(const lmgpu_accel* accel, lmgpu_accel_stats* out);

/* Host-only build (no device needed; no reference counterpart): fills the 8-wide node words (20
 * per node) and triangle records (12 floats per triangle) exactly as lmgpu_accel_build uploads
 * them. `nodes` must hold 20 * max(num_tris, 1) words and `tris` 12 * num_tris floats. */
int lmgpu_bvh8_build_host(const float* tri_p, int64_t num_tris, uint32_t* nodes, float* tris, int64_t* num_nodes,
                          int32_t* max_depth);
/* The same through the GPU builder (LMGPU_BUILDER_GPU_PLOC), copied back to host memory (no
 * reference counterpart; for tests). Same buffer sizes. Synchronous. */
int lmgpu_bvh8_build_gpu(const float* tri_p, int64_t num_tris, uint32_t* nodes, float* tris, int64_t* num_nodes,
                         int32_t* max_depth);

/* Instrumented trace (no reference counterpart; feeds the roofline's algorithmic byte count):
 * over every `sample`-th ray of the device batch, the mean number of 8-wide nodes visited and
 * of triangles tested, for closest-hit (any_hit = 0) or any-hit traversal. Synchronous. */
int lmgpu_accel_trace_counts(lmgpu_accel* accel, const void* d_rays, int64_t n, int32_t any_hit, int32_t sample,
                             double* mean_nodes, double* mean_tris);

/* ---------------------------------------------------------------------------------------------
 * Scene description for rendering. Replaces the state that renderer::pt / renderer::raycast read
 * through Scene_ (src/scene.cpp): flattened geometry with shading data, the primitive table, the
 * materials (material_{diffuse,glossy,glass,mirror}.cpp), the light list in scene-graph traversal
 * order (scene.cpp:279-286), and the camera (camera_pinhole.cpp).
 */
#define LMGPU_MAT_DIFFUSE 0
#define LMGPU_MAT_GLOSSY 1
#define LMGPU_MAT_GLASS 2
#define LMGPU_MAT_MIRROR 3
#define LMGPU_MAT_MIXTURE 4  /* material::mixture_wavefrontobj without alpha mask: diffuse + glossy */

typedef struct lmgpu_material {
    int32_t type;       /* LMGPU_MAT_* */
    float color[3];     /* diffuse and mixture: Kd; glossy: Ks; otherwise unused */
    float ax, ay;       /* glossy and mixture: GGX roughness */
    float ni;           /* glass index of refraction */
    float ks[3];        /* mixture: Ks of its glossy lobe */
    int32_t map_kd;     /* diffuse and mixture: texture whose texel replaces Kd (material_diffuse.cpp:36-40), or -1 */
    int32_t mask;       /* mixture: alpha-mask texture, 4 channels (model_wavefrontobj.cpp:403-410), or -1 */
} lmgpu_material;

/* texture::bitmap (src/texture/texture_bitmap.cpp): w x h texels of c floats (3 = RGB, 4 = RGBA) at
 * lmgpu_scene_desc::texels + offset, row-major with row 0 at the bottom (stbi's flip on load).
 * Looked up at the nearest texel of the wrapped coordinate (texture_bitmap.cpp:68-85). Image
 * textures are supported by renderer::pt and renderer::raycast. */
typedef struct lmgpu_texture {
    int32_t w, h, c, reserved;
    int64_t offset;
} lmgpu_texture;

#define LMGPU_LIGHT_AREA 0
#define LMGPU_LIGHT_ENVCONST 1
#define LMGPU_LIGHT_ENV 2
#define LMGPU_LIGHT_POINT 3        /* light::point (src/light/light_point.cpp) */
#define LMGPU_LIGHT_DIRECTIONAL 4  /* light::directional (src/light/light_directional.cpp) */

typedef struct lmgpu_light {
    int32_t type;       /* LMGPU_LIGHT_* */
    float ke[3];        /* area: Ke; envconst, point, directional: Le */
    /* area: a range of the light-triangle arrays below. The sampling CDF is built from the
     * untransformed (mesh-local) triangle areas, as light_area.cpp:68-80 does. */
    int64_t tri_offset, tri_count;
    float transform_j;  /* |det| of the light primitive's linear transform (math.h:742-745) */
    /* env: a w x h x 3 fp32 texel block at env_offset in env_texels; rot in degrees. */
    int32_t env_w, env_h;
    int64_t env_offset;
    float rot_deg, scale;
    /* point: the world-space position (the primitive's transform is not applied,
     * light_point.cpp:84-88); directional: the direction the light travels, normalized here
     * (light_directional.cpp:34-37). Unused by the other types. */
    float vec[3];
} lmgpu_light;

typedef struct lmgpu_camera {
    /* camera::pinhole props (camera_pinhole.cpp:76-97) */
    float position[3], center[3], up[3];
    float vfov, aspect;
} lmgpu_camera;

typedef struct lmgpu_scene_desc {
    /* Flattened triangles in accel-build order (the same order as lmgpu_accel_build's input). */
    int64_t num_tris;
    const float* positions;      /* num_tris x 9: world-space p1, p2, p3 (the accel-build input) */
    const float* normals;        /* num_tris x 9: per-corner normals transformed by normal_M */
    const float* geo_normals;    /* num_tris x 3: normalize(normal_M * geometry_normal(local)) */
    const int32_t* tri_prim;     /* num_tris: index into the primitive table */
    /* Primitive table: one row per flattened primitive node that carries a mesh. */
    int32_t num_prims;
    const int32_t* prim_material; /* index into materials */
    const int32_t* prim_light;    /* index into lights, or -1 */
    int32_t num_materials;
    const lmgpu_material* materials;
    /* Lights in traversal order (uniform selection, scene.cpp:374-382). At most one env light. */
    int32_t num_lights;
    const lmgpu_light* lights;
    int64_t num_light_tris;
    const float* light_tri_p;      /* num_light_tris x 9: world-space p1, p2, p3 */
    const float* light_tri_gn;     /* num_light_tris x 3: world-space geometry normal */
    const float* light_tri_area;   /* num_light_tris: mesh-local triangle area */
    int64_t num_env_texels;        /* floats in env_texels */
    const float* env_texels;
    int32_t has_camera;
    lmgpu_camera camera;
    /* Image textures (needed when a material has map_kd or mask >= 0): per triangle the three
     * corners' texture coordinates (num_tris x 6 floats, u v per corner, in the shading records'
     * order), the texture table and the texels. */
    const float* texcoords;
    int32_t num_textures;
    const lmgpu_texture* textures;
    int64_t num_texels;
    const float* texels;
} lmgpu_scene_desc;

/* Scene::build (src/scene.cpp:274-317) for the GPU renderers: uploads the description and binds
 * the accel, which must already be built over the same flattened triangles. */
int lmgpu_scene_create(lmgpu_scene** out, lmgpu_accel* accel, const lmgpu_scene_desc* desc);
int lmgpu_scene_destroy(lmgpu_scene* scene);
/* Device bytes the scene holds (geometry, shading data, tables), excluding the accel. */
int lmgpu_scene_device_bytes(const lmgpu_scene* scene, int64_t* out);

/* ---------------------------------------------------------------------------------------------
 * Film. Replaces film::bitmap (src/film/film_bitmap.cpp): an fp32 RGB accumulator on the device.
 * Pixel (x, y) is element y*w + x; row 0 is the bottom of the image (rp.y grows upward), as in
 * the reference's raster_to_pixel (include/lm/film.h:166-171).
 */
int lmgpu_film_create(lmgpu_film** out, int32_t w, int32_t h);
int lmgpu_film_destroy(lmgpu_film* film);
int lmgpu_film_clear(lmgpu_film* film);
/* Film::buffer (film_bitmap.cpp:202-208): copies h x w x 3 floats to host memory. */
/* Measurement helper (no reference counterpart): L2 read bandwidth in GB/s, from `iters` streaming
 * passes over a `bytes`-sized buffer (>= 1 MB; below the L2 size) with L1-bypassing loads. The
 * roofline of the trace kernels quotes it beside HBM, as their node arrays fit in L2. */
int lmgpu_probe_l2_bandwidth(int64_t bytes, int32_t iters, double* gbs);

/* Every pixel set to rgb (3 floats): renderer::blank's Film::clear + set_pixel loop
 * (src/renderer/renderer_blank.cpp:36-45). */
int lmgpu_film_fill(lmgpu_film* film, const float* rgb);
int lmgpu_film_read(lmgpu_film* film, float* out_rgb);
/* Device pointer to the h x w x 3 fp32 pixels (valid until the film is destroyed). */
int lmgpu_film_device_ptr(lmgpu_film* film, void** out);
/* No reference counterpart. Relative MSE of the film's estimate, from its even- and odd-pass
 * accumulators (renders with split_passes): per pixel and channel the variance of the mean is
 * (A - B)^2 * nA * nB / N^2 with A, B the even- and odd-pass means over nA, nB passes and N = nA +
 * nB, divided by (I^2 + eps) with I the estimate; averaged over pixels and channels. The error of
 * an N-pass estimate falls as 1/N, so N * rel_mse / target passes reach `target`. Needs at least
 * one pass in each accumulator. */
int lmgpu_film_rel_mse(lmgpu_film* film, double eps, double* rel_mse);

/* ---------------------------------------------------------------------------------------------
 * Renderers.
 */

/* renderer::raycast (src/renderer/renderer_raycast.cpp:48-101). color may be NULL. */
typedef struct lmgpu_raycast_params {
    float bg_color[3];
    int32_t use_constant_color;
    int32_t visualize_normal;
    int32_t has_color;
    float color[3];
} lmgpu_raycast_params;

int lmgpu_render_raycast(lmgpu_scene* scene, lmgpu_film* film, const lmgpu_raycast_params* params, void* stream);

#define LMGPU_SAMPLING_NAIVE 0
#define LMGPU_SAMPLING_NEE 1
#define LMGPU_SAMPLING_MIS 2
#define LMGPU_PRIMARY_PIXEL 0
#define LMGPU_PRIMARY_IMAGE 1

/* renderer::pt (src/renderer/renderer_pt.cpp:51-315) with scheduler::spp::sample
 * (src/scheduler.cpp:17-50). max_verts counts path vertices including the camera vertex, so a
 * maximum path length of L edges is max_verts = L + 1. Random numbers come from a Philox4x32-10
 * stream keyed by (seed, pixel * spp + sample, vertex), independent of launch shape. */
typedef struct lmgpu_pt_params {
    int64_t spp;
    int32_t max_verts;
    uint32_t seed;
    int32_t sampling_mode;      /* LMGPU_SAMPLING_* ("mis" is the reference default) */
    int32_t primary_mode;       /* LMGPU_PRIMARY_* ("pixel" is the reference default) */
    int64_t wave_paths;         /* paths in flight per wave; 0 = library default */
    int32_t accumulate;         /* 1: add to the film; the film's scale becomes 1 / (total spp) */
    int32_t instrument;         /* 1: count node visits / triangle tests on every 64th traced ray;
                                   2: on every traced ray, and record the ray with the most visits */
    int32_t split_passes;       /* 1 (no reference counterpart): keep even and odd sample passes in two
                                   accumulators of the film, for lmgpu_film_rel_mse. A film that holds
                                   split passes keeps splitting the passes later jobs add to it.
                                   Not with instrument. */
    int32_t reserved;
} lmgpu_pt_params;

typedef struct lmgpu_render_stats {
    int64_t paths;
    int64_t rays;               /* every traced segment: extension + shadow */
    int64_t extension_rays;
    int64_t shadow_rays;
    double elapsed_ms;          /* device time of the render (CUDA events) */
    double trace_ms;            /* device time inside the extension + shadow trace kernels */
    double extend_ms, shade_ms, shadow_ms, generate_ms;  /* device time per kernel kind */
    int64_t extend_launches, shadow_launches;
    /* with params->instrument: mean 8-wide nodes visited / triangles tested per traced ray */
    double ext_nodes, ext_tris, shadow_nodes, shadow_tris;
    /* with params->instrument == 2: the most nodes one ray visited, and that ray (o, tmin, d, tmax) */
    int64_t ext_max_nodes, shadow_max_nodes;
    float ext_worst_ray[8], shadow_worst_ray[8];
} lmgpu_render_stats;

/* Renders into `film` (cleared first unless params->accumulate) on `stream` and waits for it.
 * stats may be NULL. The film holds the estimate scaled by 1/spp in both primary-ray modes (image
 * mode: w*h / paths with w*h*spp paths), as renderer_pt.cpp:307-312 rescales it. The render runs as
 * one job of the device's shared wavefront (see lmgpu_batch_* below): params->wave_paths paths in
 * flight (0: 2^25, about 270 bytes each, 9 GB held by the device after the first call; 2^24 measured
 * 1.2 % slower on the 3.8M-triangle 1920x1080 64-spp frame), finished paths replaced by new ones
 * until the job drains. Instrumented renders (params->instrument) run in fixed waves instead,
 * one launch per bounce. Either way the image is the same up to the order of fp32 additions.
 * Calls on one device from several host threads take turns. */
int lmgpu_render_pt(lmgpu_scene* scene, lmgpu_film* film, const lmgpu_pt_params* params, void* stream,
                    lmgpu_render_stats* stats);

/* renderer::lt (src/renderer/renderer_lt.cpp:50-160, light tracing with next-event connections
 * to the camera) with scheduler::spi::sample (src/scheduler.cpp:114-138): num_samples light paths,
 * each started from a light chosen uniformly (path::sample_primary_ray(LE), path.h:101-118; an
 * environment light starts its rays on the disk of the scene's bounding sphere). Every surface
 * vertex but specular ones connects to the pinhole camera; the film receives the sum over paths
 * scaled by w*h / (light paths), renderer_lt.cpp:157. Light paths are numbered
 * [first_path, first_path + num_samples); path p's random numbers are the Philox stream keyed by
 * (seed, p, vertex), so a render split into calls with consecutive first_path and accumulate
 * gives the single call's image (no reference counterpart: scheduler::spi::time's rounds). */
typedef struct lmgpu_lt_params {
    int64_t num_samples;
    int64_t first_path;
    int32_t max_verts;          /* path vertices including the light and the camera vertex */
    uint32_t seed;
    int64_t wave_paths;         /* light paths per wave; 0 = 2^24 (about 230 bytes each, held by the
                                   device after the first call) */
    int32_t accumulate;         /* 1: add to the film; the scale becomes w*h / (all light paths) */
    int32_t reserved;
} lmgpu_lt_params;

/* Renders into `film` on `stream` and waits for it (the replacement of Renderer_LT_NEE::render).
 * stats may be NULL; stats->paths counts light paths. */
int lmgpu_render_lt(lmgpu_scene* scene, lmgpu_film* film, const lmgpu_lt_params* params, void* stream,
                    lmgpu_render_stats* stats);

/* renderer::bdpt (src/renderer/renderer_bdpt.cpp:297-413 over include/lm/bidir.h) with
 * scheduler::spi::sample: num_samples samples, each one eye subpath (a primary ray over the whole
 * image) and one light subpath of up to max_verts vertices, combined by every strategy (s light
 * vertices, t eye vertices, min_verts <= s + t <= max_verts) with the power-heuristic weight of
 * bidir.h:460-479; the film is scaled by w*h / (samples), renderer_bdpt.cpp:397-399. Sample p's
 * random numbers are the Philox stream keyed by (seed, p, subpath vertex), so consecutive calls
 * with first_path and accumulate add up to one render. A strategy whose own pdf is 0 contributes
 * nothing (the reference asserts it is not 0). */
#define LMGPU_BDPT_ALL 0      /* renderer::bdpt: every strategy, power heuristic (bidir.h:460-479) */
#define LMGPU_BDPT_PT_NAIVE 1 /* renderer::pt_naive_path (renderer_bdpt.cpp:63-124): s = 0 only, no light
                                 subpath, unweighted */
#define LMGPU_BDPT_PT_NEE 2   /* renderer::pt_nee_path (renderer_bdpt.cpp:129-200): per length the strategy
                                 s = 1, or s = 0 when the eye vertex it connects is specular; unweighted */
#define LMGPU_BDPT_LT_NEE 3   /* renderer::lt_nee_path (renderer_bdpt.cpp:205-288): t = 1 only, unweighted */
#define LMGPU_BDPT_OPT 4      /* renderer::bdptopt (renderer_bdptopt.cpp:315-400, 419-535): every strategy,
                                 balance heuristic over pdfs without component pdfs */
typedef struct lmgpu_bdpt_params {
    int64_t num_samples;
    int64_t first_path;
    int32_t min_verts;          /* the reference's default is 2 */
    int32_t max_verts;          /* 2..64 */
    uint32_t seed;
    int32_t accumulate;
    int64_t wave_paths;         /* samples per wave; 0 = 2^22, or fewer so that the connection queue holds
                                   at most 2^28 rays. Each sample of a wave takes 2 * max_verts * 80 bytes of
                                   vertex records and max_verts * (max_verts - 1) / 2 * 48 bytes of queue. */
    int32_t strategy;           /* LMGPU_BDPT_* */
    int32_t reserved;
} lmgpu_bdpt_params;

int lmgpu_render_bdpt(lmgpu_scene* scene, lmgpu_film* film, const lmgpu_bdpt_params* params, void* stream,
                      lmgpu_render_stats* stats);

/* ---------------------------------------------------------------------------------------------
 * Shared wavefront for many jobs (no reference counterpart: the reference renders one job at a
 * time). Each job is a built scene, a film and renderer::pt parameters; the paths of every job go
 * through the same generate / extend / shade / shadow kernels, each carrying its job id, and
 * paths that finish are replaced by new ones (from the same or the next job) until the queue is
 * drained. A job's film receives exactly what lmgpu_render_pt gives for it alone (same Philox
 * keys), up to the order of fp32 additions. Jobs may be submitted while earlier ones are still
 * in flight (continuous batching).
 */
typedef struct lmgpu_batch lmgpu_batch;

/* queue_paths: paths in flight (0 = 2^22). */
int lmgpu_batch_create(lmgpu_batch** out, int64_t queue_paths);
int lmgpu_batch_destroy(lmgpu_batch* batch);
/* Appends a job; its paths follow those of earlier jobs. Without params->accumulate the film is
 * cleared first. The scene and film must outlive the job. */
int lmgpu_batch_submit(lmgpu_batch* batch, lmgpu_scene* scene, lmgpu_film* film, const lmgpu_pt_params* params,
                       int32_t* job_id);
/* Runs the wavefront for at most max_chunks chunks of 8 bounce iterations (max_chunks <= 0: until
 * every submitted path is done) on `stream`, then refreshes the job progress the status call
 * reports. *paths_left receives the paths still in flight or not yet started. */
int lmgpu_batch_run(lmgpu_batch* batch, int32_t max_chunks, void* stream, int64_t* paths_left);
/* Progress of a job as of the last lmgpu_batch_run: leading samples-per-pixel passes whose every
 * pixel has finished, and whether the whole job is done. */
int lmgpu_batch_job_status(const lmgpu_batch* batch, int32_t job, int32_t* passes_complete, int32_t* done);
/* Changes how many samples per pixel a job renders, between runs (after lmgpu_batch_run has
 * returned): down to stop it early, back up (at most to the spp it was submitted with) to let it
 * continue. Passes of which a path has already started always complete, so the count becomes
 * max(spp, passes started) and *spp_out (may be null) receives it. Random streams stay keyed by
 * the submitted spp (pix * spp_submitted + sample), so a job stopped after N passes holds exactly
 * the first N passes of the submitted render. With split passes the film's even / odd pass counts
 * follow, so lmgpu_film_rel_mse on a job that is done reads the error of the passes it holds: the
 * loop "run until done, estimate the error, raise spp" is progressive rendering to a target error
 * (the reference's progressive schedulers, scheduler.cpp:57-109, stop on time instead). The job must
 * be its film's latest and not yet resolved. */
int lmgpu_batch_job_set_spp(lmgpu_batch* batch, int32_t job, int32_t spp, int32_t* spp_out);
/* Rescales a finished job's film (as lmgpu_render_pt does at the end of a render). */
int lmgpu_batch_resolve(lmgpu_batch* batch, int32_t job, void* stream);
/* Cumulative rays traced and device time since creation or the last reset. */
int lmgpu_batch_get_stats(const lmgpu_batch* batch, lmgpu_render_stats* out);
/* Forgets every job (buffers stay allocated). */
int lmgpu_batch_reset(lmgpu_batch* batch);
/* on != 0: runs also time every kernel (event nodes in the captured chunk); lmgpu_batch_get_stats
 * then reports extend_ms, shade_ms, shadow_ms and generate_ms (planner + camera vertices). */
int lmgpu_batch_set_timing(lmgpu_batch* batch, int32_t on);

/* No counterpart in the reference. renderer::pt for callers that must not allocate device memory:
 * hosts that hand every byte of HBM to their own pool allocator and forbid libraries from calling
 * cudaMalloc/cudaFree behind their back (a training or serving framework that reserves the device
 * at start-up, a plugin host whose memory accounting would not see the library's buffers), and
 * hosts that require a steady state free of allocations, where cudaMalloc's implicit device
 * synchronization and possible failure are not acceptable mid-run. It renders exactly like
 * lmgpu_render_pt, but its wavefront queues live in one file-scope device array of fixed size
 * (about 6.5 MiB, held by every GPU that loads the library until the process exits) instead of
 * buffers the library allocates, so at most LMGPU_NOALLOC_MAX_WAVE paths are in flight per wave
 * (params->wave_paths = 0 picks that size; larger values are rejected with
 * LMGPU_ERR_INVALID_ARGUMENT). The scene must already be created. The caller passes the output:
 * d_film, a device buffer of h x w x 3 floats, which receives the estimate scaled by 1/spp in
 * both primary modes (the scale renderer_pt.cpp:307-312 gives, as lmgpu_render_pt does);
 * params->accumulate must be 0. The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current and caches it for the life of the process. A
 * cudaDeviceReset invalidates the cached address, as it invalidates every scene and film handle of
 * the library: do not call this entry point after one. Every call shares the one array and clears what must start at zero, so calls
 * whose work overlaps on the GPU (different streams, or concurrent host threads) race: serialize
 * them. The call enqueues on `stream`, waits for it to read the error word, and calls no
 * cudaMalloc, cudaFree or other allocating routine. */
#define LMGPU_NOALLOC_MAX_WAVE 32768
int lmgpu_render_pt_noalloc(lmgpu_scene* scene, float* d_film, int32_t w, int32_t h, const lmgpu_pt_params* params,
                            void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LMGPU_H */

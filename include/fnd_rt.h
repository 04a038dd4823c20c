/*
 * fnd_rt.h — C ABI of the Foundation path-tracer pass (GB300 / sm_103a).
 *
 * The reference renderer (mos9527/Foundation) exposes one monolithic raster
 * pass: `Foundation::Renderer::Renderer(device, allocator)` with a per-frame
 * `Draw()` (src/Renderer/Renderer.hpp:39-43, src/Renderer/Renderer.cpp:367-401),
 * CHECK/BugCheck error handling (src/Core/Core.hpp:17, src/Core/Core.cpp:7-10)
 * and owner-scoped RAII handles (src/Platform/RHI/Details/Details.hpp:76-121).
 * It has no ray-tracing code at all, so every entry point below has no
 * line-for-line counterpart; each one names the reference interface whose
 * role it takes over in the new path-tracer pass.
 *
 * Conventions (all entry points):
 *  - return FND_OK (0) on success, a negative fnd_status on failure; no C++
 *    exception crosses this boundary and nothing terminates the process;
 *  - fnd_rt_last_error(ctx) gives a human-readable message for the last
 *    failure on that context;
 *  - input and output buffers are owned by the caller; device memory that the
 *    library allocates is owned by the context / scene and freed by destroy;
 *  - one CUDA stream per context; a context is not thread-safe, separate
 *    contexts may be used from separate threads;
 *  - device-side failures (traversal stack overflow, queue timeout) are
 *    latched in a device status word and returned by the next synchronising
 *    call (fnd_rt_sync, or any call made with FND_MEM_HOST buffers).
 */
#ifndef FND_RT_H
#define FND_RT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: fnd_rt_bvh_desc gained collapse_tri_cost and fnd_cache_desc
 * weight_average (both structs grew); version 1 callers are refused. */
#define FND_RT_ABI_VERSION 2u
#define FND_INVALID_ID 0xFFFFFFFFu

typedef enum fnd_status {
    FND_OK = 0,
    FND_ERR_INVALID_ARG = -1,    /* null pointer, bad size, bad flag, non-finite vertex */
    FND_ERR_OUT_OF_MEMORY = -2,  /* host or device allocation failed */
    FND_ERR_CUDA = -3,           /* a CUDA runtime call failed (message has the CUDA error) */
    FND_ERR_NO_DEVICE = -4,      /* no CUDA device / bad ordinal / not an sm_103 part */
    FND_ERR_INVALID_SCENE = -5,  /* scene too large for the node format, or depth over the stack */
    FND_ERR_STACK_OVERFLOW = -6, /* a ray needed more traversal stack than provisioned */
    FND_ERR_TIMEOUT = -7,        /* a bounded device wait ran out of iterations */
    FND_ERR_UNSUPPORTED = -8,    /* feature not available in this build */
    FND_ERR_IO = -9              /* file read / write failed */
} fnd_status;

/* Where the ray / hit buffers of a trace call live. */
enum { FND_MEM_HOST = 0, FND_MEM_DEVICE = 1 };

/* One ray: origin, [tmin, tmax] interval, direction (need not be unit).
 * 32 bytes, two 16-byte halves so a thread loads it with two vector loads. */
typedef struct fnd_ray {
    float org[3];
    float tmin;
    float dir[3];
    float tmax;
} fnd_ray;

/* Closest-hit result: original triangle index (FND_INVALID_ID on a miss) and
 * the hit distance in units of |dir| (+inf on a miss). 8 bytes. */
typedef struct fnd_hit {
    uint32_t prim;
    float t;
} fnd_hit;

typedef struct fnd_rt_ctx fnd_rt_ctx;
typedef struct fnd_rt_scene fnd_rt_scene;

/* Replaces the (device, allocator) pair handed to Renderer::Renderer
 * (src/Renderer/Renderer.hpp:41). */
typedef struct fnd_rt_desc {
    uint32_t abi_version; /* must be FND_RT_ABI_VERSION */
    int32_t device;       /* CUDA device ordinal */
    void* stream;         /* cudaStream_t to launch on; NULL: the context creates its own */
    uint32_t flags;       /* reserved, 0 */
} fnd_rt_desc;

/* BVH build parameters. The builder is binned SAH over triangle bounding-box
 * centroids, then a collapse of the binary tree into 8-wide compressed nodes. */
typedef struct fnd_rt_bvh_desc {
    uint32_t sah_bins;      /* 2..64, default 32 */
    uint32_t max_leaf_tris; /* 1..4, default 4 */
    uint32_t build_threads; /* host threads of the build and the collapse; 0: all
                               host cores. The tree does not depend on it, except
                               when a spatial-split budget runs out (split_budget) */
    uint32_t flags;         /* FND_BVH_SPATIAL_SPLITS, FND_BVH_GPU_BUILD, FND_BVH_SAH_COLLAPSE,
                               FND_BVH_GPU_CLUSTER (+ FND_BVH_CLUSTER_RADIUS(r)),
                               FND_BVH_NODE_WIDTH(w) or 0 */
    float traversal_cost;   /* SAH cost of a traversal step relative to a triangle
                               test, (0, 64]; 0: default 1 (the reference tree) */
    float split_budget;     /* FND_BVH_SPATIAL_SPLITS: references the splits may add,
                               per triangle, [0, 16]; 0: default 2. The builder stops
                               splitting where the SAH gains nothing, so a large budget
                               is a cap rather than a target (a dense soup of 1M
                               triangles settles near 6 references per triangle).
                               Build threads share the budget, so when it runs out
                               the tree can differ from one build to the next; hits
                               never do. Below the cap the tree is reproducible */
    float margin_scale;     /* box inflation relative to the default (2^-16 of the scene
                               size), [1, 2^16]; 0: 1. A scene instanced at a scale far below
                               the world's needs more (fnd_rt_instances_upload checks it) */
    float collapse_tri_cost; /* FND_BVH_SAH_COLLAPSE: cost of a triangle test relative to a
                               wide-node visit, (0, 16]; 0: default 0.3 (the fastest of
                               0.05 - 1 on the traversal kernel) */
} fnd_rt_bvh_desc;

/* Spatial splits (Stich et al. 2009): references of triangles that straddle
 * a split plane are clipped and duplicated (by default at most 2 extra
 * references per triangle, split_budget),
 * which tightens the tree of scenes with long, overlapping triangles. Hits
 * are identical either way. */
enum { FND_BVH_SPATIAL_SPLITS = 1u };
/* Build on the GPU: linear BVH over 63-bit Morton codes of the triangle
 * centroids on cubic cells (Karras 2012), or FND_BVH_GPU_CLUSTER, with SAH
 * leaf merging, collapsed to the same 8-wide format on the device. Much
 * faster to build (31M triangles in tens of ms), a few per cent slower to
 * trace than the binned-SAH tree on large flat scenes; hits are identical.
 * Up to 2^27 triangles; not combined with spatial splits; build_threads is
 * ignored. */
enum { FND_BVH_GPU_BUILD = 2u };
/* Collapse the binary tree into 8-wide nodes by the SAH-optimal dynamic
 * programme (Ylitie, Karras & Laine 2017) instead of the greedy rule: fuller
 * nodes, small subtrees merged into leaf slots of up to 4 triangles, on
 * the host build and on FND_BVH_GPU_BUILD alike; hits are identical either
 * way. */
enum { FND_BVH_SAH_COLLAPSE = 4u };
/* With FND_BVH_GPU_BUILD: the binary tree by parallel locally-ordered
 * clustering over the Morton order (Meister & Bittner 2018) instead of the
 * Karras hierarchy: each round merges the clusters that are each other's
 * nearest neighbour (least merged box area) among the r clusters on either
 * side. A slower build, a faster tree; hits are identical. */
enum { FND_BVH_GPU_CLUSTER = 8u };
/* The clustering's search radius r, 1..64, in bits 8..15 of flags; 0: 2 (the fastest
 * trees of 1 - 64 on the traversal kernel). */
#define FND_BVH_CLUSTER_RADIUS(r) ((uint32_t)(r) << 8)
/* Children per wide node, 2..8, in bits 16..19 of flags; 0: 8. The node
 * record and its test keep 8 slots whatever the width (a narrower tree has
 * more, emptier nodes): the autotuner's node-width dimension. Any build. */
#define FND_BVH_NODE_WIDTH(w) ((uint32_t)(w) << 16)

typedef struct fnd_rt_scene_info {
    uint32_t num_tris;
    uint32_t num_binary_nodes;
    uint32_t num_wide_nodes;
    uint32_t binary_depth;
    uint32_t wide_depth;
    uint32_t num_leaves;
    uint64_t node_bytes; /* device bytes of the wide nodes */
    uint64_t tri_bytes;  /* device bytes of the triangle arrays */
    double sah_cost;     /* SAH cost of the binary tree (C_trav = C_isect = 1) */
    double build_ms;     /* binary binned-SAH build, host */
    double collapse_ms;  /* collapse + compression + triangle re-layout, host */
    double upload_ms;    /* host -> device copies */
    float bounds_lo[3];
    float bounds_hi[3];
    float box_margin; /* absolute outward inflation applied to every node box */
    uint32_t num_refs; /* triangle references in the leaves (num_tris without spatial splits) */
} fnd_rt_scene_info;

/* ---- context --------------------------------------------------------- */

/* Creates a context on desc->device. Allocates the device status word and the
 * work-queue counters. Counterpart of Renderer::Renderer
 * (src/Renderer/Renderer.cpp:34-311). */
int fnd_rt_create(const fnd_rt_desc* desc, fnd_rt_ctx** out_ctx);

/* Waits for the context's stream, frees everything it owns (scenes must be
 * destroyed first). Counterpart of Renderer::~Renderer
 * (src/Renderer/Renderer.cpp:402-406), which waits for its queue to idle. */
int fnd_rt_destroy(fnd_rt_ctx* ctx);

/* Message of the last failure on ctx ("" if none); valid until the next call
 * on ctx. With ctx = NULL: the message of the calling thread's last failed
 * fnd_rt_create / fnd_rt_destroy or call made without a valid context. */
const char* fnd_rt_last_error(const fnd_rt_ctx* ctx);

/* Waits for the context's stream and returns the device status: FND_OK, or
 * the first latched device error (which is then cleared). */
int fnd_rt_sync(fnd_rt_ctx* ctx);

/* The cudaStream_t the context launches on. */
void* fnd_rt_stream(const fnd_rt_ctx* ctx);

/* Page-locked host buffers for FND_MEM_HOST calls (copies from pinned memory
 * run at full link speed). Counterpart of the host-visible staging buffers
 * the reference maps with MapSpan (src/Platform/RHI/Resource.hpp:62-68). */
int fnd_rt_host_alloc(size_t bytes, void** out_ptr);
int fnd_rt_host_free(void* ptr);

/* ---- scenes ----------------------------------------------------------- */

/* Builds the BVH on the host and uploads nodes and triangles.
 * verts: nv * 3 floats (x, y, z); idx: nt * 3 vertex indices (host memory).
 * Non-finite vertex coordinates or out-of-range indices are rejected with
 * FND_ERR_INVALID_ARG; nt == 0 gives an empty scene every ray misses.
 * Counterpart of the staging uploads of vertex / index buffers in the
 * reference renderer (src/Renderer/Renderer.cpp:133-198). */
int fnd_rt_scene_upload(fnd_rt_ctx* ctx, const float* verts, uint32_t nv, const uint32_t* idx,
                        uint32_t nt, const fnd_rt_bvh_desc* bvh, fnd_rt_scene** out_scene);

int fnd_rt_scene_info_get(const fnd_rt_scene* scene, fnd_rt_scene_info* out_info);

int fnd_rt_scene_destroy(fnd_rt_scene* scene);

/* ---- traversal -------------------------------------------------------- */

/* Closest hit for n rays: for each ray the triangle with the smallest hit t
 * in [tmin, tmax], ties broken by the lowest triangle index; t is computed by
 * the watertight ray/triangle test in FP32.
 * mem = FND_MEM_DEVICE: rays / out are device pointers, the call only enqueues
 * work on the context stream (call fnd_rt_sync to wait and read the status);
 * mem = FND_MEM_HOST: host pointers (pinned or pageable), the call copies in,
 * traces, copies out and synchronises. */
int fnd_rt_trace_closest(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_ray* rays, uint32_t n,
                         fnd_hit* out, int mem);

/* Any hit (occlusion) for n rays: out[i] = 1 if some triangle is hit with t in
 * [tmin, tmax], else 0. Same memory rules as fnd_rt_trace_closest. */
int fnd_rt_trace_any(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_ray* rays, uint32_t n,
                     uint8_t* out, int mem);

/* Traversal counters of the last trace call (device-side totals), for the
 * memory-roofline accounting: wide nodes fetched and triangles tested; and
 * for the SIMT accounting: warp steps of the node test and of the triangle
 * test (steps a warp executed, whatever its active lanes), so that
 * node_fetches / (32 * warp_node_steps) is the node phase's lane
 * utilisation and tri_tests / (32 * warp_tri_steps) the triangle phase's. */
typedef struct fnd_rt_trace_stats {
    uint64_t rays;
    uint64_t node_fetches;
    uint64_t tri_tests;
    uint64_t warp_node_steps;
    uint64_t warp_tri_steps;
} fnd_rt_trace_stats;

/* Re-runs a closest-hit trace with per-ray counters enabled (slower variant of
 * the kernel) and returns the totals. Same memory rules as trace_closest. */
int fnd_rt_trace_closest_stats(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_ray* rays,
                               uint32_t n, fnd_hit* out, int mem, fnd_rt_trace_stats* stats);

/* ---- launch shape and autotuning ----------------------------------------
 * Block size, shared-memory short-stack depth and the refill threshold of
 * the persistent traversal kernels. A context starts with the defaults
 * (128, 8, 8); fnd_rt_tune times every combination on a caller's ray batch
 * and reports the table and the fastest. No reference counterpart: the
 * reference has no compute dispatch to tune (src/Platform/RHI/Command.hpp:32-116). */
typedef struct fnd_rt_trace_config {
    uint32_t block;        /* 64, 128 or 256 threads */
    uint32_t short_stack;  /* 4, 8 or 16 entries per thread */
    uint32_t refill_min;   /* 1..32 idle lanes before a warp refills */
    uint32_t postpone_min; /* postpone a node's triangles while fewer than this many lanes
                              of the warp have triangles to test (0..32, 0: never) */
    uint32_t sort_bits;    /* 0: rays traced in input order; 6..21 (multiple of 3): rays
                              first bucketed by origin cell (Morton order on a grid over
                              the scene box) and direction octant, a key of this many
                              bits; results are unchanged, only the schedule. Single-scene
                              traces and the path tracer's secondary and shadow rays. */
} fnd_rt_trace_config;

typedef struct fnd_rt_tune_entry {
    fnd_rt_trace_config config;
    float ms;              /* best-of-reps kernel time (CUDA events) */
} fnd_rt_tune_entry;

enum { FND_QUERY_CLOSEST = 0, FND_QUERY_ANY = 1 };

int fnd_rt_set_trace_config(fnd_rt_ctx* ctx, const fnd_rt_trace_config* config);
int fnd_rt_get_trace_config(const fnd_rt_ctx* ctx, fnd_rt_trace_config* out);
/* Times every launch shape on n device rays (FND_QUERY_CLOSEST / _ANY) with
 * `reps` timed runs each, then the best shape with each coherence-order key
 * width (sort time included); fills up to table_cap entries, *table_n, *best
 * (the context keeps its own config; apply *best with fnd_rt_set_trace_config). */
int fnd_rt_tune(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_ray* rays, uint32_t n, uint32_t kind,
                uint32_t reps, fnd_rt_tune_entry* table, uint32_t table_cap, uint32_t* table_n,
                fnd_rt_trace_config* best);

/* ---- batched traversal --------------------------------------------------
 * Many scenes and ray batches of uneven sizes in ONE persistent launch: every
 * job is (scene, device rays, device output, query kind); a global work
 * counter hands rays of all jobs to the warps. The launch (counter reset +
 * kernel) is captured once in a CUDA graph and replayed by
 * fnd_rt_batch_launch. */
typedef struct fnd_rt_batch fnd_rt_batch;

typedef struct fnd_rt_batch_job {
    const fnd_rt_scene* scene;
    const fnd_ray* rays;  /* device, 16-byte aligned */
    void* out;            /* device: fnd_hit[n] (closest) or uint8_t[n] (any) */
    uint32_t n;
    uint32_t kind;        /* FND_QUERY_CLOSEST or FND_QUERY_ANY */
} fnd_rt_batch_job;

enum { FND_BATCH_NO_GRAPH = 1u };

int fnd_rt_batch_create(fnd_rt_ctx* ctx, const fnd_rt_batch_job* jobs, uint32_t njobs, uint32_t flags,
                        fnd_rt_batch** out_batch);
/* Enqueues the batch on the context stream (asynchronous; fnd_rt_sync waits). */
int fnd_rt_batch_launch(fnd_rt_batch* batch);
/* Times every launch shape on the batch, re-captures its graph with the
 * fastest and returns it (table as in fnd_rt_tune). */
int fnd_rt_batch_tune(fnd_rt_batch* batch, uint32_t reps, fnd_rt_tune_entry* table, uint32_t table_cap,
                      uint32_t* table_n, fnd_rt_trace_config* best);
int fnd_rt_batch_destroy(fnd_rt_batch* batch);

/* ---- path tracing ------------------------------------------------------
 * The reference's per-frame entry is Renderer::Draw
 * (src/Renderer/Renderer.cpp:367-401): update the camera, record, submit,
 * present. fnd_rt_render is the path-tracer pass's counterpart: one call
 * renders `spp` samples per pixel of the scene into a linear-radiance RGB
 * buffer (no swapchain: the caller owns the output). */

enum { FND_MAT_LAMBERT = 0, FND_MAT_GGX = 1, FND_MAT_EMISSIVE = 2 };

/* 48 bytes. Lambert: albedo. GGX: albedo is the specular colour F0 (Schlick),
 * roughness is the GGX alpha. Emissive: one-sided black emitter with
 * radiance `emission` on the side its triangle winding faces; `light` is the
 * index of the quad light (fnd_rt_scene_set_lights) with the same geometry,
 * used to weight BSDF-sampled hits against light sampling (-1: none). */
typedef struct fnd_material {
    uint32_t type;
    float albedo[3];
    float roughness;
    float emission[3];
    int32_t light;
    float reserved[3];
} fnd_material;

/* Parallelogram light corner + u*edge_u + v*edge_v, emitting `radiance` on
 * the side of cross(edge_u, edge_v). 48 bytes. */
typedef struct fnd_quad_light {
    float corner[3];
    float edge_u[3];
    float edge_v[3];
    float radiance[3];
} fnd_quad_light;

/* Pinhole camera in the glm::lookAt convention of the reference
 * (src/Renderer/Renderer.cpp:374-380): right-handed, looking from eye to target. */
typedef struct fnd_camera {
    float eye[3];
    float target[3];
    float up[3];
    float vfov_deg;
} fnd_camera;

/* FND_RENDER_WAVEFRONT: run every bounce as wavefront stages (no tail
 * megakernel; for comparison and testing, same results). */
enum { FND_RENDER_ACCUMULATE = 1u, FND_RENDER_WAVEFRONT = 4u };

typedef struct fnd_render_desc {
    uint32_t width, height;
    uint32_t spp;        /* samples per pixel in this call */
    uint32_t max_depth;  /* surface interactions per path, 1..64 (8) */
    uint32_t rr_start;   /* first bounce index with Russian roulette (3) */
    uint32_t flags;      /* FND_RENDER_ACCUMULATE: add to the previous calls' samples */
    uint64_t seed;       /* PCG32 seed; each pixel gets its own stream */
    fnd_camera camera;
    float sky[3];          /* constant radiance of escaping rays */
    float sun_dir[3];      /* towards the sun; zero vector: no sun */
    float sun_irradiance[3];
    uint32_t wave_paths;   /* paths in flight per wave (218 bytes of device state each),
                              0: automatic (up to 2^25) */
    uint32_t tail_paths;   /* once at most this many paths of a wave remain, one
                              megakernel finishes them; 0: automatic */
} fnd_render_desc;

typedef struct fnd_render_stats {
    uint64_t paths;
    uint64_t extension_rays;
    uint64_t shadow_rays;
    uint32_t waves;
    uint32_t samples_accumulated;
} fnd_render_stats;

/* Material per triangle (original index order) and the material table. */
int fnd_rt_scene_set_materials(fnd_rt_scene* scene, const uint32_t* tri_material, uint32_t nt,
                               const fnd_material* materials, uint32_t nm);
/* Quad lights sampled by next-event estimation. */
int fnd_rt_scene_set_lights(fnd_rt_scene* scene, const fnd_quad_light* lights, uint32_t nl);

/* Renders desc->spp samples per pixel. rgb: width*height*3 floats, row-major
 * from the top row, receiving the mean radiance over all accumulated samples;
 * host or device memory per `mem` (FND_MEM_DEVICE: asynchronous). */
int fnd_rt_render(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_render_desc* desc, float* rgb, int mem);

/* Counters of the last fnd_rt_render call (synchronises the stream). */
int fnd_rt_render_stats_get(fnd_rt_ctx* ctx, fnd_render_stats* out);

/* ---- instancing -------------------------------------------------------------
 * A two-level scene: instances of uploaded triangle scenes (bottom levels)
 * placed by affine transforms, under a top-level tree over their world
 * boxes. Traced with fnd_rt_trace_closest / fnd_rt_trace_any like any scene:
 * a hit reports prim = prim_offset of the instance + the bottom-level
 * triangle index, and t, the ray parameter (the same in world and object
 * space). Each instance's bottom level is intersected with the ray mapped by
 * the inverse transform (computed in FP64, rounded to FP32): o' = Minv (o, 1),
 * d' = Minv (d, 0), sums left to right. Ties break by the reported id.
 * A bottom level must stay alive while instanced, and its box margin must
 * cover the object-space ray origins its instances produce: an instance
 * scaled far below the world needs the bottom level uploaded with a larger
 * margin_scale (the call fails with FND_ERR_INVALID_SCENE naming the value).
 * Two-level scenes are traced and rendered (shading normals by global id are
 * made at upload; fnd_rt_scene_set_materials takes one material id per global
 * id, so instances' prim ranges should not overlap), not batched, tuned or
 * traced through the no-allocation entry point. Reference counterpart: none
 * (the reference draws one hard-coded quad). */
typedef struct fnd_rt_instance {
    const fnd_rt_scene* scene;  /* bottom level: a triangle scene of the same context */
    float transform[12];        /* object -> world, row-major 3x4: x' = M (x, y, z, 1) */
    uint32_t prim_offset;       /* hit id of the instance's triangle 0 */
} fnd_rt_instance;

int fnd_rt_instances_upload(fnd_rt_ctx* ctx, const fnd_rt_instance* instances, uint32_t n,
                            fnd_rt_scene** out_scene);

/* ---- image output ---------------------------------------------------------
 * Linear radiance (width*height RGB floats, row-major from the top row, the
 * layout fnd_rt_render writes) to R8G8B8A8_UNORM pixels, the format of the
 * reference renderer's colour target (src/Renderer/Renderer.cpp:40,81):
 * exposure, tone curve, sRGB transfer function (the target is UNORM), 8-bit
 * rounding, alpha 255. Replaces the swapchain present of Renderer::Draw
 * (Renderer.cpp:395-399) with a buffer the caller writes out. */
enum { FND_TONEMAP_CLAMP = 0u, FND_TONEMAP_REINHARD = 1u, FND_TONEMAP_ACES = 2u };

int fnd_rt_tonemap(fnd_rt_ctx* ctx, const float* rgb, uint32_t width, uint32_t height, int mem_in, float exposure,
                   uint32_t mode, uint8_t* rgba, int mem_out);

/* ---- raster pass -----------------------------------------------------------
 * CUDA restatement of the reference renderer's only pass
 * (src/Renderer/Renderer.cpp:312-366, src/Renderer/Triangle.slang): an indexed
 * triangle list of vertex_input records (Renderer.cpp:23-27) transformed by
 * proj * view * model, back faces culled (front faces counter-clockwise,
 * Renderer.cpp:127-131), no depth test, fragment = texture(uv) * (colour, 1),
 * written to an R8G8B8A8_UNORM target cleared to `clear`. Where the graphics
 * API leaves rules to the implementation this pass fixes them: vertices
 * snapped to 1/256 pixel, pixel centres at +0.5, the top-left fill rule,
 * perspective-correct interpolation, bilinear filtering with repeat
 * addressing (the reference sampler's linear filters and repeat mode on its
 * single mip level; its anisotropic taps are implementation-defined), and
 * no clipping: a triangle with a vertex behind the eye is skipped. */
typedef struct fnd_raster_vertex {
    float pos[2];
    float color[3];
    float uv[2];
} fnd_raster_vertex;

typedef struct fnd_raster_desc {
    uint32_t width, height;  /* colour target (1920 x 1080 in the reference) */
    float model[16];         /* column-major, as the uniform buffer of Renderer.cpp:28-33 */
    float view[16];
    float proj[16];
    float clear[4];          /* clear colour (the reference clears to 0, 0, 0, 1) */
    uint32_t cull_back;      /* 1: cull back faces (the reference's state) */
} fnd_raster_desc;

/* The reference's per-frame uniforms at time t seconds (Renderer.cpp:370-380):
 * model rotates 90 degrees per second about +z, view looks from (2, 2, 2) at
 * the origin with +z up, proj is an infinite perspective of 45 degrees and
 * near plane 0.1 with the y axis flipped. Host-only; no context needed. */
int fnd_rt_raster_uniforms(float time_s, float aspect, float* model, float* view, float* proj);

/* Draws ni / 3 triangles (host vertex, index and RGBA8 texture arrays) into
 * rgba (width*height*4 bytes, top row first; host or device per mem). */
int fnd_rt_raster_draw(fnd_rt_ctx* ctx, const fnd_raster_desc* desc, const fnd_raster_vertex* verts, uint32_t nv,
                       const uint16_t* idx, uint32_t ni, const uint8_t* texture, uint32_t tex_w, uint32_t tex_h,
                       uint8_t* rgba, int mem);

/* ---- radiance cache -----------------------------------------------------
 * An online-trained MLP (96 -> 5 x 64 ReLU -> 3, BF16 tensor cores, FP32
 * Adam) that predicts reflected radiance. With FND_RENDER_CACHE a render
 * call first traces `train_paths` full training paths and takes
 * `train_steps` optimiser steps on their vertices, then renders: paths end at
 * the vertex after their first non-specular bounce, where the network
 * supplies the reflected radiance. The plain tracer (no flag) stays the
 * unbiased estimator against which the cache's error is measured. No reference counterpart
 * (the reference has no ray tracer); the session state lives in the context
 * like the renderer's per-frame resources (src/Renderer/Renderer.hpp:13-36). */
enum { FND_RENDER_CACHE = 2u };
/* With FND_RENDER_CACHE: run only the cache's training paths and optimiser
 * steps of a call (the frame buffer and rgb are untouched; rgb may be NULL),
 * e.g. to train the cache before its images are accumulated. */
enum { FND_RENDER_TRAIN_ONLY = 8u };

typedef struct fnd_cache_desc {
    uint32_t train_paths;   /* training paths per render call (65,536) */
    uint32_t train_steps;   /* optimiser steps per render call (4) */
    uint32_t batch;         /* training samples per step (16,384) */
    float learning_rate;    /* Adam learning rate (1e-2) */
    float specular_alpha;   /* GGX alpha below which a vertex counts as specular (0.1) */
    uint32_t flags;         /* reserved, 0 */
    uint64_t seed;          /* weight initialisation and sampling seed */
    float weight_average;   /* [0, 1): 0 queries the latest weights; d > 0 queries an
                               exponential moving average of the optimiser's iterates,
                               a <- d a + (1 - d) w after every Adam step, divided by
                               1 - d^steps (Polyak averaging; it damps the weight noise
                               of a high learning rate). Training always uses the latest
                               weights; set_weights / load restart the average. */
} fnd_cache_desc;

typedef struct fnd_cache_stats {
    uint64_t steps;           /* optimiser steps taken */
    uint64_t samples_last;    /* training samples of the last render call */
    uint64_t queries_last;    /* cache queries of the last render wave */
    double loss_last;         /* mean relative-L2 loss of the last step */
} fnd_cache_stats;

#define FND_CACHE_NUM_PARAMS 22720u
#define FND_CACHE_NUM_FEATURES 96u

/* Creates (or re-creates) the context's cache for a scene: He-uniform
 * weights, zero Adam state, the scene's bounding box for the position
 * encoding. */
int fnd_rt_cache_create(fnd_rt_ctx* ctx, const fnd_rt_scene* scene, const fnd_cache_desc* desc);
int fnd_rt_cache_destroy(fnd_rt_ctx* ctx);
int fnd_rt_cache_stats_get(fnd_rt_ctx* ctx, fnd_cache_stats* out);
/* FP32 master weights, row-major W[K][N] per layer, layers in order. */
int fnd_rt_cache_get_weights(fnd_rt_ctx* ctx, float* out, uint32_t n);
int fnd_rt_cache_set_weights(fnd_rt_ctx* ctx, const float* w, uint32_t n);
/* Checkpoint: versioned header, weights and Adam moments. */
int fnd_rt_cache_save(fnd_rt_ctx* ctx, const char* path);
int fnd_rt_cache_load(fnd_rt_ctx* ctx, const char* path);
/* Network on explicit features (n x 96 host floats) -> n x 3 host floats. */
int fnd_rt_cache_eval(fnd_rt_ctx* ctx, const float* features, uint32_t n, float* out);
/* Gradient of the mean relative-L2 loss on explicit features / targets
 * (n x 3): grad receives FND_CACHE_NUM_PARAMS floats, loss the mean loss. */
int fnd_rt_cache_gradient(fnd_rt_ctx* ctx, const float* features, const float* targets, uint32_t n, float* grad,
                          double* loss);
/* The network's input features of n points, each 13 host floats: position,
 * outgoing direction, normal, roughness, albedo -> n x 96 host floats (the
 * BF16 values the network sees, widened to float). */
int fnd_rt_cache_encode(fnd_rt_ctx* ctx, const float* points, uint32_t n, float* out);
/* One Adam step with the given gradient (FND_CACHE_NUM_PARAMS host floats). */
int fnd_rt_cache_adam_step(fnd_rt_ctx* ctx, const float* grad, float learning_rate);

/* Closest hit without any device allocation. No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc at trace time
 * (a plugin inside a host application's frame callback, where the host
 * forbids device allocations or has handed out all device memory up front,
 * or code that must not add the device-wide synchronisation of
 * cudaMalloc / cudaFree). rays / out are HOST buffers; the scene must have
 * been uploaded beforehand. Results equal fnd_rt_trace_closest's.
 * The rays and hits are staged through one fixed file-scope device array of
 * about 2.5 MiB, which every GPU that loads this library holds until the
 * process exits; a call takes at most 65,536 rays and larger n is rejected
 * with FND_ERR_INVALID_ARG. The first call on a device resolves the array's
 * address (set-up; under lazy module loading the driver may reserve the array
 * only then), so make that first call at set-up time, while device memory is
 * still free, and before any stream capture; a set-up that failed is retried
 * by the next call. All calls share the array and it keeps the last call's
 * contents (the work counter and status word are cleared at the start of each
 * call): calls that overlap on the GPU race, so serialise them. The launch
 * uses the context's launch shape without the coherence sort.
 * stream: cudaStream_t, or NULL for the scene context's stream. Synchronous:
 * returns once the hits are in `out`; the caller's current device is left
 * unchanged. */
int fnd_rt_trace_closest_noalloc(const fnd_rt_scene* scene, const fnd_ray* rays, uint32_t n, fnd_hit* out,
                                 void* stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* FND_RT_H */

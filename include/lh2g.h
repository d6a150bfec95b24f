/* lh2g.h - C ABI of the GB300 wavefront render core (libRenderCore_GB300.so).
 *
 * A flat, allocation-owning C interface under the core's CoreAPI_Base plugin (lh2_core_api.h). Every entry
 * point returns an int status (LH2G_OK on success) and never aborts the host; the message of the last failure
 * is available from lh2g_last_error(). One context owns one CUDA stream on one device; calls on a context
 * must come from one host thread at a time.
 *
 * Each entry point names the reference interface it replaces (lib/RenderSystem/core_api_base.h of
 * Lighthouse 2, where the plugin API is a C++ vtable; the reference has no C ABI of its own).
 */
#ifndef LH2G_H
#define LH2G_H

#include "lh2g_types.h"

#if defined(__GNUC__)
#define LH2G_API __attribute__((visibility("default")))
#else
#define LH2G_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define LH2G_OK 0
#define LH2G_ERR_INVALID 1     /* bad argument or call order */
#define LH2G_ERR_CUDA 2        /* a CUDA call failed */
#define LH2G_ERR_OOM 3         /* device allocation failed */
#define LH2G_ERR_STATE 4       /* scene not finalized / no target */
#define LH2G_ERR_OVERFLOW 5    /* a device capacity was exceeded (traversal stack, node pool) */

typedef struct lh2g_context lh2g_context;

/* Per-frame statistics, the fields of CoreStats (core_api_base.h:30-64) this core fills. */
typedef struct lh2g_stats {
    uint32_t totalRays, totalExtensionRays, totalShadowRays, primaryRayCount, bounce1RayCount, deepRayCount;
    float renderTime, traceTime0, traceTime1, traceTimeX, shadowTraceTime, shadeTime, filterTime, bvhBuildTime;
    uint32_t SMcount, ccMajor, ccMinor, VRAM;
    int32_t probedInstid, probedTriid;
    float probedDist;
    uint32_t deviceStatus;          /* LH2G_STATUS_* bits reported by the kernels */
} lh2g_stats;

/* Context: replaces CreateCore (lib/rendercore_optix7/core_api.cpp:18-22) + RenderCore::Init (rendercore.cpp:219-278). */
LH2G_API int lh2g_create(int device, lh2g_context** out);
/* RenderCore::Shutdown (rendercore.cpp:984-1003). */
LH2G_API int lh2g_destroy(lh2g_context* ctx);
LH2G_API const char* lh2g_last_error(lh2g_context* ctx);

/* SetGeometry (core_api_base.h:114): 3 float4 vertices per triangle + CoreTri records; meshes in index order. */
LH2G_API int lh2g_set_geometry(lh2g_context* ctx, int meshIdx, const float* vertices4, int vertexCount, int triangleCount, const lh2g_core_tri* tris);
/* SetInstance (core_api_base.h:116): 4x4 row-major object-to-world transform; meshIdx -1 truncates the list. */
LH2G_API int lh2g_set_instance(lh2g_context* ctx, int instIdx, int meshIdx, const float* transform16);
/* FinalizeInstances (core_api_base.h:118): builds every dirty BLAS and the TLAS on the device. */
LH2G_API int lh2g_finalize_instances(lh2g_context* ctx);
/* SetMaterials (core_api_base.h:105); textures must be set first. */
LH2G_API int lh2g_set_materials(lh2g_context* ctx, const lh2g_material* materials, int count);
/* Packs materials into the 128-byte device format without a context (for inspection and tests). */
LH2G_API int lh2g_pack_materials(const lh2g_material* materials, int count, const lh2g_texture* textures, int textureCount, lh2g_gpu_material* out);
/* SetTextures (core_api_base.h:103): ARGB32 texels, MIP levels back to back. */
LH2G_API int lh2g_set_textures(lh2g_context* ctx, const lh2g_texture* textures, int count);
/* SetLights (core_api_base.h:107-110). Frames that select lights by their potentials (every estimator but the OptiX 7
 * one with its light tree, LH2G_RP_LIGHTTREE) take at most 64 lights in total (the reference's MAXISLIGHTS); the
 * light tree takes up to LH2G_MAX_TREE_LIGHTS area, point and spot lights. Also builds the light tree
 * (RenderCore::SetLights calls UpdateLightTree, rendercore_optix7/rendercore.cpp:709). */
#define LH2G_MAX_TREE_LIGHTS (1 << 16)   /* the reference's agglomerative build is quadratic: 0.4 s at 8k lights */
LH2G_API int lh2g_set_lights(lh2g_context* ctx, const lh2g_light_tri* tri, int ntri, const lh2g_point_light* point, int npoint,
                    const lh2g_spot_light* spot, int nspot, const lh2g_dir_light* dir, int ndir);
/* The light tree that lh2g_set_lights builds for these lights (RenderCore::UpdateLightTree,
 * rendercore_optix7/rendercore.cpp:625-680), host only: no context or GPU needed. Writes 2 * (ntri + npoint + nspot)
 * records of 16 32-bit words (the device LightCluster of common_classes.h:522-527: light, left, right, intensity;
 * box minimum xyz, 0; box maximum xyz, 0; normal xyz, parent) to nodes; record 0 is the root. Returns the record
 * count, or minus an error code: -LH2G_ERR_INVALID (negative counts, more than LH2G_MAX_TREE_LIGHTS lights) or
 * -LH2G_ERR_OVERFLOW (capacity, in records, too small). */
LH2G_API int lh2g_build_light_tree(const lh2g_light_tri* tri, int ntri, const lh2g_point_light* point, int npoint, const lh2g_spot_light* spot,
                                   int nspot, void* nodes, int capacity);
/* SetSkyData (core_api_base.h:112): width*height RGB floats; worldToSky16 may be NULL (identity). */
LH2G_API int lh2g_set_sky(lh2g_context* ctx, const float* rgb, int width, int height, const float* worldToSky16);
/* Blue-noise tables of the OptiX 7 estimator (LH2G_RP_OPTIX7 and adaptive frames), in the layout of the Lighthouse 2
 * RenderSystem's lib/RenderSystem/common_bluenoise.h read as bytes: sobol 256 x 256 (65536 bytes), scrambling and
 * ranking 128 x 128 x 8 (131072 bytes each). The reference's OptiX 7 core compiles them in and expands them at Init
 * (lib/rendercore_optix7/rendercore.cpp:247-256); this core takes them from its host. Without tables (or after a
 * call with NULL pointers) every sample uses xorshift numbers, as the reference does for sample indices from 64 on. */
LH2G_API int lh2g_set_blue_noise(lh2g_context* ctx, const uint8_t* sobol, const uint8_t* scrambling, const uint8_t* ranking);
/* Setting (core_api_base.h:95): "epsilon", "clampValue", "maxDepth", "rrStartDepth", "nee", and the filter
 * core's "filter" (0/1, default 0), "TAA" (0/1, default 1), "clampDirect" (2.5), "clampIndirect" (15)
 * (lib/RenderCore_Optix7Filter/rendercore.cpp:674-677, rendercore.h:32-35). With "filter" on, lh2g_render
 * renders filter-core frames (LH2G_RP_FILTER, Halton-jittered when TAA is on) and denoises them with SVGF.
 * Scheduling settings of this core (results do not change): "waveTail" (default 5; path lengths from this one on
 * run to their end in one persistent kernel; 0: one launch per stage and wave throughout) and "pipelineFrames"
 * (frames in flight, 0..8, default 6; 0 and 1 render one frame at a time; see lh2g_get_stream) and "waveOccupancy"
 * (fraction of the GPU the persistent wave kernels of one frame launch, (0, 1], default 1) and "sortConnections"
 * (1: group each wave's light connections by the light they sample before the any-hit queries, 2: the same within
 * chunks of 1,024 consecutive connections; default 0) and "sortRays" (1: group each bounce wave's extension rays by
 * direction octant before the closest-hit queries, 2: within chunks of 1,024; default 0).
 * Estimator of lh2g_render: "estimator" 0 (PrimeRef, default) or 1 (the OptiX 7 core's, LH2G_RP_OPTIX7; one camera
 * seed drawn per wave of maxDepth, where the reference draws only for the waves its loop runs), "adaptive" 1
 * (PrimeAdaptive frames, lh2g_render_adaptive). Both draw a blue-noise shift per frame from seed 0x11331445.
 * "bsdf" 1: those estimators with the Disney BSDF (LH2G_RP_DISNEY); "lightTree" 1: the OptiX 7 estimator selects
 * lights through the light tree (LH2G_RP_LIGHTTREE). */
LH2G_API int lh2g_setting(lh2g_context* ctx, const char* name, float value);
/* SetTarget (core_api_base.h:93), headless: the output is a device float4 buffer of width*height pixels. */
LH2G_API int lh2g_set_target(lh2g_context* ctx, int width, int height, int spp);
/* SetProbePos (core_api_base.h:91). */
LH2G_API int lh2g_set_probe(lh2g_context* ctx, int x, int y);
/* Render (core_api_base.h:97): converge 0 = Converge (accumulate), 1 = Restart. */
LH2G_API int lh2g_render(lh2g_context* ctx, const lh2g_view* view, int converge);
/* Render one frame with explicit estimator parameters (used by the parity tests): accumulate != 0 adds to the
 * accumulator, else it is cleared first. captureHits / captureSeeds (host, maxDepth * W*H*spp entries, may be
 * NULL) receive per-path, per-depth hit records and RNG states; counters (host, 2 * maxDepth, may be NULL)
 * receive per path length the extension and connection counts. */
LH2G_API int lh2g_render_ex(lh2g_context* ctx, const lh2g_view* view, const lh2g_render_params* params, int accumulate,
                   lh2g_hit* captureHits, uint32_t* captureSeeds, uint32_t* counters);
/* One frame of the PrimeAdaptive core (lib/RenderCore_PrimeAdaptive/rendercore.cpp:600-755): the OptiX 7 estimator
 * (LH2G_RP_OPTIX7's shading, with per-sample accumulators) over W*H*spp paths, each pixel's variance estimate
 * (finalize_shared.h:97-151) scaled by devScale, up to 24 more samples per pixel where the estimate asks for them (at
 * most W*H*spp in all; beyond that the requests of lower sample numbers, then of lower pixels, are kept), a second
 * wave of those paths, and finalizeASRender: the accumulator gets each pixel's samples divided by their count
 * (cleared first unless accumulate), the frame the accumulator divided by (samplesTaken + spp) / spp. devScale stays
 * on the device and steers the next frame towards 91-98 % of the budget (initially 10, lh2g_set_adaptive_scale).
 * params: flags LH2G_RP_NEE or 0; cameraR0 / frameSeed = the frame's two draws of RandomUInt(camRNGseed); shift =
 * the shift draw; maxDepth <= 32. captureHits / captureSeeds cover the first wave (maxDepth * W*H*spp entries);
 * counters (host, 4 * maxDepth) the first wave's then the second's per path length; stats (may be NULL): devScale for
 * the next frame, the second wave's paths and the samples requested. With any of them the call waits. */
typedef struct lh2g_adaptive_stats { float devScale; uint32_t adaptivePaths, requested; } lh2g_adaptive_stats;
LH2G_API int lh2g_render_adaptive(lh2g_context* ctx, const lh2g_view* view, const lh2g_render_params* params, int accumulate,
                                  lh2g_hit* captureHits, uint32_t* captureSeeds, uint32_t* counters, lh2g_adaptive_stats* stats);
/* devScale the next adaptive frame starts from (RenderCore_PrimeAdaptive/rendercore.h: 10) */
LH2G_API int lh2g_set_adaptive_scale(lh2g_context* ctx, float devScale);
/* lh2g_render_ex without captures, followed by an asynchronous copy of the finalized frame (W*H float4) into
 * hostFrame: returns once the work is queued; hostFrame holds the frame after lh2g_wait (or any call that waits for
 * the context). Consecutive calls overlap like other plain frames; the copy of one frame completes before the next
 * frame's finalize overwrites the device frame. Pinned host memory makes the copy overlap rendering. */
LH2G_API int lh2g_render_to_host(lh2g_context* ctx, const lh2g_view* view, const lh2g_render_params* params, int accumulate,
                                 float* hostFrame);
/* SVGF on the accumulator of the last LH2G_RP_FILTER frame (lib/RenderCore_Optix7Filter/rendercore.cpp:904-935):
 * prepareFilter (demodulation, reprojection, luminance moments), applyFilter phases 1-3 (temporal blend,
 * a-trous at steps 1, 2, 4, remodulation), then TAA + unsharpen or finalizeNoTAA into the frame buffer, whose
 * border pixels keep their contents as in the reference; then the history buffers swap. lh2g_render calls
 * this itself when the "filter" setting is on. */
LH2G_API int lh2g_filter(lh2g_context* ctx, const lh2g_filter_params* params);
/* Copies filter buffer slot LH2G_FB_* (W*H elements; LH2G_FB_ACCUM 2*W*H) to host memory. */
LH2G_API int lh2g_read_filter_buffer(lh2g_context* ctx, int slot, void* host);
/* The filter parameters lh2g_render used for its last filtered frame, and the jittered view and estimator
 * parameters of that frame (either pointer may be NULL). */
LH2G_API int lh2g_get_last_filter_frame(lh2g_context* ctx, lh2g_filter_params* filter, lh2g_view* jitteredView,
                                        lh2g_render_params* params);
/* WaitForRender (core_api_base.h:99): blocks until every frame and operation submitted on the context is done. */
LH2G_API int lh2g_wait(lh2g_context* ctx);
/* GetCoreStats (core_api_base.h:87). */
LH2G_API int lh2g_get_stats(lh2g_context* ctx, lh2g_stats* out);
/* Headless output: device pointer of the W*H float4 frame (accumulator / samples), and host read-backs. */
LH2G_API int lh2g_get_framebuffer(lh2g_context* ctx, void** devicePtr);
LH2G_API int lh2g_read_framebuffer(lh2g_context* ctx, float* host);
LH2G_API int lh2g_read_accumulator(lh2g_context* ctx, float* host);

/* The context's CUDA stream (cudaStream_t), for callers that bracket frames with their own events. Plain frames
 * (lh2g_render / lh2g_render_ex without read-backs, lh2g_render_to_host; targets up to 8M paths) run on internal
 * streams in turn (setting "pipelineFrames"), so that one frame's last waves overlap the next frame's first ones; they
 * wait for work enqueued on the context stream before them, and this call orders the context stream after every
 * frame submitted so far, so an event recorded on the returned stream afterwards completes after those frames.
 * Every call that reads results or changes the scene or target does the same. */
LH2G_API int lh2g_get_stream(lh2g_context* ctx, void** stream);
/* Per-launch device timing of the next frames (enable != 0): lh2g_get_launch_times waits for the core's stream,
 * fills ms[k] with the duration of launch k of every frame rendered since timing was enabled or since its previous
 * call (frames in order; per frame [generate, (extend, shade, connect) x waves, tail if used, finalize]), sets
 * *count to the number of those launches (up to 16384; older ones are dropped) and starts over. Timing adds one
 * event pair per launch and no host synchronisation. */
LH2G_API int lh2g_enable_launch_timing(lh2g_context* ctx, int enable);
LH2G_API int lh2g_get_launch_times(lh2g_context* ctx, float* ms, int capacity, int* count);

/* Traversal work of the last frame: out[0..3] = interior nodes visited and triangles tested by the closest-hit
 * (extend) stage, then by the any-hit (connect) stage. */
LH2G_API int lh2g_get_traversal_stats(lh2g_context* ctx, unsigned long long* out4);

/* Ray queries over the scene (the OptiX Prime query interface of lib/RenderCore_PrimeRef/rendercore.cpp:569-605,
 * formats RTP_BUFFER_FORMAT_RAY_ORIGIN_TMIN_DIRECTION_TMAX / hit float4 {u|v<<16, inst, prim, t}).
 * mode 0: closest hit into lh2g_hit[n] (prim = -1 on a miss); mode 1: any hit into uint32 occluded[n].
 * A hit has tmin < t < tmax; tmin may be negative (hits behind the origin). A ray with a NaN in its origin,
 * direction, tmin or tmax is a miss and not occluded.
 * lh2g_trace takes device pointers and a CUDA stream (NULL = the context's stream) and returns without waiting;
 * lh2g_trace_host takes host buffers and returns when the results are back on the host. */
LH2G_API int lh2g_trace(lh2g_context* ctx, const lh2g_ray* rays, void* out, long long n, int mode, void* stream);
LH2G_API int lh2g_trace_host(lh2g_context* ctx, const lh2g_ray* rays, void* out, long long n, int mode);

/* Allocation-free frame render. No counterpart in the reference (its cores always allocate their buffers).
 * For callers that cannot call cudaMalloc when they render: a host with a fixed device-memory budget and its
 * own allocator (a game engine or plugin host that owns all device memory), or a process that must not grow
 * its device footprint after start-up. It renders one frame like lh2g_render_ex
 * (same kernels, same results) with all scratch memory of the wavefront stages in a static device array
 * compiled into the library (about 6 MB, held by every GPU that loads it until the process exits), and adds
 * the frame's per-pixel sums to accumDevice (caller-owned device memory, width*height float4).
 * Limit: width * height * spp <= LH2G_NOALLOC_MAX_PATHS, else LH2G_ERR_OVERFLOW. The scene comes from ctx,
 * which must be finalized; no render target is needed. stream may be NULL (legacy default stream). The first
 * call on a device (and the first in any other CUDA context on it, e.g. after cudaDeviceReset) looks up the
 * array's device address (cudaGetSymbolAddress); make that first call before any stream capture. All calls share
 * the array and it keeps the last call's contents: calls whose GPU work overlaps (other streams, threads or
 * contexts on the same device) race. statusHost (may be NULL) receives the frame's LH2G_STATUS_* word (traversal
 * stack overflow, step limit, copy timeout: the frame is then incomplete), copied on the stream: read it after the stream has
 * completed (pinned memory) or on return (pageable memory, which makes the copy synchronous). */
#define LH2G_NOALLOC_MAX_PATHS 32768
LH2G_API int lh2g_render_noalloc(lh2g_context* ctx, const lh2g_view* view, const lh2g_render_params* params, float* accumDevice,
                                 void* stream, uint32_t* statusHost);

/* ---- SoftRasterizer core ----
 * Replaces RenderCore_SoftRasterizer's Render (lib/RenderCore_SoftRasterizer/rendercore.cpp:213-227 over
 * rasterizer.cpp:66-171,225-240): z-buffered scanline rasterisation of the context's instances (meshes, instance
 * transforms, materials' base colour or colour texture) into the target set by lh2g_set_target (3..8192 pixels per
 * side; spp is ignored), with the reference core's fixed projection (focal length = target width), its near plane
 * at z = -0.2, back-face culling by the triangles' face normals and flat shading by their object-space normal z.
 * Pixels are RGBA8 words, 0 where nothing was drawn (the reference's memset) and for the one-pixel border it never
 * draws; instances that share a mesh all take the transform set last for it (the reference's scene graph holds
 * one transform per mesh). Results equal the reference core's pixel for pixel and its z-buffer bit for bit.
 * The frame runs on the context stream; pixelsHost / depthHost (W*H words, may be NULL) receive the image and the
 * z-buffer (interpolated 1/z of each drawn pixel, 0 elsewhere), and stats (may be NULL) the frame's counts; with
 * any of them the call returns when the frame is done. lh2g_raster_pixels_device gives the device image of the
 * last frame (valid until the next raster frame or lh2g_destroy; NULL before the first). */
typedef struct lh2g_raster_stats {
    uint32_t instancesDrawn;   /* instances the mesh culling kept */
    uint32_t triangles;        /* their triangles */
    uint32_t smallTriangles;   /* triangles rasterised one per thread that offered fragments */
    uint32_t bigTriangles;     /* triangles rasterised by blocks of 8 rows x 512 columns, a warp per row */
    uint32_t fragments;        /* fragments offered to the depth test (1/z < 0) */
    uint32_t status;           /* nonzero: a triangle named a missing material (not drawn) */
} lh2g_raster_stats;
LH2G_API int lh2g_raster_render(lh2g_context* ctx, const lh2g_view* view, uint32_t* pixelsHost, float* depthHost, lh2g_raster_stats* stats);
LH2G_API uint32_t* lh2g_raster_pixels_device(lh2g_context* ctx);
/* the last raster frame's pixels (its W*H words) to host memory; waits for the context stream */
LH2G_API int lh2g_raster_read(lh2g_context* ctx, uint32_t* pixelsHost);

/* ---- serving loop (no counterpart in the reference, whose cores render one frame at a time) ----
 * Render and ray-query jobs of several resident scenes, continuously batched: jobs are admitted smallest first
 * (oldest first once one has waited 0.2 s) while their paths fit in the server's path capacity (the admission
 * unit, 48 B x 2 + 64 B of queue memory per path plus 16 B of per-path radiance), and the paths of every admitted
 * job share one set of wavefront queues; one CUDA graph per tick advances every in-flight path by one vertex.
 * Express jobs (at most "expressMaxPaths" paths, off by default) skip the queues: each of their paths is traced to
 * its end within one tick by one thread, beside the waves, so a small job finishes in one tick instead of one tick
 * per bounce. A job's image is the per-pixel sum of its
 * samples (what lh2g_render_ex with accumulate = 0 leaves in the accumulator), bit for bit the same whatever else
 * is in flight. Ray queries run concurrently on a second stream. Scenes are finalized contexts, added by
 * reference: they must outlive the server and stay unchanged while it runs. Host buffers passed to submit must
 * stay valid until the job is done; pinned memory makes the copies asynchronous. */
typedef struct lh2g_server lh2g_server;
typedef struct lh2g_job_times { double submit, admit, done; } lh2g_job_times;   /* seconds on a steady clock */
typedef struct lh2g_server_stats {
    unsigned long long ticks, raysTraced;
    long long jobsDone, pathsInFlight, pending;
    uint32_t deviceStatus;
    long long loopLaunches;            /* launches of the device-side tick loop ("deviceLoop"; 0 with host-driven ticks) */
} lh2g_server_stats;
LH2G_API int lh2g_server_create(int device, long long pathCapacity, lh2g_server** out);
LH2G_API int lh2g_server_destroy(lh2g_server* server);   /* finishes the jobs it holds first */
/* Scheduling settings, applied to jobs admitted afterwards: "expressMaxPaths" (default 0: no express jobs; a
 * path traced whole by one thread is slower than the waves, so express jobs only pay when the GPU is otherwise
 * idle), "expressBudget" (express paths per tick, default 1048576), "tickBudget" (new queue paths per tick,
 * default clamp(capacity, 2^20, 2^22)), "maxWaitSeconds" (0.2), "largeJobPaths" (default 2^23; 0 = none: render jobs
 * of at least this many paths skip the shared queues and run one at a time as plain frames on the server's own
 * stream beside the ticks, needing no queue memory), "deviceLoop" (1 default: one graph launch runs ticks on the
 * device inside a conditional WHILE node until a job finishes, a job is submitted, the work runs out or "loopTicks"
 * ticks (default 256) have run, the device admitting the further ranges of jobs already admitted; 0: the host
 * launches every tick's graph, two in flight). Results do not depend on them. */
LH2G_API int lh2g_server_setting(lh2g_server* server, const char* name, double value);
LH2G_API const char* lh2g_server_last_error(lh2g_server* server);
LH2G_API int lh2g_server_add_scene(lh2g_server* server, lh2g_context* scene, int* sceneId);
/* hostOut: width * height float4. Filter frames (LH2G_RP_FILTER) are not served. */
LH2G_API int lh2g_server_submit_render(lh2g_server* server, int sceneId, const lh2g_view* view, const lh2g_render_params* params,
                                       float* hostOut, long long* jobId);
/* ray query as lh2g_trace_host: mode 0 closest hit into lh2g_hit[n], 1 any hit into uint32[n]; 1 <= n < 2^31 */
LH2G_API int lh2g_server_submit_trace(lh2g_server* server, int sceneId, const lh2g_ray* hostRays, long long n, int mode, void* hostOut,
                                      long long* jobId);
/* waits up to timeoutMs for a job: LH2G_OK when done (times filled), LH2G_ERR_STATE on timeout */
LH2G_API int lh2g_server_wait(lh2g_server* server, long long jobId, int timeoutMs, lh2g_job_times* times);
LH2G_API int lh2g_server_release(lh2g_server* server, long long jobId);   /* forgets a finished job */
LH2G_API int lh2g_server_get_stats(lh2g_server* server, lh2g_server_stats* out);

/* ---- radiance cache (no counterpart in the reference): a hash-grid + one-blob encoded 4 x 64 ReLU MLP with
 * bf16 weights, trained online with Adam on the relative L2 loss, inference and training on the tensor cores.
 * A query is 16 floats: position xyz, roughness, outgoing direction xyz, 0, normal xyz, 0, albedo rgb, 0; a
 * prediction and a training target are 4 floats (rgb, 0). Parameters: LH2G_NRC_MLP_PARAMS fp32 weights (row-major
 * [out][in] per layer: 64x64 four times, then 3x64) and LH2G_NRC_GRID_PARAMS fp32 grid features (12 levels x 2^19
 * entries x 2). */
#define LH2G_NRC_MLP_PARAMS 16576
#define LH2G_NRC_GRID_PARAMS 12582912
typedef struct lh2g_nrc lh2g_nrc;
typedef struct lh2g_nrc_config {
    float sceneMin[3], sceneMax[3];   /* box the hash grid spans */
    float learningRate;               /* Adam step (1e-3 when 0) */
    uint32_t seed;                    /* initial parameters */
} lh2g_nrc_config;
LH2G_API int lh2g_nrc_create(int device, const lh2g_nrc_config* config, lh2g_nrc** out);
LH2G_API int lh2g_nrc_destroy(lh2g_nrc* cache);
LH2G_API const char* lh2g_nrc_last_error(lh2g_nrc* cache);
/* encoding geometry (for CPU checkers): per-level resolution, dense flag, and bmin xyz + 1 / extent xyz */
LH2G_API int lh2g_nrc_get_spec(lh2g_nrc* cache, int* res12, int* dense12, float* bminInv6);
LH2G_API int lh2g_nrc_set_params(lh2g_nrc* cache, const float* mlp, const float* grid);   /* either may be NULL; resets Adam */
LH2G_API int lh2g_nrc_get_params(lh2g_nrc* cache, float* mlp, float* grid);
/* the accumulated gradients (a train call with update = 0 leaves them; update = 1 applies and clears them) */
LH2G_API int lh2g_nrc_get_grads(lh2g_nrc* cache, float* mlp, float* grid);
/* device buffers, asynchronous on stream (NULL: the cache's stream) */
LH2G_API int lh2g_nrc_infer(lh2g_nrc* cache, const float* queries, long long n, float* out, void* stream);
LH2G_API int lh2g_nrc_train(lh2g_nrc* cache, const float* queries, const float* targets, long long n, int update, float* lossOut,
                            void* stream);
/* one Adam step with the gradients accumulated by train calls with update = 0 (then cleared) */
LH2G_API int lh2g_nrc_apply_update(lh2g_nrc* cache, void* stream);
/* as lh2g_nrc_infer / lh2g_nrc_train (update = 1) for a count that earlier device work leaves at countDevice
 * (a uint32, at most maxCount are used): no host round trip. An empty training batch leaves the parameters
 * unchanged (the Adam step count still advances). */
LH2G_API int lh2g_nrc_infer_counted(lh2g_nrc* cache, const float* queries, const uint32_t* countDevice, long long maxCount, float* out,
                                    void* stream);
LH2G_API int lh2g_nrc_train_counted(lh2g_nrc* cache, const float* queries, const float* targets, const uint32_t* countDevice,
                                    long long maxCount, void* stream);
/* the mean loss of the last training batch (waits for the device) */
LH2G_API int lh2g_nrc_last_loss(lh2g_nrc* cache, float* loss);
/* One frame with the radiance cache (like lh2g_render_ex with accumulate): a path ends at its first vertex from
 * path length 2 on that a diffuse bounce leads to and adds throughput x cache(query) there; one in sixteen of
 * them trace on and their radiance from that vertex on, divided by the throughput into it, trains the cache after the frame
 * (train != 0, at most 65536 samples, one Adam step). The plain estimator is unchanged everywhere else.
 * With stats == NULL the call returns once the frame is queued, and consecutive frames overlap like plain frames
 * (their cache work stays in submission order: each frame's inference sees the previous frame's update);
 * with stats it waits for the frame and reports its query and training-sample counts and training loss. */
typedef struct lh2g_nrc_frame_stats { uint32_t queries, trainSamples; float loss; } lh2g_nrc_frame_stats;
LH2G_API int lh2g_render_nrc(lh2g_context* ctx, lh2g_nrc* cache, const lh2g_view* view, const lh2g_render_params* params, int accumulate,
                             int train, lh2g_nrc_frame_stats* stats);
/* Self-test of the bounded tensor-core waits: a kernel waits on an mbarrier that nothing arrives on, gives up
 * after `limit` polls and sets *status to 1 (the error word every timed-out wait of the cache kernels raises);
 * the device stays usable. */
LH2G_API int lh2g_nrc_wait_selftest(int device, uint32_t limit, uint32_t* status);
/* host buffers, synchronous */
LH2G_API int lh2g_nrc_infer_host(lh2g_nrc* cache, const float* queries, long long n, float* out);
LH2G_API int lh2g_nrc_train_host(lh2g_nrc* cache, const float* queries, const float* targets, long long n, int update, float* lossOut);

#ifdef __cplusplus
}
#endif
#endif

/* lh2o.h - CPU ORACLE of the GB300 wavefront render core.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker that the CUDA path is compared against, and the
 * timed CPU baseline of the benchmark. Nothing in the product links, loads or calls it; only tests/,
 * __graft_entry__.smoke() and bench.py (its CPU-baseline leg and --impl reference arm) may.
 *
 * It restates, in plain C++ on the host, the reference's path for one frame:
 *   - primary rays        lib/RenderCore_PrimeRef/kernels/camera.h:39-68
 *   - shading             lib/RenderCore_PrimeRef/kernels/pathtracer.h:45-168 with the BSDF of
 *                         lib/sharedBSDFs/lambert.h:32-125, lights of lib/CUDA/shared_kernel_code/lights_shared.h,
 *                         materials of lib/CUDA/shared_kernel_code/material_shared.h:42-206
 *   - shadow connections  lib/RenderCore_PrimeRef/kernels/connections.h:22-34
 *   - the wave loop       lib/RenderCore_PrimeRef/rendercore.cpp:535-632, run per path depth-first, which is
 *                         equivalent because every random number depends only on (path, depth).
 * and, as other estimators, the OptiX 7 core's (lib/rendercore_optix7/kernels/pathtracer.h:54-238 with
 * optix/.optix.cu:71-129: MIS, blue noise, path regularisation, one diffuse bounce) and the PrimeAdaptive core's
 * adaptive frames (lib/RenderCore_PrimeAdaptive/rendercore.cpp:600-755, kernels/camera.h, kernels/pathtracer.h,
 * lib/CUDA/shared_kernel_code/finalize_shared.h:71-151).
 * Ray traversal in the reference is closed NVIDIA code (OptiX / OptiX Prime), so the oracle brings its own
 * scalar binned-SAH BVH2 and a brute-force intersector; both return the closest hit with ties broken by the
 * lowest (instance, primitive).
 */
#ifndef LH2O_H
#define LH2O_H

#include "../include/lh2g_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lh2o_scene lh2o_scene;

lh2o_scene* lh2o_create(void);
void lh2o_destroy(lh2o_scene* s);

/* Scene setters: same meaning as the core's CoreAPI_Base setters (core_api_base.h:103-118). */
int lh2o_set_geometry(lh2o_scene* s, int meshIdx, const float* vertices4, int vertexCount, int triangleCount,
                      const lh2g_core_tri* tris);
int lh2o_set_instance(lh2o_scene* s, int instIdx, int meshIdx, const float* transform16);
int lh2o_set_materials(lh2o_scene* s, const lh2g_material* mats, int count);
int lh2o_set_textures(lh2o_scene* s, const lh2g_texture* tex, int count);
int lh2o_set_lights(lh2o_scene* s, const lh2g_light_tri* tri, int ntri, const lh2g_point_light* pt, int npt,
                    const lh2g_spot_light* spot, int nspot, const lh2g_dir_light* dir, int ndir);
/* the light tree lh2o_set_lights built (2 * (area + point + spot lights) records of 16 words, record 0 the root);
 * returns the record count (out NULL: the count only), -1 if capacity (in records) is too small */
int lh2o_light_tree(const lh2o_scene* s, void* out, int capacity);
int lh2o_set_sky(lh2o_scene* s, const float* rgb, int width, int height, const float* worldToSky16);
/* Builds the BVHs (BVH2 per mesh + BVH2 over instances). Must follow the setters, precede tracing. */
int lh2o_finalize(lh2o_scene* s);

/* Ray queries. mode 0: closest hit into hits (prim = -1 on miss); mode 1: any hit, occluded[i] = 0/1.
 * brute != 0 tests every triangle of every instance (the check of the BVH). */
int lh2o_trace(lh2o_scene* s, const lh2g_ray* rays, long long n, int mode, int brute, lh2g_hit* hits,
               uint32_t* occluded, int nthreads);

/* Closest hit with unquantised barycentrics (t, instance, primitive, u, v per ray; prim = -1 on a miss). */
int lh2o_trace_raw(lh2o_scene* s, const lh2g_ray* rays, long long n, float* t, int* inst, int* prim, float* u, float* v,
                   int nthreads);

/* One frame of the path tracer. pixelAccum (W*H float4) receives += the sum over the frame's samples of each
 * path's radiance (rgb; w = primary hit distance when LH2G_RP_DEPTH_W). pixelAccum64 (optional, W*H*4
 * doubles) receives the same sums accumulated in FP64. counters (optional, 2*maxDepth) receive per path
 * length the number of extension rays and shadow rays written. capture (optional) receives per-path,
 * per-depth hits and RNG states (maxDepth * W*H*spp entries each). Returns 0 on success. */
int lh2o_render(lh2o_scene* s, const lh2g_view* view, const lh2g_render_params* p, float* pixelAccum,
                double* pixelAccum64, uint32_t* counters, lh2g_capture* capture, int nthreads);

/* Blue-noise tables of the OptiX 7 estimator (lib/RenderSystem/common_bluenoise.h layout, 8 bits per entry):
 * sobol 256 x 256, scrambling and ranking 128 x 128 x 8 each. NULL pointers remove them. */
int lh2o_set_blue_noise(lh2o_scene* s, const uint8_t* sobol, const uint8_t* scrambling, const uint8_t* ranking);

/* One frame of the PrimeAdaptive core (lib/RenderCore_PrimeAdaptive/rendercore.cpp:600-755): spp samples per pixel
 * with the OptiX 7 estimator, a per-pixel variance estimate scaled by *devScale, up to 24 more samples per pixel
 * where it asks for them (at most W*H*spp in all; *devScale is then steered towards 91-98 % of that budget), and
 * finalizeASRender: accum (W*H float4) += each pixel's samples divided by their count; frame (optional) =
 * accum / frames. p->cameraR0 and p->frameSeed are the frame's two draws of RandomUInt(camRNGseed), p->shift the
 * blue-noise shift. counters (optional, 4 * maxDepth): per path length the extension and connection counts of the
 * first wave, then of the second. adaptivePaths: the second wave's path count. frameAccOut, featuresOut (W*H*spp
 * float4) and deviationOut (W*H) are optional copies of the intermediate buffers; capture covers the first wave. */
int lh2o_render_adaptive(lh2o_scene* s, const lh2g_view* view, const lh2g_render_params* p, float* accum, float* frame, float* devScale,
                         uint32_t* counters, uint32_t* adaptivePaths, float* frameAccOut, float* featuresOut, float* deviationOut,
                         lh2g_capture* capture, int nthreads);

/* SVGF feature buffers of a LH2G_RP_FILTER frame, W*H entries each, written for the paths of sample 0 of a
 * frame with samplesTaken == 0 (RenderCore_Optix7Filter/kernels/pathtracer.h:95-232). features: uint4;
 * worldPos, deltaDepth: float4. The caller keeps them between frames (features.w carries the history count). */
typedef struct lh2o_features { uint32_t* features; float* worldPos; float* deltaDepth; } lh2o_features;

/* lh2o_render with feature output. For LH2G_RP_FILTER frames pixelAccum (and pixelAccum64) hold 2*W*H float4:
 * the direct half, then the indirect half. */
int lh2o_render_ex(lh2o_scene* s, const lh2g_view* view, const lh2g_render_params* p, float* pixelAccum,
                   double* pixelAccum64, uint32_t* counters, lh2g_capture* capture, const lh2o_features* feat, int nthreads);

/* SVGF state of one render target: the buffers of RenderCore_Optix7Filter/rendercore.cpp:350-364 (W*H entries,
 * float4 unless noted), owned by the caller. lh2o_svgf_frame swaps the history pointers inside the struct
 * exactly as the GPU core swaps its buffers, so the same slot names can be compared after every frame. */
typedef struct lh2o_svgf {
    int width, height;
    uint32_t* features;                  /* uint4, written by lh2o_render_ex */
    float* worldPos;                     /* written by lh2o_render_ex */
    float* prevWorldPos;
    float* deltaDepth;                   /* written by lh2o_render_ex */
    float* motion;                       /* float2 */
    float* moments;
    float* prevMoments;
    float* shading;
    float* filteredIN;
    float* filteredOUT;
    float* prevPixels;
    float* taaPixels;                    /* TAA output (the reference updates 'shading' in place) */
    float* target;                       /* the frame: border pixels are never written */
} lh2o_svgf;

/* prepareFilter, applyFilter x 3, TAA + unsharpen or finalizeNoTAA, history swaps
 * (RenderCore_Optix7Filter/rendercore.cpp:904-935). accum: 2*W*H float4 of the frame. */
int lh2o_svgf_frame(lh2o_svgf* f, const float* accum, const lh2g_filter_params* fp, int nthreads);

/* Radiance cache (no reference counterpart): the encoding, the network's outputs and the gradients of the mean
 * relative L2 loss, with the GPU kernels' rounding points when emulate != 0 (fp16 grid features, bf16 weights,
 * activations and loss gradients; sums in double), and one Adam step (beta1 0.9, beta2 0.99, eps 1e-15). Grid
 * and weight layouts are those of lh2g_nrc_set_params; gMlp / gGrid are added to (double, same layouts). */
typedef struct lh2o_nrc_spec { int res[12]; int dense[12]; float bmin[3], inv[3]; } lh2o_nrc_spec;
void lh2o_nrc_encode(const lh2o_nrc_spec* spec, const float* grid, const float* query16, float* e64);
int lh2o_nrc_forward(const lh2o_nrc_spec* spec, const float* grid, const float* mlp, const float* queries, long long n, float* out4,
                     int emulate, int nthreads);
/* outputs in double, without the GPU's rounding (finite-difference checks) */
int lh2o_nrc_forward64(const lh2o_nrc_spec* spec, const float* grid, const float* mlp, const float* queries, long long n, double* out3);
int lh2o_nrc_gradients(const lh2o_nrc_spec* spec, const float* grid, const float* mlp, const float* queries, const float* targets,
                       long long n, int emulate, double* gMlp, double* gGrid, double* loss);
void lh2o_nrc_adam(float* p, float* m, float* v, const float* g, long long n, float lr, long long step);

/* SoftRasterizer core (lib/RenderCore_SoftRasterizer/rasterizer.cpp:66-171,201-240, rendercore.cpp:213-222):
 * one frame of W x H RGBA8 pixels (0 where nothing was drawn) and the z-buffer of interpolated 1/z (0 where
 * nothing was drawn; may be null); fragments = depth-test passes (may be null). W, H in 3..8192. */
int lh2o_raster(lh2o_scene* s, const lh2g_view* view, int W, int H, uint32_t* pixels, float* zbuffer, uint64_t* fragments);

/* Small pure functions exported for the pinning tests against the reference's own headers. */
uint32_t lh2o_wanghash(uint32_t s);
/* blueNoiseSampler4 over an expanded table (5 * 65536 + 64 entries) */
void lh2o_bluenoise4(const uint32_t* bn, int x, int y, int sampleIndex, int sampleDimension, float* out4);
float lh2o_random_float(uint32_t* seed);
void lh2o_random_barycentrics(float r0, float* out3);
uint32_t lh2o_pack_normal(const float* n3);
void lh2o_unpack_normal(uint32_t p, float* out3);
void lh2o_diffuse_cos(float r0, float r1, float* out3);
void lh2o_tangent2world(const float* v3, const float* n3, float* out3);
void lh2o_consistent_normal(const float* d3, const float* in3, float alpha, float* out3);
void lh2o_sincos(float x, float* s, float* c);
float lh2o_expf(float x);
float lh2o_log2f(float x);
float lh2o_logf(float x);
float lh2o_powf(float x, float y);
float lh2o_atan2f(float y, float x);
float lh2o_acosf(float x);
uint16_t lh2o_float2half(float f);
float lh2o_half2float(uint16_t h);
void lh2o_pack_material(const lh2g_material* m, const uint32_t* texFirstPixel, const uint32_t* texWH,
                        lh2g_gpu_material* out);
void lh2o_invert4x4(const float* m16, float* out16);
uint32_t lh2o_pack_normal2(const float* n3);
void lh2o_unpack_normal2(uint32_t p, float* out3);
uint32_t lh2o_hdr_to_rgb32(const float* c3);
void lh2o_rgb32_to_hdr(uint32_t c, int min1, float* out3);
void lh2o_combine_to_float4(const float* a3, const float* b3, float* out4);
void lh2o_split_float4(const float* x4, float* direct3, float* indirect3);
void lh2o_rgb_to_ycocg(const float* rgb3, float* out3);
void lh2o_ycocg_to_rgb(const float* ycocg3, float* out3);
float lh2o_luminance(const float* rgb3);
float lh2o_mitchell_netravali(float v);
/* prepareFilter's camera constants (prevPos, prevE, prevRight, prevUp as 4 float4) for a target of height h */
void lh2o_svgf_view(const lh2g_view* v, int h, float* out16);

#ifdef __cplusplus
}
#endif
#endif

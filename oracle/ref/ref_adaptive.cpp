/* ref_adaptive.cpp - the PrimeAdaptive core's kernels compiled for the host (TEST INFRASTRUCTURE ONLY).
 *
 * Built by oracle/ref/Makefile from the reference tree: lib/RenderCore_PrimeAdaptive/kernels/{camera,pathtracer,
 * connections}.h (generateEyeRaysKernel, generateEyeRaysKernelAdaptive, shadeKernel, finalizeConnectionKernel, their
 * launch wrappers cut off) with the Lambert BSDF (lib/sharedBSDFs/lambert.h, the alternative kernels/bsdf.h offers),
 * and estimateVarianceKernel / finalizeASRenderKernel of lib/CUDA/shared_kernel_code/finalize_shared.h. A test drives
 * the core's RenderImpl (lib/RenderCore_PrimeAdaptive/rendercore.cpp:600-755) through these entry points with the
 * oracle standing in for the closed OptiX Prime queries. Every launch runs its threads one at a time in index order,
 * so the compaction atomics hand out slots in thread order. */
#include "ref_shim.h"
#include <vector>
#include "helper_math.h"
#include "common_settings.h"
#include "common_types.h"
#include "common_classes.h"
#include "common_functions.h"

namespace refad {
#include "ref_globals.h"
/* CLAMPINTENSITY of the core's core_settings.h (CLAMPFIREFLIES on): scales a contribution whose largest channel
 * exceeds clampValue down to it, w untouched */
#define CLAMPINTENSITY                                                                                                         \
    {                                                                                                                          \
        const float v_ = max(contribution.x, max(contribution.y, contribution.z));                                             \
        if (v_ > clampValue) {                                                                                                 \
            const float m_ = clampValue / v_;                                                                                  \
            contribution.x *= m_, contribution.y *= m_, contribution.z *= m_;                                                  \
        }                                                                                                                      \
    }
#include "lambert.h"
#include "inc_ad/pathtracer.h"
#include "inc_ad/camera.h"
#include "inc_ad/connections.h"
/* the finalize kernels' globals: the render-target surface as a float4 array, powf(x, 2) and powf(x, 128) as
 * repeated squarings (the oracle's own), like the other CUDA math calls ref_shim.h routes */
static float4* debugData;
static float4* refTarget;
static int refTargetW;
struct RefSurface {};
static RefSurface renderTarget;
template <typename T>
static inline void surf2Dwrite(T v, RefSurface, int xBytes, int y, cudaSurfaceBoundaryMode) { refTarget[xBytes / (int)sizeof(T) + y * refTargetW] = v; }
static inline float ref_powf(float x, float y) {
    if (y == 2.0f) return x * x;
    if (y == 128.0f) { for (int i = 0; i < 7; i++) x = x * x; return x; }
    return std::pow(x, y);
}
#define powf(x, y) ref_powf(x, y)
#include "finalize_shared.h"
#undef powf
}  // namespace refad

using namespace refad;

static void grid1(long long n, void (*body)(void*), void* ctx) {
    blockDim.x = blockDim.y = blockDim.z = 1;
    threadIdx.x = threadIdx.y = threadIdx.z = 0;
    blockIdx.y = blockIdx.z = 0;
    for (long long i = 0; i < n; i++) { blockIdx.x = (uint)i; body(ctx); }
}
static void grid2(int w, int h, void (*body)(void*), void* ctx) {
    blockDim.x = blockDim.y = blockDim.z = 1;
    threadIdx.x = threadIdx.y = threadIdx.z = 0;
    blockIdx.z = 0;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) { blockIdx.x = (uint)x, blockIdx.y = (uint)y; body(ctx); }
}

extern "C" {

void ref_ad_set_scene(void* instDescs, void* mats, void* tri, int ntri, void* pt, int npt, void* spot, int nspot, void* dir, int ndir,
                      uint32_t* texels, float geoEps, float clampVal, int maxPathLength, float* sky4, int skyW, int skyH) {
    instanceDescriptors = (CoreInstanceDesc*)instDescs;
    materials = (CUDAMaterial4*)mats;
    triLights = (CoreLightTri*)tri, pointLights = (CorePointLight*)pt, spotLights = (CoreSpotLight*)spot, directionalLights = (CoreDirectionalLight*)dir;
    lightCounts = make_int4(ntri, npt, nspot, ndir);
    argb32 = (uchar4*)texels;
    skywidth = skyW, skyheight = skyH, skyPixels = (float4*)sky4;
    geometryEpsilon = geoEps;
    clampValue = clampVal;
    MAXPATHLENGTH_RT = maxPathLength;
}

/* lib/RenderCore_PrimeAdaptive/kernels/.cuda.cu:174-198 */
void ref_ad_init_extend(int pathCount) {
    memset(counters, 0, sizeof(Counters));
    counters->activePaths = (uint)pathCount, counters->totalExtensionRays = (uint)pathCount;
}
void ref_ad_init_stage2() { counters->activePaths = 0, counters->extensionRays = 0, counters->shadowRays = 0; }
void ref_ad_next() {
    counters->totalExtensionRays += counters->extensionRays;
    counters->activePaths = counters->extensionRays;
    counters->extensionRays = 0;
}
void ref_ad_counters(uint32_t* out3) { out3[0] = counters->activePaths, out3[1] = counters->extensionRays, out3[2] = counters->shadowRays; }
void ref_ad_set_active(uint32_t n) { counters->activePaths = n; }
void ref_ad_set_shadow(uint32_t n) { counters->shadowRays = n; }

struct GenArgs { Ray4* rays; float4* ps; uint R0; const uint* bn; int pass; float3 pos, right, up; float aperture; float3 p1; float distortion; int4 sp; int n; const float* dev; };
static void gen_body(void* c) {
    GenArgs* a = (GenArgs*)c;
    generateEyeRaysKernel(a->rays, a->ps, a->R0, a->bn, a->pass, a->pos, a->right, a->up, a->aperture, a->p1, a->distortion, a->sp, a->n);
}
static void gen2_body(void* c) {
    GenArgs* a = (GenArgs*)c;
    generateEyeRaysKernelAdaptive(a->dev, a->rays, a->ps, a->R0, (uint)a->pass, a->bn, a->pos, a->right, a->up, a->aperture, a->p1, a->distortion,
                                  a->sp, a->n);
}
static GenArgs gen_args(void* rays, void* ps, uint32_t R0, const uint32_t* bn, int pass, const float* pos, float aperture, const float* right,
                        const float* up, const float* p1, float distortion, int w, int h, int spp) {
    GenArgs a;
    a.rays = (Ray4*)rays, a.ps = (float4*)ps, a.R0 = R0, a.bn = bn, a.pass = pass;
    a.pos = make_float3(pos[0], pos[1], pos[2]), a.right = make_float3(right[0], right[1], right[2]), a.up = make_float3(up[0], up[1], up[2]);
    a.aperture = aperture, a.p1 = make_float3(p1[0], p1[1], p1[2]), a.distortion = distortion;
    a.sp = make_int4(w + (h << 16), spp, 0, 0);
    a.dev = nullptr;
    return a;
}
/* generateEyeRays (camera.h:39-87): W*H*spp primary rays */
void ref_ad_generate(void* rays, void* ps, uint32_t R0, const uint32_t* bn, int pass, const float* pos, float aperture, const float* right,
                     const float* up, const float* p1, float distortion, int w, int h, int spp) {
    GenArgs a = gen_args(rays, ps, R0, bn, pass, pos, aperture, right, up, p1, distortion, w, h, spp);
    a.n = w * h * spp;
    grid1(a.n, gen_body, &a);
}
/* generateEyeRaysAdaptive (camera.h:96-157): W*H*24 threads, the rays of those a pixel's deviation asks for */
void ref_ad_generate_adaptive(const float* deviation, void* rays, void* ps, uint32_t R0, int pass, const uint32_t* bn, const float* pos,
                              float aperture, const float* right, const float* up, const float* p1, float distortion, int w, int h, int spp) {
    GenArgs a = gen_args(rays, ps, R0, bn, pass, pos, aperture, right, up, p1, distortion, w, h, spp);
    a.dev = deviation;
    a.n = w * h * 24;
    grid1(a.n, gen2_body, &a);
}

struct ShadeArgs {
    float4* acc; float4* feat; uint stride; Ray4* rays; float4* ps; Intersection* hits; Ray4* raysOut; float4* psOut; Ray4* conn; float4* pot;
    uint R0, shift; const uint* bn; int pass, pathLength, w, h; float spread; int n;
};
static void shade_body(void* c) {
    ShadeArgs* a = (ShadeArgs*)c;
    shadeKernel(a->acc, a->feat, a->stride, a->rays, a->ps, a->hits, a->raysOut, a->psOut, a->conn, a->pot, a->R0, a->shift, a->bn, a->pass, -1,
                a->pathLength, a->w, a->h, a->spread, a->n);
}
void ref_ad_shade(int pathCount, float* frameAcc, float* features, void* rays, void* ps, void* hits, void* raysOut, void* psOut, void* connections,
                  void* potentials, uint32_t R0, uint32_t shift, const uint32_t* bn, int pass, int pathLength, int w, int h, float spreadAngle, int nee) {
    ShadeArgs a;
    a.acc = (float4*)frameAcc, a.feat = (float4*)features, a.stride = 0, a.rays = (Ray4*)rays, a.ps = (float4*)ps, a.hits = (Intersection*)hits;
    a.raysOut = (Ray4*)raysOut, a.psOut = (float4*)psOut, a.conn = nee ? (Ray4*)connections : nullptr, a.pot = (float4*)potentials;
    a.R0 = R0, a.shift = shift, a.bn = bn, a.pass = pass, a.pathLength = pathLength, a.w = w, a.h = h, a.spread = spreadAngle, a.n = pathCount;
    grid1(pathCount, shade_body, &a);
}

struct ConnArgs { float4* acc; uint* hb; float4* pot; int n; };
static void conn_body(void* c) { ConnArgs* a = (ConnArgs*)c; finalizeConnectionKernel(a->acc, a->hb, a->pot, a->n); }
void ref_ad_finalize_connections(int rayCount, float* frameAcc, uint32_t* hitBits, void* potentials) {
    ConnArgs a{(float4*)frameAcc, hitBits, (float4*)potentials, rayCount};
    grid1(rayCount, conn_body, &a);
}

struct VarArgs { const float4* acc; const float4* feat; float* dev; float scale; int w, h, spp; };
static void var_body(void* c) { VarArgs* a = (VarArgs*)c; estimateVarianceKernel(a->acc, a->feat, a->dev, a->scale, a->w, a->h, a->spp); }
void ref_ad_estimate_variance(const float* frameAcc, const float* features, float* deviation, float scale, int w, int h, int spp) {
    VarArgs a{(const float4*)frameAcc, (const float4*)features, deviation, scale, w, h, spp};
    grid2(w, h, var_body, &a);
}

struct FinArgs { const float4* facc; float4* acc; int w, h, spp; float scale; };
static void fin_body(void* c) { FinArgs* a = (FinArgs*)c; finalizeASRenderKernel(a->facc, a->acc, a->w, a->h, a->spp, a->scale); }
/* finalizeASRender (finalize_shared.h:86-93) with the surface written to target (W*H float4) */
void ref_ad_finalize(const float* frameAcc, float* accumulator, float* target, int w, int h, int samplesTaken, int spp) {
    refTarget = (float4*)target, refTargetW = w;
    const int frame = samplesTaken / spp;
    FinArgs a{(const float4*)frameAcc, (float4*)accumulator, w, h, spp, 1.0f / (float)frame};
    grid2(w, h, fin_body, &a);
}
}

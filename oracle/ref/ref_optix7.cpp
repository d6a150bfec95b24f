/* ref_optix7.cpp - the OptiX 7 core's shading kernel and ray-generation helpers compiled for the host
 * (TEST INFRASTRUCTURE ONLY).
 *
 * Built by oracle/ref/Makefile from the reference tree: lib/rendercore_optix7/kernels/pathtracer.h (shadeKernel, with
 * its launch wrapper cut off) and the blue-noise, lens and eye-ray helpers of lib/rendercore_optix7/optix/.optix.cu
 * (the lines from blueNoiseSampler4 to generateEyeRay, cut out of that file because the rest of it is OptiX
 * device code), with the Lambert BSDF (lib/sharedBSDFs/lambert.h, the alternative kernels/bsdf.h offers). A test
 * drives the OptiX 7 core's wave loop (lib/rendercore_optix7/rendercore.cpp:874-922) through these entry points with
 * the oracle standing in for optixTrace. Every launch runs its threads one at a time in index order. */
#include "ref_shim.h"
#include <vector>
#include "helper_math.h"
#include "common_settings.h"
#include "common_types.h"
#include "common_classes.h"
#include "common_functions.h"

/* Built three times: as is with the Lambert BSDF (entry points ref_o7_*), and with -DREF_O7_DISNEY with the Disney BSDF
 * (the default branch of the core's kernels/bsdf.h: lib/sharedBSDFs/ggxmdf.h, frosted.h, disney.h; entry points
 * ref_o7d_*). The Disney build reads copies the Makefile makes in $(OUT)/inc_o7d: the three BSDF headers with their
 * CUDA branches selected (the samplers' sincosf form and the adjoint parameter), and pathtracer.h with its unset
 * newBsdfPdf (pathtracer.h:219) zero-initialised, so that a sampler exit that leaves it unset ends the path on the
 * host as the restatement does. logf and powf go to the oracle's own functions, as the other transcendentals do.
 * The third build (-DREF_O7_LTREE -DLIGHTTREE, entry points ref_o7t_*, Lambert BSDF) selects lights through the light
 * tree: it reads copies in $(OUT)/inc_o7t of pathtracer.h with its two light-tree calls (pathtracer.h:145,187)
 * taking the place of the potential-based ones they sit beside as comments, and of
 * shared_kernel_code/lights_shared.h with the tree typed as the device LightCluster layout (ref_globals.h's
 * DevLightCluster; the host build of common_classes.h has the host layout) and each child box's three random
 * numbers drawn x, y, z in that order (the order the CUDA compiler evaluates make_float3's arguments; g++ evaluates
 * them right to left). */
#if defined(REF_O7_LTREE)
#define REF_NS refo7t
#define O7(name) ref_o7t_##name
#elif defined(REF_O7_DISNEY)
#define REF_NS refo7d
#define O7(name) ref_o7d_##name
extern "C" float lh2o_logf(float x);
extern "C" float lh2o_powf(float x, float y);
#else
#define REF_NS refo7
#define O7(name) ref_o7_##name
#endif

namespace REF_NS {
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
#if defined(REF_O7_LTREE)
#include "lambert.h"
#include "inc_o7t/pathtracer.h"
#elif defined(REF_O7_DISNEY)
using std::abs;
#define logf(x) lh2o_logf(x)
#define powf(x, y) lh2o_powf(x, y)
#include "inc_o7d/ggxmdf.h"
#include "inc_o7d/frosted.h"
#include "inc_o7d/disney.h"
#include "inc_o7d/pathtracer.h"
#else
#include "lambert.h"
#include "inc_o7/pathtracer.h"
#endif
/* the fields of Params (lib/rendercore_optix7/core_settings.h:113-133) that the ray-generation helpers read */
struct RefParams { float4 posLensSize; float3 right, up, p1; float geometryEpsilon, distortion; int3 scrsize; int pass, phase, shift; uint* blueNoise; };
static RefParams params;
#include "inc_o7/optix_raygen.h"
}  // namespace REF_NS

using namespace REF_NS;

static void grid1(long long n, void (*body)(long long, void*), void* ctx) {
    blockDim.x = blockDim.y = blockDim.z = 1;
    threadIdx.x = threadIdx.y = threadIdx.z = 0;
    blockIdx.y = blockIdx.z = 0;
    for (long long i = 0; i < n; i++) { blockIdx.x = (uint)i; body(i, ctx); }
}

extern "C" {

/* scene: all pointers stay owned by the caller; sky4 holds the sky and then its 64x scaled-down copy;
 * blueNoise: 5 * 65536 entries plus padding (the expanded tables of rendercore.cpp:247-256) */
void O7(set_scene)(void* instDescs, void* mats, void* tri, int ntri, void* pt, int npt, void* spot, int nspot, void* dir, int ndir,
                      uint32_t* texels, float geoEps, float clampVal, int maxPathLength, float* sky4, int skyW, int skyH, uint32_t* blueNoise) {
    instanceDescriptors = (CoreInstanceDesc*)instDescs;
    materials = (CUDAMaterial4*)mats;
    triLights = (CoreLightTri*)tri, pointLights = (CorePointLight*)pt, spotLights = (CoreSpotLight*)spot, directionalLights = (CoreDirectionalLight*)dir;
    lightCounts = make_int4(ntri, npt, nspot, ndir);
    argb32 = (uchar4*)texels;
    skywidth = skyW, skyheight = skyH, skyPixels = (float4*)sky4;
    geometryEpsilon = geoEps;
    clampValue = clampVal;
    MAXPATHLENGTH_RT = maxPathLength;
    params.blueNoise = blueNoise;
}

/* InitCountersForExtend / InitCountersSubsequent (lib/rendercore_optix7/kernels/.cuda.cu:191-212) */
void O7(init_counters)(int pathCount) {
    memset(counters, 0, sizeof(Counters));
    counters->activePaths = (uint)pathCount, counters->totalExtensionRays = (uint)pathCount;
}
void O7(next_counters)() {
    counters->totalExtensionRays += counters->extensionRays;
    counters->activePaths = counters->extensionRays;
    counters->extended = counters->shaded = 0;
    counters->extensionRays = 0;
}
void O7(counters)(uint32_t* out2) { out2[0] = counters->extensionRays, out2[1] = counters->shadowRays; }
void O7(set_shadow_count)(uint32_t n) { counters->shadowRays = n; }

/* the first part of setupPrimaryRay (optix/.optix.cu:112-121): the eye ray of every path and its path state
 * (the optixTrace that follows it there is the caller's) */
struct GenArgs { float4* ps; uint stride; };
static void gen_body(long long i, void* c) {
    GenArgs* a = (GenArgs*)c;
    const uint pathIdx = (uint)i;
    const uint pixelIdx = pathIdx % (params.scrsize.x * params.scrsize.y);
    const uint sampleIdx = pathIdx / (params.scrsize.x * params.scrsize.y) + params.pass;
    uint seed = WangHash(pathIdx * 16789 + params.pass * 1791);
    float3 O, D;
    generateEyeRay(O, D, pixelIdx, sampleIdx, seed);
    a->ps[pathIdx] = make_float4(O, __uint_as_float((pathIdx << 6) + 1));
    a->ps[pathIdx + a->stride] = make_float4(D, 0);
}
void O7(generate)(float* pathStates, int w, int h, int spp, int pass, int shift, const float* pos, float aperture, const float* right,
                     const float* up, const float* p1, float distortion) {
    params.posLensSize = make_float4(pos[0], pos[1], pos[2], aperture);
    params.right = make_float3(right[0], right[1], right[2]), params.up = make_float3(up[0], up[1], up[2]);
    params.p1 = make_float3(p1[0], p1[1], p1[2]);
    params.distortion = distortion, params.scrsize = make_int3(w, h, spp), params.pass = pass, params.shift = shift;
    params.geometryEpsilon = geometryEpsilon;
    GenArgs a{(float4*)pathStates, (uint)(w * h * spp)};
    grid1((long long)w * h * spp, gen_body, &a);
}

struct ShadeArgs {
    float4* acc; uint stride; float4* ps; float4* hits; float4* conn; uint R0, shift; int pass, pathLength, w, h; float spread; uint n;
};
static void shade_body(long long, void* c) {
    ShadeArgs* a = (ShadeArgs*)c;
    shadeKernel(a->acc, a->stride, a->ps, a->hits, a->conn, a->R0, a->shift, params.blueNoise, a->pass, -1, a->pathLength, a->w, a->h, a->spread, a->n);
}
void O7(shade)(int pathCount, float* accumulator, float* pathStates, float* hits, float* connections, uint32_t R0, uint32_t shift, int pass,
                  int pathLength, int w, int h, int spp, float spreadAngle, int nee) {
    ShadeArgs a;
    a.acc = (float4*)accumulator, a.stride = (uint)(w * h * spp), a.ps = (float4*)pathStates, a.hits = (float4*)hits;
    a.conn = nee ? (float4*)connections : nullptr, a.R0 = R0, a.shift = shift, a.pass = pass, a.pathLength = pathLength;
    a.w = w, a.h = h, a.spread = spreadAngle, a.n = (uint)pathCount;
    grid1(pathCount, shade_body, &a);
}

/* the part of generateShadowRay (optix/.optix.cu:142-154) after optixTrace: unoccluded connections add their
 * contribution and 1 in w to the pixel */
void O7(finalize_connections)(int count, float* accumulator, const float* connections, const uint32_t* occluded, int stride) {
    const float4* cd = (const float4*)connections;
    float4* acc = (float4*)accumulator;
    for (int i = 0; i < count; i++) {
        if (occluded[i]) continue;
        const float4 E4 = cd[i + stride * 2 * 2];
        const int pixelIdx = __float_as_int(E4.w);
        if (pixelIdx < stride) acc[pixelIdx] += make_float4(E4.x, E4.y, E4.z, 1);
    }
}

#if defined(REF_O7_LTREE)
/* the light tree the light-selection code reads (records of the device LightCluster; owned by the caller) */
void O7(set_light_tree)(void* records) { lightTree = (DevLightCluster*)records; }
#endif

/* blueNoiseSampler4 of tools_shared.h:324-337 (the shading kernels' copy) */
void O7(bluenoise4)(const uint32_t* bn, int x, int y, int sampleIndex, int sampleDimension, float* out4) {
    const float4 r = blueNoiseSampler4(bn, x, y, sampleIndex, sampleDimension);
    out4[0] = r.x, out4[1] = r.y, out4[2] = r.z, out4[3] = r.w;
}
}

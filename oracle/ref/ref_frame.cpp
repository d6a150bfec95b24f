/* ref_frame.cpp - the reference's own path-tracer kernels compiled for the host (TEST INFRASTRUCTURE ONLY).
 *
 * Compiled by oracle/ref/Makefile straight from the reference tree (include paths point into it; nothing is
 * copied). Exposes the kernels as extern "C" entry points that run one "launch" over all job indices
 * serially, so a test can drive the reference's wave loop (lib/RenderCore_PrimeRef/rendercore.cpp:551-611)
 * with the oracle standing in for the closed OptiX Prime ray queries. */
#include "ref_shim.h"
#include "helper_math.h"
#include "common_settings.h"
#include "common_types.h"
#include "common_classes.h"
#include "common_functions.h"

namespace refcore {
/* kernel globals, lib/RenderCore_PrimeRef/kernels/.cuda.cu:22-43 (triLights is the name lights_shared.h reads) */
static CoreInstanceDesc* instanceDescriptors;
struct CUDAMaterial4 { uint4 baseData4, parameters, t0data4, t1data4, n0data4, n1data4, sdata4, rdata4; };
static CUDAMaterial4* materials;
static CoreLightTri* triLights;
static CorePointLight* pointLights;
static CoreSpotLight* spotLights;
static CoreDirectionalLight* directionalLights;
static int4 lightCounts;
static uchar4* argb32;
static float4* argb128;
static uchar4* nrm32;
static float4* skyPixels;
static int skywidth, skyheight;
static mat4 worldToSky;
/* device layout of LightCluster (common_classes.h:522-527); only referenced by the unused light-tree code */
struct DevLightCluster { int light; int left, right; float intensity; float4 bmin, bmax; float4 N; };
static DevLightCluster* lightTree;
static const bool adjoint = false; /* lambert.h reads the CUDA-only 'adjoint' parameter */
static float geometryEpsilon = 1e-3f;
static float clampValue = 10.0f;
/* lib/RenderCore_PrimeRef/core_settings.h:74-84, 101-135, 151-153 (device-visible parts) */
struct Counters { uint activePaths, extensionRays, shadowRays, totalExtensionRays, totalShadowRays; int probedInstid, probedTriid; float probedDist; };
static Counters counterStore;
static Counters* counters = &counterStore;
struct Ray4 { float4 O4, D4; };
struct Intersection { float t; int triid, instid; float u, v; };
#define NOHIT -1
#define ISDIELECTRIC (1 << 0)
#define DIFFUSEMAPISHDR (1 << 1)
#define HASDIFFUSEMAP (1 << 2)
#define HASNORMALMAP (1 << 3)
#define HASSPECULARITYMAP (1 << 4)
#define HASROUGHNESSMAP (1 << 5)
#define ISANISOTROPIC (1 << 6)
#define HAS2NDNORMALMAP (1 << 7)
#define HAS2NDDIFFUSEMAP (1 << 9)
#define HASSMOOTHNORMALS (1 << 11)
#define HASALPHA (1 << 12)
#define MAT_ISDIELECTRIC (flags & ISDIELECTRIC)
#define MAT_DIFFUSEMAPISHDR (flags & DIFFUSEMAPISHDR)
#define MAT_HASDIFFUSEMAP (flags & HASDIFFUSEMAP)
#define MAT_HASNORMALMAP (flags & HASNORMALMAP)
#define MAT_HASSPECULARITYMAP (flags & HASSPECULARITYMAP)
#define MAT_HASROUGHNESSMAP (flags & HASROUGHNESSMAP)
#define MAT_HAS2NDNORMALMAP (flags & HAS2NDNORMALMAP)
#define MAT_HAS2NDDIFFUSEMAP (flags & HAS2NDDIFFUSEMAP)
#define MAT_HASSMOOTHNORMALS (flags & HASSMOOTHNORMALS)
#define MAT_HASALPHA (flags & HASALPHA)
#define CONSISTENTNORMALS
#define BILINEAR
#ifndef REF_MAXPATHLENGTH
#define REF_MAXPATHLENGTH 3
#endif
static int MAXPATHLENGTH_RT = REF_MAXPATHLENGTH;
#define MAXPATHLENGTH MAXPATHLENGTH_RT

#include "tools_shared.h"
#include "sampling_shared.h"
#include "material_shared.h"
#include "lights_shared.h"
#include "lambert.h"
/* PrimeRef's shadeKernel calls the BSDF sampler without the r5 argument of the shared Lambert BSDF */
static inline float3 SampleBSDF(const ShadingData shadingData, float3 iN, const float3 N, const float3 T, const float3 wo,
                                const float distance, const float r3, const float r4, float3& wi, float& pdf, bool& specular) {
    return SampleBSDF(shadingData, iN, N, T, wo, distance, r3, r4, 0.0f, wi, pdf, specular);
}
#include "pathtracer.h"
#include "camera.h"
#include "connections.h"
}  // namespace refcore

ref_dim3 threadIdx, blockIdx, blockDim;
using namespace refcore;

static void run_grid(long long n, void (*body)(void*), void* ctx) {
    blockDim.x = 1, blockDim.y = blockDim.z = 1;
    threadIdx.x = threadIdx.y = threadIdx.z = 0;
    blockIdx.y = blockIdx.z = 0;
    for (long long i = 0; i < n; i++) { blockIdx.x = (uint)i; body(ctx); }
}

extern "C" {

/* scene: all pointers stay owned by the caller */
void ref_set_scene(void* instDescs, void* mats, void* tri, int ntri, void* pt, int npt, void* spot, int nspot, void* dir, int ndir,
                   uint32_t* texels, float geoEps, int maxPathLength, float* sky4, int skyW, int skyH) {
    instanceDescriptors = (CoreInstanceDesc*)instDescs;
    materials = (CUDAMaterial4*)mats;
    triLights = (CoreLightTri*)tri, pointLights = (CorePointLight*)pt, spotLights = (CoreSpotLight*)spot, directionalLights = (CoreDirectionalLight*)dir;
    lightCounts = make_int4(ntri, npt, nspot, ndir);
    argb32 = (uchar4*)texels;
    skywidth = skyW, skyheight = skyH, skyPixels = (float4*)sky4;
    geometryEpsilon = geoEps;
    MAXPATHLENGTH_RT = maxPathLength;
}

void ref_init_counters(int pathCount) {
    counters->activePaths = pathCount, counters->extensionRays = 0, counters->shadowRays = 0;
    counters->totalExtensionRays = pathCount, counters->totalShadowRays = 0;
}
void ref_next_counters(uint32_t* out3) {
    out3[0] = counters->extensionRays, out3[1] = counters->shadowRays, out3[2] = 0;
    counters->totalExtensionRays += counters->extensionRays;
    counters->totalShadowRays += counters->shadowRays;
    counters->activePaths = counters->extensionRays;
    counters->extensionRays = 0, counters->shadowRays = 0;
}

struct GenArgs { Ray4* rays; float4* ps; uint R0; int pass; float3 pos, right, up; float aperture; float3 p1; int4 sp; int n; };
static void gen_body(void* c) {
    GenArgs* a = (GenArgs*)c;
    generateEyeRaysKernel(a->rays, a->ps, a->R0, a->pass, a->pos, a->right, a->up, a->aperture, a->p1, a->sp, a->n);
}
void ref_generate(void* rays, void* pathStates, uint32_t R0, int pass, const float* pos, const float* right, const float* up,
                  float aperture, const float* p1, int w, int h, int spp) {
    GenArgs a;
    a.rays = (Ray4*)rays, a.ps = (float4*)pathStates, a.R0 = R0, a.pass = pass;
    a.pos = make_float3(pos[0], pos[1], pos[2]), a.right = make_float3(right[0], right[1], right[2]);
    a.up = make_float3(up[0], up[1], up[2]), a.aperture = aperture, a.p1 = make_float3(p1[0], p1[1], p1[2]);
    a.sp = make_int4(w + (h << 16), spp, 0, 0);
    a.n = w * h * spp;
    run_grid(a.n, gen_body, &a);
}

struct ShadeArgs {
    float4* acc; uint stride; Ray4* rays; float4* ps; Intersection* hits; Ray4* raysOut; float4* psOut; Ray4* conn; float4* pot;
    uint R0; int pass, probe, pathLength, w, h; float spread; float3 p1, p2, p3, pos; int n;
};
static void shade_body(void* c) {
    ShadeArgs* a = (ShadeArgs*)c;
    shadeKernel(a->acc, a->stride, a->rays, a->ps, a->hits, a->raysOut, a->psOut, a->conn, a->pot, a->R0, a->pass, a->probe,
                a->pathLength, a->w, a->h, a->spread, a->p1, a->p2, a->p3, a->pos, a->n);
}
void ref_shade(int pathCount, float* accumulator, void* rays, void* pathStates, void* hits, void* raysOut, void* pathStatesOut,
               void* connections, void* potentials, uint32_t R0, int pass, int pathLength, int w, int h, float spreadAngle, int nee) {
    ShadeArgs a;
    a.acc = (float4*)accumulator, a.stride = (uint)(w * h), a.rays = (Ray4*)rays, a.ps = (float4*)pathStates, a.hits = (Intersection*)hits;
    a.raysOut = (Ray4*)raysOut, a.psOut = (float4*)pathStatesOut, a.conn = nee ? (Ray4*)connections : 0, a.pot = (float4*)potentials;
    a.R0 = R0, a.pass = pass, a.probe = -1, a.pathLength = pathLength, a.w = w, a.h = h, a.spread = spreadAngle;
    a.p1 = a.p2 = a.p3 = a.pos = make_float3(0, 0, 0);
    a.n = pathCount;
    run_grid(pathCount, shade_body, &a);
}

struct ConnArgs { float4* acc; uint* hb; float4* pot; int n; };
static void conn_body(void* c) { ConnArgs* a = (ConnArgs*)c; finalizeConnectionKernel(a->acc, a->hb, a->pot, a->n); }
void ref_finalize_connections(int rayCount, float* accumulator, uint32_t* hitBits, void* potentials) {
    ConnArgs a;
    a.acc = (float4*)accumulator, a.hb = hitBits, a.pot = (float4*)potentials, a.n = rayCount;
    run_grid(rayCount, conn_body, &a);
}

/* pure functions */
uint32_t ref_wanghash(uint32_t s) { return WangHash(s); }
float ref_random_float(uint32_t* s) { return RandomFloat(*s); }
void ref_random_barycentrics(float r0, float* o) { float3 b = RandomBarycentrics(r0); o[0] = b.x, o[1] = b.y, o[2] = b.z; }
uint32_t ref_pack_normal(const float* n) { return PackNormal(make_float3(n[0], n[1], n[2])); }
void ref_unpack_normal(uint32_t p, float* o) { float3 n = UnpackNormal(p); o[0] = n.x, o[1] = n.y, o[2] = n.z; }
void ref_diffuse_cos(float r0, float r1, float* o) { float3 v = DiffuseReflectionCosWeighted(r0, r1); o[0] = v.x, o[1] = v.y, o[2] = v.z; }
void ref_tangent2world(const float* v, const float* n, float* o) {
    float3 r = Tangent2World(make_float3(v[0], v[1], v[2]), make_float3(n[0], n[1], n[2])); o[0] = r.x, o[1] = r.y, o[2] = r.z;
}
void ref_consistent_normal(const float* d, const float* in, float alpha, float* o) {
    float3 r = ConsistentNormal(make_float3(d[0], d[1], d[2]), make_float3(in[0], in[1], in[2]), alpha); o[0] = r.x, o[1] = r.y, o[2] = r.z;
}
void ref_invert4x4(const float* m, float* o) { mat4 a; memcpy(a.cell, m, 64); mat4 r = a.Inverted(); memcpy(o, r.cell, 64); }
}

extern "C" void ref_debug_shading(int inst, int prim, float u, float v, const float* d3, float* out) {
    ShadingData sd;
    float3 N, iN, fN, T;
    const CoreTri4* tris = (const CoreTri4*)instanceDescriptors[inst].triangles;
    GetShadingData(make_float3(d3[0], d3[1], d3[2]), u, v, 0.001f, tris[prim], inst, sd, N, iN, fN, T);
    out[0] = sd.color.x, out[1] = sd.color.y, out[2] = sd.color.z;
    out[3] = __uint_as_float(sd.parameters.x);
    out[4] = fN.x, out[5] = fN.y, out[6] = fN.z;
    out[7] = __uint_as_float(tris[prim].v4.w == 0 ? 0 : __float_as_uint(tris[prim].v4.w));
}

/* ref_frame.cpp - the reference's own path-tracer kernels compiled for the host (TEST INFRASTRUCTURE ONLY).
 *
 * Compiled by oracle/ref/Makefile straight from the reference tree (include paths point into it; nothing is
 * copied). Exposes the kernels as extern "C" entry points that run one "launch" over all job indices
 * serially, so a test can drive the reference's wave loop (lib/RenderCore_PrimeRef/rendercore.cpp:551-611)
 * with the oracle standing in for the closed OptiX Prime ray queries. */
#include "ref_shim.h"
#include <vector>
#include "helper_math.h"
#include "common_settings.h"
#include "common_types.h"
#include "common_classes.h"
#include "common_functions.h"

namespace refcore {
#include "ref_globals.h"
#include "lambert.h"
/* PrimeRef's shadeKernel calls the BSDF sampler without the r5 argument of the shared Lambert BSDF */
static inline float3 SampleBSDF(const ShadingData shadingData, float3 iN, const float3 N, const float3 T, const float3 wo,
                                const float distance, const float r3, const float r4, float3& wi, float& pdf, bool& specular) {
    return SampleBSDF(shadingData, iN, N, T, wo, distance, r3, r4, 0.0f, wi, pdf, specular);
}
#include "pathtracer.h"
#include "camera.h"
#include "connections.h"

/* SVGF kernels (finalize_shared.h): the globals they write, the render-target surface as a float4 array, and
 * powf(x, 128) routed like the oracle's (seven squarings), as the other CUDA math calls are routed by ref_shim.h */
static float4* debugData;
static float4* refTarget;
static int refTargetW;
struct RefSurface {};
static RefSurface renderTarget;
template <typename T>
static inline void surf2Dwrite(T v, RefSurface, int xBytes, int y, cudaSurfaceBoundaryMode) { refTarget[xBytes / (int)sizeof(T) + y * refTargetW] = v; }
static inline float ref_powf(float x, float y) {
    if (y == 128.0f) { for (int i = 0; i < 7; i++) x = x * x; return x; }
    return std::pow(x, y);
}
#define powf(x, y) ref_powf(x, y)
#include "finalize_shared.h"
#undef powf
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

/* SVGF kernels over a W x H grid, one call per pixel in row-major order */
static void run_grid2(int w, int h, void (*body)(void*), void* ctx) {
    blockDim.x = blockDim.y = blockDim.z = 1;
    threadIdx.x = threadIdx.y = threadIdx.z = 0;
    blockIdx.z = 0;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) { blockIdx.x = (uint)x, blockIdx.y = (uint)y; body(ctx); }
}
struct PrepArgs {
    const float4* acc; uint4* feat; const float4 *wp, *pwp; float4* shading; float2* motion; float4 *mom, *pmom; const float4* dd;
    float4 pos, E, right, up; float j0, j1, pj0, pj1; int w, h; float scale, cd, ci; int stationary;
};
static void prep_body(void* c) {
    PrepArgs* a = (PrepArgs*)c;
    prepareFilterKernel(a->acc, a->feat, a->wp, a->pwp, a->shading, a->motion, a->mom, a->pmom, a->dd, a->pos, a->E, a->right, a->up, a->j0,
                        a->j1, a->pj0, a->pj1, a->w, a->h, a->scale, a->cd, a->ci, a->stationary);
}
void ref_svgf_prepare(const float* accum, uint32_t* features, const float* worldPos, const float* prevWorldPos, float* shading, float* motion,
                      float* moments, float* prevMoments, const float* deltaDepth, const float* view16, float j0, float j1, float prevj0,
                      float prevj1, int w, int h, float scale, float clampDirect, float clampIndirect, int camIsStationary) {
    static std::vector<float4> dbg;
    dbg.resize((size_t)w * h);
    debugData = dbg.data();
    PrepArgs a;
    a.acc = (const float4*)accum, a.feat = (uint4*)features, a.wp = (const float4*)worldPos, a.pwp = (const float4*)prevWorldPos;
    a.shading = (float4*)shading, a.motion = (float2*)motion, a.mom = (float4*)moments, a.pmom = (float4*)prevMoments;
    a.dd = (const float4*)deltaDepth;
    const float4* v = (const float4*)view16;
    a.pos = v[0], a.E = v[1], a.right = v[2], a.up = v[3];
    a.j0 = j0, a.j1 = j1, a.pj0 = prevj0, a.pj1 = prevj1, a.w = w, a.h = h, a.scale = scale, a.cd = clampDirect, a.ci = clampIndirect;
    a.stationary = camIsStationary;
    run_grid2(w, h, prep_body, &a);
}
struct ApplyArgs {
    const uint4* feat; const float4 *pwp, *wp, *dd; const float2* motion; const float4* mom; const float4 *A, *B; float4* C;
    uint w, h; int phase; uint last;
};
static void apply_body(void* c) {
    ApplyArgs* a = (ApplyArgs*)c;
    applyFilterKernel(a->feat, a->pwp, a->wp, a->dd, a->motion, a->mom, a->A, a->B, a->C, a->w, a->h, a->phase, a->last);
}
void ref_svgf_apply(const uint32_t* features, const float* prevWorldPos, const float* worldPos, const float* deltaDepth, const float* motion,
                    const float* moments, const float* A, const float* B, float* C, int w, int h, int phase, int lastPass) {
    ApplyArgs a;
    a.feat = (const uint4*)features, a.pwp = (const float4*)prevWorldPos, a.wp = (const float4*)worldPos, a.dd = (const float4*)deltaDepth;
    a.motion = (const float2*)motion, a.mom = (const float4*)moments, a.A = (const float4*)A, a.B = (const float4*)B, a.C = (float4*)C;
    a.w = (uint)w, a.h = (uint)h, a.phase = phase, a.last = (uint)lastPass;
    run_grid2(w, h, apply_body, &a);
}
/* TAApassKernel updates its input in place while neighbouring threads read it; here every pixel sees the input
 * unchanged (each result goes to out and the input is restored before the next pixel) */
struct TaaArgs { float4 *px, *prev; const float2* motion; uint w, h; const float4* in; float4* out; };
static void taa_body(void* c) {
    TaaArgs* a = (TaaArgs*)c;
    TAApassKernel(a->px, a->prev, 0, 0, nullptr, nullptr, a->motion, a->w, a->h);
    const size_t i = (size_t)blockIdx.x + (size_t)blockIdx.y * a->w;
    a->out[i] = a->px[i];
    a->px[i] = a->in[i];
}
void ref_svgf_taa(const float* pixels, float* prevPixels, const float* motion, float* out, int w, int h) {
    std::vector<float4> work((const float4*)pixels, (const float4*)pixels + (size_t)w * h);
    TaaArgs a;
    a.px = work.data(), a.prev = (float4*)prevPixels, a.motion = (const float2*)motion, a.w = (uint)w, a.h = (uint)h;
    a.in = (const float4*)pixels, a.out = (float4*)out;
    run_grid2(w, h, taa_body, &a);
}
struct FinArgs { const float4* px; uint w, h; int mode; };
static void fin_body(void* c) {
    FinArgs* a = (FinArgs*)c;
    if (a->mode) unsharpenTAAKernel(a->px, a->w, a->h);
    else finalizeNoTAAKernel((float4*)a->px, a->w, a->h);
}
void ref_svgf_finalize(const float* pixels, float* target, int w, int h, int taa) {
    refTarget = (float4*)target, refTargetW = w;
    FinArgs a;
    a.px = (const float4*)pixels, a.w = (uint)w, a.h = (uint)h, a.mode = taa;
    run_grid2(w, h, fin_body, &a);
}
/* tools_shared.h / sampling_shared.h packing helpers */
uint32_t ref_pack_normal2(const float* n) { return PackNormal2(make_float3(n[0], n[1], n[2])); }
void ref_unpack_normal2(uint32_t p, float* o) { float3 n = UnpackNormal2(p); o[0] = n.x, o[1] = n.y, o[2] = n.z; }
uint32_t ref_hdr_to_rgb32(const float* c) { return HDRtoRGB32(make_float3(c[0], c[1], c[2])); }
void ref_rgb32_to_hdr(uint32_t c, int min1, float* o) { float3 v = min1 ? RGB32toHDRmin1(c) : RGB32toHDR(c); o[0] = v.x, o[1] = v.y, o[2] = v.z; }
void ref_combine_to_float4(const float* a, const float* b, float* o) {
    float4 r = CombineToFloat4(make_float3(a[0], a[1], a[2]), make_float3(b[0], b[1], b[2])); o[0] = r.x, o[1] = r.y, o[2] = r.z, o[3] = r.w;
}
void ref_split_float4(const float* x, float* d, float* i) {
    float4 v = make_float4(x[0], x[1], x[2], x[3]);
    float3 a = GetDirectFromFloat4(v), b = GetIndirectFromFloat4(v);
    d[0] = a.x, d[1] = a.y, d[2] = a.z, i[0] = b.x, i[1] = b.y, i[2] = b.z;
}
void ref_rgb_to_ycocg(const float* c, float* o) { float3 v = RGBToYCoCg(make_float3(c[0], c[1], c[2])); o[0] = v.x, o[1] = v.y, o[2] = v.z; }
void ref_ycocg_to_rgb(const float* c, float* o) { float3 v = YCoCgToRGB(make_float3(c[0], c[1], c[2])); o[0] = v.x, o[1] = v.y, o[2] = v.z; }
float ref_luminance(const float* c) { return Luminance(make_float3(c[0], c[1], c[2])); }
float ref_mitchell_netravali(float v) { return mitchellNetravali(v); }

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

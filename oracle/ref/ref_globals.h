/* ref_globals.h - the device globals and defines the reference's kernels read, for compiling them on the host
 * (TEST INFRASTRUCTURE ONLY). Included inside one namespace per harness translation unit (ref_frame.cpp,
 * ref_optix7.cpp, ref_adaptive.cpp), so that each core's kernels, which share names, get their own copies; then
 * the shared device code of lib/CUDA/shared_kernel_code is included by the including file. */
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
/* the counters of lib/RenderCore_PrimeRef/core_settings.h:74-84 (PrimeAdaptive's are the same) with the extra
 * fields of lib/rendercore_optix7/core_settings.h:96-110; kernels read them by name */
struct Counters { uint activePaths, shaded, generated, connected, extended, extensionRays, shadowRays, totalExtensionRays, totalShadowRays;
                  int probedInstid, probedTriid; float probedDist; };
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

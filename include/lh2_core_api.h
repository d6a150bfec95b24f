/* lh2_core_api.h - the Lighthouse 2 RenderCore plugin interface, as implemented by libRenderCore_GB300.so.
 *
 * A RenderSystem loads the core exactly as lib/RenderSystem/core_api_base.cpp:97-130 does:
 *   dlopen("libRenderCore_GB300.so", RTLD_NOW | RTLD_GLOBAL); dlsym("CreateCore"); api->Init();
 * and then calls it through the CoreAPI_Base vtable below, whose member order, signatures and argument
 * layouts are those of lib/RenderSystem/core_api_base.h:81-119 (Itanium C++ ABI, g++). The data types are
 * declared here with the byte layouts of lib/RenderSystem/common_classes.h (CUDA vector types: float2/int2/
 * uint2 8-byte aligned, float4 16-byte aligned), so arrays built by the RenderSystem pass through unchanged.
 *
 * Headless target: SetTarget reads only width and height from the GLTexture; the rendered image is a device
 * float4 buffer (lh2g_get_framebuffer on the context returned by GB300_GetContext).
 */
#ifndef LH2_CORE_API_H
#define LH2_CORE_API_H

#include <cstdint>
#include <vector_types.h>

#include "lh2g.h"

namespace lighthouse2 {

typedef unsigned int uint;

enum Convergence { Converge = 0, Restart = 1 };

/* common_classes.h:452-475 */
struct ViewPyramid {
    float3 pos, p1, p2, p3;
    float aperture, spreadAngle, imagePlane, focalDistance, distortion;
};

/* common_types.h:460-464: 16 floats, row-major */
class mat4 {
public:
    float cell[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    static mat4 Identity() { return mat4(); }
};

/* lib/platform/system.h:220-237 (only the data members matter to a core) */
class GLTexture {
public:
    uint ID = 0;
    uint width = 0, height = 0;
};

/* common_classes.h:57-97 */
typedef lh2g_core_tri CoreTri;

/* common_classes.h:336-359 (host layout) */
enum TexelStorage { ARGB32 = 0, ARGB128, NRM32 };
struct CoreTexDesc {
    union { float4* fdata; uchar4* idata; };
    uint width = 0, height = 0, flags = 0, pixelCount = 0, firstPixel = 0, MIPlevels = 1;
    TexelStorage storage = ARGB32;
};

/* common_classes.h:219-328 */
enum class MaterialType : char { DISNEY = 0 };
class CoreMaterial {
public:
    struct Vec3Value { float3 value; int textureID; float scale; float2 uvscale, uvoffset; uint2 size; };
    struct ScalarValue { float value; int textureID; int component; float scale; float2 uvscale, uvoffset; uint2 size; };
    Vec3Value color, detailColor, normals, detailNormals;
    uint flags;
    Vec3Value absorption;
    ScalarValue metallic, subsurface, specular, roughness, specularTint, anisotropic, sheen, sheenTint, clearcoat, clearcoatGloss,
        transmission, eta;
    ScalarValue reflection, refraction, ior;
    MaterialType pbrtMaterialType : 8;
    ScalarValue urough, vrough;
    Vec3Value Ks;
    Vec3Value eta_rgb;
    ScalarValue sigma;
    bool thin;
    ScalarValue specTrans, diffTrans;
    Vec3Value scatterDistance;
    ScalarValue flatness;
    Vec3Value Kr;
    Vec3Value opacity;
};

/* common_classes.h:365-446 */
typedef lh2g_light_tri CoreLightTri;
typedef lh2g_point_light CorePointLight;
typedef lh2g_spot_light CoreSpotLight;
typedef lh2g_dir_light CoreDirectionalLight;

/* core_api_base.h:30-64 */
struct CoreStats {
    char* deviceName = 0;
    uint SMcount = 0;
    uint ccMajor = 0, ccMinor = 0;
    uint VRAM = 0;
    uint argb32TexelCount = 0, argb128TexelCount = 0, nrm32TexelCount = 0;
    float bvhBuildTime = 0;
    uint totalRays = 0, totalExtensionRays = 0, totalShadowRays = 0;
    float renderTime = 0, frameOverhead = 0;
    uint primaryRayCount = 0;
    float traceTime0 = 0;
    uint bounce1RayCount = 0;
    float traceTime1 = 0;
    uint deepRayCount = 0;
    float traceTimeX = 0, shadowTraceTime = 0, shadeTime = 0, filterTime = 0;
    int probedInstid = 0, probedTriid = -1;
    float probedDist = 0;
    float3 probedWorldPos;
};

/* core_api_base.h:81-119 */
class CoreAPI_Base {
public:
    virtual CoreStats GetCoreStats() const = 0;
    virtual void Init() = 0;
    virtual void SetProbePos(const int2 pos) = 0;
    virtual void SetTarget(GLTexture* target, const uint spp) = 0;
    virtual void Setting(const char* name, float value) = 0;
    virtual void Render(const ViewPyramid& view, const Convergence converge, bool async) = 0;
    virtual void WaitForRender() = 0;
    virtual void Shutdown() = 0;
    virtual void SetTextures(const CoreTexDesc* tex, const int textureCount) = 0;
    virtual void SetMaterials(CoreMaterial* mat, const int materialCount) = 0;
    virtual void SetLights(const CoreLightTri* triLights, const int triLightCount, const CorePointLight* pointLights, const int pointLightCount,
                           const CoreSpotLight* spotLights, const int spotLightCount, const CoreDirectionalLight* directionalLights,
                           const int directionalLightCount) = 0;
    virtual void SetSkyData(const float3* pixels, const uint width, const uint height, const mat4& worldToLight = mat4()) = 0;
    virtual void SetGeometry(const int meshIdx, const float4* vertexData, const int vertexCount, const int triangleCount, const CoreTri* triangles) = 0;
    virtual void SetInstance(const int instanceIdx, const int modelIdx, const mat4& transform = mat4::Identity()) = 0;
    virtual void FinalizeInstances() = 0;
};

}  // namespace lighthouse2

extern "C" {
/* core_api.cpp:18-22 of the reference cores: the plugin factory. */
LH2G_API lighthouse2::CoreAPI_Base* CreateCore();
/* The C-ABI context behind a core created by CreateCore (errors: lh2g_last_error on it). */
LH2G_API lh2g_context* GB300_GetContext(lighthouse2::CoreAPI_Base* core);
}

#endif

/* rendercore.cu - the Lighthouse 2 plugin face of the GB300 core: CoreAPI_Base on top of the C ABI.
 *
 * Mirrors the reference core's host class (lib/RenderCore_PrimeRef/rendercore.cpp, lib/rendercore_optix7/
 * rendercore.cpp): same setter semantics, CoreMaterial converted to the core's material description, errors
 * kept in the context (lh2g_last_error) instead of aborting the process. Async Render runs on the context's
 * CUDA stream; WaitForRender waits for it (replacing the Win32 render thread of rendercore.cpp:803-847).
 */
#include <cstring>
#include <vector>

#include "lh2_core_api.h"

using namespace lighthouse2;

namespace {

lh2g_map_ref map_of(int tex, float2 s, float2 o) {
    lh2g_map_ref m;
    m.texture = tex, m.uvscale[0] = s.x, m.uvscale[1] = s.y, m.uvoffset[0] = o.x, m.uvoffset[1] = o.y;
    return m;
}

class RenderCoreGB300 : public CoreAPI_Base {
public:
    lh2g_context* ctx = nullptr;
    CoreStats stats;
    std::vector<lh2g_texture> tex;

    CoreStats GetCoreStats() const override {
        CoreStats s = stats;
        lh2g_stats g;
        if (ctx && lh2g_get_stats(ctx, &g) == LH2G_OK) {
            s.SMcount = g.SMcount, s.ccMajor = g.ccMajor, s.ccMinor = g.ccMinor, s.VRAM = g.VRAM;
            s.bvhBuildTime = g.bvhBuildTime;
            s.totalRays = g.totalRays, s.totalExtensionRays = g.totalExtensionRays, s.totalShadowRays = g.totalShadowRays;
            s.renderTime = g.renderTime, s.primaryRayCount = g.primaryRayCount, s.bounce1RayCount = g.bounce1RayCount, s.deepRayCount = g.deepRayCount;
            s.probedInstid = g.probedInstid, s.probedTriid = g.probedTriid, s.probedDist = g.probedDist;
        }
        return s;
    }
    void Init() override { if (!ctx) lh2g_create(0, &ctx); }
    void SetProbePos(const int2 pos) override { lh2g_set_probe(ctx, pos.x, pos.y); }
    void SetTarget(GLTexture* target, const uint spp) override { if (target) lh2g_set_target(ctx, (int)target->width, (int)target->height, (int)spp); }
    /* "rasterizer" 1: Render draws the SoftRasterizer core's frame (RenderCore_SoftRasterizer/rendercore.cpp:213-227)
     * instead of path tracing; read it with lh2g_raster_read / lh2g_raster_pixels_device */
    bool raster = false;
    void Setting(const char* name, float value) override {
        if (!strcmp(name, "rasterizer")) raster = value != 0.0f;
        else lh2g_setting(ctx, name, value);
    }
    void Render(const ViewPyramid& view, const Convergence converge, bool async) override {
        lh2g_view v;
        memcpy(&v, &view, sizeof(v));
        if (raster) lh2g_raster_render(ctx, &v, nullptr, nullptr, nullptr);
        else lh2g_render(ctx, &v, converge == Restart ? 1 : 0);
        if (!async) lh2g_wait(ctx);
    }
    void WaitForRender() override { lh2g_wait(ctx); }
    void Shutdown() override { if (ctx) lh2g_destroy(ctx); ctx = nullptr; }
    void SetTextures(const CoreTexDesc* t, const int n) override {
        tex.resize(n);
        for (int i = 0; i < n; i++) {
            tex[i].texels = (const uint32_t*)t[i].idata;
            tex[i].width = t[i].width, tex[i].height = t[i].height, tex[i].flags = t[i].flags;
            tex[i].pixelCount = t[i].pixelCount, tex[i].firstPixel = 0, tex[i].MIPlevels = t[i].MIPlevels, tex[i].storage = (int32_t)t[i].storage;
        }
        lh2g_set_textures(ctx, tex.data(), n);
    }
    void SetMaterials(CoreMaterial* mat, const int n) override {
        std::vector<lh2g_material> m(n);
        for (int i = 0; i < n; i++) {
            const CoreMaterial& c = mat[i];
            lh2g_material& g = m[i];
            memset(&g, 0, sizeof(g));
            g.color[0] = c.color.value.x, g.color[1] = c.color.value.y, g.color[2] = c.color.value.z;
            g.absorption[0] = c.absorption.value.x, g.absorption[1] = c.absorption.value.y, g.absorption[2] = c.absorption.value.z;
            g.metallic = c.metallic.value, g.subsurface = c.subsurface.value, g.specular = c.specular.value, g.roughness = c.roughness.value;
            g.specularTint = c.specularTint.value, g.anisotropic = c.anisotropic.value, g.sheen = c.sheen.value, g.sheenTint = c.sheenTint.value;
            g.clearcoat = c.clearcoat.value, g.clearcoatGloss = c.clearcoatGloss.value, g.transmission = c.transmission.value, g.eta = c.eta.value;
            g.flags = c.flags;
            g.color_map = map_of(c.color.textureID, c.color.uvscale, c.color.uvoffset);
            g.detail_color_map = map_of(c.detailColor.textureID, c.detailColor.uvscale, c.detailColor.uvoffset);
            g.normal_map = map_of(c.normals.textureID, c.normals.uvscale, c.normals.uvoffset);
            g.detail_normal_map = map_of(c.detailNormals.textureID, c.detailNormals.uvscale, c.detailNormals.uvoffset);
            g.specular_map = map_of(c.specular.textureID, c.specular.uvscale, c.specular.uvoffset);
            g.roughness_map = map_of(c.roughness.textureID, c.roughness.uvscale, c.roughness.uvoffset);
        }
        lh2g_set_materials(ctx, m.data(), n);
    }
    void SetLights(const CoreLightTri* a, const int na, const CorePointLight* p, const int np, const CoreSpotLight* s, const int ns,
                   const CoreDirectionalLight* d, const int nd) override {
        lh2g_set_lights(ctx, a, na, p, np, s, ns, d, nd);
    }
    void SetSkyData(const float3* pixels, const uint w, const uint h, const mat4& worldToLight) override {
        lh2g_set_sky(ctx, (const float*)pixels, (int)w, (int)h, worldToLight.cell);
    }
    void SetGeometry(const int meshIdx, const float4* v, const int vc, const int tc, const CoreTri* t) override {
        lh2g_set_geometry(ctx, meshIdx, (const float*)v, vc, tc, t);
    }
    void SetInstance(const int idx, const int mesh, const mat4& T) override { lh2g_set_instance(ctx, idx, mesh, T.cell); }
    void FinalizeInstances() override { lh2g_finalize_instances(ctx); }
};

}  // namespace

extern "C" {
LH2G_API CoreAPI_Base* CreateCore() { return new RenderCoreGB300(); }
LH2G_API lh2g_context* GB300_GetContext(CoreAPI_Base* core) { return core ? static_cast<RenderCoreGB300*>(core)->ctx : nullptr; }
}

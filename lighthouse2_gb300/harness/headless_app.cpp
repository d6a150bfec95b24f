/* headless_app.cpp - a headless Lighthouse 2 application: loads a render core by name through the plugin
 * interface and drives it the way the reference's RenderSystem and apps do, with no window and no GL.
 *
 *   loading       lib/RenderSystem/core_api_base.cpp:97-127: dlopen("lib" + name + ".so", RTLD_NOW | RTLD_GLOBAL),
 *                 else dlopen(name); dlsym("CreateCore"); Init()
 *   scene sync    RenderSystem::SynchronizeSceneData, lib/RenderSystem/rendersystem.cpp:50-211: textures, then
 *                 materials (CoreMaterial, host_material.h field by field), then geometry per mesh in index order,
 *                 lights, sky, then every instance and SetInstance(count, -1) to truncate, FinalizeInstances
 *   frame loop    apps/tinyapp/main.cpp:61-100: per frame apply the scene change (an instance moved:
 *                 SetInstance + FinalizeInstances, as the RenderSystem does for dirty instances), Render(view,
 *                 Restart | Converge, async = true), WaitForRender, GetCoreStats
 *   output        the headless target: the core's frame read through its C ABI (GB300_GetContext +
 *                 lh2g_read_framebuffer, found with dlsym) and appended to a file; one line of statistics per
 *                 frame on stdout. With the setting rasterizer=1 the core draws the SoftRasterizer core's frame
 *                 and the file gets its RGBA8 words (lh2g_raster_read)
 *
 * usage: headless_app <core name or library path> <scene file> <frames file> <output file> <width> <height> <spp>
 *                     [setting=value ...]
 * File formats: lighthouse2_gb300/scenefile.py.
 */
#include <dlfcn.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "lh2_core_api.h"

using namespace lighthouse2;

namespace {

struct Reader {
    FILE* f = nullptr;
    bool ok = true;
    template <typename T>
    void read(T* dst, size_t n) {
        if (n && fread(dst, sizeof(T), n, f) != n) ok = false;
    }
    template <typename T>
    T get() {
        T v{};
        read(&v, 1);
        return v;
    }
};

struct Mesh {
    std::vector<float4> verts;
    std::vector<CoreTri> tris;
};
struct Instance {
    int mesh;
    mat4 T;
};
struct Texture {
    uint width, height;
    std::vector<uint32_t> texels;
};
struct Scene {
    std::vector<Mesh> meshes;
    std::vector<Instance> instances;
    std::vector<lh2g_material> materials;
    std::vector<Texture> textures;
    std::vector<CoreLightTri> triLights;
    std::vector<CorePointLight> pointLights;
    std::vector<CoreSpotLight> spotLights;
    std::vector<CoreDirectionalLight> dirLights;
    uint skyW = 0, skyH = 0;
    std::vector<float3> sky;
};
struct Frame {
    ViewPyramid view;
    int converge;
    int instance, mesh;
    mat4 T;
};

bool load_scene(const char* path, Scene& s) {
    Reader r;
    r.f = fopen(path, "rb");
    if (!r.f) return false;
    char magic[8];
    r.read(magic, 8);
    if (memcmp(magic, "LH2GSCN1", 8) != 0) { fclose(r.f); return false; }
    uint c[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    r.read(c, 10);
    /* a truncated or foreign file must fail here, not allocate from garbage counts */
    const uint limit = 1u << 28;
    bool sane = r.ok && c[8] < (1u << 16) && c[9] < (1u << 16);
    for (int k = 0; k < 8; k++) sane = sane && c[k] < limit;
    if (!sane) { fclose(r.f); return false; }
    s.meshes.resize(c[0]), s.instances.resize(c[1]), s.materials.resize(c[2]), s.textures.resize(c[3]);
    s.triLights.resize(c[4]), s.pointLights.resize(c[5]), s.spotLights.resize(c[6]), s.dirLights.resize(c[7]);
    s.skyW = c[8], s.skyH = c[9];
    for (Mesh& m : s.meshes) {
        const uint n = r.get<uint>();
        if (!r.ok || n >= limit) { fclose(r.f); return false; }
        m.verts.resize(3 * (size_t)n), m.tris.resize(n);
        r.read(m.verts.data(), m.verts.size());
        r.read(m.tris.data(), n);
    }
    for (Instance& in : s.instances) {
        in.mesh = r.get<int>();
        r.read(in.T.cell, 16);
    }
    r.read(s.materials.data(), s.materials.size());
    for (Texture& t : s.textures) {
        t.width = r.get<uint>(), t.height = r.get<uint>();
        const uint n = r.get<uint>();
        if (!r.ok || n >= limit) { fclose(r.f); return false; }
        t.texels.resize(n);
        r.read(t.texels.data(), t.texels.size());
    }
    r.read(s.triLights.data(), s.triLights.size());
    r.read(s.pointLights.data(), s.pointLights.size());
    r.read(s.spotLights.data(), s.spotLights.size());
    r.read(s.dirLights.data(), s.dirLights.size());
    s.sky.resize((size_t)s.skyW * s.skyH);
    r.read(s.sky.data(), s.sky.size());
    fclose(r.f);
    return r.ok;
}

bool load_frames(const char* path, std::vector<Frame>& frames) {
    Reader r;
    r.f = fopen(path, "rb");
    if (!r.f) return false;
    char magic[8];
    r.read(magic, 8);
    if (memcmp(magic, "LH2GFRM1", 8) != 0) { fclose(r.f); return false; }
    const uint n = r.get<uint>();
    if (!r.ok || n >= (1u << 20)) { fclose(r.f); return false; }
    frames.resize(n);
    for (Frame& f : frames) {
        r.read(&f.view, 1);
        f.converge = r.get<int>();
        f.instance = r.get<int>(), f.mesh = r.get<int>();
        r.read(f.T.cell, 16);
    }
    fclose(r.f);
    return r.ok;
}

/* the RenderSystem's material as the reference's host code fills CoreMaterial (unused fields keep the
 * HostMaterial defaults: no texture, scale 1) */
CoreMaterial::Vec3Value vec3(const float* v, const lh2g_map_ref* map) {
    CoreMaterial::Vec3Value x;
    memset(&x, 0, sizeof(x));
    x.value.x = v ? v[0] : 0.0f, x.value.y = v ? v[1] : 0.0f, x.value.z = v ? v[2] : 0.0f;
    x.textureID = map ? map->texture : -1;
    x.scale = 1.0f;
    x.uvscale.x = map ? map->uvscale[0] : 1.0f, x.uvscale.y = map ? map->uvscale[1] : 1.0f;
    x.uvoffset.x = map ? map->uvoffset[0] : 0.0f, x.uvoffset.y = map ? map->uvoffset[1] : 0.0f;
    return x;
}
CoreMaterial::ScalarValue scalar(float v, const lh2g_map_ref* map = nullptr) {
    CoreMaterial::ScalarValue x;
    memset(&x, 0, sizeof(x));
    x.value = v;
    x.textureID = map ? map->texture : -1;
    x.scale = 1.0f;
    x.uvscale.x = map ? map->uvscale[0] : 1.0f, x.uvscale.y = map ? map->uvscale[1] : 1.0f;
    x.uvoffset.x = map ? map->uvoffset[0] : 0.0f, x.uvoffset.y = map ? map->uvoffset[1] : 0.0f;
    return x;
}
CoreMaterial core_material(const lh2g_material& g) {
    CoreMaterial c;
    memset(&c, 0, sizeof(c));
    c.color = vec3(g.color, &g.color_map);
    c.detailColor = vec3(nullptr, &g.detail_color_map);
    c.normals = vec3(nullptr, &g.normal_map);
    c.detailNormals = vec3(nullptr, &g.detail_normal_map);
    c.flags = g.flags;
    c.absorption = vec3(g.absorption, nullptr);
    c.metallic = scalar(g.metallic), c.subsurface = scalar(g.subsurface), c.specular = scalar(g.specular, &g.specular_map);
    c.roughness = scalar(g.roughness, &g.roughness_map), c.specularTint = scalar(g.specularTint), c.anisotropic = scalar(g.anisotropic);
    c.sheen = scalar(g.sheen), c.sheenTint = scalar(g.sheenTint), c.clearcoat = scalar(g.clearcoat), c.clearcoatGloss = scalar(g.clearcoatGloss);
    c.transmission = scalar(g.transmission), c.eta = scalar(g.eta);
    return c;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 8) {
        fprintf(stderr, "usage: %s <core> <scene> <frames> <output> <width> <height> <spp> [setting=value ...]\n", argv[0]);
        return 2;
    }
    Scene scene;
    std::vector<Frame> frames;
    if (!load_scene(argv[2], scene)) { fprintf(stderr, "cannot read scene %s\n", argv[2]); return 2; }
    if (!load_frames(argv[3], frames)) { fprintf(stderr, "cannot read frames %s\n", argv[3]); return 2; }
    const uint W = (uint)atoi(argv[5]), H = (uint)atoi(argv[6]), spp = (uint)atoi(argv[7]);

    /* CoreAPI_Base::CreateCoreAPI (core_api_base.cpp:97-127) */
    const std::string name = argv[1];
    void* lib = dlopen(("lib" + name + ".so").c_str(), RTLD_NOW | RTLD_GLOBAL);
    if (!lib) lib = dlopen(name.c_str(), RTLD_NOW | RTLD_GLOBAL);
    if (!lib) { fprintf(stderr, "cannot load core %s: %s\n", name.c_str(), dlerror()); return 3; }
    typedef CoreAPI_Base* (*createCoreFunction)();
    const createCoreFunction createCore = (createCoreFunction)dlsym(lib, "CreateCore");
    typedef lh2g_context* (*contextFunction)(CoreAPI_Base*);
    const contextFunction getContext = (contextFunction)dlsym(lib, "GB300_GetContext");
    typedef int (*readFunction)(lh2g_context*, float*);
    const readFunction readFrame = (readFunction)dlsym(lib, "lh2g_read_framebuffer");
    typedef int (*rasterReadFunction)(lh2g_context*, uint32_t*);
    const rasterReadFunction readRaster = (rasterReadFunction)dlsym(lib, "lh2g_raster_read");
    if (!createCore || !getContext || !readFrame || !readRaster) { fprintf(stderr, "core %s lacks its entry points\n", name.c_str()); return 3; }
    CoreAPI_Base* core = createCore();
    core->Init();

    /* SynchronizeSceneData (rendersystem.cpp:203-211) */
    std::vector<CoreTexDesc> tex(scene.textures.size());
    for (size_t i = 0; i < tex.size(); i++) {
        Texture& t = scene.textures[i];
        tex[i].idata = reinterpret_cast<uchar4*>(t.texels.data());
        tex[i].width = t.width, tex[i].height = t.height, tex[i].flags = 0;
        tex[i].pixelCount = (uint)t.texels.size(), tex[i].firstPixel = 0, tex[i].MIPlevels = 5, tex[i].storage = ARGB32;
    }
    core->SetTextures(tex.data(), (int)tex.size());
    std::vector<CoreMaterial> mats;
    for (const lh2g_material& g : scene.materials) mats.push_back(core_material(g));
    core->SetMaterials(mats.data(), (int)mats.size());
    for (size_t k = 0; k < scene.meshes.size(); k++) {
        Mesh& m = scene.meshes[k];
        core->SetGeometry((int)k, m.verts.data(), (int)m.verts.size(), (int)m.tris.size(), m.tris.data());
    }
    core->SetLights(scene.triLights.data(), (int)scene.triLights.size(), scene.pointLights.data(), (int)scene.pointLights.size(),
                    scene.spotLights.data(), (int)scene.spotLights.size(), scene.dirLights.data(), (int)scene.dirLights.size());
    if (!scene.sky.empty()) core->SetSkyData(scene.sky.data(), scene.skyW, scene.skyH, mat4());
    for (size_t k = 0; k < scene.instances.size(); k++) core->SetInstance((int)k, scene.instances[k].mesh, scene.instances[k].T);
    core->SetInstance((int)scene.instances.size(), -1);
    core->FinalizeInstances();

    bool raster = false;
    for (int a = 8; a < argc; a++) {
        const char* eq = strchr(argv[a], '=');
        if (!eq) continue;
        const std::string key(argv[a], eq - argv[a]);
        if (key == "rasterizer") raster = atof(eq + 1) != 0.0;
        core->Setting(key.c_str(), (float)atof(eq + 1));
    }
    GLTexture target;
    target.width = W, target.height = H;
    core->SetTarget(&target, spp);

    FILE* out = fopen(argv[4], "wb");
    if (!out) { fprintf(stderr, "cannot write %s\n", argv[4]); return 2; }
    std::vector<float> pixels(4 * (size_t)W * H);
    std::vector<uint32_t> words((size_t)W * H);
    int status = 0;
    for (size_t k = 0; k < frames.size(); k++) {
        const Frame& f = frames[k];
        if (f.instance >= 0) {   /* a moved instance: the RenderSystem re-sends it and finalizes */
            core->SetInstance(f.instance, f.mesh, f.T);
            core->FinalizeInstances();
        }
        core->Render(f.view, f.converge ? Restart : Converge, true);
        core->WaitForRender();
        const CoreStats st = core->GetCoreStats();
        if (raster) {
            if (readRaster(getContext(core), words.data()) != 0) { status = 4; break; }
            fwrite(words.data(), sizeof(uint32_t), words.size(), out);
        } else {
            if (readFrame(getContext(core), pixels.data()) != 0) { status = 4; break; }
            fwrite(pixels.data(), sizeof(float), pixels.size(), out);
        }
        printf("{\"frame\": %zu, \"totalRays\": %u, \"totalExtensionRays\": %u, \"totalShadowRays\": %u, \"primaryRayCount\": %u, "
               "\"renderTime_ms\": %.4f, \"bvhBuildTime_ms\": %.4f, \"SMcount\": %u}\n",
               k, st.totalRays, st.totalExtensionRays, st.totalShadowRays, st.primaryRayCount, st.renderTime, st.bvhBuildTime, st.SMcount);
    }
    fclose(out);
    core->Shutdown();
    return status;
}

/* ref_raster.cpp - the reference's SoftRasterizer core compiled for the host (TEST INFRASTRUCTURE ONLY).
 *
 * Compiled by oracle/ref/Makefile from the reference tree: lib/RenderCore_SoftRasterizer/rasterizer.cpp and
 * rendercore.cpp (each with its include of core_settings.h removed: that header pulls in the OpenGL platform
 * library), the mat4 operators of lib/platform/system.cpp, and rasterizer.h / rendercore.h by path. The OpenGL
 * texture upload that ends RenderCore::Render (rendercore.cpp:224-226) is caught by a stub that copies the
 * pixels out. The entry point drives the core through its own RenderCore methods, as the RenderSystem does. */
#include <cstdio>
#include <cstdlib>
#include <cassert>
#include <vector>
#include "helper_math.h"
#include "common_settings.h"
#include "common_types.h"
#include "common_classes.h"
#include "lh2g_types.h"

#define MALLOC64(x) ((x) == 0 ? 0 : aligned_alloc(64, (x)))
#define FREE64(x) free(x)
using std::vector;

#include "mat4_ops.h"

/* the OpenGL surface of the RenderSystem, reduced to what the core reads, and the upload it ends with */
typedef unsigned int GLuint;
namespace lighthouse2 {
class GLTexture { public: GLuint ID = 0; uint width = 0, height = 0; };
}
#define GL_TEXTURE_2D 0
#define GL_RGBA 0
#define GL_UNSIGNED_BYTE 0
static const uint* g_uploaded = nullptr;
static inline void glBindTexture(int, GLuint) {}
static inline void glTexImage2D(int, int, int, int, int, int, int, int, const void* p) { g_uploaded = (const uint*)p; }

#include "core_api_base.h"
#include "rasterizer.h"
#include "rendercore.h"
using namespace lh2core;
#include "rasterizer_body.h"
#include "rendercore_body.h"

extern "C" {

/* One frame of the reference core over a scene given in the C ABI's host layouts (lh2g_core_tri is CoreTri's
 * host layout). Returns the uploaded pixels and Rasterizer::zbuffer. A fresh core per call. */
int ref_raster(int W, int H, int nMesh, const int* triCount, const float* const* verts, const lh2g_core_tri* const* tris, int nInst,
               const int* instMesh, const float* instT, int nMat, const lh2g_material* mats, int nTex, const lh2g_texture* tex,
               const lh2g_view* v, uint* pixels, float* zbuf) {
    RenderCore* core = new RenderCore();
    core->Init();
    GLTexture target;
    target.width = W, target.height = H;
    core->SetTarget(&target, 1);
    std::vector<CoreTexDesc> td(nTex);
    for (int i = 0; i < nTex; i++) {
        td[i].idata = (uchar4*)tex[i].texels;
        td[i].width = tex[i].width, td[i].height = tex[i].height, td[i].pixelCount = tex[i].pixelCount;
    }
    if (nTex) core->SetTextures(td.data(), nTex);
    std::vector<CoreMaterial> cm(nMat);
    for (int i = 0; i < nMat; i++) {
        memset((void*)&cm[i], 0, sizeof(CoreMaterial));
        cm[i].color.value = make_float3(mats[i].color[0], mats[i].color[1], mats[i].color[2]);
        cm[i].color.textureID = mats[i].color_map.texture;
    }
    core->SetMaterials(cm.data(), nMat);
    for (int m = 0; m < nMesh; m++) core->SetGeometry(m, (const float4*)verts[m], 3 * triCount[m], triCount[m], (const CoreTri*)tris[m]);
    for (int i = 0; i < nInst; i++) {
        mat4 T;
        memcpy(T.cell, instT + 16 * i, 64);
        core->SetInstance(i, instMesh[i], T);
    }
    ViewPyramid view;
    view.pos = make_float3(v->pos[0], v->pos[1], v->pos[2]);
    view.p1 = make_float3(v->p1[0], v->p1[1], v->p1[2]);
    view.p2 = make_float3(v->p2[0], v->p2[1], v->p2[2]);
    view.p3 = make_float3(v->p3[0], v->p3[1], v->p3[2]);
    g_uploaded = nullptr;
    core->Render(view, Restart, false);
    if (!g_uploaded) return 1;
    memcpy(pixels, g_uploaded, sizeof(uint) * (size_t)W * H);
    if (zbuf) memcpy(zbuf, Rasterizer::zbuffer, sizeof(float) * (size_t)W * H);
    /* the core's scene graph and meshes stay allocated (the static scene root owns them): test harness */
    return 0;
}

}  // extern "C"

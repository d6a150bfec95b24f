/* ref_lighttree.cpp - the OptiX 7 core's light-tree build compiled for the host (TEST INFRASTRUCTURE ONLY).
 *
 * Built by oracle/ref/Makefile from the reference tree: RenderCore::UpdateLightTreeNormals, FindBestMatch and
 * UpdateLightTree (lib/rendercore_optix7/rendercore.cpp:571-680, cut out of that file into
 * $(OUT)/inc_lt/lighttree_body.h) as members of a stand-in RenderCore that holds only the light buffers they read,
 * with CoreBuffer reduced to a host array. The LightCluster constructors come from a copy of
 * lib/RenderSystem/common_classes.h in $(OUT)/inc_lt whose leaf constructors reset their box before growing it
 * (bounds.Reset()): the originals grow a box that nothing initialised, whose contents C++ leaves indeterminate. */
#include "ref_shim.h"
#include <vector>
#include "helper_math.h"
#include "common_settings.h"
#include "common_types.h"
#include "common_classes.h"

namespace reflt {
enum { ON_HOST = 1, ON_DEVICE = 2, STAGED = 4 };
template <class T>
struct CoreBuffer {
    std::vector<T> v;
    CoreBuffer(int n, int) : v((size_t)n) {}
    T* HostPtr() { return v.data(); }
    T* DevPtr() { return v.data(); }
    int GetSize() const { return (int)v.size(); }
    void StageCopyToDevice() {}
};
static void stageLightTree(LightCluster*) {}
struct RenderCore {
    CoreBuffer<CoreLightTri>* triLightBuffer = nullptr;
    CoreBuffer<CorePointLight>* pointLightBuffer = nullptr;
    CoreBuffer<CoreSpotLight>* spotLightBuffer = nullptr;
    CoreBuffer<LightCluster>* lightTree = nullptr;
    void UpdateLightTreeNormals(const int node);
    int FindBestMatch(int* todo, const int idx, const int N);
    void UpdateLightTree();
};
#include "lighttree_body.h"
}  // namespace reflt

extern "C" {
/* the tree UpdateLightTree builds for these lights (CoreLightTri / CorePointLight / CoreSpotLight arrays): its
 * (ntri + npt + nspot) * 2 records of 64 bytes to out; returns the record count (-1: capacity too small) */
int ref_light_tree(const void* tri, int ntri, const void* pt, int npt, const void* spot, int nspot, void* out, int capacity) {
    using namespace reflt;
    RenderCore rc;
    rc.triLightBuffer = new CoreBuffer<CoreLightTri>(ntri, ON_HOST);
    rc.pointLightBuffer = new CoreBuffer<CorePointLight>(npt, ON_HOST);
    rc.spotLightBuffer = new CoreBuffer<CoreSpotLight>(nspot, ON_HOST);
    if (ntri) memcpy(rc.triLightBuffer->HostPtr(), tri, sizeof(CoreLightTri) * ntri);
    if (npt) memcpy(rc.pointLightBuffer->HostPtr(), pt, sizeof(CorePointLight) * npt);
    if (nspot) memcpy(rc.spotLightBuffer->HostPtr(), spot, sizeof(CoreSpotLight) * nspot);
    int n = 0;
    if (ntri + npt + nspot > 0) {   /* (with no lights UpdateLightTree would read past its empty list) */
        rc.UpdateLightTree();
        n = rc.lightTree->GetSize();
        static_assert(sizeof(LightCluster) == 64, "the host LightCluster is the device record");
        if (n <= capacity) memcpy(out, rc.lightTree->HostPtr(), sizeof(LightCluster) * n);
        else n = -1;
    }
    delete rc.triLightBuffer, delete rc.pointLightBuffer, delete rc.spotLightBuffer, delete rc.lightTree;
    return n;
}
}

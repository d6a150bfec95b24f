/* core_types.cuh - device-side data layout of the GB300 render core (HBM resident).
 *
 *   BVH8 node (80 B, 5 x uint4): a compressed wide node in the spirit of Ylitie, Karras and Laine,
 *   "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs" (HPG 2017): a float origin p,
 *   three 8-bit power-of-two scale exponents, and per child six 8-bit box planes quantised outward
 *   (child box = p + q * 2^(e-127)). Child slot meta byte:
 *     0x00                empty slot
 *     0x80 | k            internal child, node index childBase + k
 *     (count << 5) | off  leaf child of 1..3 primitives at prim slots [primBase + off, + count)
 *   Leaf primitives of one node are stored contiguously, in node creation order.
 *
 *   Triangle intersection record (48 B, 3 x float4): v0 (w = primitive index within its mesh),
 *   e1 = v1 - v0, e2 = v2 - v0, stored in leaf order.
 *
 *   Path state SoA (one float4 per field, stride = path capacity):
 *     O4 = origin xyz, w = path index;  D4 = direction xyz, w = flags;  T4 = throughput rgb.
 */
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "lh2g_types.h"

namespace lh2g {

struct BVH8Node {
    float px, py, pz;
    uint32_t ebits;          /* e.x | e.y << 8 | e.z << 16 | imask << 24 */
    uint32_t childBase, primBase;
    uint32_t meta[2];        /* 8 meta bytes */
    uint32_t qlox[2], qloy[2], qloz[2], qhix[2], qhiy[2], qhiz[2];
};
static_assert(sizeof(BVH8Node) == 80, "BVH8 node must be 80 bytes");

/* Instance record for traversal (64 B): inverse transform rows (object <- world), BLAS root, mesh. */
struct alignas(16) InstanceGPU {   /* read as four float4 by the traversal */
    float inv[12];
    uint32_t blasRoot;       /* 0xffffffff: empty mesh */
    uint32_t mesh;
    uint32_t pad0, pad1;
};
static_assert(sizeof(InstanceGPU) == 64, "InstanceGPU must be four float4");

/* Everything the kernels read about the scene. Passed by value. */
struct SceneGPU {
    const uint4* nodes;              /* BVH8 node pool (BLAS + TLAS) */
    const float4* triData;           /* 3 float4 per leaf slot */
    const InstanceGPU* inst;
    const uint32_t* tlasPrims;       /* TLAS leaf slot -> instance index */
    uint32_t tlasRoot;               /* 0xffffffff: no instances */
    int instCount;
    /* shading */
    const float4* const* instTris;   /* per instance: CoreTri4 array of its mesh */
    const float4* instInvRows;       /* per instance: rows A, B, C of the inverse transform (3 float4) */
    const uint4* materials;          /* 8 uint4 per material */
    int nMaterials;
    const uint32_t* texels;          /* ARGB32, all textures back to back */
    const float4* triLights;         /* 6 float4 per area light */
    const float4* pointLights;       /* 2 float4 */
    const float4* spotLights;        /* 3 float4 */
    const float4* dirLights;         /* 2 float4 */
    int nTri, nPoint, nSpot, nDir;
    const float4* lightTree;         /* light-tree records, 4 float4 each (light_tree.h); record 0 the root */
    int nTreeNodes;
    const float4* skyPixels;
    int skyW, skyH;
    float4 worldToSky[3];            /* rows of the 3x3 part */
    const float4* skySmall;          /* (skyW >> 6) x (skyH >> 6) tile averages, read by the OptiX 7 estimator after a bounce */
    const uint32_t* blueNoise;       /* expanded blue-noise tables (5 * 65536 + 64 entries); null: xorshift numbers only */
};

/* Per-frame parameters. */
struct FrameGPU {
    int W, H, spp, maxDepth, rrStart, samplesTaken;
    uint32_t cameraR0;
    uint32_t frameSeed;              /* LH2G_RP_FILTER: shading R0 = frameSeed + depth * 91771 */
    float eps;
    int flags;
    float spreadAngle, aperture;
    float3 pos, p1, right, up;
    int64_t P;                       /* paths in the frame */
    int64_t stride;                  /* capacity of the SoA buffers */
    /* the OptiX 7 / PrimeAdaptive estimators (LH2G_RP_OPTIX7, LH2G_RP_ADAPTIVE) */
    uint32_t shift;                  /* blue-noise tile shift */
    uint32_t pass;                   /* the shading kernel's 'pass' (sample index of layer 0) */
    uint32_t r0Base, r0Depth;        /* PrimeAdaptive shading seed: r0Base + depth * r0Depth */
    float clampValue;
    float distortion;
    /* a band of rows [rowBegin, rowBegin + rowCount) of the W x H frame (bandPix = W * rowCount; 0: the whole frame);
     * a path's local index l maps to its index in the whole frame, which seeds its random numbers */
    int rowBegin, rowCount;
    uint32_t bandPix;
};

/* the index in the whole frame of the band's path l */
__device__ __forceinline__ uint32_t global_path(const FrameGPU& F, const uint32_t l) {
    if (!F.bandPix) return l;
    return (l / F.bandPix) * ((uint32_t)F.W * (uint32_t)F.H) + (uint32_t)F.rowBegin * (uint32_t)F.W + l % F.bandPix;
}

/* Device counters of one frame. extension[d] counts extension rays written while shading path length
 * d+1 (the queue of the next wave), shadow[d] the connections; status holds error bits. */
struct Counters {
    uint32_t extension[64];
    uint32_t shadow[64];
    uint32_t fetch[4 * 64];          /* persistent-kernel work counters, one per (kernel, depth) */
    uint32_t status;
    uint32_t probeInst, probePrim;
    float probeDist;
    unsigned long long travStats[4];   /* extend: nodes, triangles; connect: nodes, triangles */
    uint32_t hitCount[64], missCount[64];   /* per path length: queue slots placed in the shading order so far */
};

/* Path flags. The OptiX 7 / PrimeAdaptive estimators keep them in the low 6 bits of O4.w, above them the path's
 * slot: bits 0-3 the reference's S_* flags, bits 4-5 the ray's tmin (0: 0, 1: the geometry epsilon, 2: EPSILON) */
constexpr uint32_t S_BOUNCEDTWICE = 8;   /* (S_SPECULAR 1, S_BOUNCED 2 and S_VIASPECULAR 4 as in the other estimators) */
constexpr uint32_t MIS_TMIN_SHIFT = 4, MIS_TMIN_EPS = 1u << 4, MIS_TMIN_EPSILON = 2u << 4;
constexpr int MIS_SLOT_BITS = 26;   /* slots below 2^26 (67M paths) */

/* (the LH2G_STATUS_* bits of the device status word are in lh2g_types.h) */

}  // namespace lh2g

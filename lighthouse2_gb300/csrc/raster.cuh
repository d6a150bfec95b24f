/* raster.cuh - the SoftRasterizer core on the GPU: z-buffered scanline rasterisation of the scene's instances.
 *
 * Semantics of lib/RenderCore_SoftRasterizer/rasterizer.cpp:66-171 (Mesh::Render): per triangle back-face culling,
 * clipping against the near and left planes, projection, edge walks into per-row outlines and span fills with
 * perspective-correct texture coordinates; a fragment replaces the pixel when its interpolated 1/z is below the
 * z-buffer's. The reference runs triangles one after another, so a pixel ends with the fragment of smallest 1/z,
 * the earliest triangle among equal ones. Here every triangle runs at once:
 *   pass 1 (k_rs_cover): each fragment with 1/z < 0 offers the key (~bits(1/z)) << 32 | triangle order to its pixel
 *          by a 64-bit atomicMin, which leaves exactly the fragment the sequential z-test keeps;
 *   pass 2 (k_rs_color): the triangles that offered fragments run again and the fragment whose key won writes the
 *          texel colour.
 * Every interpolant is the reference's running sum (x0 += dx per row, u0 += du per pixel, ...), recomputed the
 * same way in both passes, so the GPU's pixels and z-buffer equal the sequential result bit for bit. Triangles
 * covering more than a few dozen pixels are queued instead and run as one block per (triangle, 8-row chunk,
 * 512-column segment) (k_rs_big), a warp per row; a warp per queued triangle first walks its edges once and leaves
 * their running values at every chunk's first row (k_rs_edges), so a chunk starts there. */
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace lh2g {

/* one instance the mesh culling kept: its object-to-camera rows, its triangles and their place in draw order */
struct RasterInst {
    float M[12];               /* rows 0..2 of transform x localTransform (rasterizer.cpp:187) */
    const float4* verts;       /* 3 per triangle */
    const float4* tris;        /* CoreTri4 records, 13 float4 per triangle (texture coordinates) */
    const float4* norms;       /* per triangle: face normal xyz, material index bits (launch_raster_pack) */
    uint32_t first;            /* draw order of its first triangle among the kept instances' triangles */
    uint32_t count;
};

/* a material as the rasterizer reads it (rendercore.cpp:166-185): a packed colour, or a texture's level 0 */
struct RasterMat { uint32_t diffuse, texFirst, width, height; };   /* width 0: untextured */

struct RasterFrame {
    int W, H;
    float4 nearPlane, leftPlane;     /* Rasterizer::frustum[0], [1]: the two planes triangles are clipped against */
    const RasterInst* inst;
    int nInst;
    uint32_t total;                  /* triangles of the kept instances */
    const RasterMat* mats;
    uint32_t nMats;
    const uint32_t* texels;
    uint32_t* pixels;                /* W x H RGBA8 */
    unsigned long long* keys;        /* W x H depth keys, all ones = empty */
    uint32_t* list;                  /* pass 1 -> pass 2: small triangles that offered fragments */
    uint2* big;                      /* triangles for the block path: draw order, first chunk */
    uint2* owner;                    /* per chunk of RS_CHUNK rows: its triangle's draw order and the chunk's index in it */
    float4* ck;                      /* per chunk and edge: the edge's running x, z, u, v at the chunk's first row */
    uint32_t ckCap;                  /* chunks the two arrays above hold */
    uint32_t* counters;              /* [0] list, [1] big, [2] fragments offered, [3] status (bad material), [4] chunks */
};

constexpr int RS_CHUNK = 8;          /* rows per block of the big-triangle path (a warp per row) */

/* a mesh's per-triangle face normal and material (16 B, from the CoreTri4 records) for the first pass */
void launch_raster_pack(const float4* tris, uint32_t n, float4* norms, cudaStream_t st);
/* the frame's two passes on `st` (keys and pixels must be cleared and counters zeroed before) */
void launch_raster(const RasterFrame& R, int smCount, cudaStream_t st);
/* the z-buffer of the reference (interpolated 1/z of the kept fragment, 0 where none) from the depth keys */
void launch_raster_depth(const RasterFrame& R, float* zbuffer, cudaStream_t st);

}  // namespace lh2g

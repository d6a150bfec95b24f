/* nrc.cuh - the radiance cache: a multiresolution hash grid plus one-blob encoding feeding a 4 x 64 ReLU MLP.
 *
 * No counterpart in the reference (its estimators trace every path to its end). The cache follows the published
 * neural radiance caching scheme (Mueller, Rousselle, Novak, Keller, "Real-time Neural Radiance Caching for Path
 * Tracing", SIGGRAPH 2021) with the multiresolution hash encoding of Mueller, Evans, Schied, Keller ("Instant
 * Neural Graphics Primitives", SIGGRAPH 2022), written from those descriptions:
 *
 *   query     16 floats: position xyz + roughness, outgoing direction xyz, normal xyz, albedo rgb
 *   encoding  64 inputs: 12 hash-grid levels x 2 features (resolutions 16 .. 2048, geometric; 2^19 entries per
 *             level, dense below that size, else the spatial hash x ^ 2654435761 y ^ 805459861 z; trilinear),
 *             one-blob (4 triangular bins) of the direction's and of the normal's spherical angles and of the
 *             roughness, the albedo, a constant 1, zeros
 *   network   64 -> 64 -> 64 -> 64 -> 64 -> 3, ReLU between layers, no biases, bf16 weights and activations,
 *             fp32 accumulation; the output layer is padded to 16 rows
 *   loss      relative L2: (y - t)^2 / (y^2 + 0.01) with y held constant in the denominator, mean over the batch
 *             and the 3 channels
 *   update    Adam (beta1 0.9, beta2 0.99, eps 1e-15) on fp32 master parameters; the kernels read bf16 weights
 *             and fp16 grid features written by the update
 */
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "device_math.cuh"

namespace lh2g {
namespace nrc {

constexpr int IN = 64, HID = 64, OUT = 3, OUTP = 16, LAYERS = 5;
constexpr int LEVELS = 12, LOG2T = 19, TABLE = 1 << LOG2T, FEAT = 2;
constexpr int WMASTER = 4 * HID * IN + OUT * HID;   /* fp32 master weights, row-major [out][in] per layer */
constexpr int WDEV = 4 * HID * IN + OUTP * HID;     /* bf16 device weights, output layer padded to 16 rows */
constexpr long long GRID_PARAMS = (long long)LEVELS * TABLE * FEAT;
#ifndef LH2G_NRC_LEVEL_UNROLL
#define LH2G_NRC_LEVEL_UNROLL 12  /* tuning switch: hash-grid levels encoded per loop iteration (12: all) */
#endif
constexpr int LEVEL_UNROLL = LH2G_NRC_LEVEL_UNROLL;

/* encoding parameters computed on the host */
struct GridSpec {
    float bmin[3], inv[3];   /* position -> [0, 1]^3 */
    int res[LEVELS];         /* cells per axis */
    int dense[LEVELS];       /* 1: (res + 1)^3 <= TABLE, direct indexing */
};

__device__ __forceinline__ uint32_t grid_index(const GridSpec& G, int l, uint32_t x, uint32_t y, uint32_t z) {
    if (G.dense[l]) {
        const uint32_t r1 = (uint32_t)G.res[l] + 1u;
        return x + r1 * (y + r1 * z);
    }
    return ((x * 1u) ^ (y * 2654435761u) ^ (z * 805459861u)) & (uint32_t)(TABLE - 1);
}

/* cell and interpolation weights of one level: the 8 corners are (i + (c & 1), j + (c >> 1 & 1), k + (c >> 2)) */
struct Cell {
    uint32_t i, j, k;
    float fx, fy, fz;
};
__device__ __forceinline__ Cell grid_cell(const GridSpec& G, int l, const float3 p) {
    const float r = (float)G.res[l];
    const float x = p.x * r, y = p.y * r, z = p.z * r;
    Cell c;
    c.i = (uint32_t)min(f2i(floorf(x)), G.res[l] - 1), c.j = (uint32_t)min(f2i(floorf(y)), G.res[l] - 1);
    c.k = (uint32_t)min(f2i(floorf(z)), G.res[l] - 1);
    c.fx = x - (float)c.i, c.fy = y - (float)c.j, c.fz = z - (float)c.k;
    return c;
}
__device__ __forceinline__ float corner_weight(const Cell& c, int corner) {
    return ((corner & 1) ? c.fx : 1.0f - c.fx) * ((corner & 2) ? c.fy : 1.0f - c.fy) * ((corner & 4) ? c.fz : 1.0f - c.fz);
}

__device__ __forceinline__ float3 unit_position(const GridSpec& G, const float4 q0) {
    return make_float3(fminf(fmaxf((q0.x - G.bmin[0]) * G.inv[0], 0.0f), 1.0f), fminf(fmaxf((q0.y - G.bmin[1]) * G.inv[1], 0.0f), 1.0f),
                       fminf(fmaxf((q0.z - G.bmin[2]) * G.inv[2], 0.0f), 1.0f));
}

/* four triangular bins centred at 1/8, 3/8, 5/8, 7/8 */
__device__ __forceinline__ void one_blob4(float x, float* out) {
#pragma unroll
    for (int i = 0; i < 4; i++) out[i] = fmaxf(0.0f, 1.0f - fabsf(x * 4.0f - ((float)i + 0.5f)));
}

/* spherical angles of a unit vector, both in [0, 1] */
__device__ __forceinline__ void sph01(const float3 d, float& th, float& ph) {
    th = acos_at(fminf(fmaxf(d.z, -1.0f), 1.0f)) * INVPI;
    ph = atan2_at(d.y, d.x) * INV2PI + 0.5f;
}

/* the 64 network inputs of a query (fp32; the kernels round them to bf16) */
__device__ __forceinline__ void encode(const GridSpec& G, const __half2* __restrict__ grid, const float4* q, float* e) {
    const float3 p = unit_position(G, q[0]);
    /* levels in groups of LEVEL_UNROLL so that several levels' gathers are in flight at once (the encoding is
     * bound by the latency of these L2 reads) */
#pragma unroll LEVEL_UNROLL
    for (int l = 0; l < LEVELS; l++) {
        const Cell c = grid_cell(G, l, p);
        float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
        for (int corner = 0; corner < 8; corner++) {
            const uint32_t idx = grid_index(G, l, c.i + (corner & 1), c.j + ((corner >> 1) & 1), c.k + (corner >> 2));
            const float2 v = __half22float2(__ldg(grid + (size_t)l * TABLE + idx));
            const float w = corner_weight(c, corner);
            f0 = f0 + w * v.x, f1 = f1 + w * v.y;
        }
        e[2 * l] = f0, e[2 * l + 1] = f1;
    }
    float th, ph;
    sph01(make_float3(q[1].x, q[1].y, q[1].z), th, ph);
    one_blob4(th, e + 24), one_blob4(ph, e + 28);
    sph01(make_float3(q[2].x, q[2].y, q[2].z), th, ph);
    one_blob4(th, e + 32), one_blob4(ph, e + 36);
    one_blob4(fminf(fmaxf(q[0].w, 0.0f), 1.0f), e + 40);
    e[44] = q[3].x, e[45] = q[3].y, e[46] = q[3].z, e[47] = 1.0f;
#pragma unroll
    for (int i = 48; i < IN; i++) e[i] = 0.0f;
}

}  // namespace nrc
}  // namespace lh2g

/* nrc.cu - radiance-cache kernels: inference, training (forward, loss, backward), Adam, and the C ABI.
 *
 * Matrix products run on the fifth-generation tensor cores (tcgen05, tc.cuh): a CTA of 128 threads holds a tile
 * of 128 queries, one per thread and per TMEM lane. Each layer is D[128 x N] = A[128 x 64] * W^T with A (bf16
 * activations) and W (bf16 weights, [N x 64]) in shared memory and D (fp32) in tensor memory; 4 MMAs of K = 16
 * per layer, issued by thread 0, completion through an mbarrier. The backward pass propagates the loss gradient
 * with the same instruction (D = delta * W, with W^T staged in shared memory); the weight gradients, sums over the
 * 128 rows of a tile of delta^T * activation, accumulate in each thread's registers on the FP32 pipes and reach
 * global memory once per CTA. Hash-grid gradients are scattered with atomics.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "lh2g.h"
#include "nrc.cuh"
#include "tc.cuh"

namespace lh2g {
namespace nrc {

constexpr int TILE = 128;
constexpr uint32_t WAIT_LIMIT = 1u << 24;
constexpr uint32_t LAYER_BYTES = HID * IN * 2;            /* 8 KB */
constexpr uint32_t OUT_LAYER_BYTES = OUTP * IN * 2;       /* 2 KB */
constexpr uint32_t WEIGHT_BYTES = 4 * LAYER_BYTES + OUT_LAYER_BYTES;
constexpr uint32_t ACT_BYTES = TILE * IN * 2;             /* 16 KB */
constexpr uint32_t ERR_TIMEOUT = 1u;

__host__ __device__ constexpr int layer_rows(int l) { return l < 4 ? HID : OUTP; }
__host__ __device__ constexpr uint32_t layer_offset(int l) { return (uint32_t)l * LAYER_BYTES; }   /* bytes, also in the global bf16 array */

/* 8 consecutive bf16 of row r, columns 8c .. 8c + 7, of a K-major tile with K columns */
__device__ __forceinline__ void st_row8(unsigned char* tile, uint32_t r, uint32_t c, uint32_t K, const uint4 v) {
    *reinterpret_cast<uint4*>(tile + tc::kmajor_offset(r, 8u * c, K)) = v;
}
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ float bf16_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t u) { return __uint_as_float(u & 0xffff0000u); }

/* a row of 64 fp32 values as bf16 into row r of a K = 64 tile */
__device__ __forceinline__ void store_row64(unsigned char* tile, uint32_t r, const float* v) {
#pragma unroll
    for (int c = 0; c < 8; c++)
        st_row8(tile, r, c, 64, make_uint4(pack_bf16(v[8 * c], v[8 * c + 1]), pack_bf16(v[8 * c + 2], v[8 * c + 3]),
                                           pack_bf16(v[8 * c + 4], v[8 * c + 5]), pack_bf16(v[8 * c + 6], v[8 * c + 7])));
}

/* the bf16 weights of all layers from global memory into K-major shared tiles (and, when Wt != nullptr, each layer
 * transposed: W_l^T as a [64 x rows_l] K-major tile) */
__device__ void stage_weights(const __nv_bfloat16* __restrict__ W, unsigned char* Ws, unsigned char* Wt) {
    const uint16_t* w = reinterpret_cast<const uint16_t*>(W);
    for (int l = 0; l < LAYERS; l++) {
        const int rows = layer_rows(l);
        const uint16_t* src = w + layer_offset(l) / 2;
        for (int idx = threadIdx.x; idx < rows * 8; idx += blockDim.x) {
            const int r = idx >> 3, c = idx & 7;
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(src + r * IN + 8 * c));
            st_row8(Ws + layer_offset(l), (uint32_t)r, (uint32_t)c, IN, v);
        }
        if (Wt)
            for (int idx = threadIdx.x; idx < rows * IN; idx += blockDim.x) {
                const int n = idx / IN, k = idx % IN;
                *reinterpret_cast<uint16_t*>(Wt + layer_offset(l) + tc::kmajor_offset((uint32_t)k, (uint32_t)n, (uint32_t)rows)) = __ldg(src + n * IN + k);
            }
    }
}

/* D[128 x N] (+)= A[128 x K] * B[N x K]^T on the tensor core, issued by the calling thread (no commit); with accumulate
 * the first K step adds to D too */
__device__ __forceinline__ void issue_mma(uint32_t dTmem, uint32_t aAddr, uint32_t bAddr, int K, int N, bool accumulate) {
    const uint32_t sbo = (uint32_t)K * 16u;
    const uint32_t idesc = tc::idesc_bf16_f32(TILE, N);
    for (int s = 0; s < K / 16; s++)
        tc::mma_bf16(dTmem, tc::smem_desc(aAddr + (uint32_t)s * 256u, 128u, sbo), tc::smem_desc(bAddr + (uint32_t)s * 256u, 128u, sbo), idesc,
                     (accumulate || s > 0) ? 1u : 0u);
}
/* D[128 x N] = A[128 x K] * B[N x K]^T on the tensor core (thread 0 issues, then commits to mbar) */
__device__ __forceinline__ void issue_gemm(uint32_t dTmem, uint32_t aAddr, uint32_t bAddr, int K, int N, uint64_t* mbar) {
    tc::fence_after_sync();
    issue_mma(dTmem, aAddr, bAddr, K, N, false);
    tc::mma_commit(mbar);
}

/* the row of this thread from D (columns [0, 16 * chunks)) */
__device__ __forceinline__ void read_row(uint32_t tmem, int chunks, float* v) {
    const uint32_t lane = (threadIdx.x & ~31u) << 16;   /* warp w reads lanes 32 w .. 32 w + 31 */
    for (int c = 0; c < chunks; c++) tc::tmem_ld16(tmem + lane + (uint32_t)(16 * c), v + 16 * c);
}

struct Shared {
    uint64_t mbar;
    uint32_t tmem;
    uint32_t failed;
};

/* shared memory of a kernel: the header, then 1 KB aligned tiles */
__device__ __forceinline__ unsigned char* tiles_base(unsigned char* dyn) {
    return reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(dyn) + sizeof(Shared) + 1023) & ~(uintptr_t)1023);
}
constexpr uint32_t SMEM_SLACK = 1024 + 64;

/* ---------------------------------------------------------------------------------------------------------
 * inference: out[i] = MLP(encode(query[i])), 4 floats per query (rgb, 0)
 * ------------------------------------------------------------------------------------------------------- */
/* tuning switch: query tiles per CTA (1 or 2). With 2, a CTA of 256 threads encodes two tiles of 128 queries at
 * once and issues both tiles' products per layer under one commit: the weights are staged once for both, and more
 * warps per SM wait on the hash-grid gathers (3 CTAs of 8 warps instead of 4 of 4). Measured 5 % slower (1M queries
 * in 0.675 against 0.645 ms): the gathers are bound by L2 sector traffic (96 gathers of 4 B per query, each a
 * 32-byte sector, about 5 TB/s of L2 reads), not by the warps waiting on them. 1 is the default. */
#ifndef LH2G_NRC_INFER_TILES
#define LH2G_NRC_INFER_TILES 1
#endif
constexpr int INFER_TILES = LH2G_NRC_INFER_TILES;
static_assert(INFER_TILES == 1 || INFER_TILES == 2, "one or two tiles per CTA");
constexpr uint32_t INFER_SMEM = WEIGHT_BYTES + INFER_TILES * ACT_BYTES + SMEM_SLACK;
constexpr uint32_t INFER_TMEM_COLS = 64 * INFER_TILES;

__global__ void __launch_bounds__(TILE * INFER_TILES) k_infer(const GridSpec G, const __half2* __restrict__ grid, const __nv_bfloat16* __restrict__ W,
                                                              const float4* __restrict__ queries, const long long nMax, const uint32_t* __restrict__ nDev,
                                                              float4* __restrict__ out, uint32_t* errors) {
    /* query count: nMax, or the count a previous kernel left in device memory (at most nMax) */
    const long long n = nDev ? min((long long)*nDev, nMax) : nMax;
    extern __shared__ unsigned char dyn[];
    Shared& sh = *reinterpret_cast<Shared*>(dyn);
    unsigned char* Ws = tiles_base(dyn);
    /* this thread's tile of the CTA and its row in it; its warp reads TMEM lanes 32 (warp % 4) .. + 31 */
    const uint32_t sub = threadIdx.x / TILE, row = threadIdx.x % TILE;
    unsigned char* A = Ws + WEIGHT_BYTES + sub * ACT_BYTES;
    if (threadIdx.x < 32) {
        tc::tmem_alloc(&sh.tmem, INFER_TMEM_COLS);
        tc::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        tc::mbar_init(&sh.mbar, 1);
        tc::mbar_fence_init();
        sh.failed = 0;
    }
    stage_weights(W, Ws, nullptr);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = sh.tmem, a0 = tc::smem_u32(Ws + WEIGHT_BYTES), wAddr = tc::smem_u32(Ws);
    const uint32_t myD = tmem + 64u * sub + ((row & ~31u) << 16);
    uint32_t phase = 0;
    const long long tiles = (n + TILE - 1) / TILE;
    for (long long t = (long long)blockIdx.x * INFER_TILES; t < tiles; t += (long long)gridDim.x * INFER_TILES) {
        const long long q = (t + sub) * TILE + row;
        float v[IN];
        if (q < n) {
            float4 qq[4];
#pragma unroll
            for (int i = 0; i < 4; i++) qq[i] = __ldg(queries + 4 * q + i);
            encode(G, grid, qq, v);
        } else {
#pragma unroll
            for (int i = 0; i < IN; i++) v[i] = 0.0f;
        }
        store_row64(A, row, v);
        for (int l = 0; l < LAYERS; l++) {
            tc::fence_proxy_async();
            tc::fence_before_sync();
            __syncthreads();
            if (threadIdx.x == 0) {
                tc::fence_after_sync();
                for (int s2 = 0; s2 < INFER_TILES; s2++)
                    issue_mma(tmem + 64u * (uint32_t)s2, a0 + (uint32_t)s2 * ACT_BYTES, wAddr + layer_offset(l), IN, layer_rows(l), false);
                tc::mma_commit(&sh.mbar);
            }
            if (!tc::mbar_wait(&sh.mbar, phase, WAIT_LIMIT)) sh.failed = 1;
            phase ^= 1u;
            tc::fence_after_sync();
            if (l < LAYERS - 1) {
#pragma unroll
                for (int c = 0; c < 4; c++) tc::tmem_ld16(myD + (uint32_t)(16 * c), v + 16 * c);
#pragma unroll
                for (int i = 0; i < HID; i++) v[i] = fmaxf(v[i], 0.0f);
                store_row64(A, row, v);
            } else {
                float y[16];
                tc::tmem_ld16(myD, y);
                if (q < n) out[q] = make_float4(y[0], y[1], y[2], 0.0f);
            }
        }
        tc::fence_before_sync();
        __syncthreads();
        if (__syncthreads_or(sh.failed)) break;
    }
    __syncthreads();
    if (threadIdx.x == 0 && sh.failed) atomicOr(errors, ERR_TIMEOUT);
    tc::fence_after_sync();
    if (threadIdx.x < 32) tc::tmem_dealloc(tmem, INFER_TMEM_COLS);
}

/* ---------------------------------------------------------------------------------------------------------
 * training: one pass over n samples accumulates the gradients of the mean relative L2 loss into gW (fp32, master
 * layout) and gGrid, and the loss into *loss
 * ------------------------------------------------------------------------------------------------------- */
constexpr uint32_t DELTA_BYTES = TILE * HID * 2;
constexpr uint32_t GRADT_BYTES = HID * TILE * 2;   /* a [64 x 128] bf16 tile: delta_j^T or act_j^T */
constexpr uint32_t TRAIN_SMEM = 2 * WEIGHT_BYTES + 5 * ACT_BYTES + DELTA_BYTES + 2 * GRADT_BYTES + SMEM_SLACK;
/* TMEM: columns 0..63 the forward / backward products, 64 (j + 1) .. 64 (j + 2) - 1 the sums of dW_j (j = 0..3) */
constexpr uint32_t TRAIN_TMEM_COLS = 512;

__device__ __forceinline__ void load_row8(const unsigned char* tile, uint32_t r, uint32_t col8, uint32_t K, float* v) {
    const uint4 u = *reinterpret_cast<const uint4*>(tile + tc::kmajor_offset(r, col8, K));
    v[0] = bf16_lo(u.x), v[1] = bf16_hi(u.x), v[2] = bf16_lo(u.y), v[3] = bf16_hi(u.y);
    v[4] = bf16_lo(u.z), v[5] = bf16_hi(u.z), v[6] = bf16_lo(u.w), v[7] = bf16_hi(u.w);
}

/* column b of a [64 x TILE] K-major tile (K = TILE): 64 bf16 values, element (n, b) */
__device__ __forceinline__ void store_col64(unsigned char* tile, uint32_t b, const float* v) {
#pragma unroll
    for (int n = 0; n < 64; n += 2) {
        const uint32_t u = pack_bf16(v[n], v[n + 1]);
        *reinterpret_cast<uint16_t*>(tile + tc::kmajor_offset((uint32_t)n, b, TILE)) = (uint16_t)(u & 0xffffu);
        *reinterpret_cast<uint16_t*>(tile + tc::kmajor_offset((uint32_t)n + 1u, b, TILE)) = (uint16_t)(u >> 16);
    }
}
/* row r of a K = 64 tile, bit for bit, into column r of a [64 x TILE] K-major tile */
__device__ __forceinline__ void transpose_row64(const unsigned char* src, unsigned char* dst, uint32_t r) {
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const uint4 u = *reinterpret_cast<const uint4*>(src + tc::kmajor_offset(r, 8u * c, IN));
        const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
            *reinterpret_cast<uint16_t*>(dst + tc::kmajor_offset(8u * c + 2u * i, r, TILE)) = (uint16_t)(w[i] & 0xffffu);
            *reinterpret_cast<uint16_t*>(dst + tc::kmajor_offset(8u * c + 2u * i + 1u, r, TILE)) = (uint16_t)(w[i] >> 16);
        }
    }
}

__global__ void __launch_bounds__(TILE, 1) k_train(const GridSpec G, const __half2* __restrict__ grid, const __nv_bfloat16* __restrict__ W,
                                                   const float4* __restrict__ queries, const float4* __restrict__ targets, const long long nMax,
                                                   const uint32_t* __restrict__ nDev, float* __restrict__ gW, float* __restrict__ gGrid,
                                                   float* __restrict__ loss, uint32_t* errors) {
    const long long n = nDev ? min((long long)*nDev, nMax) : nMax;
    extern __shared__ unsigned char dyn[];
    Shared& sh = *reinterpret_cast<Shared*>(dyn);
    unsigned char* Ws = tiles_base(dyn);
    unsigned char* Wt = Ws + WEIGHT_BYTES;
    unsigned char* act = Wt + WEIGHT_BYTES;          /* act_0 (inputs) .. act_4, [128 x 64] each */
    unsigned char* delta = act + 5 * ACT_BYTES;      /* delta_j, [128 x rows_j] */
    /* the weight-gradient product of hidden layer j, dW_j = delta_j^T act_j (sum over the tile's rows), on the tensor
     * core: A = delta_j^T [64 x 128] (K = the tile's rows) in deltaT, B = act_j^T [64 x 128] in actT. The MMA is
     * M = 128: its rows 64..127 read the 16 KB after deltaT (actT) and land in TMEM lanes 64..127, which are never
     * read. dW_j accumulates over the CTA's tiles in TMEM columns 64 (j + 1) .. 64 (j + 2), lanes 0..63. */
    unsigned char* deltaT = delta + DELTA_BYTES;
    unsigned char* actT = deltaT + GRADT_BYTES;
    if (threadIdx.x < 32) {
        tc::tmem_alloc(&sh.tmem, TRAIN_TMEM_COLS);
        tc::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        tc::mbar_init(&sh.mbar, 1);
        tc::mbar_fence_init();
        sh.failed = 0;
    }
    stage_weights(W, Ws, Wt);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = sh.tmem, wAddr = tc::smem_u32(Ws), wtAddr = tc::smem_u32(Wt), actAddr = tc::smem_u32(act), dAddr = tc::smem_u32(delta);
    const uint32_t dtAddr = tc::smem_u32(deltaT), atAddr = tc::smem_u32(actT);
    const uint32_t r = threadIdx.x;
    /* the output layer's gradient (16 x 64) on the FP32 pipes: row n4, columns k0 .. k0 + 7 of this thread */
    const uint32_t k0 = (r & 7) * 8, n4 = r >> 3;
    float gw4[8];
#pragma unroll
    for (int i = 0; i < 8; i++) gw4[i] = 0.0f;
    bool anyTile = false;   /* the TMEM gradient columns hold sums once the first tile has run */
    float lossSum = 0.0f;
    const float invCount = 1.0f / (3.0f * (float)n);
    uint32_t phase = 0;
    const long long tiles = (n + TILE - 1) / TILE;
    for (long long t = blockIdx.x; t < tiles; t += gridDim.x) {
        const long long q = t * TILE + r;
        const bool valid = q < n;
        float4 qq[4];
        float v[IN];
        if (valid) {
#pragma unroll
            for (int i = 0; i < 4; i++) qq[i] = __ldg(queries + 4 * q + i);
            encode(G, grid, qq, v);
        } else {
#pragma unroll
            for (int i = 0; i < IN; i++) v[i] = 0.0f;
        }
        store_row64(act, r, v);
        /* forward */
        float y[16];
#pragma unroll 1
        for (int j = 0; j < LAYERS; j++) {
            tc::fence_proxy_async();
            tc::fence_before_sync();
            __syncthreads();
            if (r == 0) issue_gemm(tmem, actAddr + (uint32_t)j * ACT_BYTES, wAddr + layer_offset(j), IN, layer_rows(j), &sh.mbar);
            if (!tc::mbar_wait(&sh.mbar, phase, WAIT_LIMIT)) sh.failed = 1;
            phase ^= 1u;
            tc::fence_after_sync();
            if (j < LAYERS - 1) {
                read_row(tmem, 4, v);
#pragma unroll
                for (int i = 0; i < HID; i++) v[i] = fmaxf(v[i], 0.0f);
                store_row64(act + (uint32_t)(j + 1) * ACT_BYTES, r, v);
            } else {
                read_row(tmem, 1, y);
            }
        }
        /* loss and its gradient with respect to the output (rows past n contribute nothing) */
        float dy[16];
#pragma unroll
        for (int c = 0; c < 16; c++) dy[c] = 0.0f;
        if (valid) {
            const float4 tg = __ldg(targets + q);
            const float tt[3] = {tg.x, tg.y, tg.z};
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const float den = y[c] * y[c] + 0.01f, e = y[c] - tt[c];
                lossSum += e * e / den * invCount;
                dy[c] = 2.0f * e / den * invCount;
            }
        }
        st_row8(delta, r, 0, OUTP, make_uint4(pack_bf16(dy[0], dy[1]), pack_bf16(dy[2], dy[3]), pack_bf16(dy[4], dy[5]), pack_bf16(dy[6], dy[7])));
        st_row8(delta, r, 1, OUTP, make_uint4(pack_bf16(dy[8], dy[9]), pack_bf16(dy[10], dy[11]), pack_bf16(dy[12], dy[13]), pack_bf16(dy[14], dy[15])));
        /* backward: layer j = 4 .. 0 */
#pragma unroll
        for (int j = LAYERS - 1; j >= 0; j--) {
            const int Nj = layer_rows(j);
            const unsigned char* aj = act + (uint32_t)j * ACT_BYTES;
            if (j < LAYERS - 1) transpose_row64(aj, actT, r);   /* act_j^T, the weight-gradient product's B */
            tc::fence_proxy_async();
            tc::fence_before_sync();
            __syncthreads();
            /* dL/d act_j = delta_j * W_j and, for the hidden layers, dW_j += delta_j^T act_j, on the tensor core ... */
            if (r == 0) {
                tc::fence_after_sync();
                issue_mma(tmem, dAddr, wtAddr + layer_offset(j), Nj, HID, false);
                if (j < LAYERS - 1) issue_mma(tmem + 64u * (uint32_t)(j + 1), dtAddr, atAddr, TILE, HID, anyTile);
                tc::mma_commit(&sh.mbar);
            }
            /* ... while the output layer's gradient (16 rows) accumulates on the FP32 pipes */
            if (j == LAYERS - 1) {
#pragma unroll 2
                for (uint32_t b = 0; b < (uint32_t)TILE; b++) {
                    float a8[8];
                    load_row8(aj, b, k0, IN, a8);
                    const float d = __uint_as_float((uint32_t)*reinterpret_cast<const uint16_t*>(delta + tc::kmajor_offset(b, n4, OUTP)) << 16);
#pragma unroll
                    for (int i = 0; i < 8; i++) gw4[i] += d * a8[i];
                }
            }
            if (!tc::mbar_wait(&sh.mbar, phase, WAIT_LIMIT)) sh.failed = 1;
            phase ^= 1u;
            tc::fence_after_sync();
            float g[HID];
            read_row(tmem, 4, g);
            tc::fence_before_sync();
            __syncthreads();   /* every thread is done with delta_j */
            if (j > 0) {
                /* delta_{j-1} = dL/d act_j where act_j > 0 (the ReLU of layer j - 1) */
                float m[8];
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    load_row8(aj, r, 8 * c, IN, m);
#pragma unroll
                    for (int i = 0; i < 8; i++) g[8 * c + i] = m[i] > 0.0f ? g[8 * c + i] : 0.0f;
                }
                store_row64(delta, r, g);
                store_col64(deltaT, r, g);   /* delta_{j-1}^T, the next weight-gradient product's A */
            } else if (valid) {
                /* dL/d inputs: the hash-grid features receive it through the trilinear weights */
                const float3 p = unit_position(G, qq[0]);
                for (int l = 0; l < LEVELS; l++) {
                    const Cell c = grid_cell(G, l, p);
#pragma unroll
                    for (int corner = 0; corner < 8; corner++) {
                        const uint32_t idx = grid_index(G, l, c.i + (corner & 1), c.j + ((corner >> 1) & 1), c.k + (corner >> 2));
                        const float w = corner_weight(c, corner);
                        float* dst = gGrid + ((size_t)l * TABLE + idx) * 2;
                        atomicAdd(dst, w * g[2 * l]);
                        atomicAdd(dst + 1, w * g[2 * l + 1]);
                    }
                }
            }
        }
        anyTile = true;
        if (__syncthreads_or(sh.failed)) break;
    }
    /* this CTA's gradient sums and loss: the hidden layers' from TMEM (lanes 0..63 = rows of dW_j, warps 0 and 1) */
    tc::fence_after_sync();
    if (anyTile && r < (uint32_t)HID)
        for (int l = 0; l < 4; l++) {
            float g[HID];
            read_row(tmem + 64u * (uint32_t)(l + 1), 4, g);
#pragma unroll
            for (int k = 0; k < IN; k++) atomicAdd(gW + l * HID * IN + r * IN + k, g[k]);
        }
    if (n4 < (uint32_t)OUT)
#pragma unroll
        for (int i = 0; i < 8; i++) atomicAdd(gW + 4 * HID * IN + n4 * IN + k0 + i, gw4[i]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) lossSum += __shfl_xor_sync(0xffffffffu, lossSum, off);
    if ((r & 31) == 0) atomicAdd(loss, lossSum);
    __syncthreads();
    if (r == 0 && sh.failed) atomicOr(errors, ERR_TIMEOUT);
    tc::fence_after_sync();
    if (r < 32) tc::tmem_dealloc(tmem, TRAIN_TMEM_COLS);
}

/* ---------------------------------------------------------------------------------------------------------
 * Adam on fp32 master parameters (gradients cleared), writing the copy the kernels read
 * ------------------------------------------------------------------------------------------------------- */
__global__ void k_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v, float* __restrict__ g, const long long n, const float lr,
                       const float c1, const float c2, __nv_bfloat16* __restrict__ outBf16, __half* __restrict__ outHalf,
                       const uint32_t* __restrict__ batchDev) {
    if (batchDev && *batchDev == 0u) return;   /* an empty training batch (counted on the device) changes nothing */
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-15f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * (gi * gi);
        const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        m[i] = mi, v[i] = vi, p[i] = pi, g[i] = 0.0f;
        if (outBf16) outBf16[i] = __float2bfloat16_rn(pi);
        if (outHalf) outHalf[i] = __float2half_rn(pi);
    }
}

/* Self-test of the bounded waits: an mbarrier that nothing arrives on. The wait gives up after `limit` polls and
 * the kernel reports it, the failure path every tensor-core wait of this file takes. */
__global__ void k_wait_probe(const uint32_t limit, uint32_t* status) {
    __shared__ uint64_t mbar;
    if (threadIdx.x == 0) {
        tc::mbar_init(&mbar, 1);
        tc::mbar_fence_init();
    }
    __syncthreads();
    const bool done = tc::mbar_wait(&mbar, 0, limit);
    if (!__syncthreads_and(done) && threadIdx.x == 0) atomicOr(status, ERR_TIMEOUT);
}

__global__ void k_to_copies(const float* __restrict__ p, const long long n, __nv_bfloat16* __restrict__ outBf16, __half* __restrict__ outHalf) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (outBf16) outBf16[i] = __float2bfloat16_rn(p[i]);
        if (outHalf) outHalf[i] = __float2half_rn(p[i]);
    }
}

}  // namespace nrc
}  // namespace lh2g

using namespace lh2g;
using namespace lh2g::nrc;

struct lh2g_nrc {
    int device = 0;
    cudaStream_t st = nullptr;
    std::string err;
    GridSpec G;
    float lr = 1e-3f;
    long long step = 0;
    float *pW = nullptr, *mW = nullptr, *vW = nullptr, *gW = nullptr;   /* WMASTER */
    __nv_bfloat16* Wdev = nullptr;                                      /* WDEV */
    float *pG = nullptr, *mG = nullptr, *vG = nullptr, *gG = nullptr;   /* GRID_PARAMS */
    __half* grid16 = nullptr;
    float* dLoss = nullptr;
    uint32_t* dErr = nullptr;
    int blocksInfer = 0, blocksTrain = 0;
};

namespace {

int nfail(lh2g_nrc* c, int code, const std::string& m) {
    if (c) c->err = m;
    return code;
}
#define NCK(call)                                                                                        \
    do {                                                                                                 \
        const cudaError_t _e = (call);                                                                   \
        if (_e != cudaSuccess) return nfail(c, LH2G_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

uint32_t rng_next(uint64_t& s) {   /* splitmix64 */
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return (uint32_t)((z ^ (z >> 31)) >> 32);
}
float rng_uniform(uint64_t& s, float a) { return ((float)rng_next(s) * (1.0f / 4294967296.0f) * 2.0f - 1.0f) * a; }

int launch_copies(lh2g_nrc* c) {
    k_to_copies<<<256, 256, 0, c->st>>>(c->pW, WMASTER, c->Wdev, nullptr);
    k_to_copies<<<1024, 256, 0, c->st>>>(c->pG, GRID_PARAMS, nullptr, c->grid16);
    NCK(cudaGetLastError());
    return LH2G_OK;
}

int check_errors(lh2g_nrc* c) {
    uint32_t e = 0;
    NCK(cudaMemcpyAsync(&e, c->dErr, 4, cudaMemcpyDeviceToHost, c->st));
    NCK(cudaStreamSynchronize(c->st));
    if (e) return nfail(c, LH2G_ERR_CUDA, "radiance cache: a tensor-core completion wait ran out");
    return LH2G_OK;
}

}  // namespace

extern "C" {

int lh2g_nrc_create(int device, const lh2g_nrc_config* cfg, lh2g_nrc** out) {
    if (!cfg || !out) return LH2G_ERR_INVALID;
    *out = nullptr;
    lh2g_nrc* c = new lh2g_nrc();
    c->device = device;
    c->lr = cfg->learningRate > 0 ? cfg->learningRate : 1e-3f;
    for (int a = 0; a < 3; a++) {
        const float ext = cfg->sceneMax[a] - cfg->sceneMin[a];
        c->G.bmin[a] = cfg->sceneMin[a];
        c->G.inv[a] = ext > 0 ? 1.0f / ext : 1.0f;
    }
    const double growth = std::exp(std::log(2048.0 / 16.0) / (LEVELS - 1));
    for (int l = 0; l < LEVELS; l++) {
        c->G.res[l] = (int)std::floor(16.0 * std::pow(growth, (double)l));
        const double cells = std::pow((double)c->G.res[l] + 1.0, 3.0);
        c->G.dense[l] = cells <= (double)TABLE ? 1 : 0;
    }
    auto fail = [&](int code) { lh2g_nrc_destroy(c); return code; };
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) return fail(LH2G_ERR_CUDA);
    bool ok = true;
    for (float** q : {&c->pW, &c->mW, &c->vW, &c->gW}) ok = ok && cudaMalloc((void**)q, sizeof(float) * WMASTER) == cudaSuccess;
    for (float** q : {&c->pG, &c->mG, &c->vG, &c->gG}) ok = ok && cudaMalloc((void**)q, sizeof(float) * GRID_PARAMS) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&c->Wdev, sizeof(__nv_bfloat16) * WDEV) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&c->grid16, sizeof(__half) * GRID_PARAMS) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&c->dLoss, 16) == cudaSuccess && cudaMalloc((void**)&c->dErr, 16) == cudaSuccess;
    if (!ok) return fail(LH2G_ERR_OOM);
    /* initial parameters: Xavier-uniform weights, grid features uniform in +-1e-4 */
    std::vector<float> w(WMASTER), g(GRID_PARAMS);
    uint64_t seed = cfg->seed ? cfg->seed : 0x1234567ull;
    for (int l = 0; l < LAYERS; l++) {
        const int rows = l < 4 ? HID : OUT;
        const float a = std::sqrt(6.0f / (float)(IN + rows));
        for (int i = 0; i < rows * IN; i++) w[(size_t)l * HID * IN + i] = rng_uniform(seed, a);
    }
    for (auto& x : g) x = rng_uniform(seed, 1e-4f);
    ok = cudaMemcpy(c->pW, w.data(), sizeof(float) * WMASTER, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(c->pG, g.data(), sizeof(float) * GRID_PARAMS, cudaMemcpyHostToDevice) == cudaSuccess;
    /* on the cache's own (non-blocking) stream, ordered before the copies below: a legacy-stream memset would not be */
    for (float* q : {c->mW, c->vW, c->gW}) ok = ok && cudaMemsetAsync(q, 0, sizeof(float) * WMASTER, c->st) == cudaSuccess;
    for (float* q : {c->mG, c->vG, c->gG}) ok = ok && cudaMemsetAsync(q, 0, sizeof(float) * GRID_PARAMS, c->st) == cudaSuccess;
    ok = ok && cudaMemsetAsync(c->Wdev, 0, sizeof(__nv_bfloat16) * WDEV, c->st) == cudaSuccess &&
         cudaMemsetAsync(c->dErr, 0, 16, c->st) == cudaSuccess && cudaMemsetAsync(c->dLoss, 0, 16, c->st) == cudaSuccess;
    ok = ok && cudaFuncSetAttribute(k_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)INFER_SMEM) == cudaSuccess;
    ok = ok && cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TRAIN_SMEM) == cudaSuccess;
    /* all of the unified L1 / shared storage as shared memory, so that several inference CTAs share an SM: the
     * hash-grid gathers of the encoding are latency bound and want warps to hide it */
    ok = ok && cudaFuncSetAttribute(k_infer, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared) == cudaSuccess;
    if (!ok) return fail(LH2G_ERR_CUDA);
    int sms = 1, per = 0, smemSM = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaDeviceGetAttribute(&smemSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_infer, TILE * INFER_TILES, INFER_SMEM) != cudaSuccess) per = 0;
    /* resident CTAs per SM: what shared memory allows with the carveout above (1 KB reserved per CTA; the
     * calculator may assume a smaller carveout), at most what the SM's 512 TMEM columns hold. Surplus CTAs would
     * only wait: the kernel strides over its tiles. */
    per = std::max(per, smemSM / (int)(INFER_SMEM + 1024));
    c->blocksInfer = sms * std::max(1, std::min(per, (int)(512 / INFER_TMEM_COLS)));
    c->blocksTrain = sms;
    if (launch_copies(c) != LH2G_OK || cudaStreamSynchronize(c->st) != cudaSuccess) return fail(LH2G_ERR_CUDA);
    *out = c;
    return LH2G_OK;
}

int lh2g_nrc_destroy(lh2g_nrc* c) {
    if (!c) return LH2G_ERR_INVALID;
    cudaSetDevice(c->device);
    if (c->st) cudaStreamSynchronize(c->st);
    for (void* q : {(void*)c->pW, (void*)c->mW, (void*)c->vW, (void*)c->gW, (void*)c->pG, (void*)c->mG, (void*)c->vG, (void*)c->gG,
                    (void*)c->Wdev, (void*)c->grid16, (void*)c->dLoss, (void*)c->dErr})
        if (q) cudaFree(q);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
    return LH2G_OK;
}

const char* lh2g_nrc_last_error(lh2g_nrc* c) { return c ? c->err.c_str() : "null cache"; }

int lh2g_nrc_get_spec(lh2g_nrc* c, int* res12, int* dense12, float* bminInv6) {
    if (!c || !res12 || !dense12 || !bminInv6) return LH2G_ERR_INVALID;
    for (int l = 0; l < LEVELS; l++) res12[l] = c->G.res[l], dense12[l] = c->G.dense[l];
    for (int a = 0; a < 3; a++) bminInv6[a] = c->G.bmin[a], bminInv6[3 + a] = c->G.inv[a];
    return LH2G_OK;
}

int lh2g_nrc_set_params(lh2g_nrc* c, const float* mlp, const float* grid) {
    if (!c) return LH2G_ERR_INVALID;
    cudaSetDevice(c->device);
    if (mlp) NCK(cudaMemcpyAsync(c->pW, mlp, sizeof(float) * WMASTER, cudaMemcpyHostToDevice, c->st));
    if (grid) NCK(cudaMemcpyAsync(c->pG, grid, sizeof(float) * GRID_PARAMS, cudaMemcpyHostToDevice, c->st));
    for (float* q : {c->mW, c->vW, c->gW}) NCK(cudaMemsetAsync(q, 0, sizeof(float) * WMASTER, c->st));
    for (float* q : {c->mG, c->vG, c->gG}) NCK(cudaMemsetAsync(q, 0, sizeof(float) * GRID_PARAMS, c->st));
    c->step = 0;
    const int r = launch_copies(c);
    if (r != LH2G_OK) return r;
    NCK(cudaStreamSynchronize(c->st));
    return LH2G_OK;
}

int lh2g_nrc_get_params(lh2g_nrc* c, float* mlp, float* grid) {
    if (!c) return LH2G_ERR_INVALID;
    cudaSetDevice(c->device);
    if (mlp) NCK(cudaMemcpyAsync(mlp, c->pW, sizeof(float) * WMASTER, cudaMemcpyDeviceToHost, c->st));
    if (grid) NCK(cudaMemcpyAsync(grid, c->pG, sizeof(float) * GRID_PARAMS, cudaMemcpyDeviceToHost, c->st));
    NCK(cudaStreamSynchronize(c->st));
    return LH2G_OK;
}

int lh2g_nrc_get_grads(lh2g_nrc* c, float* mlp, float* grid) {
    if (!c) return LH2G_ERR_INVALID;
    cudaSetDevice(c->device);
    if (mlp) NCK(cudaMemcpyAsync(mlp, c->gW, sizeof(float) * WMASTER, cudaMemcpyDeviceToHost, c->st));
    if (grid) NCK(cudaMemcpyAsync(grid, c->gG, sizeof(float) * GRID_PARAMS, cudaMemcpyDeviceToHost, c->st));
    NCK(cudaStreamSynchronize(c->st));
    return LH2G_OK;
}

static int infer_launch(lh2g_nrc* c, const float* queries, long long nMax, const uint32_t* nDev, float* out, void* stream) {
    cudaSetDevice(c->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : c->st;
    const long long tiles = (nMax + TILE - 1) / TILE;
    const int blocks = (int)std::min<long long>((tiles + INFER_TILES - 1) / INFER_TILES, c->blocksInfer);
    k_infer<<<blocks, TILE * INFER_TILES, INFER_SMEM, st>>>(c->G, reinterpret_cast<const __half2*>(c->grid16), c->Wdev, reinterpret_cast<const float4*>(queries), nMax,
                                             nDev, reinterpret_cast<float4*>(out), c->dErr);
    NCK(cudaGetLastError());
    return LH2G_OK;
}

int lh2g_nrc_infer(lh2g_nrc* c, const float* queries, long long n, float* out, void* stream) {
    if (!c || (n > 0 && (!queries || !out)) || n < 0) return LH2G_ERR_INVALID;
    if (n == 0) return LH2G_OK;
    return infer_launch(c, queries, n, nullptr, out, stream);
}

int lh2g_nrc_infer_counted(lh2g_nrc* c, const float* queries, const uint32_t* countDevice, long long maxCount, float* out, void* stream) {
    if (!c || !countDevice || maxCount < 0 || (maxCount > 0 && (!queries || !out))) return LH2G_ERR_INVALID;
    if (maxCount == 0) return LH2G_OK;
    return infer_launch(c, queries, maxCount, countDevice, out, stream);
}

static int adam_launch(lh2g_nrc* c, cudaStream_t st, const uint32_t* batchDev) {
    c->step++;
    const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)c->step)));
    const float c2 = (float)(1.0 / (1.0 - std::pow(0.99, (double)c->step)));
    k_adam<<<64, 256, 0, st>>>(c->pW, c->mW, c->vW, c->gW, WMASTER, c->lr, c1, c2, c->Wdev, nullptr, batchDev);
    k_adam<<<2048, 256, 0, st>>>(c->pG, c->mG, c->vG, c->gG, GRID_PARAMS, c->lr, c1, c2, nullptr, c->grid16, batchDev);
    NCK(cudaGetLastError());
    return LH2G_OK;
}

int lh2g_nrc_apply_update(lh2g_nrc* c, void* stream) {
    if (!c) return LH2G_ERR_INVALID;
    cudaSetDevice(c->device);
    return adam_launch(c, stream ? (cudaStream_t)stream : c->st, nullptr);
}

static int train_launch(lh2g_nrc* c, const float* queries, const float* targets, long long nMax, const uint32_t* nDev, cudaStream_t st) {
    NCK(cudaMemsetAsync(c->dLoss, 0, 4, st));
    const long long tiles = (nMax + TILE - 1) / TILE;
    const int blocks = (int)std::min<long long>(tiles, c->blocksTrain);
    k_train<<<blocks, TILE, TRAIN_SMEM, st>>>(c->G, reinterpret_cast<const __half2*>(c->grid16), c->Wdev, reinterpret_cast<const float4*>(queries),
                                             reinterpret_cast<const float4*>(targets), nMax, nDev, c->gW, c->gG, c->dLoss, c->dErr);
    NCK(cudaGetLastError());
    return LH2G_OK;
}

int lh2g_nrc_train_counted(lh2g_nrc* c, const float* queries, const float* targets, const uint32_t* countDevice, long long maxCount, void* stream) {
    if (!c || !countDevice || maxCount <= 0 || !queries || !targets) return LH2G_ERR_INVALID;
    cudaSetDevice(c->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : c->st;
    const int r = train_launch(c, queries, targets, maxCount, countDevice, st);
    return r != LH2G_OK ? r : adam_launch(c, st, countDevice);
}

int lh2g_nrc_last_loss(lh2g_nrc* c, float* loss) {
    if (!c || !loss) return LH2G_ERR_INVALID;
    cudaSetDevice(c->device);
    NCK(cudaDeviceSynchronize());   /* training may have run on any stream */
    NCK(cudaMemcpy(loss, c->dLoss, 4, cudaMemcpyDeviceToHost));
    uint32_t e = 0;
    NCK(cudaMemcpy(&e, c->dErr, 4, cudaMemcpyDeviceToHost));
    if (e) return nfail(c, LH2G_ERR_CUDA, "radiance cache: a tensor-core completion wait ran out");
    return LH2G_OK;
}

int lh2g_nrc_train(lh2g_nrc* c, const float* queries, const float* targets, long long n, int update, float* lossOut, void* stream) {
    if (!c || n <= 0 || !queries || !targets) return LH2G_ERR_INVALID;
    cudaSetDevice(c->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : c->st;
    int r0 = train_launch(c, queries, targets, n, nullptr, st);
    if (r0 != LH2G_OK) return r0;
    if (update) {
        const int r = adam_launch(c, st, nullptr);
        if (r != LH2G_OK) return r;
    }
    if (lossOut) {
        NCK(cudaMemcpyAsync(lossOut, c->dLoss, 4, cudaMemcpyDeviceToHost, st));
        NCK(cudaStreamSynchronize(st));
        uint32_t e = 0;
        NCK(cudaMemcpy(&e, c->dErr, 4, cudaMemcpyDeviceToHost));
        if (e) return nfail(c, LH2G_ERR_CUDA, "radiance cache: a tensor-core completion wait ran out");
    }
    return LH2G_OK;
}

int lh2g_nrc_wait_selftest(int device, uint32_t limit, uint32_t* status) {
    if (!status || limit == 0) return LH2G_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return LH2G_ERR_CUDA;
    uint32_t* d = nullptr;
    if (cudaMalloc((void**)&d, 4) != cudaSuccess) return LH2G_ERR_OOM;
    bool ok = cudaMemset(d, 0, 4) == cudaSuccess;
    if (ok) {
        k_wait_probe<<<1, 32>>>(limit, d);
        ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess;
    }
    ok = ok && cudaMemcpy(status, d, 4, cudaMemcpyDeviceToHost) == cudaSuccess;
    cudaFree(d);
    return ok ? LH2G_OK : LH2G_ERR_CUDA;
}

/* host-memory forms (tests, small batches): copy in, run on the cache's stream, copy out */
int lh2g_nrc_infer_host(lh2g_nrc* c, const float* queries, long long n, float* out) {
    if (!c || n <= 0 || !queries || !out) return LH2G_ERR_INVALID;
    cudaSetDevice(c->device);
    float *dq = nullptr, *dout = nullptr;
    NCK(cudaMalloc((void**)&dq, sizeof(float) * 16 * (size_t)n));
    if (cudaMalloc((void**)&dout, sizeof(float) * 4 * (size_t)n) != cudaSuccess) { cudaFree(dq); return nfail(c, LH2G_ERR_OOM, "infer_host"); }
    int r = LH2G_OK;
    if (cudaMemcpy(dq, queries, sizeof(float) * 16 * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess) r = LH2G_ERR_CUDA;
    if (r == LH2G_OK) r = lh2g_nrc_infer(c, dq, n, dout, nullptr);
    if (r == LH2G_OK) r = check_errors(c);
    if (r == LH2G_OK && cudaMemcpy(out, dout, sizeof(float) * 4 * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess) r = LH2G_ERR_CUDA;
    cudaFree(dq), cudaFree(dout);
    return r;
}

int lh2g_nrc_train_host(lh2g_nrc* c, const float* queries, const float* targets, long long n, int update, float* lossOut) {
    if (!c || n <= 0 || !queries || !targets) return LH2G_ERR_INVALID;
    cudaSetDevice(c->device);
    float *dq = nullptr, *dt = nullptr;
    NCK(cudaMalloc((void**)&dq, sizeof(float) * 16 * (size_t)n));
    if (cudaMalloc((void**)&dt, sizeof(float) * 4 * (size_t)n) != cudaSuccess) { cudaFree(dq); return nfail(c, LH2G_ERR_OOM, "train_host"); }
    int r = LH2G_OK;
    if (cudaMemcpy(dq, queries, sizeof(float) * 16 * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dt, targets, sizeof(float) * 4 * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess)
        r = LH2G_ERR_CUDA;
    float loss = 0.0f;
    if (r == LH2G_OK) r = lh2g_nrc_train(c, dq, dt, n, update, &loss, nullptr);
    if (r == LH2G_OK && lossOut) *lossOut = loss;
    cudaFree(dq), cudaFree(dt);
    return r;
}

}  // extern "C"

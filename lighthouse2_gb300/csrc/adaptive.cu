/* adaptive.cu - the device stages of a PrimeAdaptive frame (lib/RenderCore_PrimeAdaptive/rendercore.cpp:600-755).
 *
 * Between its two wave loops the reference core estimates each pixel's variance (estimateVarianceKernel,
 * lib/CUDA/shared_kernel_code/finalize_shared.h:97-151), lets up to 24 threads per pixel ask for one more sample each
 * (generateEyeRaysKernelAdaptive, kernels/camera.h:96-139: sample S when !(S > deviation)), caps the total at the
 * frame's W*H*spp paths, steers devScale towards 91-98 % of that budget on the host (rendercore.cpp:670-680), and after
 * the second loop adds each pixel's samples, divided by their count, to the accumulator (finalizeASRenderKernel,
 * finalize_shared.h:71-93). Here all of it stays on the device:
 *   k_ad_estimate   the variance estimate, each pixel's sample count, a histogram of the counts
 *   k_ad_budget     one thread: the budget cap, the devScale step (kept on the device for the next frame), and where
 *                   the cap cuts: the reference's compaction atomics keep the first budget-many requests in their
 *                   order of arrival; this core keeps the first in thread order (thread = pixel + (S - 1) * W*H), i.e.
 *                   every request with S below S*, and those with S = S* of the first `room` pixels asking for it
 *   k_ad_flag/k_ad_kept + two exclusive scans   per pixel its kept count and its first second-wave slot
 *   k_ad_generate   the kept primary rays, slot order = pixel order, S ascending within a pixel
 *   k_ad_finalize   per pixel: each sample layer's first-wave sum plus its second-wave paths (S order), the layers
 *                   summed, divided by their sample count, added to the accumulator; the frame
 * The second wave's paths shade as their sample layer (pixel + (S % spp) * W*H) but accumulate into their own slot,
 * so paths that share a layer never write the same memory.
 */
#include "kernels.cuh"
#include "wavefront.cuh"

namespace lh2g {

namespace {

/* estimateVarianceKernel for pixel (x, y) over the first wave's sample layers (powf(x, 2) written as x * x) */
__device__ float estimate_variance(const float4* __restrict__ acc, const float4* __restrict__ features, const int x, const int y, const int W,
                                   const int H, const int spp) {
    const int64_t WH = (int64_t)W * H;
    const float x1 = (float)max(0, x - 4), y1 = (float)max(0, y - 4), x2 = (float)min(W - 1, x + 4), y2 = (float)min(H - 1, y + 4);
    float3 total = mk3(0);
    float weightSum = 0;
    for (int i = 0; i < spp; i++) {
        const float3 Nlocal = UnpackNormal2(__float_as_uint(__ldg(&features[x + (int64_t)y * W + i * WH].w)));
        for (int v = (int)y1; v <= y2; v++)
            for (int u = (int)x1; u <= x2; u++) {
                const int64_t a = u + (int64_t)v * W + i * WH;
                const float4 feature = __ldg(features + a);
                const float3 normal = UnpackNormal2(__float_as_uint(feature.w));
                const float3 albedo = xyz(feature);
                const float3 smp = xyz(__ldg(acc + a));
                const float3 lighting = make_float3(smp.x / fmaxf(albedo.x, 0.001f), smp.y / fmaxf(albedo.y, 0.001f), smp.z / fmaxf(albedo.z, 0.001f));
                const uint32_t dx = (uint32_t)abs(x - u), dy = (uint32_t)abs(y - v);
                const float xweight = dx == 1 ? 0.9f : (dx == 2 ? 0.75f : (dx == 3 ? 0.55f : (dx == 4 ? 0.35f : 1.0f)));
                const float yweight = dy == 1 ? 0.9f : (dy == 2 ? 0.75f : (dy == 3 ? 0.55f : (dy == 4 ? 0.35f : 1.0f)));
                const float c = fmaxf(0.0001f, dot(normal, Nlocal));
                const float weight = xweight * yweight * (c * c);
                weightSum += weight;
                total = total + lighting * weight;
            }
    }
    const float3 average = total * (1.0f / weightSum);
    float variance = 0;
    for (int i = 0; i < spp; i++) {
        const int64_t a = x + (int64_t)y * W + i * WH;
        const float3 albedo = xyz(__ldg(features + a));
        const float3 smp = xyz(__ldg(acc + a));
        const float3 lighting = make_float3(smp.x / fmaxf(albedo.x, 0.001f), smp.y / fmaxf(albedo.y, 0.001f), smp.z / fmaxf(albedo.z, 0.001f));
        const float d = Luminance(lighting) - Luminance(average);
        variance += d * d;
    }
    variance /= 3.0f * (float)spp;
    return (variance + EPSILON) / (Luminance(average) + EPSILON);
}

__global__ void __launch_bounds__(256) k_ad_estimate(const FrameGPU F, const float4* __restrict__ acc, const float4* __restrict__ features,
                                                     float* __restrict__ deviation, uint32_t* __restrict__ want, AdaptiveState* state) {
    __shared__ uint32_t hist[25];
    if (threadIdx.x < 25) hist[threadIdx.x] = 0;
    __syncthreads();
    const int64_t WH = (int64_t)F.W * F.H;
    const int64_t px = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (px < WH) {
        const float d = estimate_variance(acc, features, (int)(px % F.W), (int)(px / F.W), F.W, F.H, F.spp) * state->devScale;
        deviation[px] = d;
        uint32_t c = 0;
        for (uint32_t S = 1; S <= 24; S++) if (!((float)S > d)) c = S;   /* the threads of a pixel that generate a ray */
        want[px] = c;
        atomicAdd(&hist[c], 1u);
    }
    __syncthreads();
    if (threadIdx.x < 25 && hist[threadIdx.x]) atomicAdd(&state->hist[threadIdx.x], hist[threadIdx.x]);
}

/* one thread: the budget cap, the devScale step (rendercore.cpp:670-680) and where the cap cuts the requests */
__global__ void k_ad_budget(const FrameGPU F, AdaptiveState* state) {
    if (threadIdx.x || blockIdx.x) return;
    unsigned long long total = 0;
    for (int k = 1; k <= 24; k++) total += (unsigned long long)k * state->hist[k];
    const float budget = (float)(F.W * F.H * F.spp);
    uint32_t pathCount = (uint32_t)total;
    if ((float)pathCount > budget) pathCount = (uint32_t)budget;
    float ds = state->devScale;
    const float fc = (float)pathCount;
    if (fc > 0.98f * budget) ds *= 0.92f;
    else if (fc > 0.96f * budget) ds *= 0.98f;
    else if (fc < 0.91f * budget) ds *= 1.08f;
    else if (fc < 0.94f * budget) ds *= 1.02f;
    state->devScale = ds;
    state->requested = (uint32_t)total;
    state->pathCount = pathCount;
    uint32_t sStar = 25, room = 0;
    if (total > pathCount) {
        unsigned long long before = 0;
        for (uint32_t S = 1; S <= 24; S++) {
            unsigned long long n = 0;   /* pixels asking for sample S */
            for (uint32_t k = S; k <= 24; k++) n += state->hist[k];
            if (before + n > pathCount) { sStar = S, room = (uint32_t)(pathCount - before); break; }
            before += n;
        }
    }
    state->sStar = sStar, state->room = room;
}

__global__ void k_ad_flag(const int64_t n, const uint32_t* __restrict__ want, uint32_t* __restrict__ flag, const AdaptiveState* state) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flag[i] = want[i] >= state->sStar ? 1u : 0u;
}
__global__ void k_ad_kept(const int64_t n, const uint32_t* __restrict__ want, const uint32_t* __restrict__ rank, uint32_t* __restrict__ kept,
                          const AdaptiveState* state) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t w = want[i], s = state->sStar;
    kept[i] = w < s ? w : s - 1u + (rank[i] < state->room ? 1u : 0u);
}

/* exclusive scan of n <= 2^26 uint32: 4096 per block (1024 threads x 4), the block sums scanned by one block of
 * 1024 threads (16 per thread), then added back */
constexpr int SCAN_BLOCK = 1024, SCAN_ITEMS = 4, SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warpSums[32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if ((int)lane >= o) x += y;
    }
    if (lane == 31) warpSums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (blockDim.x >> 5) ? warpSums[lane] : 0u;
        const uint32_t w0 = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if ((int)lane >= o) w += y;
        }
        warpSums[lane] = w - w0;
        if (lane == 31) *total = w;
    }
    __syncthreads();
    const uint32_t r = x - v + warpSums[warp];
    __syncthreads();
    return r;
}
__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_tiles(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint32_t* __restrict__ sums,
                                                          const int64_t n) {
    __shared__ uint32_t tot;
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS], s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) v[k] = base + k < n ? in[base + k] : 0u, s += v[k];
    uint32_t run = block_exclusive_scan(s, &tot);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}
__global__ void __launch_bounds__(SCAN_BLOCK) k_scan_sums(uint32_t* sums, const int tiles) {
    __shared__ uint32_t tot;
    constexpr int PER = 16;
    uint32_t v[PER], s = 0;
    const int base = threadIdx.x * PER;
#pragma unroll
    for (int k = 0; k < PER; k++) v[k] = base + k < tiles ? sums[base + k] : 0u, s += v[k];
    uint32_t run = block_exclusive_scan(s, &tot);
#pragma unroll
    for (int k = 0; k < PER; k++) {
        if (base + k < tiles) sums[base + k] = run;
        run += v[k];
    }
}
__global__ void k_scan_add(uint32_t* __restrict__ out, const uint32_t* __restrict__ sums, const int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += sums[i / SCAN_TILE];
}

/* the second wave's primary rays: pixel px's kept samples S = 1..kept[px] in slots first[px] + S - 1 */
__global__ void __launch_bounds__(256) k_ad_generate(const SceneGPU S, const FrameGPU F, const WaveBuffers B, const uint32_t* __restrict__ kept,
                                                     const uint32_t* __restrict__ first, uint32_t* __restrict__ slotLayer, const uint32_t R1) {
    const int64_t WH = (int64_t)F.W * F.H;
    const int64_t px = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (px >= WH) return;
    const uint32_t k = kept[px], f = first[px];
    const int sx = (int)(px % F.W), sy = (int)(px / F.W);
    for (uint32_t s = 1; s <= k; s++) {
        const uint32_t slot = f + s - 1;
        const uint32_t thread = (uint32_t)(px + (int64_t)(s - 1) * WH);
        float3 O, D;
        primary_adaptive(S, F, sx, sy, s + F.pass, thread, R1, O, D);   /* sample index S + spp + samplesTaken (F.pass of the second wave) */
        B.O[0][slot] = make_float4(O.x, O.y, O.z, __uint_as_float((slot << 6) | S_SPECULAR | MIS_TMIN_EPS));
        B.D[0][slot] = make_float4(D.x, D.y, D.z, __uint_as_float(0u));
        B.T[0][slot] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
        B.pathAcc[slot] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        slotLayer[slot] = (uint32_t)(px + (int64_t)(s % (uint32_t)F.spp) * WH);
    }
}

/* finalizeASRenderKernel after both waves: accum += (sum of the sample layers) / their sample count */
__global__ void __launch_bounds__(256) k_ad_finalize(const FrameGPU F, const float4* __restrict__ layers, const float4* __restrict__ extra,
                                                     const uint32_t* __restrict__ kept, const uint32_t* __restrict__ first, float4* __restrict__ accum,
                                                     float4* __restrict__ frame, const float scale, const int overwrite) {
    const int64_t WH = (int64_t)F.W * F.H;
    const int64_t px = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (px >= WH) return;
    const uint32_t k = kept[px], f = first[px];
    float4 q = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int i = 0; i < F.spp; i++) {
        float4 v = layers[px + i * WH];
        for (uint32_t s = 1; s <= k; s++)
            if (s % (uint32_t)F.spp == (uint32_t)i) v = v + extra[f + s - 1];
        q = q + v;
    }
    const float4 add = q * (1.0f / q.w);
    float4 a = overwrite ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : accum[px];
    a = a + add;
    accum[px] = a;
    frame[px] = a * scale;
}

}  // namespace

void launch_adaptive_estimate(const FrameGPU& F, const WaveBuffers& B, float* deviation, uint32_t* want, AdaptiveState* state, cudaStream_t st) {
    const int64_t WH = (int64_t)F.W * F.H;
    k_ad_estimate<<<(unsigned)((WH + 255) / 256), 256, 0, st>>>(F, B.pathAcc, B.misFeatures, deviation, want, state);
    k_ad_budget<<<1, 32, 0, st>>>(F, state);
}

void exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t* sums, const int64_t n, cudaStream_t st) {
    const int tiles = (int)((n + SCAN_TILE - 1) / SCAN_TILE);
    k_scan_tiles<<<tiles, SCAN_BLOCK, 0, st>>>(in, out, sums, n);
    k_scan_sums<<<1, SCAN_BLOCK, 0, st>>>(sums, tiles);
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, sums, n);
}

void launch_adaptive_keep(const FrameGPU& F, const uint32_t* want, uint32_t* tmp, uint32_t* rank, uint32_t* kept, uint32_t* first, uint32_t* sums,
                          const AdaptiveState* state, cudaStream_t st) {
    const int64_t WH = (int64_t)F.W * F.H;
    const unsigned blocks = (unsigned)((WH + 255) / 256);
    k_ad_flag<<<blocks, 256, 0, st>>>(WH, want, tmp, state);
    exclusive_scan(tmp, rank, sums, WH, st);
    k_ad_kept<<<blocks, 256, 0, st>>>(WH, want, rank, kept, state);
    exclusive_scan(kept, first, sums, WH, st);
}

void launch_adaptive_generate(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, const uint32_t* kept, const uint32_t* first,
                              uint32_t* slotLayer, uint32_t R1, cudaStream_t st) {
    const int64_t WH = (int64_t)F.W * F.H;
    k_ad_generate<<<(unsigned)((WH + 255) / 256), 256, 0, st>>>(S, F, B, kept, first, slotLayer, R1);
}

void launch_adaptive_finalize(const FrameGPU& F, const float4* layers, const float4* extra, const uint32_t* kept, const uint32_t* first, float4* accum,
                              float4* frame, float scale, int overwrite, cudaStream_t st) {
    const int64_t WH = (int64_t)F.W * F.H;
    k_ad_finalize<<<(unsigned)((WH + 255) / 256), 256, 0, st>>>(F, layers, extra, kept, first, accum, frame, scale, overwrite);
}

}  // namespace lh2g

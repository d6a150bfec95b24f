/* svgf.cu - spatiotemporal variance-guided filtering of a filter-core frame on the GB300.
 *
 * The pass sequence of lib/RenderCore_Optix7Filter/rendercore.cpp:904-935 over the kernels of
 * lib/CUDA/shared_kernel_code/finalize_shared.h:
 *   prepare    demodulate direct / indirect light by the albedo, clamp, reproject (analytic for diffuse pixels,
 *              diamond search for specular ones), temporal luminance moments, history count   (:169-291)
 *   apply 1-3  5x5 a-trous (corners cut) at steps 1, 2, 4 with normal, depth, material and luminance stops;
 *              phase 1 blends with the clamped history, phase 3 remodulates and takes the square root (:320-476)
 *   taa        Mitchell-Netravali history read, YCoCg clamp at +-1.25 sigma                  (:498-539)
 *   unsharpen  sharpen and square into the frame, border pixels untouched                     (:553-576)
 *   or finalizeNoTAA                                                                          (:587-595)
 * One thread per pixel; 32 x 8 blocks so that a warp reads one row segment of every buffer (coalesced 128-bit
 * loads) and the a-trous neighbourhoods of a block overlap in L1. Everything is HBM / L2 bound: per pass each
 * pixel reads a few float4 of its own and hits cache for its neighbours.
 * The TAA pass reads the phase-3 image and writes a separate buffer: the reference updates its input in place
 * while neighbouring threads still read it.
 */
#include "fp_exact.h"
#include "svgf.cuh"

namespace lh2g {
namespace {

constexpr int BX = 32, BY = 8;

/* w * 0.0001 rounded as the reference's float * double product; out of line so that only warps with a lane
 * on a material edge execute it (inlined, it is if-converted into every tap) */
__device__ __noinline__ float material_stop(const float w) { return mul_float_by_double(w, DBL_1EM4_MANT, DBL_1EM4_EXP); }

struct Px {
    int x, y;
    size_t i;
};
__device__ __forceinline__ bool pixel(const int W, const int H, Px& p) {
    p.x = threadIdx.x + blockIdx.x * blockDim.x;
    p.y = threadIdx.y + blockIdx.y * blockDim.y;
    p.i = (size_t)p.x + (size_t)p.y * W;
    return p.x < W && p.y < H;
}

/* ---- reprojection helpers (finalize_shared.h:169-215, sampling_shared.h:111-220) ---- */
struct Reproject {
    const float4* __restrict__ prevWorldPos;
    int w, h;
    __device__ float4 world(int x, int y) const {
        if (x >= 0 && y >= 0 && x < w && y < h) return __ldg(prevWorldPos + (size_t)x + (size_t)y * w);
        return make_float4(1e20f, 1e20f, 1e20f, __uint_as_float(0));
    }
    __device__ float WorldDistance(int px, int py, const float4& cur) const {
        const float4 p = world(px, py);
        const float3 localNormal = UnpackNormal2(__float_as_uint(cur.w)), prevNormal = UnpackNormal2(__float_as_uint(p.w));
        if ((__float_as_uint(p.w) & 3u) != 1u) return 1e21f;   /* only specular pixels are searched */
        if (dot(localNormal, prevNormal) < 0.85f) return 1e21f;
        return length(xyz(cur - p));
    }
    __device__ float FineWorldDistance(const float2 pixel, const float4& cur) const {
        const int x0 = f2i(pixel.x), y0 = f2i(pixel.y);
        const float fx = pixel.x - floorf(pixel.x), fy = pixel.y - floorf(pixel.y);
        const float w0 = (1 - fx) * (1 - fy), w1 = fx * (1 - fy), w2 = (1 - fx) * fy, w3 = fx * fy;
        const float d0 = WorldDistance(x0, y0, cur), d1 = WorldDistance(x0 + 1, y0, cur);
        const float d2 = WorldDistance(x0, y0 + 1, cur), d3 = WorldDistance(x0 + 1, y0 + 1, cur);
        float totalWeight = 0, totalDist = 0;
        if (d0 < 1e20f) totalDist += d0 * w0, totalWeight += w0;
        if (d1 < 1e20f) totalDist += d1 * w1, totalWeight += w1;
        if (d2 < 1e20f) totalDist += d2 * w2, totalWeight += w2;
        if (d3 < 1e20f) totalDist += d3 * w3, totalWeight += w3;
        return totalWeight == 0 ? 1e20f : totalDist / totalWeight;
    }
    __device__ int RefineHistoryPos(float2& pos, const float2 offset, const float4& cur, float& bestDist, const float step) const {
        int bestTap = 0;
        const float2 c0 = make_float2(pos.x - step, pos.y), c1 = make_float2(pos.x + step, pos.y);
        const float2 c2 = make_float2(pos.x, pos.y - step), c3 = make_float2(pos.x, pos.y + step);
        float d;
        d = FineWorldDistance(c0 + offset, cur); if (d < bestDist) bestDist = d, pos = c0, bestTap = 1;
        d = FineWorldDistance(c1 + offset, cur); if (d < bestDist) bestDist = d, pos = c1, bestTap = 2;
        d = FineWorldDistance(c2 + offset, cur); if (d < bestDist) bestDist = d, pos = c2, bestTap = 3;
        d = FineWorldDistance(c3 + offset, cur); if (d < bestDist) bestDist = d, pos = c3, bestTap = 4;
        return bestTap;
    }
    /* bilinear weights of the 2x2 block ending at (floor u, floor v); taps whose normal (dot < minDot) or
     * specularity disagree with the pixel get weight 0; returns false when no tap qualifies */
    __device__ bool taps(const float4& localPos, const float3& localNormal, float u, float v, float minDot, size_t a[4], float wt[4],
                         float& sum) const {
        const int iu1 = f2i(floorf(u)), iv1 = f2i(floorf(v)), iu0 = max(0, iu1 - 1), iv0 = max(0, iv1 - 1);
        if (iu1 >= w || iv1 >= h || iu1 < 0 || iv1 < 0) return false;
        const float fu = u - floorf(u), fv = v - floorf(v);
        a[0] = (size_t)iu0 + (size_t)iv0 * w, a[1] = (size_t)iu1 + (size_t)iv0 * w;
        a[2] = (size_t)iu0 + (size_t)iv1 * w, a[3] = (size_t)iu1 + (size_t)iv1 * w;
        const uint32_t spec = __float_as_uint(localPos.w) & 3u;
        wt[0] = (1 - fu) * (1 - fv), wt[1] = fu * (1 - fv), wt[2] = (1 - fu) * fv, wt[3] = 1 - (wt[0] + wt[1] + wt[2]);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint32_t n = __float_as_uint(__ldg(&prevWorldPos[a[k]].w));
            if (dot(UnpackNormal2(n), localNormal) < minDot || (n & 3u) != spec) wt[k] = 0;
        }
        sum = wt[0] + wt[1] + wt[2] + wt[3];
        return sum != 0;
    }
};

/* ---- prepareFilterKernel ---- */
__global__ void __launch_bounds__(BX* BY) k_prepare(const SvgfBuffers b, const SvgfArgs a) {
    Px p;
    if (!pixel(a.W, a.H, p)) return;
    const size_t WH = (size_t)a.W * a.H;
    uint4 feature = b.features[p.i];
    const float3 direct = xyz(__ldg(b.accum + p.i)) * a.scale;
    const float4 localWorldPos = __ldg(b.worldPos + p.i);
    const float3 albedo = RGB32toHDRmin1(feature.x);
    const float3 indirect = xyz(__ldg(b.accum + p.i + WH)) * a.scale;
    const float3 reciAlbedo = make_float3(1.0f / albedo.x, 1.0f / albedo.y, 1.0f / albedo.z);
    const float3 directLight = fmin3(direct * reciAlbedo, a.clampDirect);
    const float3 indirectLight = fmin3(indirect * reciAlbedo, a.clampIndirect);
    b.shading[p.i] = CombineToFloat4(directLight, indirectLight);
    float lumDirect = Luminance(directLight), lumDirect2 = lumDirect * lumDirect;
    float lumIndirect = Luminance(indirectLight), lumIndirect2 = lumIndirect * lumIndirect;
    const Reproject R{b.prevWorldPos, a.W, a.H};
    float2 prevPixelPos;
    if (((feature.w >> 4) & 3u) == 0) {
        /* diffuse: project the world position into the previous camera */
        const SvgfView& V = a.view;
        const float3 dd = normalize(xyz(localWorldPos - V.prevPos));
        const float4 D = make_float4(dd.x, dd.y, dd.z, 0);
        const float3 ss = xyz(V.prevPos) + xyz(D) * (V.prevPos.w / dot4(V.prevE, D));
        const float4 S = make_float4(ss.x, ss.y, ss.z, 0);
        prevPixelPos = make_float2(dot4(S, V.prevRight) - V.prevRight.w - a.j0, dot4(S, V.prevUp) - V.prevUp.w - a.j1);
    } else {
        prevPixelPos = make_float2((float)p.x, (float)p.y);
        if (!a.camIsStationary) {
            /* specular: diamond search, at most 25 refinements */
            float bestDist = length(xyz(localWorldPos - __ldg(b.prevWorldPos + p.i))), stepSize = 5.0f;
            const float2 offset = make_float2(a.j0 - a.prevj0, a.j1 - a.prevj1);
            for (int iter = 0; iter < 25; iter++) {
                const int tap = R.RefineHistoryPos(prevPixelPos, offset, localWorldPos, bestDist, stepSize);
                if (tap == 0) { stepSize *= 0.45f; if (stepSize < 0.05f) break; }
            }
        }
    }
    prevPixelPos = prevPixelPos + make_float2(0.5f, 0.5f);
    const float ppx = prevPixelPos.x, ppy = prevPixelPos.y;
    bool hit = false;
    if (ppx >= 0 && ppx < (float)a.W && ppy >= 0 && ppy < (float)a.H) {
        const float3 localNormal = UnpackNormal2(feature.y);
        size_t t[4];
        float wt[4], sum;
        if (R.taps(localWorldPos, localNormal, ppx, ppy, 0.95f, t, wt, sum)) {
            const float4 h = (wt[0] * __ldg(b.prevMoments + t[0]) + wt[1] * __ldg(b.prevMoments + t[1]) + wt[2] * __ldg(b.prevMoments + t[2]) +
                              wt[3] * __ldg(b.prevMoments + t[3])) * (1.0f / sum);
            if (h.x > -1) {
                lumDirect = 0.2f * lumDirect + 0.8f * h.x;
                lumDirect2 = 0.2f * lumDirect2 + 0.8f * h.y;
                lumIndirect = 0.2f * lumIndirect + 0.8f * h.z;
                lumIndirect2 = 0.2f * lumIndirect2 + 0.8f * h.w;
                if ((feature.w & 15u) < 15u) feature.w++;
                hit = true;
            }
        }
    }
    if (!hit) feature.w &= 0xfffffff0u;
    b.features[p.i].w = feature.w;
    b.motion[p.i] = prevPixelPos;
    b.moments[p.i] = make_float4(lumDirect, lumDirect2, lumIndirect, lumIndirect2);
}

/* ---- applyFilterKernel ---- */
#ifndef LH2G_SVGF_UNROLL
#define LH2G_SVGF_UNROLL 0   /* tuning switch: 0 rolled tap loops, 1 inner loop unrolled, 2 both unrolled */
#endif
/* The neighbours of a block's pixels (the block and a halo of 2 steps) are unpacked once per block into shared
 * memory, four float4 per pixel: normal + depth, albedo + material id, direct light + its luminance, indirect light
 * + its luminance; the taps read them there (unpacked per tap, the 20 taps of a pixel repeat the work of their
 * neighbours). Columns are clamped to the image as the taps clamp them; rows outside the image are loaded clamped
 * and never read. */
template <int PHASE>
struct ApplyTile {
    static constexpr int STEP = 1 << (PHASE - 1), TW = BX + 4 * STEP, TH = BY + 4 * STEP, N = TW * TH;
    static constexpr size_t BYTES = 4 * sizeof(float4) * N;
};

template <int PHASE>
__global__ void __launch_bounds__(BX* BY) k_apply(const SvgfBuffers b, const SvgfArgs a, const float4* __restrict__ A, const float4* __restrict__ B,
                                                  float4* __restrict__ C) {
    using T = ApplyTile<PHASE>;
    extern __shared__ float4 tile[];
    float4 *tN = tile, *tA = tile + T::N, *tD = tile + 2 * T::N, *tI = tile + 3 * T::N;
    const int x0 = (int)(blockIdx.x * BX) - 2 * T::STEP, y0 = (int)(blockIdx.y * BY) - 2 * T::STEP;
    for (int t = threadIdx.y * BX + threadIdx.x; t < T::N; t += BX * BY) {
        const int u = min(max(x0 + t % T::TW, 0), a.W - 1), v = min(max(y0 + t / T::TW, 0), a.H - 1);
        const size_t q = (size_t)u + (size_t)v * a.W;
        const uint4 nf = __ldg(b.features + q);
        const float4 nc = __ldg(A + q);
        const float3 n = UnpackNormal2(nf.y), al = RGB32toHDR(nf.x), di = GetDirect(nc), in = GetIndirect(nc);
        tN[t] = make_float4(n.x, n.y, n.z, __uint_as_float(nf.z));
        tA[t] = make_float4(al.x, al.y, al.z, __uint_as_float(nf.w >> 4));
        tD[t] = make_float4(di.x, di.y, di.z, Luminance(di));
        tI[t] = make_float4(in.x, in.y, in.z, Luminance(in));
    }
    __syncthreads();
    Px p;
    if (!pixel(a.W, a.H, p)) return;
    const int w = a.W, h = a.H, x = p.x, y = p.y;
    const uint4 lf = __ldg(b.features + p.i);
    const float3 localNormal = UnpackNormal2(lf.y);
    const float3 localColor = RGB32toHDR(lf.x);
    const uint32_t localMatID = lf.w >> 4;
    float directWeightSum = 1, indirectWeightSum = 1;
    const float4 own = __ldg(A + p.i);
    float3 directSum = directWeightSum * GetDirect(own);
    float3 indirectSum = indirectWeightSum * GetIndirect(own);
    const float localDirect = Luminance(GetDirect(own)), localIndirect = Luminance(GetIndirect(own));
    const float localDepth = __uint_as_float(lf.z);
    const float4 dd = __ldg(b.deltaDepth + p.i);
    const float localDdx = dd.z, localDdy = dd.w;
    const float sigma = 10.0f * oneoverpow2(PHASE - 1);
    const float factor = (lf.w & 15u) == 0 ? 400.0f : 1.0f;
    const float4 m = __ldg(b.moments + p.i);
    const float var_dir = m.y - m.x * m.x, var_ind = m.w - m.z * m.z;
    const float rdir = -1.0f / (sigma * factor * sqrtf(var_dir + 0.00001f) + 0.00001f);
    const float rind = -1.0f / (sigma * factor * sqrtf(var_ind + 0.00001f) + 0.00001f);
    constexpr int step = 1 << (PHASE - 1);
    /* the tap loops stay rolled (LH2G_SVGF_UNROLL 0): unrolled, the 20 tap bodies overflow the instruction cache
     * and warps stall on instruction fetch */
#if LH2G_SVGF_UNROLL >= 2
#pragma unroll
#else
#pragma unroll 1
#endif
    for (int vv = -2; vv <= 2; vv++) {
        const int v = vv * step + y;
        const int r = (vv == 2 || vv == -2) ? 1 : 2;
        if (v < 0 || v >= h) continue;
#if LH2G_SVGF_UNROLL >= 1
#pragma unroll
#else
#pragma unroll 1
#endif
        for (int uu = -2; uu <= 2; uu++) {
            if (uu < -r || uu > r || (uu == 0 && vv == 0)) continue;
            /* the tap's column, clamped to the image, is tile column x - x0 + uu * step (the tile holds clamped columns) */
            const int t = (x - x0 + uu * step) + (v - y0) * T::TW;
            const float4 tn = tN[t], ta = tA[t], td = tD[t], ti = tI[t];
            const float w_dist = (float)(uu * uu + vv * vv) * (-1.0f / 7.5f);
            const float3 nDirect = make_float3(td.x, td.y, td.z), nIndirect = make_float3(ti.x, ti.y, ti.z);
            float w_normal = pow128(fmaxf(0.0f, dot(make_float3(tn.x, tn.y, tn.z), localNormal)));
            const float expected = localDepth + localDdx * (float)(uu * step) + localDdy * (float)(vv * step);
            const float depthError = fabsf(expected - tn.w);
            const float expectedDifference = fabsf(expected - localDepth);
            const float w_depth = depthError / fmaxf(0.00001f, (0.5f + (float)PHASE * 0.5f) * expectedDifference);
            /* material stop: the reference multiplies by the double literal 0.0001 here, i.e. in double; the same
             * float comes from exact integer arithmetic (no FP64 instruction) */
            if (__float_as_uint(ta.w) != localMatID) w_normal = material_stop(w_normal);
            else w_normal = w_normal * dot(localColor, make_float3(ta.x, ta.y, ta.z));
            float w_dir = w_normal * exp_cw(fabsf(localDirect - td.w) * rdir + w_dist - w_depth);
            float w_ind = w_normal * exp_cw(fabsf(localIndirect - ti.w) * rind + w_dist - w_depth);
            if (!isfinite(w_dir)) w_dir = 0;
            if (!isfinite(w_ind)) w_ind = 0;
            directSum = directSum + nDirect * w_dir, directWeightSum += w_dir;
            indirectSum = indirectSum + nIndirect * w_ind, indirectWeightSum += w_ind;
        }
    }
    float3 directFiltered = directSum * (1.0f / fmaxf(0.0001f, directWeightSum));
    float3 indirectFiltered = indirectSum * (1.0f / fmaxf(0.0001f, indirectWeightSum));
    if (PHASE == 1) {
        const float2 mv = __ldg(b.motion + p.i);
        const int ix = f2i(mv.x), iy = f2i(mv.y);
        const Reproject R{b.prevWorldPos, w, h};
        size_t t[4];
        float wt[4], sum;
        if (ix >= 0 && ix < w && iy >= 0 && iy < h && R.taps(__ldg(b.worldPos + p.i), localNormal, mv.x, mv.y, 0.975f, t, wt, sum)) {
            float3 prevDirect = wt[0] * GetDirect(__ldg(B + t[0])), prevIndirect = wt[0] * GetIndirect(__ldg(B + t[0]));
#pragma unroll
            for (int k = 1; k < 4; k++) {
                const float4 hb = __ldg(B + t[k]);
                prevDirect = prevDirect + wt[k] * GetDirect(hb), prevIndirect = prevIndirect + wt[k] * GetIndirect(hb);
            }
            prevDirect = RGBToYCoCg(prevDirect * (1.0f / sum)), prevIndirect = RGBToYCoCg(prevIndirect * (1.0f / sum));
            /* neighbourhood clamp in YCoCg, +-0.75 sigma over the 3x3 block of the unfiltered input */
            float3 dirAvg = RGBToYCoCg(directFiltered), dirVar = dirAvg * dirAvg;
            float3 indAvg = RGBToYCoCg(indirectFiltered), indVar = indAvg * indAvg;
            auto add = [&](size_t q) {
                const float4 c4 = __ldg(A + q);
                const float3 f = RGBToYCoCg(GetDirect(c4)), g = RGBToYCoCg(GetIndirect(c4));
                dirAvg = dirAvg + f, dirVar = dirVar + f * f, indAvg = indAvg + g, indVar = indVar + g * g;
            };
            const size_t i = p.i;
            if (x > 1) {
                if (y > 1) add(i - w - 1);
                add(i - 1);
                if (y < h - 1) add(i + w - 1);
            }
            if (y > 1) add(i - w);
            if (y < h - 1) add(i + w);
            if (x < w - 1) {
                if (y > 1) add(i + 1 - w);
                add(i + 1);
                if (y < h - 1) add(i + 1 + w);
            }
            dirAvg = dirAvg * (1.0f / 9.0f), dirVar = dirVar * (1.0f / 9.0f), indAvg = indAvg * (1.0f / 9.0f), indVar = indVar * (1.0f / 9.0f);
            float3 sd = fmax3(0.0f, dirVar - dirAvg * dirAvg), si = fmax3(0.0f, indVar - indAvg * indAvg);
            sd = make_float3(sqrtf(sd.x), sqrtf(sd.y), sqrtf(sd.z)), si = make_float3(sqrtf(si.x), sqrtf(si.y), sqrtf(si.z));
            prevDirect = clamp3(prevDirect, dirAvg - 0.75f * sd, dirAvg + 0.75f * sd);
            prevIndirect = clamp3(prevIndirect, indAvg - 0.75f * si, indAvg + 0.75f * si);
            directFiltered = directFiltered * 0.1f + YCoCgToRGB(prevDirect) * 0.9f;
            indirectFiltered = indirectFiltered * 0.1f + YCoCgToRGB(prevIndirect) * 0.9f;
        }
    }
    if (PHASE == 3) {
        const float3 c = (directFiltered + indirectFiltered) * RGB32toHDR(lf.x);
        C[p.i] = make_float4(sqrtf(c.x), sqrtf(c.y), sqrtf(c.z), 1);
    } else {
        C[p.i] = CombineToFloat4(directFiltered, indirectFiltered);
    }
}

/* ---- TAApassKernel: reads 'pixels' and the history, writes 'out' ---- */
__global__ void __launch_bounds__(BX* BY) k_taa(const SvgfBuffers b, const SvgfArgs a, const float4* __restrict__ pixels,
                                                const float4* __restrict__ prev, float4* __restrict__ out) {
    Px p;
    if (!pixel(a.W, a.H, p)) return;
    const int w = a.W, h = a.H, x = p.x, y = p.y;
    float3 px = xyz(__ldg(pixels + p.i));
    const float2 mv = __ldg(b.motion + p.i);
    const float ppx = mv.x - 0.5f, ppy = mv.y - 0.5f;
    if (ppx >= 0 && ppx < (float)w && ppy >= 0 && ppy < (float)h) {
        const float3 newPixel = RGBToYCoCg(px);
        /* ReadTexelBmitchellNetravali (sampling_shared.h:117-134) */
        const int x1 = f2i(ppx - 2.0f), y1 = f2i(ppy - 2.0f);
        float totalWeight = 0;
        float4 total = make_float4(0, 0, 0, 0);
        for (int yy = y1; yy < y1 + 4; yy++)
            for (int xx = x1; xx < x1 + 4; xx++)
                if (xx >= 0 && yy > 0 && xx < w && yy < h) {
                    const float weight = MitchellNetravali((float)xx - ppx) * MitchellNetravali((float)yy - ppy);
                    total = total + __ldg(prev + (size_t)xx + (size_t)yy * w) * weight;
                    totalWeight += weight;
                }
        float3 history = RGBToYCoCg(xyz(total * (1.0f / totalWeight)));
        float3 colorAvg = newPixel, colorVar = newPixel * newPixel;
        auto add = [&](size_t q) { const float3 f = RGBToYCoCg(xyz(__ldg(pixels + q))); colorAvg = colorAvg + f, colorVar = colorVar + f * f; };
        const size_t i = p.i;
        if (x > 1) {
            if (y > 1) add(i - w - 1);
            add(i - 1);
            if (y < h - 1) add(i + w - 1);
        }
        if (y > 1) add(i - w);
        if (y < h - 1) add(i + w);
        if (x < w - 1) {
            if (y > 1) add(i + 1 - w);
            add(i + 1);
            if (y < h - 1) add(i + 1 + w);
        }
        colorAvg = colorAvg * (1.0f / 9.0f), colorVar = colorVar * (1.0f / 9.0f);
        float3 sigma = fmax3(0.0f, colorVar - colorAvg * colorAvg);
        sigma = make_float3(sqrtf(sigma.x), sqrtf(sigma.y), sqrtf(sigma.z));
        history = clamp3(history, colorAvg - 1.25f * sigma, colorAvg + 1.25f * sigma);
        px = YCoCgToRGB(newPixel * 0.1f + history * 0.9f);
        if (isnan(px.x + px.y + px.z)) px = YCoCgToRGB(newPixel);
    }
    const float3 c = fmin3(10.0f, px);
    out[p.i] = make_float4(c.x, c.y, c.z, 0);
}

/* ---- unsharpenTAAKernel: sharpen, square (gamma is applied again downstream) ---- */
__global__ void __launch_bounds__(BX* BY) k_unsharpen(const SvgfArgs a, const float4* __restrict__ pixels, float4* __restrict__ target) {
    Px p;
    if (!pixel(a.W, a.H, p)) return;
    const int w = a.W, x = p.x, y = p.y;
    if (x == 0 || y == 0 || x >= a.W - 1 || y >= a.H - 1) return;
    auto P = [&](int xx, int yy) { return __ldg(pixels + (size_t)xx + (size_t)yy * w); };
    const float4 p0 = P(x - 1, y - 1), p1 = P(x, y - 1), p2 = P(x + 1, y - 1), p3 = P(x + 1, y);
    const float4 p4 = P(x + 1, y + 1), p5 = P(x, y + 1), p6 = P(x - 1, y + 1), p7 = P(x - 1, y);
    const float4 c = P(x, y);
    const float4 blur = 0.35f * p0 + 0.5f * p1 + 0.35f * p2 + 0.5f * p3 + 0.35f * p4 + 0.5f * p5 + 0.35f * p6 + 0.5f * p7;
    const float4 sharp = c * 2.7f - 0.5f * blur;
    const float4 v = make_float4(fmaxf(c.x, sharp.x), fmaxf(c.y, sharp.y), fmaxf(c.z, sharp.z), fmaxf(c.w, sharp.w));
    target[p.i] = make_float4(v.x * v.x, v.y * v.y, v.z * v.z, 0);
}

/* ---- finalizeNoTAAKernel ---- */
__global__ void __launch_bounds__(BX* BY) k_finalize_no_taa(const SvgfArgs a, const float4* __restrict__ pixels, float4* __restrict__ target) {
    Px p;
    if (!pixel(a.W, a.H, p)) return;
    if (p.x == 0 || p.y == 0 || p.x >= a.W - 1 || p.y >= a.H - 1) return;
    const float4 v = __ldg(pixels + p.i);
    target[p.i] = make_float4(sqrtf(v.x), sqrtf(v.y), sqrtf(v.z), 0);
}

}  // namespace

void launch_svgf(const SvgfBuffers& b, const SvgfArgs& a, bool taa, cudaStream_t st) {
    const dim3 block(BX, BY), grid((a.W + BX - 1) / BX, (a.H + BY - 1) / BY);
    k_prepare<<<grid, block, 0, st>>>(b, a);
    static const bool attrs = [] {   /* the phase-3 tile (48 x 24 pixels, 72 KB) exceeds the 48 KB default */
        cudaFuncSetAttribute(k_apply<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ApplyTile<1>::BYTES);
        cudaFuncSetAttribute(k_apply<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ApplyTile<2>::BYTES);
        cudaFuncSetAttribute(k_apply<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ApplyTile<3>::BYTES);
        return true;
    }();
    (void)attrs;
    k_apply<1><<<grid, block, ApplyTile<1>::BYTES, st>>>(b, a, b.shading, b.filteredIN, b.filteredOUT);
    k_apply<2><<<grid, block, ApplyTile<2>::BYTES, st>>>(b, a, b.filteredOUT, nullptr, b.filteredIN);
    k_apply<3><<<grid, block, ApplyTile<3>::BYTES, st>>>(b, a, b.filteredIN, nullptr, b.shading);
    if (taa) {
        k_taa<<<grid, block, 0, st>>>(b, a, b.shading, b.prevPixels, b.taaPixels);
        k_unsharpen<<<grid, block, 0, st>>>(a, b.taaPixels, b.target);
    } else {
        k_finalize_no_taa<<<grid, block, 0, st>>>(a, b.shading, b.target);
    }
}

}  // namespace lh2g

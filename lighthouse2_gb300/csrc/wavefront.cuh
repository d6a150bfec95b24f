/* wavefront.cuh - per-path device code shared by the frame kernels (kernels.cu) and the serving loop (server.cu):
 * the primary ray of a path, the shading of one path vertex, the hit record of a traversal. */
#pragma once
#include "kernels.cuh"
#include "shading.cuh"
#include "disney.cuh"
#include "svgf.cuh"
#include "traverse.cuh"

namespace lh2g {
namespace {

constexpr int WAVE_BLOCK = 128;
static_assert(WAVE_BLOCK == LH2G_TRAV_BLOCK, "traversal kernels run LH2G_TRAV_BLOCK threads per block");
constexpr int NRC_DEPTH = 2;   /* first path length at which radiance-cache frames query the cache */
#ifndef LH2G_NRC_TRAIN_SHIFT
#define LH2G_NRC_TRAIN_SHIFT 4
#endif
/* 1 in 2^LH2G_NRC_TRAIN_SHIFT cached paths trace on and train the cache (1 in 16: the survey's budget) */
constexpr uint32_t NRC_TRAIN_MASK = (1u << LH2G_NRC_TRAIN_SHIFT) - 1u;
constexpr uint32_t S_CACHED = 8;   /* radiance-cache frames: the path has recorded its cache vertex */

__device__ __forceinline__ uint32_t lanemask_lt() { uint32_t m; asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m)); return m; }

/* tuning switch: 1 (default) queues a frame's primary rays in 8 x 4 pixel tiles (LH2G_TILE_W), so that each warp of the first wave
 * (and, through the compaction that keeps a warp's survivors together, of the later ones) holds a compact patch of
 * the image instead of a 32-pixel strip of one row; 0 queues them in path order. The queue slot is only where a
 * path waits: every per-path quantity is indexed by the path, so results do not change. */
#ifndef LH2G_TILE_PRIMARY
#define LH2G_TILE_PRIMARY 1
#endif
#ifndef LH2G_TILE_W
#define LH2G_TILE_W 8   /* tile width; the height is 32 / width */
#endif
/* the (band-local) path index of primary queue slot q: per sample layer of W x rows pixels, rows in groups of TH,
 * each group in tiles of TW columns (the last tile narrower when W is not a multiple of TW, the last group lower
 * when rows is not a multiple of TH), a tile's pixels row by row */
__device__ __forceinline__ uint32_t primary_slot_path(const FrameGPU& F, const uint32_t q) {
#if LH2G_TILE_PRIMARY
    constexpr uint32_t TW = LH2G_TILE_W, TH = 32 / LH2G_TILE_W;
    static_assert(TW * TH == 32, "a tile is a warp");
    const uint32_t W = (uint32_t)F.W, rows = F.bandPix ? F.bandPix / W : (uint32_t)F.H, layerSize = W * rows;
    const uint32_t layer = q / layerSize, r0 = q - layer * layerSize;
    const uint32_t g = r0 / (TH * W), r = r0 - g * TH * W;
    const uint32_t rg = min(TH, rows - TH * g);
    const uint32_t t = r / (TW * rg), u = r - t * TW * rg;
    const uint32_t wt = min(TW, W - TW * t);
    const uint32_t dy = u / wt, dx = u - dy * wt;
    return layer * layerSize + (TH * g + dy) * W + TW * t + dx;
#else
    (void)F;
    return q;
#endif
}

/* Primary ray of path jobIndex (lib/RenderCore_PrimeRef/kernels/camera.h:39-68; pixel corner without lens for
 * LH2G_RP_FILTER frames, RenderCore_Optix7Filter/optix/.optix.cu:66-100). */
__device__ __forceinline__ void primary_ray(const FrameGPU& F, const uint32_t local, float3& O, float3& D) {
    const uint32_t jobIndex = global_path(F, local);   /* the path's index in the whole frame */
    const uint32_t x = jobIndex % (uint32_t)F.W;
    uint32_t y = jobIndex / (uint32_t)F.W;
    y %= (uint32_t)F.H;
    uint32_t seed = WangHash(jobIndex + F.cameraR0);
    const float r0 = RandomFloat(seed), r1 = RandomFloat(seed);
    const float r2 = RandomFloat(seed), r3 = RandomFloat(seed);
    float3 posOnPixel, posOnLens;
    if (F.flags & LH2G_RP_FILTER) {
        /* filter core: pixel corner of the jittered view, no lens (RenderCore_Optix7Filter/optix/.optix.cu:66-100) */
        const float u = (float)x * (1.0f / (float)F.W), v = (float)y * (1.0f / (float)F.H);
        posOnPixel = F.p1 + u * F.right + v * F.up;
        posOnLens = F.pos;
    } else {
        posOnPixel = F.p1 + ((float)x + r0) * (F.right / (float)F.W) + ((float)y + r1) * (F.up / (float)F.H);
        const float blade = (float)f2i(r2 * 9);
        float rr2 = (r2 - blade * (1.0f / 9.0f)) * 9.0f, rr1 = r3;
        float x1, y1, x2, y2;
        sincos_cw(blade * PI / 4.5f, &x1, &y1);
        sincos_cw((blade + 1.0f) * PI / 4.5f, &x2, &y2);
        if ((rr1 + rr2) > 1) rr1 = 1.0f - rr1, rr2 = 1.0f - rr2;
        const float xr = x1 * rr1 + x2 * rr2;
        const float yr = y1 * rr1 + y2 * rr2;
        posOnLens = F.pos + F.aperture * (F.right * xr + F.up * yr);
    }
    O = posOnLens;
    D = normalize(posOnPixel - posOnLens);
}

struct ShadeOut {
    bool ext, shadow;
    float4 eO, eD, eT;
    float4 sO, sD, sE;
};

/* The shading order of a queue of `count` rays with their hit records. A ray that hit nothing shades in a few
 * instructions (sky, no connection, no extension), one that hit a surface in thousands; shaded in queue order, a
 * warp of a bounce wave runs the long path with the few lanes whose ray hit. Each tile of PART_TILE consecutive
 * slots puts its hit slots, in queue order, at one place of the front of `order` (counter *hitCount) and its
 * missed ones at one place of the back (*missCount), so that the shading warps run one kind of path; with the
 * tiles' hits kept together, consecutive connections and extension rays still come from nearby slots. Launched
 * with PART_TILE threads per block; both counters start at zero. */
constexpr uint32_t PART_TILE = 512;
__device__ __forceinline__ void partition_queue(const float4* __restrict__ hits, const uint32_t count, uint32_t* __restrict__ order,
                                                uint32_t* hitCount, uint32_t* missCount) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    __shared__ uint32_t hitsBefore[PART_TILE / 32], validBefore[PART_TILE / 32], base[2];
    for (uint32_t t0 = blockIdx.x * PART_TILE; t0 < count; t0 += gridDim.x * PART_TILE) {   /* uniform in the block */
        const uint32_t s = t0 + threadIdx.x;
        const bool valid = s < count;
        const bool hit = valid && __float_as_int(__ldg(&hits[s].z)) != NOHIT;
        const uint32_t hm = __ballot_sync(0xffffffffu, hit), vm = __ballot_sync(0xffffffffu, valid);
        if (lane == 0) hitsBefore[warp] = __popc(hm), validBefore[warp] = __popc(vm);
        __syncthreads();
        if (warp == 0) {   /* exclusive prefix over the 16 warps, the tile's bases in the order */
            const uint32_t h0 = lane < PART_TILE / 32 ? hitsBefore[lane] : 0u, v0 = lane < PART_TILE / 32 ? validBefore[lane] : 0u;
            uint32_t h = h0, v = v0;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t h2 = __shfl_up_sync(0xffffffffu, h, off), v2 = __shfl_up_sync(0xffffffffu, v, off);
                if ((int)lane >= off) h += h2, v += v2;
            }
            if (lane < PART_TILE / 32) hitsBefore[lane] = h - h0, validBefore[lane] = v - v0;
            if (lane == PART_TILE / 32 - 1) {
                base[0] = h ? atomicAdd(hitCount, h) : 0u;
                base[1] = v - h ? atomicAdd(missCount, v - h) : 0u;
            }
        }
        __syncthreads();
        if (valid) {
            const uint32_t lt = lanemask_lt();
            const uint32_t pos = hit ? base[0] + hitsBefore[warp] + __popc(hm & lt)
                                     : count - 1u - (base[1] + (validBefore[warp] - hitsBefore[warp]) + __popc(vm & ~hm & lt));
            order[pos] = s;
        }
        __syncthreads();   /* the next tile rewrites the prefixes */
    }
}

/* Shading of one path vertex (lib/RenderCore_PrimeRef/kernels/pathtracer.h:45-168, with the filter core's
 * feature gathering for LH2G_RP_FILTER): o4, d4, t4 = the path's ray state, hit = its closest hit. Radiance goes
 * to the path's own accumulator; a connection and an extension ray are returned in out. */
__device__ __forceinline__ void shade_core(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, const int depth, const float4 o4,
                                           const float4 d4, const float4 t4, const float4 hit, ShadeOut& out, float* pot) {
    const uint32_t pathIdx = __float_as_uint(o4.w);
    uint32_t FLAGS = __float_as_uint(d4.w);
    const float3 O = xyz(o4), D = xyz(d4);
    float3 throughput = xyz(t4);
    const int PRIM = __float_as_int(hit.z), INST = __float_as_int(hit.y);
    const float HIT_T = hit.w;
    const size_t capIdx = (size_t)(depth - 1) * F.P + pathIdx;
    const bool filt = (F.flags & LH2G_RP_FILTER) != 0;
    const uint32_t R0 = filt ? F.frameSeed + (uint32_t)depth * 91771u : (uint32_t)F.samplesTaken * 7907u + (uint32_t)depth * 91771u;
    /* radiance goes to the indirect half once the path has bounced off a diffuse vertex */
    const uint32_t half = filt && (FLAGS & S_BOUNCED) ? 1u : 0u;
    float4* accP = B.pathAcc + (half ? F.P : 0) + pathIdx;
    /* SVGF data of sample 0 (RenderCore_Optix7Filter/kernels/pathtracer.h:95-104) */
    const uint32_t WH = (uint32_t)F.W * (uint32_t)F.H;
    const bool firstHitToBeStored = filt && (FLAGS & S_BOUNCED) == 0 && pathIdx / WH + (uint32_t)F.samplesTaken == 0;
    const uint32_t isSpecular = (FLAGS & S_VIASPECULAR) ? 1u : 0u;
    if (depth == 1 && firstHitToBeStored) {
        PackFeatures(B.features + pathIdx, 0, 0, 1e34f, 0, 0);
        B.worldPos[pathIdx] = make_float4(0, 0, 0, __uint_as_float(0));
        B.deltaDepth[pathIdx] = make_float4(0, 0, 0, 0);
    }
    float4 acc = *accP;
    if ((F.flags & LH2G_RP_DEPTH_W) && depth == 1) acc.w += PRIM == NOHIT ? 10000.0f : HIT_T;
    if (PRIM == NOHIT) {
        const float3 c = throughput * SampleSkydome(S, D);
        acc.x += c.x, acc.y += c.y, acc.z += c.z;
        *accP = acc;
        if (firstHitToBeStored) {
            const uint32_t packedNormal = PackNormal2(D * -1.0f) + isSpecular;
            PackFeatures(B.features + pathIdx, HDRtoRGB32(c), packedNormal, HIT_T, isSpecular, 0);
            const float3 far = O + 50000 * D;
            B.worldPos[pathIdx] = make_float4(far.x, far.y, far.z, __uint_as_float(packedNormal));
            B.deltaDepth[pathIdx] = make_float4(0, 0, 0, 0);
        }
        if (B.capSeeds) B.capSeeds[capIdx] = 0;
        return;
    }
    const uint32_t bary = __float_as_uint(hit.x);
    const float HIT_U = (float)(bary & 65535u) * (1.0f / 65535.0f);
    const float HIT_V = (float)(bary >> 16) * (1.0f / 65535.0f);
    Shading sd;
    float3 N, iN, fN, T;
    const float3 I = O + HIT_T * D;
    const float coneWidth = F.spreadAngle * HIT_T;
    GetShadingData(S, D, HIT_U, HIT_V, coneWidth, INST, PRIM, sd, N, iN, fN, T);
    const bool nee = (F.flags & LH2G_RP_NEE) != 0;
    auto matID = [&]() {   /* ShadingData::matID is never assigned in the reference; the material index is what it names */
        return min(__float_as_uint(__ldg(S.instTris[INST] + (size_t)PRIM * 13 + 1).w), (uint32_t)(S.nMaterials - 1));
    };
    auto derivatives = [&]() {
        return DepthDerivatives((int)(pathIdx % (uint32_t)F.W), (int)(pathIdx / (uint32_t)F.W), F.W, F.H, HIT_T, I, N, F.p1, F.right, F.up, F.pos);
    };
    if (IsEmissive(sd)) {
        const float DdotNL = -dot(D, N);
        if (DdotNL > 0) {
            const float3 c = throughput * sd.color;
            if (depth == 1 || (FLAGS & S_SPECULAR) || !nee) acc.x += c.x, acc.y += c.y, acc.z += c.z;
        }
        *accP = acc;
        if (firstHitToBeStored) {
            const uint32_t packedNormal = PackNormal2(N) + isSpecular;
            PackFeatures(B.features + pathIdx, HDRtoRGB32(sd.color), packedNormal, HIT_T, isSpecular, matID());
            B.worldPos[pathIdx] = make_float4(I.x, I.y, I.z, __uint_as_float(packedNormal));
            B.deltaDepth[pathIdx] = derivatives();
        }
        if (B.capSeeds) B.capSeeds[capIdx] = 0;
        return;
    }
    *accP = acc;
    if ((F.flags & LH2G_RP_NRC) && depth >= NRC_DEPTH && (FLAGS & (S_SPECULAR | S_CACHED)) == 0) {
        /* radiance cache, at the first vertex from path length 2 on that a diffuse bounce leads to (after a specular
         * bounce the path footprint is still small: it traces on): the query of this vertex (looking back along the
         * ray), the throughput that reaches it and the radiance gathered before it; a training path
         * (NRC_TRAIN_MASK) traces on, the others end here */
        const bool train = (WangHash(pathIdx * 3u + F.cameraR0) & NRC_TRAIN_MASK) == 0u;
        const float side = dot(D, N) > 0 ? -1.0f : 1.0f;
        float4* rec = B.nrcRec + pathIdx;
        const int64_t P = F.P;
        rec[0] = make_float4(I.x, I.y, I.z, ROUGHNESS(sd));
        rec[P] = make_float4(-D.x, -D.y, -D.z, 0.0f);
        rec[2 * P] = make_float4(fN.x * side, fN.y * side, fN.z * side, 0.0f);
        rec[3 * P] = make_float4(sd.color.x, sd.color.y, sd.color.z, 0.0f);
        rec[4 * P] = make_float4(throughput.x, throughput.y, throughput.z, train ? 2.0f : 1.0f);
        rec[5 * P] = make_float4(acc.x, acc.y, acc.z, 0.0f);
        if (!train) {
            if (B.capSeeds) B.capSeeds[capIdx] = 0;
            return;
        }
        FLAGS |= S_CACHED;
    }
    if (ROUGHNESS(sd) <= 0.001f || TRANSMISSION(sd) > 0.999f) FLAGS |= S_SPECULAR; else FLAGS &= ~S_SPECULAR;
    uint32_t seed = WangHash(global_path(F, pathIdx) * 17u + R0);
    if (firstHitToBeStored) {
        if (FLAGS & S_SPECULAR) {
            B.features[pathIdx].x = HDRtoRGB32(sd.color);   /* modulated by the first diffuse vertex later */
        } else {
            float3 albedo = sd.color;
            if (FLAGS & S_VIASPECULAR) albedo = albedo * RGB32toHDR(B.features[pathIdx].x);
            /* the reference writes flip ? -fN : fN with flip = +-1, which always takes the first branch */
            const uint32_t packedNormal = PackNormal2(fN * -1.0f) + isSpecular;
            PackFeatures(B.features + pathIdx, HDRtoRGB32(albedo), packedNormal, HIT_T, isSpecular, matID());
            B.worldPos[pathIdx] = make_float4(I.x, I.y, I.z, __uint_as_float(packedNormal));
            B.deltaDepth[pathIdx] = derivatives();
        }
    }
    const float faceDir = (dot(D, N) > 0) ? -1.0f : 1.0f;
    if (faceDir == 1) sd.transmittance = mk3(0);
    if ((FLAGS & S_SPECULAR) == 0 && nee) {
        const float q0 = RandomFloat(seed), q1 = RandomFloat(seed);
        float pickProb = 0, lightPdf = 0;
        float3 lightColor = mk3(0);
        int picked = 0;
        float3 L = RandomPointOnLight(S, q0, q1, I, fN * faceDir, pickProb, lightPdf, lightColor, pot, WAVE_BLOCK, picked) - I;
        const float dist = length(L);
        L = L * (1.0f / dist);
        const float NdotL = dot(L, fN * faceDir);
        if (NdotL > 0 && lightPdf > 0) {
            float bsdfPdf;
            const float3 sampledBSDF = EvaluateBSDF(sd, fN, L, bsdfPdf) * ROUGHNESS(sd);
            const float3 contribution = throughput * sampledBSDF * lightColor * (NdotL / (pickProb * lightPdf));
            const float3 SO = SafeOrigin(I, L, N, F.eps);
            out.shadow = true;
            out.sO = make_float4(SO.x, SO.y, SO.z, __uint_as_float(pathIdx));
            out.sD = make_float4(L.x, L.y, L.z, dist - 2 * F.eps);
            /* w: bit 0 the radiance half (filter frames), bits 1..6 the light (connections may be grouped by it) */
            out.sE = make_float4(contribution.x, contribution.y, contribution.z, __uint_as_float(half | ((uint32_t)picked << 1)));
        }
    }
    if (depth == F.maxDepth && firstHitToBeStored) {
        /* the path ends before its first diffuse bounce (RenderCore_Optix7Filter/kernels/pathtracer.h:288-299) */
        const uint32_t packedNormal = PackNormal2(N) + isSpecular;
        PackFeatures(B.features + pathIdx, 0, packedNormal, HIT_T, isSpecular, 0);
        B.worldPos[pathIdx] = make_float4(I.x, I.y, I.z, __uint_as_float(packedNormal));
    }
    float3 R;
    float newBsdfPdf;
    bool specular = false;
    const float q3 = RandomFloat(seed), q4 = RandomFloat(seed), q5 = RandomFloat(seed);
    const float3 bsdf = SampleBSDF(sd, fN, N, D * -1.0f, HIT_T, q3, q4, R, newBsdfPdf, specular);
    if (B.capSeeds) B.capSeeds[capIdx] = seed;
    if (newBsdfPdf < EPSILON || isnan(newBsdfPdf)) return;
    if (specular) FLAGS |= S_SPECULAR;
    const float pr = depth == F.maxDepth ? 0.0f : (((FLAGS & S_SPECULAR) || depth < F.rrStart) ? 1.0f : SurvivalProbability(bsdf));
    if (pr <= q5) return;
    throughput = throughput * (bsdf * fabsf(dot(fN, R)) / (pr * newBsdfPdf));
    if (!(FLAGS & S_SPECULAR)) FLAGS |= S_BOUNCED; else FLAGS |= S_VIASPECULAR;
    const float3 EO = SafeOrigin(I, R, N, F.eps);
    out.ext = true;
    out.eO = make_float4(EO.x, EO.y, EO.z, __uint_as_float(pathIdx));
    out.eD = make_float4(R.x, R.y, R.z, __uint_as_float(FLAGS));
    out.eT = make_float4(throughput.x, throughput.y, throughput.z, 0.0f);
}

/* ======================================================================================================
 * The OptiX 7 core's estimator (lib/rendercore_optix7/kernels/pathtracer.h:54-238, ray generation of
 * optix/.optix.cu:71-129) and the PrimeAdaptive core's variant (lib/RenderCore_PrimeAdaptive/kernels/pathtracer.h,
 * camera.h), with the Lambert BSDF. Path state: O4.w = slot << 6 | flags (S_* bits 0-3, tmin class bits 4-5),
 * D4.w = the packed normal of the previous vertex, T4 = throughput (bsdf * cos, the pdf not yet divided out) and
 * w = the pdf of the bounce that led here. Radiance goes to pathAcc[slot]; a slot's RNG identity is slotLayer[slot]
 * in the adaptive second wave, else the slot itself.
 * ==================================================================================================== */
constexpr uint32_t MIS_FLAG_MASK = 63u;

LH2G_DEV uint32_t PackNormal(const float3 N) {   /* tools_shared.h:101-107 */
    const float f = 65535.0f / fmaxf(sqrtf(8.0f * N.z + 8.0f), 0.0001f);
    return f2u(N.x * f + 32767.0f) + (f2u(N.y * f + 32767.0f) << 16);
}
LH2G_DEV float3 UnpackNormal(const uint32_t p) {   /* tools_shared.h:108-120 */
    float4 nn = make_float4(u2f23(p & 65535u) * (2.0f / 65535.0f), u2f23(p >> 16) * (2.0f / 65535.0f), 0.0f, 0.0f);
    nn = nn + make_float4(-1.0f, -1.0f, 1.0f, -1.0f);
    float l = dot(make_float3(nn.x, nn.y, nn.z), make_float3(-nn.x, -nn.y, -nn.w));
    nn.z = l, l = sqrtf(l), nn.x *= l, nn.y *= l;
    return make_float3(nn.x, nn.y, nn.z) * 2.0f + mk3(0.0f, 0.0f, -1.0f);
}

/* blueNoiseSampler4 (tools_shared.h:324-337) over the expanded tables */
LH2G_DEV float4 blue_noise4(const uint32_t* __restrict__ bn, const int x, const int y, const int sampleIndex, const int sampleDimension) {
    const uint4 r = __ldg(reinterpret_cast<const uint4*>(bn + sampleDimension + (x + y * 128) * 8 + 65536 * 3));
    const int rsi1 = (sampleIndex ^ (int)r.x) & 255, rsi2 = (sampleIndex ^ (int)r.y) & 255;
    const int rsi3 = (sampleIndex ^ (int)r.z) & 255, rsi4 = (sampleIndex ^ (int)r.w) & 255;
    const int v1 = (int)__ldg(bn + sampleDimension + 0 + rsi1 * 256), v2 = (int)__ldg(bn + sampleDimension + 1 + rsi2 * 256);
    const int v3 = (int)__ldg(bn + sampleDimension + 2 + rsi3 * 256), v4 = (int)__ldg(bn + sampleDimension + 3 + rsi4 * 256);
    const uint4 b = __ldg(reinterpret_cast<const uint4*>(bn + (sampleDimension & 7) + (x + y * 128) * 8 + 65536));
    return make_float4((0.5f + (float)(v1 ^ (int)b.x)) * (1.0f / 256.0f), (0.5f + (float)(v2 ^ (int)b.y)) * (1.0f / 256.0f),
                       (0.5f + (float)(v3 ^ (int)b.z)) * (1.0f / 256.0f), (0.5f + (float)(v4 ^ (int)b.w)) * (1.0f / 256.0f));
}

/* RayTarget (lib/RenderSystem/common_functions.h:29-50) */
LH2G_DEV float3 ray_target(const int sx, const int sy, const float r0, const float r1, const int W, const int H, const float distortion,
                           const float3 p1, const float3 right, const float3 up) {
    if (distortion == 0) {
        const float u = ((float)sx + r0) * (1.0f / W);
        const float v = ((float)sy + r1) * (1.0f / H);
        return p1 + u * right + v * up;
    }
    const float tx = sx / (float)W - 0.5f, ty = sy / (float)H - 0.5f;
    const float rr = tx * tx + ty * ty;
    const float rq = sqrtf(rr) * (1.0f + distortion * rr + distortion * rr * rr);
    const float theta = atan2_at(tx, ty);
    float st, ct;
    sincos_cw(theta, &st, &ct);
    const float bx = (st * rq + 0.5f) * W;
    const float by = (ct * rq + 0.5f) * H;
    return p1 + (bx + r0) * (right / (float)W) + (by + r1) * (up / (float)H);
}

/* RandomPointOnLens (optix/.optix.cu:71-83; RenderCore_PrimeAdaptive/kernels/camera.h:22-33) */
LH2G_DEV float3 lens_point(const float r0, float r1, const float3 pos, const float aperture, const float3 right, const float3 up) {
    const float blade = (float)f2i(r0 * 9);
    float r2 = (r0 - blade * (1.0f / 9.0f)) * 9.0f;
    float x1, y1, x2, y2;
    sincos_cw(blade * PI / 4.5f, &x1, &y1);
    sincos_cw((blade + 1.0f) * PI / 4.5f, &x2, &y2);
    if ((r1 + r2) > 1) r1 = 1.0f - r1, r2 = 1.0f - r2;
    const float xr = x1 * r1 + x2 * r2;
    const float yr = y1 * r1 + y2 * r2;
    return pos + aperture * (right * xr + up * yr);
}

/* the primary ray of path pathIdx of an OptiX 7 frame (optix/.optix.cu:85-121) */
__device__ __forceinline__ void primary_optix7(const SceneGPU& S, const FrameGPU& F, const uint32_t pathIdx, float3& O, float3& D) {
    const uint32_t WH = (uint32_t)F.W * (uint32_t)F.H;
    const uint32_t pixelIdx = pathIdx % WH;
    const uint32_t sampleIdx = pathIdx / WH + (uint32_t)F.samplesTaken;
    uint32_t seed = WangHash(pathIdx * 16789u + (uint32_t)F.samplesTaken * 1791u);
    const int sx = (int)(pixelIdx % (uint32_t)F.W), sy = (int)(pixelIdx / (uint32_t)F.W);
    float4 r4;
    if (sampleIdx < 64 && S.blueNoise) {
        r4 = blue_noise4(S.blueNoise, (sx + (int)(F.shift & 127u)) & 127, (sy + (int)(F.shift >> 24)) & 127, (int)sampleIdx, 0);
    } else {
        r4.x = RandomFloat(seed), r4.y = RandomFloat(seed);
        r4.z = RandomFloat(seed), r4.w = RandomFloat(seed);
    }
    O = lens_point(r4.x, r4.z, F.pos, F.aperture, F.right, F.up);
    D = normalize(ray_target(sx, sy, r4.y, r4.w, F.W, F.H, F.distortion, F.p1, F.right, F.up) - O);
}

/* the primary ray of pixel (sx, sy) with sample index sampleIdx in a PrimeAdaptive frame (camera.h:39-80, 96-139) */
__device__ __forceinline__ void primary_adaptive(const SceneGPU& S, const FrameGPU& F, const int sx, const int sy, const uint32_t sampleIdx,
                                                 const uint32_t thread, const uint32_t R0, float3& O, float3& D) {
    float4 r4;
    if (sampleIdx < 64 && S.blueNoise) {
        r4 = blue_noise4(S.blueNoise, sx & 127, sy & 127, (int)sampleIdx, 0);
    } else {
        uint32_t seed = WangHash(thread + R0);
        r4.x = RandomFloat(seed), r4.y = RandomFloat(seed);
        r4.z = RandomFloat(seed), r4.w = RandomFloat(seed);
    }
    O = lens_point(r4.x, r4.z, F.pos, F.aperture, F.right, F.up);
    D = normalize(ray_target(sx, sy, r4.y, r4.w, F.W, F.H, F.distortion, F.p1, F.right, F.up) - O);
}

/* SampleSmallSkydome (tools_shared.h:204-211) */
LH2G_DEV float3 sample_small_sky(const SceneGPU& S, const float3& Dw) {
    const uint32_t w = (uint32_t)S.skyW >> 6, h = (uint32_t)S.skyH >> 6;
    if (w == 0 || h == 0 || !S.skySmall) return mk3(0);
    const float4 m0 = S.worldToSky[0], m1 = S.worldToSky[1], m2 = S.worldToSky[2];
    const float3 D = -make_float3(m0.x * Dw.x + m0.y * Dw.y + m0.z * Dw.z, m1.x * Dw.x + m1.y * Dw.y + m1.z * Dw.z, m2.x * Dw.x + m2.y * Dw.y + m2.z * Dw.z);
    float p = atan2_at(D.y, D.x);
    p = (p < 0) ? (p + 2 * PI) : p;
    const float theta = acos_at(D.z < -1.f ? -1.f : (D.z > 1.f ? 1.f : D.z));
    const uint32_t u = f2u((float)w * p * INV2PI - 0.5f);
    const uint32_t v = f2u((float)h * theta * INVPI - 0.5f);
    const uint32_t idx = u + v * w;
    return idx < w * h ? xyz(__ldg(S.skySmall + idx)) : mk3(0);
}

/* LightPickProb (lights_shared.h:158-177): the chance that light idx would have been picked from O with normal N,
 * the tri lights' potential taken at the light point I */
LH2G_DEV float light_pick_prob(const SceneGPU& S, const int idx, const float3& O, const float3& N, const float3& I) {
    const int lights = S.nTri + S.nPoint + S.nSpot + S.nDir;
    float sum = 0, mine = 0;
    for (int i = 0; i < lights; i++) {
        float c;
        if (i < S.nTri) {
            const float4* l = S.triLights + (size_t)i * 6;
            const float4 c4 = __ldg(l), n4 = __ldg(l + 1);
            float3 L = I - O;
            const float att = 1.0f / dot(L, L);
            L = normalize(L);
            const float LNdotL = fmaxf(0.0f, -dot(xyz(n4), L));
            const float NdotL = fmaxf(0.0f, dot(N, L));
            c = c4.w * LNdotL * NdotL * att;
        } else if (i < S.nTri + S.nPoint) {
            c = PotentialPoint(S, i - S.nTri, O, N);
        } else if (i < S.nTri + S.nPoint + S.nSpot) {
            c = PotentialSpot(S, i - S.nTri - S.nPoint, O, N);
        } else {
            c = PotentialDir(S, i - S.nTri - S.nPoint - S.nSpot, N);
        }
        if (i == idx) mine = c;
        sum += c;
    }
    if (sum <= 0) return 0.0f;
    return (idx >= 0 && idx < lights) ? mine / sum : 0.0f;
}

/* CLAMPINTENSITY (rendercore_optix7/core_settings.h:191-194) and FIXNAN_FLOAT3 (common_settings.h:66) */
LH2G_DEV void clamp_intensity(float3& c, const float clampValue) {
    const float v = fmaxf(c.x, fmaxf(c.y, c.z));
    if (v > clampValue) { const float m = clampValue / v; c.x *= m, c.y *= m, c.z *= m; }
}
LH2G_DEV void fix_nan(float3& a) { if (!isfinite(a.x + a.y + a.z)) a = mk3(0); }

/* the ray's tmin from its flags */
LH2G_DEV float mis_tmin(const uint32_t flags, const float eps) {
    const uint32_t c = (flags >> MIS_TMIN_SHIFT) & 3u;
    return c == 1u ? eps : (c == 2u ? EPSILON : 0.0f);
}

/* Shading of one path vertex of the OptiX 7 / PrimeAdaptive estimators. */
__device__ __forceinline__ void shade_mis(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, const int depth, const float4 o4,
                                          const float4 d4, const float4 t4, const float4 hit, ShadeOut& out, float* pot) {
    const bool optix7 = (F.flags & LH2G_RP_OPTIX7) != 0;
    const uint32_t word = __float_as_uint(o4.w);
    const uint32_t slot = word >> 6;
    uint32_t FLAGS = word & 15u;
    const uint32_t pathIdx = B.slotLayer ? __ldg(B.slotLayer + slot) : slot;
    const float3 O = xyz(o4), D = xyz(d4);
    float3 throughput = xyz(t4);
    const float bsdfPdf = t4.w;
    const int PRIM = __float_as_int(hit.z), INST = __float_as_int(hit.y);
    const float HIT_T = hit.w;
    const size_t capIdx = (size_t)(depth - 1) * F.P + slot;
    const uint32_t WH = (uint32_t)F.W * (uint32_t)F.H;
    const uint32_t sampleIdx = pathIdx / WH + F.pass;
    float4* accP = B.pathAcc + slot;
    /* PrimeAdaptive: albedo and normal of the first diffuse-led vertex, for the variance estimate (first wave only) */
    float4* feat = (B.misFeatures && (FLAGS & S_BOUNCED) == 0) ? B.misFeatures + pathIdx : nullptr;
    if (PRIM == NOHIT) {
        const float3 skyPixel = (FLAGS & S_BOUNCED) ? sample_small_sky(S, D) : SampleSkydome(S, D);
        float3 contribution = throughput * skyPixel * (1.0f / bsdfPdf);
        clamp_intensity(contribution, F.clampValue);
        fix_nan(contribution);
        float4 acc = *accP;
        acc.x += contribution.x, acc.y += contribution.y, acc.z += contribution.z;
        *accP = acc;
        if (feat) *feat = make_float4(contribution.x, contribution.y, contribution.z, __uint_as_float(PackNormal2(D * -1.0f)));
        if (B.capSeeds) B.capSeeds[capIdx] = 0;
        return;
    }
    const float HIT_U = (float)(__float_as_uint(hit.x) & 65535u) * (1.0f / 65535.0f);
    const float HIT_V = (float)(__float_as_uint(hit.x) >> 16) * (1.0f / 65535.0f);
    Shading sd;
    float3 N, iN, fN, T;
    const float3 I = O + HIT_T * D;
    const bool disneyBsdf = (F.flags & LH2G_RP_DISNEY) != 0;   /* kernels/bsdf.h's default branch: disney.h */
    GetShadingData(S, D, HIT_U, HIT_V, F.spreadAngle * HIT_T, INST, PRIM, sd, N, iN, fN, T, disneyBsdf);
    if (feat) *feat = make_float4(sd.color.x, sd.color.y, sd.color.z, __uint_as_float(PackNormal2(iN)));
    const uint32_t tminBits = optix7 ? MIS_TMIN_EPS : 0u;
    if (sd.flags & 1) {   /* alpha: the ray continues behind the surface */
        if (B.capSeeds) B.capSeeds[capIdx] = 0;
        if (depth >= F.maxDepth) return;
        fix_nan(throughput);
        out.ext = true;
        if (optix7) {
            const float3 P = I + D * F.eps;
            out.eO = make_float4(P.x, P.y, P.z, __uint_as_float((slot << 6) | FLAGS | MIS_TMIN_EPS));
            out.eD = d4;
        } else {
            out.eO = make_float4(I.x, I.y, I.z, __uint_as_float((slot << 6) | FLAGS | MIS_TMIN_EPSILON));
            out.eD = make_float4(D.x, D.y, D.z, __uint_as_float(0u));
        }
        out.eT = make_float4(throughput.x, throughput.y, throughput.z, bsdfPdf);
        return;
    }
    if (IsEmissive(sd)) {
        const float DdotNL = -dot(D, N);
        if (DdotNL > 0) {
            float3 contribution = mk3(0);
            if (depth == 1 || (FLAGS & S_SPECULAR) || !(F.flags & LH2G_RP_NEE)) {
                contribution = sd.color;   /* the reference leaves the throughput out here */
            } else {
                const float3 lastN = UnpackNormal(__float_as_uint(d4.w));
                const float4 tv = __ldg(S.instTris[INST] + (size_t)PRIM * 13 + 5);   /* T, area */
                const float lightPdf = (HIT_T * HIT_T) / (fabsf(dot(D, N)) * tv.w);
                const int ltri = __float_as_int(__ldg(S.instTris[INST] + (size_t)PRIM * 13).w);
                float pickProb;
                if (F.flags & LH2G_RP_LIGHTTREE) {   /* the shading seed, as the reference draws it before this branch */
                    uint32_t seed = WangHash(pathIdx * 17u + xorshift_n(F.cameraR0, depth - 1) + (uint32_t)depth * 91771u);
                    pickProb = light_pick_prob_tree(S, ltri, lastN, I, seed);
                } else {
                    pickProb = light_pick_prob(S, ltri, O, lastN, I);
                }
                if ((bsdfPdf + lightPdf * pickProb) > 0) contribution = throughput * sd.color * (1.0f / (bsdfPdf + lightPdf * pickProb));
            }
            clamp_intensity(contribution, F.clampValue);
            fix_nan(contribution);
            float4 acc = *accP;
            acc.x += contribution.x, acc.y += contribution.y, acc.z += contribution.z;
            *accP = acc;
        }
        if (B.capSeeds) B.capSeeds[capIdx] = 0;
        return;
    }
    if (FLAGS & S_BOUNCED) sd.params[0] |= 255u << 24;   /* path regularisation: roughness 1 after a bounce */
    if (ROUGHNESS(sd) <= 0.001f || TRANSMISSION(sd) > 0.5f) FLAGS |= S_SPECULAR; else FLAGS &= ~S_SPECULAR;
    const float faceDir = (dot(D, N) > 0) ? -1.0f : 1.0f;
    if (faceDir == 1) sd.transmittance = mk3(0);
    throughput = throughput * (1.0f / bsdfPdf);
    const uint32_t R0 = optix7 ? xorshift_n(F.cameraR0, depth - 1) + (uint32_t)depth * 91771u : F.r0Base + (uint32_t)depth * F.r0Depth;
    uint32_t seed = WangHash(pathIdx * 17u + R0);
    float4 r4;
    if (sampleIdx < 64 && S.blueNoise) {
        const uint32_t x = ((pathIdx % (uint32_t)F.W) + (F.shift & 127u)) & 127u;
        const uint32_t y = ((pathIdx / (uint32_t)F.W) + (F.shift >> 24)) & 127u;
        r4 = blue_noise4(S.blueNoise, (int)x, (int)y, (int)sampleIdx, 4 * depth - 4);
    } else {
        r4.x = RandomFloat(seed), r4.y = RandomFloat(seed);
        r4.z = RandomFloat(seed), r4.w = RandomFloat(seed);
    }
    if ((FLAGS & S_SPECULAR) == 0 && (F.flags & LH2G_RP_NEE)) {
        float pickProb = 0, lightPdf = 0;
        float3 lightColor = mk3(0);
        int picked = 0;
        float3 L = ((F.flags & LH2G_RP_LIGHTTREE) ? RandomPointOnLightTree(S, r4.x, r4.y, seed, I, fN * faceDir, pickProb, lightPdf, lightColor, picked)
                                                  : RandomPointOnLight(S, r4.x, r4.y, I, fN * faceDir, pickProb, lightPdf, lightColor, pot, WAVE_BLOCK,
                                                                       picked)) - I;
        const float dist = length(L);
        L = L * (1.0f / dist);
        const float NdotL = dot(L, fN * faceDir);
        if (NdotL > 0 && lightPdf > 0) {
            float lbsdfPdf;
            /* lambert.h defines BSDF_HAS_PURE_SPECULARS: its value is scaled by ROUGHNESS (pathtracer.h:194-198) */
            const float3 sampledBSDF = disneyBsdf ? disney::EvaluateBSDF(sd, fN, T, D * -1.0f, L, lbsdfPdf)
                                                  : EvaluateBSDF(sd, fN, L, lbsdfPdf) * ROUGHNESS(sd);
            if (lbsdfPdf > 0) {
                float3 contribution = throughput * sampledBSDF * lightColor * (NdotL / (pickProb * lightPdf + lbsdfPdf));
                fix_nan(contribution);
                clamp_intensity(contribution, F.clampValue);
                const float3 SO = SafeOrigin(I, L, N, F.eps);
                out.shadow = true;
                out.sO = make_float4(SO.x, SO.y, SO.z, __uint_as_float(slot));
                out.sD = make_float4(L.x, L.y, L.z, dist - 2 * F.eps);
                out.sE = make_float4(contribution.x, contribution.y, contribution.z, __uint_as_float((uint32_t)picked << 1));
            }
        }
    }
    /* one diffuse bounce at most (ENOUGH_BOUNCES = S_BOUNCED), or the maximum path length */
    if ((FLAGS & S_BOUNCED) || depth == F.maxDepth) { if (B.capSeeds) B.capSeeds[capIdx] = seed; return; }
    float3 R = mk3(0);
    float newBsdfPdf = 0.0f;   /* the Disney sampler leaves it unset on its early exits: the path ends there */
    bool specular = false;
    const float r5 = RandomFloat(seed);   /* lambert.h's SampleBSDF draws it and does not use it */
    const float3 bsdf = disneyBsdf ? disney::SampleBSDF(sd, fN, N, T, D * -1.0f, HIT_T, r4.z, r4.w, r5, R, newBsdfPdf, specular)
                                   : SampleBSDF(sd, fN, N, D * -1.0f, HIT_T, r4.z, r4.w, R, newBsdfPdf, specular);
    if (newBsdfPdf < EPSILON || isnan(newBsdfPdf)) { if (B.capSeeds) B.capSeeds[capIdx] = seed; return; }
    if (specular) FLAGS |= S_SPECULAR;
    const float pr = ((FLAGS & S_SPECULAR) || (FLAGS & S_BOUNCED) == 0) ? 1.0f : SurvivalProbability(bsdf);
    if (pr < RandomFloat(seed)) { if (B.capSeeds) B.capSeeds[capIdx] = seed; return; }
    throughput = throughput * (1 / pr);
    if (B.capSeeds) B.capSeeds[capIdx] = seed;
    const uint32_t packedNormal = PackNormal(fN * faceDir);
    if (!(FLAGS & S_SPECULAR)) FLAGS |= (FLAGS & S_BOUNCED) ? S_BOUNCEDTWICE : S_BOUNCED; else FLAGS |= S_VIASPECULAR;
    const float3 EO = SafeOrigin(I, R, N, F.eps);
    fix_nan(throughput);
    const float3 tn = throughput * bsdf * fabsf(dot(fN, R));
    out.ext = true;
    out.eO = make_float4(EO.x, EO.y, EO.z, __uint_as_float((slot << 6) | FLAGS | tminBits));
    out.eD = make_float4(R.x, R.y, R.z, __uint_as_float(packedNormal));
    out.eT = make_float4(tn.x, tn.y, tn.z, newBsdfPdf);
}

__device__ __forceinline__ float4 hit_record(const bool found, const HitRec& best) {
    if (found) return make_float4(__uint_as_float(f2u(65535.0f * best.u) + (f2u(65535.0f * best.v) << 16)), __int_as_float(best.inst),
                                  __int_as_float(best.prim), best.t);
    return make_float4(__uint_as_float(0u), __int_as_float(0), __int_as_float(NOHIT), 1e34f);
}

}  // namespace
}  // namespace lh2g

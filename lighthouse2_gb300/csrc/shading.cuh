/* shading.cuh - device shading of the GB300 render core: material fetch, shading frame, texture filtering,
 * light selection and the Lambert BSDF with pure specular reflection / refraction.
 *
 * Semantics follow, operation by operation, lib/CUDA/shared_kernel_code/material_shared.h:42-206 (shading
 * frame with consistent normals; OptiX7 barycentric convention w V0 + u V1 + v V2), sampling_shared.h:29-104
 * (bilinear / trilinear ARGB32 fetch), lights_shared.h:37-105 and 225-313 (importance selection over at most
 * 64 lights; the potentials are recomputed instead of stored, which yields the same values), tools_shared.h
 * (normals, origin offset, sky dome) and lib/sharedBSDFs/lambert.h:32-125.
 */
#pragma once
#include <cuda_fp16.h>
#include "core_types.cuh"
#include "device_math.cuh"

namespace lh2g {

constexpr uint32_t MAT_HASDIFFUSEMAP = 1u << 2, MAT_HASNORMALMAP = 1u << 3, MAT_HASSPECULARITYMAP = 1u << 4,
                   MAT_HASROUGHNESSMAP = 1u << 5, MAT_HAS2NDNORMALMAP = 1u << 7, MAT_HAS2NDDIFFUSEMAP = 1u << 9,
                   MAT_HASSMOOTHNORMALS = 1u << 11;

struct Shading {
    float3 color;
    float3 transmittance;
    uint32_t params[4];
    int flags;
    float4 tint;   /* the Disney BSDF's tint (xyz) and luminance (w) of the base colour; set when GetShadingData is asked */
};

/* material_shared.h:19-35: the CIE XYZ conversions of the base colour's tint */
LH2G_DEV float4 tint_of(const float3 rgb) {
    const float3 xyz = make_float3(fmaxf(0.0f, 0.412453f * rgb.x + 0.357580f * rgb.y + 0.180423f * rgb.z),
                                   fmaxf(0.0f, 0.212671f * rgb.x + 0.715160f * rgb.y + 0.072169f * rgb.z),
                                   fmaxf(0.0f, 0.019334f * rgb.x + 0.119193f * rgb.y + 0.950227f * rgb.z));
    if (!(xyz.y > 0)) return make_float4(1.0f, 1.0f, 1.0f, xyz.y);
    const float3 n = xyz * (1.0f / xyz.y);
    return make_float4(fmaxf(0.0f, 3.240479f * n.x - 1.537150f * n.y - 0.498535f * n.z),
                       fmaxf(0.0f, -0.969256f * n.x + 1.875992f * n.y + 0.041556f * n.z),
                       fmaxf(0.0f, 0.055648f * n.x - 0.204043f * n.y + 1.057311f * n.z), xyz.y);
}

LH2G_DEV float char2flt(uint32_t a, int s) { return ((float)((a >> s) & 255u)) * (1.0f / 255.0f); }
LH2G_DEV float ROUGHNESS(const Shading& sd) { return fmaxf(0.001f, char2flt(sd.params[0], 24)); }
LH2G_DEV float TRANSMISSION(const Shading& sd) { return char2flt(sd.params[2], 16); }
LH2G_DEV float ETA(const Shading& sd) { return __uint_as_float(sd.params[3]); }
LH2G_DEV bool IsEmissive(const Shading& sd) { return sd.color.x > 1.0f || sd.color.y > 1.0f || sd.color.z > 1.0f; }

LH2G_DEV float4 uchar4_to_float4(uint32_t v) {
    const float r = 1.0f / 256.0f;
    return make_float4((float)(v & 255u) * r, (float)((v >> 8) & 255u) * r, (float)((v >> 16) & 255u) * r, (float)(v >> 24) * r);
}

LH2G_DEV float4 FetchTexel(const uint32_t* __restrict__ tex, const float2 texCoord, const int o, const int w, const int h) {
    const float2 tc = make_float2((fmaxf(texCoord.x + 1000, 0.0f) * w) - 0.5f, (fmaxf(texCoord.y + 1000, 0.0f) * h) - 0.5f);
    const int iu = f2i(tc.x) % w;
    const int iv = f2i(tc.y) % h;
    const float fu = tc.x - floorf(tc.x);
    const float fv = tc.y - floorf(tc.y);
    const float w0 = (1 - fu) * (1 - fv);
    const float w1 = fu * (1 - fv);
    const float w2 = (1 - fu) * fv;
    const float w3 = 1 - (w0 + w1 + w2);
    const int iu1 = (iu + 1) % w, iv1 = (iv + 1) % h;
    const float4 p0 = uchar4_to_float4(__ldg(tex + o + iu + iv * w));
    const float4 p1 = uchar4_to_float4(__ldg(tex + o + iu1 + iv * w));
    const float4 p2 = uchar4_to_float4(__ldg(tex + o + iu + iv1 * w));
    const float4 p3 = uchar4_to_float4(__ldg(tex + o + iu1 + iv1 * w));
    return p0 * w0 + p1 * w1 + p2 * w2 + p3 * w3;
}

LH2G_DEV float4 FetchTexelTrilinear(const uint32_t* __restrict__ tex, const float lambda, const float2 texCoord, const int offset, const int width, const int height) {
    int level0 = 0, level1 = 0;
    float f = 0;
    if (lambda >= 0) level0 = min(MIPLEVELCOUNT - 1, f2i(lambda)), level1 = min(MIPLEVELCOUNT - 1, level0 + 1), f = lambda - floorf(lambda);
    const float scale = (float)(width * height) * 1.3333333333f;
    const int o0 = offset + f2i(scale * (1 - __uint_as_float((uint32_t)(127 - 2 * level0) << 23)));
    const int o1 = offset + f2i(scale * (1 - __uint_as_float((uint32_t)(127 - 2 * level1) << 23)));
    const float4 p0 = FetchTexel(tex, texCoord, o0, width >> level0, height >> level0);
    const float4 p1 = FetchTexel(tex, texCoord, o1, width >> level1, height >> level1);
    return (1 - f) * p0 + f * p1;
}

LH2G_DEV float2 map_uvscale(const uint4 m) { return make_float2(half2float(m.y & 0xffffu), half2float(m.y >> 16)); }
LH2G_DEV float2 map_uvoffs(const uint4 m) { return make_float2(half2float(m.z & 0xffffu), half2float(m.z >> 16)); }

LH2G_DEV float3 ConsistentNormal(const float3& D, const float3& iN, const float alpha) {
    const float t = PI - 2 * alpha, q = (t * t) / (PI * (PI + (2 * PI - 4) * alpha));
    const float b = dot(D, iN), g = 1 + q * (b - 1), rho = sqrtf(q * (1 + g) / (1 + b));
    const float3 Rc = (g + rho * b) * iN - (rho * D);
    return normalize(D + Rc);
}

/* GetShadingData + SetupFrame for triangle prim of instance inst. */
LH2G_DEV void GetShadingData(const SceneGPU& S, const float3 D, const float u, const float v, const float coneWidth, const int inst,
                             const int prim, Shading& sd, float3& N, float3& iN, float3& fN, float3& T, const bool withTint = false) {
    const float4* tri = S.instTris[inst] + (size_t)prim * 13;
    const float4 t1 = __ldg(tri + 1), t2 = __ldg(tri + 2), t3 = __ldg(tri + 3), t4 = __ldg(tri + 4), t5 = __ldg(tri + 5), t7 = __ldg(tri + 7);
    const uint4* mat = S.materials + (size_t)min(__float_as_uint(t1.w), (uint32_t)(S.nMaterials - 1)) * 8;
    const uint4 base = __ldg(mat), params = __ldg(mat + 1);
    const uint32_t flags = base.w;
    sd.color = make_float3(half2float(base.x & 0xffffu), half2float(base.x >> 16), half2float(base.y & 0xffffu));
    sd.transmittance = make_float3(half2float(base.y >> 16), half2float(base.z & 0xffffu), half2float(base.z >> 16));
    sd.params[0] = params.x, sd.params[1] = params.y, sd.params[2] = params.z, sd.params[3] = params.w;
    sd.flags = 0;
    if (withTint) sd.tint = tint_of(sd.color);
    N = iN = fN = make_float3(t2.w, t3.w, t4.w);
    T = xyz(t5);
    const float w = 1 - (u + v);
    if (flags & MAT_HASSMOOTHNORMALS) iN = normalize(w * xyz(t2) + u * xyz(t3) + v * xyz(t4));
    const float4 rA = __ldg(S.instInvRows + 3 * inst), rB = __ldg(S.instInvRows + 3 * inst + 1), rC = __ldg(S.instInvRows + 3 * inst + 2);
    const float3 A = xyz(rA), B = xyz(rB), C = xyz(rC);
    N = normalize(N.x * A + N.y * B + N.z * C);
    iN = normalize(iN.x * A + iN.y * B + iN.z * C);
    const bool backSide = dot(D, N) > 0;
    const float alpha = w * t7.x + u * t7.y + v * t7.z;
    iN = (backSide ? -1.0f : 1.0f) * ConsistentNormal(D * -1.0f, backSide ? (iN * -1.0f) : iN, alpha);
    fN = iN;
    if (!(flags & (MAT_HASDIFFUSEMAP | MAT_HAS2NDDIFFUSEMAP | MAT_HASSPECULARITYMAP | MAT_HASNORMALMAP | MAT_HAS2NDNORMALMAP | MAT_HASROUGHNESSMAP))) return;
    const float4 t0 = __ldg(tri);
    const float ww = 1 - (u + v);
    const float tu = ww * t0.x + u * t0.y + v * t0.z;
    const float tv = ww * t1.x + u * t1.y + v * t1.z;
    if (flags & MAT_HASDIFFUSEMAP) {
        const float lambda = t7.w + log2_at(coneWidth * (1.0f / fabsf(dot(D, N))));
        const uint4 m0 = __ldg(mat + 2);
        const float2 uvscale = map_uvscale(m0), uvoffs = map_uvoffs(m0);
        const float4 texel = FetchTexelTrilinear(S.texels, lambda, uvscale * (uvoffs + make_float2(tu, tv)), (int)m0.w, (int)(m0.x & 0xffffu), (int)(m0.x >> 16));
        if (texel.w < 0.5f) { sd.flags |= 1; return; }
        sd.color = sd.color * xyz(texel);
        if (flags & MAT_HAS2NDDIFFUSEMAP) {
            const uint4 m1 = __ldg(mat + 3);
            const float2 uvscale1 = map_uvscale(m1), uvoffs1 = map_uvoffs(m1);
            sd.color = sd.color + (xyz(FetchTexel(S.texels, uvscale1 * (uvoffs1 + make_float2(tu, tv)), (int)m1.w, (int)(m1.x & 0xffffu), (int)(m1.x >> 16))) - mk3(0.5f));
        }
    }
    if (flags & MAT_HASNORMALMAP) {
        const float3 Bt = xyz(__ldg(tri + 6));
        const uint4 n0 = __ldg(mat + 4);
        const uint32_t part3 = base.z;
        const float n0scale = copysignf(-0.0001f + 0.0001f * exp_cw(0.1f * fabsf((float)((part3 >> 8) & 255u) - 128.0f)), (float)((part3 >> 8) & 255u) - 128.0f);
        const float2 uvscale = map_uvscale(n0), uvoffs = map_uvoffs(n0);
        float3 sn = (xyz(FetchTexel(S.texels, uvscale * (uvoffs + make_float2(tu, tv)), (int)n0.w, (int)(n0.x & 0xffffu), (int)(n0.x >> 16))) - mk3(0.5f)) * 2.0f;
        sn.x *= n0scale, sn.y *= n0scale;
        if (flags & MAT_HAS2NDNORMALMAP) {
            const uint4 n1 = __ldg(mat + 5);
            const float n1scale = copysignf(-0.0001f + 0.0001f * exp_cw(0.1f * ((float)((part3 >> 16) & 255u) - 128.0f)), (float)((part3 >> 16) & 255u) - 128.0f);
            const float2 uvscale1 = map_uvscale(n1), uvoffs1 = map_uvoffs(n1);
            float3 l1 = (xyz(FetchTexel(S.texels, uvscale1 * (uvoffs1 + make_float2(tu, tv)), (int)n1.w, (int)(n1.x & 0xffffu), (int)(n1.x >> 16))) - mk3(0.5f)) * 2.0f;
            l1.x *= n1scale, l1.y *= n1scale;
            sn = sn + l1;
        }
        sn = normalize(sn);
        fN = normalize(sn.x * T + sn.y * Bt + sn.z * iN);
    }
    if (flags & MAT_HASROUGHNESSMAP) {
        const uint4 rm = __ldg(mat + 7);
        const float2 uvscale = map_uvscale(rm), uvoffs = map_uvoffs(rm);
        const float4 texel = FetchTexel(S.texels, uvscale * (uvoffs + make_float2(tu, tv)), (int)rm.w, (int)(rm.x & 0xffffu), (int)(rm.x >> 16));
        sd.params[0] = (sd.params[0] & 0x00ffffffu) + ((uint32_t)f2i(texel.y * 255.0f) << 24);
        sd.params[0] = (sd.params[0] & 0xffffff00u) + (uint32_t)f2i(texel.x * 255.0f);
    }
}

/* ---- Lambert BSDF ---- */
LH2G_DEV float sqr(float x) { return x * x; }
LH2G_DEV float Fr_L(float VDotN, float eio) {
    if (VDotN < 0.0f) { eio = 1.0f / eio; VDotN = fabsf(VDotN); }
    const float SinThetaT2 = sqr(eio) * (1.0f - VDotN * VDotN);
    if (SinThetaT2 > 1.0f) return 1.0f;
    const float LDotN = sqrtf(1.0f - SinThetaT2);
    const float r1 = (VDotN - eio * LDotN) / (VDotN + eio * LDotN);
    const float r2 = (LDotN - eio * VDotN) / (LDotN + eio * VDotN);
    return 0.5f * (sqr(r1) + sqr(r2));
}
LH2G_DEV bool Refract_L(const float3 wi, const float3 n, const float eta, float3& wt) {
    const float cosThetaI = fabsf(dot(n, wi));
    const float sin2ThetaI = fmaxf(0.0f, 1.0f - cosThetaI * cosThetaI);
    const float sin2ThetaT = eta * eta * sin2ThetaI;
    if (sin2ThetaT >= 1) return false;
    const float cosThetaT = sqrtf(1.0f - sin2ThetaT);
    wt = eta * (wi * -1.0f) + (eta * cosThetaI - cosThetaT) * n;
    return true;
}
LH2G_DEV float3 EvaluateBSDF(const Shading& sd, const float3 iN, const float3 wi, float& pdf) {
    if (TRANSMISSION(sd) > 0.999f || ROUGHNESS(sd) <= 0.001f) { pdf = 0; return mk3(0); }
    pdf = fabsf(dot(wi, iN)) * INVPI;
    return sd.color * INVPI;
}
LH2G_DEV void SetupTangentSpace(const float3& N, float3& T, float3& B) {
    const float sign = copysignf(1.0f, N.z);
    const float a = -1.0f / (sign + N.z);
    const float b = N.x * N.y * a;
    B = make_float3(1.0f + sign * N.x * N.x * a, sign * b, -sign * N.x);
    T = make_float3(b, sign + N.y * N.y * a, -N.y);
}
LH2G_DEV float3 Tangent2World(const float3& V, const float3& N) {
    float3 T, B;
    SetupTangentSpace(N, T, B);
    return V.x * T + V.y * B + V.z * N;
}
LH2G_DEV float3 DiffuseReflectionCosWeighted(const float r0, const float r1) {
    const float term1 = TWOPI * r0, term2 = sqrtf(1 - r1);
    float s, c;
    sincos_cw(term1, &s, &c);
    return make_float3(c * term2, s * term2, sqrtf(r1));
}
LH2G_DEV float3 SampleBSDF(const Shading& sd, float3 iN, const float3 N, const float3 wo, const float distance, const float r3, const float r4,
                           float3& wi, float& pdf, bool& specular) {
    const float flip = (dot(wo, N) < 0) ? -1.0f : 1.0f;
    iN = iN * flip;
    specular = true, pdf = 1;
    float3 bsdf;
    const float TRANS = TRANSMISSION(sd);
    if (r4 < TRANS) {
        const float eio = flip < 0 ? (1.0f / ETA(sd)) : ETA(sd), F = Fr_L(dot(iN, wo), eio);
        float3 beer = mk3(1);
        beer.x = exp_cw(-sd.transmittance.x * distance * 2.0f);
        beer.y = exp_cw(-sd.transmittance.y * distance * 2.0f);
        beer.z = exp_cw(-sd.transmittance.z * distance * 2.0f);
        if (r3 < F) {
            wi = reflect(wo * -1.0f, iN);
            bsdf = sd.color * beer * (1 / fabsf(dot(iN, wi)));
        } else {
            if (!Refract_L(wo, iN, eio, wi)) return mk3(0);
            return sd.color * beer * 1.0f * (1 / fabsf(dot(iN, wi)));
        }
    } else {
        const float R = ROUGHNESS(sd);
        const float pReflect = 1 - R;
        if (r3 < pReflect) {
            wi = reflect(wo * -1.0f, iN);
            bsdf = sd.color * (1.0f / fabsf(dot(iN, wi)));
        } else {
            const float r5 = (r3 - pReflect) / (1 - pReflect);
            const float r6 = (r4 - TRANS) / (1 - TRANS);
            wi = normalize(Tangent2World(DiffuseReflectionCosWeighted(r5, r6), iN));
            pdf = fmaxf(0.0f, dot(wi, iN)) * INVPI;
            specular = false;
            bsdf = sd.color * INVPI;
        }
    }
    if (dot(N * flip, wi) <= 0) pdf = 0;
    return bsdf;
}

/* ---- lights ---- */
LH2G_DEV float3 RandomBarycentrics(const float r0) {
    const uint32_t uf = f2u(r0 * 4294967296.0f);
    float2 A = make_float2(1, 0), B = make_float2(0, 1), C = make_float2(0, 0);
    for (int i = 0; i < 16; ++i) {
        const int d = (int)((uf >> (2 * (15 - i))) & 0x3u);
        float2 An, Bn, Cn;
        if (d == 0) An = (B + C) * 0.5f, Bn = (A + C) * 0.5f, Cn = (A + B) * 0.5f;
        else if (d == 1) An = A, Bn = (A + B) * 0.5f, Cn = (A + C) * 0.5f;
        else if (d == 2) An = (B + A) * 0.5f, Bn = B, Cn = (B + C) * 0.5f;
        else An = (C + A) * 0.5f, Bn = (C + B) * 0.5f, Cn = C;
        A = An, B = Bn, C = Cn;
    }
    const float2 r = (A + B + C) * 0.3333333f;
    return make_float3(r.x, r.y, 1 - r.x - r.y);
}

LH2G_DEV float PotentialTri(const SceneGPU& S, const int idx, const float3& I, const float3& N, const float3& bary) {
    const float4* l = S.triLights + (size_t)idx * 6;
    const float4 c4 = __ldg(l), n4 = __ldg(l + 1), v0 = __ldg(l + 3), v1 = __ldg(l + 4), v2 = __ldg(l + 5);
    float3 L = bary.x * xyz(v0) + bary.y * xyz(v1) + bary.z * xyz(v2);
    L = L - I;
    const float att = 1.0f / dot(L, L);
    L = normalize(L);
    const float LNdotL = fmaxf(0.0f, -dot(xyz(n4), L));
    const float NdotL = fmaxf(0.0f, dot(N, L));
    return c4.w * LNdotL * NdotL * att;
}
LH2G_DEV float PotentialPoint(const SceneGPU& S, const int idx, const float3& I, const float3& N) {
    const float4 p = __ldg(S.pointLights + (size_t)idx * 2);
    const float3 L = xyz(p) - I;
    const float NdotL = fmaxf(0.0f, dot(N, normalize(L)));
    const float att = 1.0f / dot(L, L);
    return p.w * NdotL * att;
}
LH2G_DEV float PotentialSpot(const SceneGPU& S, const int idx, const float3& I, const float3& N) {
    const float4 p = __ldg(S.spotLights + (size_t)idx * 3), r = __ldg(S.spotLights + (size_t)idx * 3 + 1), d4 = __ldg(S.spotLights + (size_t)idx * 3 + 2);
    float3 L = xyz(p) - I;
    const float att = 1.0f / dot(L, L);
    L = normalize(L);
    const float d = (fmaxf(0.0f, -dot(L, xyz(d4))) - r.w) / (p.w - r.w);
    const float NdotL = fmaxf(0.0f, dot(N, L));
    const float LNdotL = fmaxf(0.0f, fminf(1.0f, d));
    return (r.x + r.y + r.z) * LNdotL * NdotL * att;
}
LH2G_DEV float PotentialDir(const SceneGPU& S, const int idx, const float3& N) {
    const float4 d = __ldg(S.dirLights + (size_t)idx * 2);
    const float LNdotL = fmaxf(0.0f, -(d.x * N.x + d.y * N.y + d.z * N.z));
    return d.w * LNdotL;
}
LH2G_DEV float Potential(const SceneGPU& S, int i, const float3& I, const float3& N, const float3& bary) {
    if (i < S.nTri) return PotentialTri(S, i, I, N, bary);
    i -= S.nTri;
    if (i < S.nPoint) return PotentialPoint(S, i, I, N);
    i -= S.nPoint;
    if (i < S.nSpot) return PotentialSpot(S, i, I, N);
    return PotentialDir(S, i - S.nSpot, N);
}

/* pot: this thread's slice of a potential array (entry i at pot[i * stride]), as the reference's local
 * potential[MAXISLIGHTS] array (lights_shared.h:232); it lives in shared memory. */
LH2G_DEV float3 RandomPointOnLight(const SceneGPU& S, float r0, float r1, const float3& I, const float3& N, float& pickProb, float& lightPdf, float3& lightColor,
                                   float* pot, const int stride, int& picked) {
    const int lights = S.nTri + S.nPoint + S.nSpot + S.nDir;
    const float lightCount = (float)lights;
    const float3 bary = RandomBarycentrics(r0);
    float sum = 0, total = 0;
    int lightIdx = 0;
    for (int i = 0; i < lights; i++) {
        const float c = Potential(S, i, I, N, bary);
        pot[i * stride] = c;
        sum += c;
    }
    if (sum <= 0) { lightPdf = 0; return mk3(1); }
    r1 *= sum;
    for (int i = 0; i < lights; i++) {
        total += pot[i * stride];
        if (total >= r1) { lightIdx = i; break; }
    }
    pickProb = pot[lightIdx * stride] / sum;
    lightIdx = max(0, min(lightIdx, f2i(lightCount) - 1));
    picked = lightIdx;
    if (lightIdx < S.nTri) {
        const float4* l = S.triLights + (size_t)lightIdx * 6;
        const float4 n4 = __ldg(l + 1), r4 = __ldg(l + 2), v0 = __ldg(l + 3), v1 = __ldg(l + 4), v2 = __ldg(l + 5);
        lightColor = xyz(r4);
        const float3 P = bary.x * xyz(v0) + bary.y * xyz(v1) + bary.z * xyz(v2);
        float3 L = I - P;
        const float sqDist = dot(L, L);
        L = normalize(L);
        const float LNdotL = L.x * n4.x + L.y * n4.y + L.z * n4.z;
        const float reciSolidAngle = sqDist / (n4.w * LNdotL);
        lightPdf = (LNdotL > 0 && dot(L, N) < 0) ? reciSolidAngle : 0;
        return P;
    } else if (lightIdx < S.nTri + S.nPoint) {
        const float4* l = S.pointLights + (size_t)(lightIdx - S.nTri) * 2;
        const float4 p = __ldg(l), r = __ldg(l + 1);
        const float3 P = xyz(p);
        const float3 L = P - I;
        const float sqDist = dot(L, L);
        lightColor = xyz(r) / sqDist;
        lightPdf = dot(L, N) > 0 ? 1.0f : 0.0f;
        return P;
    } else if (lightIdx < S.nTri + S.nPoint + S.nSpot) {
        const float4* l = S.spotLights + (size_t)(lightIdx - S.nTri - S.nPoint) * 3;
        const float4 V0 = __ldg(l), V1 = __ldg(l + 1), Dd = __ldg(l + 2);
        const float3 P = xyz(V0);
        float3 L = I - P;
        const float sqDist = dot(L, L);
        L = normalize(L);
        const float d = (fmaxf(0.0f, L.x * Dd.x + L.y * Dd.y + L.z * Dd.z) - V1.w) / (V0.w - V1.w);
        const float LNdotL = fminf(1.0f, d);
        lightPdf = (LNdotL > 0 && dot(L, N) < 0) ? (sqDist / LNdotL) : 0;
        lightColor = xyz(V1);
        return P;
    } else {
        const float4* l = S.dirLights + (size_t)(lightIdx - S.nTri - S.nPoint - S.nSpot) * 2;
        const float4 d4 = __ldg(l), r4 = __ldg(l + 1);
        const float3 L = xyz(d4);
        lightColor = xyz(r4);
        const float NdotL = dot(L, N);
        lightPdf = NdotL < 0 ? 1.0f : 0.0f;
        return I - 1000.0f * L;
    }
}

/* ---- stochastic lightcuts through the light tree (LH2G_RP_LIGHTTREE) ----
 * Records of 4 float4 (light_tree.h): (light, left, right, intensity), box min, box max, (normal, parent). */
LH2G_DEV int4 tree_head(const SceneGPU& S, const int node) {
    const float4 h = __ldg(S.lightTree + (size_t)node * 4);
    return make_int4(__float_as_int(h.x), __float_as_int(h.y), __float_as_int(h.z), __float_as_int(h.w));
}

/* CalculateChildNodeWeights (lights_shared.h:120-156): the chance of the left child of node from I with normal N,
 * the mean of the two bounds the distances to the children's boxes give; six numbers drawn from seed, three for a
 * random point in each child's box (drawn x, y, z in that order, the order the CUDA compiler evaluates the
 * reference's make_float3 arguments in). As in the reference, wmax_k takes the left child's F and intensity. */
LH2G_DEV float light_tree_left_weight(const SceneGPU& S, const int node, const float3& I, const float3& N, uint32_t& seed) {
    const int4 h = tree_head(S, node);
    const int left = h.y, right = h.z;
    const float4* tl = S.lightTree + (size_t)left * 4;
    const float4* tr = S.lightTree + (size_t)right * 4;
    const float3 b1j = xyz(__ldg(tl + 1)), b2j = xyz(__ldg(tl + 2));
    const float3 b1k = xyz(__ldg(tr + 1)), b2k = xyz(__ldg(tr + 2));
    const float3 diag_j = b2j - b1j, diag_k = b2k - b1k;
    const float3 LN = xyz(__ldg(S.lightTree + (size_t)node * 4 + 3));
    const float3 Bj = 0.5f * diag_j, Bk = 0.5f * diag_k;
    const float3 Cj = (b1j + b2j) * 0.5f, Ck = (b1k + b2k) * 0.5f;
    const float3 Dj = Cj - I, Dk = Ck - I;
    const float3 min_j = make_float3(fmaxf(Dj.x - Bj.x, 0.0f), fmaxf(Dj.y - Bj.y, 0.0f), fmaxf(Dj.z - Bj.z, 0.0f));
    const float3 min_k = make_float3(fmaxf(Dk.x - Bk.x, 0.0f), fmaxf(Dk.y - Bk.y, 0.0f), fmaxf(Dk.z - Bk.z, 0.0f));
    const float dist2j = dot(min_j, min_j), dist2k = dot(min_k, min_k);
    const float3 max_j = Dj + Bj, max_k = Dk + Bk;
    const float dist2j_max = dot(max_j, max_j), dist2k_max = dot(max_k, max_k);
    const float Ij = __int_as_float(tree_head(S, left).w), Ik = __int_as_float(tree_head(S, right).w);
    const float rj0 = RandomFloat(seed), rj1 = RandomFloat(seed), rj2 = RandomFloat(seed);
    const float3 Rj = b1j + (b2j - b1j) * make_float3(rj0, rj1, rj2);
    const float rk0 = RandomFloat(seed), rk1 = RandomFloat(seed), rk2 = RandomFloat(seed);
    const float3 Rk = b1k + (b2k - b1k) * make_float3(rk0, rk1, rk2);
    const float3 Lj = normalize(Rj - I), Lk = normalize(Rk - I);
    float Fj = fmaxf(0.001f, dot(N, Lj)), Fk = fmaxf(0.001f, dot(N, Lk));
    if (dot(LN, LN) > 0.001f) Fj *= fmaxf(0.001f, dot(LN, Lj * -1.0f)), Fk *= fmaxf(0.001f, dot(LN, Lk * -1.0f));
    const bool insideBoth = dist2j == 0 && dist2k == 0;
    const float wmin_j = (Fj * Ij) / (insideBoth ? 1.0f : fmaxf(0.0001f, dist2j));
    const float wmin_k = (Fk * Ik) / (insideBoth ? 1.0f : fmaxf(0.0001f, dist2k));
    const float wmax_j = (Fj * Ij) / fmaxf(0.0001f, dist2j_max);
    const float wmax_k = (Fj * Ij) / fmaxf(0.0001f, dist2k_max);
    const float pmin_j = wmin_j / (wmin_j + wmin_k);
    const float pmax_j = wmax_j / (wmax_j + wmax_k);
    return 0.5f * (pmin_j + pmax_j);
}

/* LightPickProbLTree (lights_shared.h:198-217): the chance that the tree picks area light idx, the product of the
 * branch chances from its leaf (record idx + 1) up to the root, the weights taken at I (the light point, as the
 * reference passes it) with normal N. A leaf without a parent (a one-light tree: the reference would read
 * record -1) ends the walk. */
LH2G_DEV float light_pick_prob_tree(const SceneGPU& S, const int idx, const float3& N, const float3& I, uint32_t& seed) {
    int node = idx + 1;
    float pickProb = 1;
    for (int guard = 0; guard < S.nTreeNodes && node > 0 && node < S.nTreeNodes; guard++) {
        const int parent = __float_as_int(__ldg(S.lightTree + (size_t)node * 4 + 3).w);
        if (parent < 0) break;
        const float p = light_tree_left_weight(S, parent, I, N, seed);
        if (tree_head(S, parent).y == node) pickProb *= p; else pickProb *= 1 - p;
        node = parent;
    }
    return pickProb;
}

/* RandomPointOnLightLTree (lights_shared.h:322-395): walk from the root, at each interior node to the left child
 * with its weight's chance (r1 rescaled to the chosen branch), then a point on the leaf's light as
 * RandomPointOnLight does. picked: the light's index over area, point and spot lights. A scene without tree lights
 * gives lightPdf 0. */
LH2G_DEV float3 RandomPointOnLightTree(const SceneGPU& S, float r0, float r1, uint32_t& seed, const float3& I, const float3& N, float& pickProb,
                                       float& lightPdf, float3& lightColor, int& picked) {
    pickProb = 1;
    if (S.nTreeNodes <= 0) { lightPdf = 0; return mk3(1); }
    int node = 0, lightIdx = 0;
    for (int guard = 0; guard <= S.nTreeNodes; guard++) {
        const int4 h = tree_head(S, node);
        if (h.y == -1) { lightIdx = h.x; break; }
        const float p_j = light_tree_left_weight(S, node, I, N, seed);
        if (r1 < p_j) node = h.y, r1 *= 1.0f / p_j, pickProb *= p_j;
        else node = h.z, r1 = (r1 - p_j) / (1 - p_j), pickProb *= 1 - p_j;
    }
    if (lightIdx & (1 << 30)) {
        const int k = lightIdx - (1 << 30);
        picked = S.nTri + k;
        const float4* l = S.pointLights + (size_t)k * 2;
        const float4 p = __ldg(l), r = __ldg(l + 1);
        const float3 P = xyz(p);
        const float3 L = P - I;
        const float sqDist = dot(L, L);
        lightColor = xyz(r) / sqDist;
        lightPdf = dot(L, N) > 0 ? 1.0f : 0.0f;
        return P;
    } else if (lightIdx & (1 << 29)) {
        const int k = lightIdx - (1 << 29);
        picked = S.nTri + S.nPoint + k;
        const float4* l = S.spotLights + (size_t)k * 3;
        const float4 V0 = __ldg(l), V1 = __ldg(l + 1), Dd = __ldg(l + 2);
        const float3 P = xyz(V0);
        float3 L = I - P;
        const float sqDist = dot(L, L);
        L = normalize(L);
        const float d = (fmaxf(0.0f, L.x * Dd.x + L.y * Dd.y + L.z * Dd.z) - V1.w) / (V0.w - V1.w);
        const float LNdotL = fminf(1.0f, d);
        lightPdf = (LNdotL > 0 && dot(L, N) < 0) ? (sqDist / LNdotL) : 0;
        lightColor = xyz(V1);
        return P;
    } else {
        picked = lightIdx;
        const float3 bary = RandomBarycentrics(r0);
        const float4* l = S.triLights + (size_t)lightIdx * 6;
        const float4 n4 = __ldg(l + 1), r4 = __ldg(l + 2), v0 = __ldg(l + 3), v1 = __ldg(l + 4), v2 = __ldg(l + 5);
        lightColor = xyz(r4);
        const float3 P = bary.x * xyz(v0) + bary.y * xyz(v1) + bary.z * xyz(v2);
        float3 L = I - P;
        const float sqDist = dot(L, L);
        L = normalize(L);
        const float LNdotL = L.x * n4.x + L.y * n4.y + L.z * n4.z;
        const float reciSolidAngle = sqDist / (n4.w * LNdotL);
        lightPdf = (LNdotL > 0 && dot(L, N) < 0) ? reciSolidAngle : 0;
        return P;
    }
}

LH2G_DEV float3 SampleSkydome(const SceneGPU& S, const float3& Dw) {
    if (S.skyW <= 0 || S.skyH <= 0) return mk3(0);
    const float4 m0 = S.worldToSky[0], m1 = S.worldToSky[1], m2 = S.worldToSky[2];
    const float3 D = -make_float3(m0.x * Dw.x + m0.y * Dw.y + m0.z * Dw.z, m1.x * Dw.x + m1.y * Dw.y + m1.z * Dw.z, m2.x * Dw.x + m2.y * Dw.y + m2.z * Dw.z);
    float p = atan2_at(D.y, D.x);
    p = (p < 0) ? (p + 2 * PI) : p;
    const float theta = acos_at(D.z < -1.f ? -1.f : (D.z > 1.f ? 1.f : D.z));
    const uint32_t u = f2u((float)S.skyW * p * INV2PI - 0.5f);
    const uint32_t v = f2u((float)S.skyH * theta * INVPI - 0.5f);
    const uint32_t idx = u + v * (uint32_t)S.skyW;
    return idx < (uint32_t)(S.skyW * S.skyH) ? xyz(__ldg(S.skyPixels + idx)) : mk3(0);
}

LH2G_DEV float SurvivalProbability(const float3& albedo) { return fminf(1.0f, fmaxf(fmaxf(albedo.x, albedo.y), albedo.z)); }
LH2G_DEV float3 SafeOrigin(const float3& O, const float3& R, const float3& N, const float geoEpsilon) {
    return O + N * (dot(N, R) > 0 ? geoEpsilon : -geoEpsilon);
}

}  // namespace lh2g

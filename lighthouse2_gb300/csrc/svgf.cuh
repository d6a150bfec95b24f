/* svgf.cuh - SVGF wire formats and helpers shared by the shading stage (feature gathering) and the filter.
 *
 * Formats of lib/CUDA/shared_kernel_code/tools_shared.h, written out in the evaluation order of that file:
 *   normal    10 bits per component at bits 2, 12, 22 ((n + 1) * 511); bits 0-1 hold the specular flag
 *   albedo    10:11:11 unsigned fixed point of min(1, c)
 *   light     two rgb triples as 5:11 unsigned fixed point in the bits of one float4 (direct in x, y;
 *             indirect in z, w), clamped at 31.999, so every field is below 65534 (the third field's word is
 *             masked to 23 bits when unpacked, which keeps every word the packer writes unchanged)
 * Fields are turned into floats with u2f23 (exact, no conversion instruction): the a-trous taps unpack ~290
 * fields per pixel and pass.
 *   features  uint4 {albedo, normal | specular, depth bits, history (4 bits) | specular << 4 | material << 6}
 */
#pragma once
#include "device_math.cuh"

namespace lh2g {

constexpr uint32_t S_BOUNCED = 2;        /* path has left a diffuse vertex (RenderCore_Optix7Filter/kernels/pathtracer.h:30) */
constexpr uint32_t S_VIASPECULAR = 4;    /* path has seen a specular vertex */

LH2G_DEV float4 operator-(float4 a, float4 b) { return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
LH2G_DEV float dot4(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
LH2G_DEV float3 fmin3(float a, float3 b) { return make_float3(fminf(a, b.x), fminf(a, b.y), fminf(a, b.z)); }
LH2G_DEV float3 fmin3(float3 a, float b) { return make_float3(fminf(a.x, b), fminf(a.y, b), fminf(a.z, b)); }
LH2G_DEV float3 fmax3(float a, float3 b) { return make_float3(fmaxf(a, b.x), fmaxf(a, b.y), fmaxf(a, b.z)); }
LH2G_DEV float clampf(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
LH2G_DEV float3 clamp3(float3 v, float3 a, float3 b) { return make_float3(clampf(v.x, a.x, b.x), clampf(v.y, a.y, b.y), clampf(v.z, a.z, b.z)); }

LH2G_DEV uint32_t PackNormal2(const float3 N) {
    const uint32_t x = min(f2u((N.x + 1) * 511), 1023u);
    const uint32_t y = min(f2u((N.y + 1) * 511), 1023u);
    const uint32_t z = min(f2u((N.z + 1) * 511), 1023u);
    return (x << 2u) + (y << 12u) + (z << 22u);
}
LH2G_DEV float3 UnpackNormal2(const uint32_t pi) {
    const uint32_t x = (pi >> 2u) & 1023u, y = (pi >> 12u) & 1023u, z = pi >> 22u;
    return make_float3(u2f23(x) * (1.0f / 511.0f) - 1, u2f23(y) * (1.0f / 511.0f) - 1, u2f23(z) * (1.0f / 511.0f) - 1);
}
LH2G_DEV uint32_t HDRtoRGB32(const float3& c) {
    const uint32_t r = f2u(1023.0f * fminf(1.0f, c.x));
    const uint32_t g = f2u(2047.0f * fminf(1.0f, c.y));
    const uint32_t b = f2u(2047.0f * fminf(1.0f, c.z));
    return (r << 22) + (g << 11) + b;
}
LH2G_DEV float3 RGB32toHDR(const uint32_t c) {
    return make_float3(u2f23(c >> 22) * (1.0f / 1023.0f), u2f23((c >> 11) & 2047u) * (1.0f / 2047.0f), u2f23(c & 2047u) * (1.0f / 2047.0f));
}
LH2G_DEV float3 RGB32toHDRmin1(const uint32_t c) {
    return make_float3(u2f23(max(1u, c >> 22)) * (1.0f / 1023.0f), u2f23(max(1u, (c >> 11) & 2047u)) * (1.0f / 2047.0f),
                       u2f23(max(1u, c & 2047u)) * (1.0f / 2047.0f));
}
/* PackFeatures (RenderCore_Optix7Filter/kernels/pathtracer.h:44-47); the history count in w & 15 survives */
LH2G_DEV void PackFeatures(uint4* f, const uint32_t albedo, const uint32_t packedNormal, const float t, const uint32_t isSpecular,
                           const uint32_t matid) {
    const uint32_t w = (isSpecular << 4) + (matid << 6) + (f->w & 15u);
    *f = make_uint4(albedo, packedNormal, __float_as_uint(t), w);
}
/* calculateDepthDerivatives (RenderCore_Optix7Filter/kernels/pathtracer.h:48-57) with the plane through the hit
 * point I and the world-space geometric normal N (the reference uses the object-space vertex 0 and face normal,
 * the same plane for an identity instance transform); p2, p3 are the view's p2 - p1 and p3 - p1 */
LH2G_DEV float4 DepthDerivatives(const int x, const int y, const int w, const int h, const float depth, const float3& I, const float3& N,
                                 const float3& p1, const float3& p2, const float3& p3, const float3& pos) {
    const float3 rayDXDir = normalize((p1 + (float)(x + 0.5f + 1) * (1.0f / w) * p2 + (float)(y + 0.5f) * (1.0f / h) * p3) - pos);
    const float rayDXDepth = dot(I - pos, N) / dot(N, rayDXDir);
    const float3 rayDYDir = normalize((p1 + (float)(x + 0.5f) * (1.0f / w) * p2 + (float)(y + 0.5f + 1) * (1.0f / h) * p3) - pos);
    const float rayDYDepth = dot(I - pos, N) / dot(N, rayDYDir);
    return make_float4(0, 0, rayDXDepth - depth, rayDYDepth - depth);
}

LH2G_DEV float Luminance(const float3 rgb) { return 0.299f * fminf(rgb.x, 10.0f) + 0.587f * fminf(rgb.y, 10.0f) + 0.114f * fminf(rgb.z, 10.0f); }
LH2G_DEV float3 RGBToYCoCg(const float3 RGB) {
    const float3 rgb = fmin3(4.0f, RGB);
    const float Y = dot(rgb, make_float3(1, 2, 1)) * 0.25f;
    const float Co = dot(rgb, make_float3(2, 0, -2)) * 0.25f + (0.5f * 256.0f / 255.0f);
    const float Cg = dot(rgb, make_float3(-1, 2, -1)) * 0.25f + (0.5f * 256.0f / 255.0f);
    return make_float3(Y, Co, Cg);
}
LH2G_DEV float3 YCoCgToRGB(const float3 c) {
    const float Y = c.x, Co = c.y - (0.5f * 256.0f / 255.0f), Cg = c.z - (0.5f * 256.0f / 255.0f);
    return make_float3(Y + Co - Cg, Y + Cg, Y - Co - Cg);
}
LH2G_DEV float4 CombineToFloat4(const float3& A, const float3& B) {
    const uint32_t Ar = f2u(fminf(A.x, 31.999f) * 2048.0f), Ag = f2u(fminf(A.y, 31.999f) * 2048.0f), Ab = f2u(fminf(A.z, 31.999f) * 2048.0f);
    const uint32_t Br = f2u(fminf(B.x, 31.999f) * 2048.0f), Bg = f2u(fminf(B.y, 31.999f) * 2048.0f), Bb = f2u(fminf(B.z, 31.999f) * 2048.0f);
    return make_float4(__uint_as_float((Ar << 16) + Ag), __uint_as_float(Ab), __uint_as_float((Br << 16) + Bg), __uint_as_float(Bb));
}
LH2G_DEV float3 GetDirect(const float4& X) {
    const uint32_t v0 = __float_as_uint(X.x), v1 = __float_as_uint(X.y);
    return make_float3(u2f23(v0 >> 16) * (1.0f / 2048.0f), u2f23(v0 & 65535u) * (1.0f / 2048.0f), u2f23(v1 & 0x7fffffu) * (1.0f / 2048.0f));
}
LH2G_DEV float3 GetIndirect(const float4& X) {
    const uint32_t v2 = __float_as_uint(X.z), v3 = __float_as_uint(X.w);
    return make_float3(u2f23(v2 >> 16) * (1.0f / 2048.0f), u2f23(v2 & 65535u) * (1.0f / 2048.0f), u2f23(v3 & 0x7fffffu) * (1.0f / 2048.0f));
}
LH2G_DEV float oneoverpow2(const int p) { return __uint_as_float((uint32_t)(127 - p) << 23); }
/* x^128 by seven squarings (the reference calls powf(x, 128)) */
LH2G_DEV float pow128(float x) {
#pragma unroll
    for (int i = 0; i < 7; i++) x = x * x;
    return x;
}
/* Mitchell-Netravali cubic with B = C = 1/3 (sampling_shared.h:22-27) */
LH2G_DEV float MitchellNetravali(const float v) {
    const float B = 1.0f / 3.0f, C = 1.0f / 3.0f, x = fabsf(v), x2 = x * x, x3 = x2 * x;
    if (x < 1) return (1.0f / 6.0f) * ((12 - 9 * B - 6 * C) * x3 + (-18 + 12 * B + 6 * C) * x2 + (6 - 2 * B));
    else if (x < 2) return 1.0f / 6.0f * ((-B - 6 * C) * x3 + (6 * B + 30 * C) * x2 + (-12 * B - 48 * C) * x + (8 * B + 24 * C));
    return 0.0f;
}

/* The previous camera as a plane and two screen axes scaled to pixels (prepareFilter's host part,
 * finalize_shared.h:293-314). Computed on the host. */
struct SvgfView { float4 prevPos, prevE, prevRight, prevUp; };

/* Device buffers of the filter (W*H entries). */
struct SvgfBuffers {
    uint4* features;
    float4* worldPos;
    float4* prevWorldPos;
    float4* deltaDepth;
    float2* motion;
    float4* moments;
    float4* prevMoments;
    float4* shading;
    float4* filteredIN;
    float4* filteredOUT;
    float4* prevPixels;
    float4* taaPixels;
    float4* accum;       /* 2*W*H: direct, indirect */
    float4* target;      /* the frame */
};

struct SvgfArgs {
    int W, H;
    float scale;         /* 1 / samplesTaken */
    float j0, j1, prevj0, prevj1;
    float clampDirect, clampIndirect;
    int camIsStationary;
    SvgfView view;
};

/* prepare, apply x 3, TAA + unsharpen or finalizeNoTAA; the caller swaps the history pointers afterwards */
void launch_svgf(const SvgfBuffers& b, const SvgfArgs& a, bool taa, cudaStream_t st);

}  // namespace lh2g

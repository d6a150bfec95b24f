/* device_math.cuh - device arithmetic of the GB300 render core.
 *
 * The library is compiled with --fmad=false, -prec-div=true, -prec-sqrt=true and without fast-math: every
 * expression below rounds exactly like the reference's formulas written out in IEEE single precision, and
 * fused multiply-adds appear only where written explicitly (in conservative culling code whose result does
 * not feed shading). Vector helpers use the evaluation order of lib/CUDA/helper_math.h.
 */
#pragma once
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#define LH2G_DEV static __device__ __forceinline__

namespace lh2g {

LH2G_DEV float3 mk3(float x, float y, float z) { return make_float3(x, y, z); }
LH2G_DEV float3 mk3(float s) { return make_float3(s, s, s); }
LH2G_DEV float3 xyz(const float4& a) { return make_float3(a.x, a.y, a.z); }
LH2G_DEV float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
LH2G_DEV float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
LH2G_DEV float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
LH2G_DEV float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
LH2G_DEV float3 operator*(float3 a, float b) { return make_float3(a.x * b, a.y * b, a.z * b); }
LH2G_DEV float3 operator*(float b, float3 a) { return make_float3(b * a.x, b * a.y, b * a.z); }
LH2G_DEV float3 operator/(float3 a, float b) { return make_float3(a.x / b, a.y / b, a.z / b); }
LH2G_DEV float3 operator+(float3 a, float b) { return make_float3(a.x + b, a.y + b, a.z + b); }
LH2G_DEV float3 operator+(float b, float3 a) { return make_float3(b + a.x, b + a.y, b + a.z); }
LH2G_DEV float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
LH2G_DEV float2 operator*(float2 a, float2 b) { return make_float2(a.x * b.x, a.y * b.y); }
LH2G_DEV float2 operator*(float2 a, float b) { return make_float2(a.x * b, a.y * b); }
LH2G_DEV float4 operator+(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
LH2G_DEV float4 operator*(float4 a, float b) { return make_float4(a.x * b, a.y * b, a.z * b, a.w * b); }
LH2G_DEV float4 operator*(float b, float4 a) { return make_float4(b * a.x, b * a.y, b * a.z, b * a.w); }
LH2G_DEV float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
LH2G_DEV float3 cross(float3 a, float3 b) { return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
LH2G_DEV float length(float3 v) { return sqrtf(dot(v, v)); }
LH2G_DEV float3 normalize(float3 v) { const float inv = 1.0f / sqrtf(dot(v, v)); return v * inv; }
LH2G_DEV float3 reflect(float3 i, float3 n) { return i - 2.0f * n * dot(n, i); }

constexpr float PI = 3.14159265358979323846264f;
constexpr float INVPI = 0.31830988618379067153777f;
constexpr float INV2PI = 0.15915494309189533576888f;
constexpr float TWOPI = 6.28318530717958647692528f;
constexpr float EPSILON = 0.0001f;
constexpr int MIPLEVELCOUNT = 5;
constexpr int NOHIT = -1;
constexpr uint32_t S_SPECULAR = 1;

/* three-input minimum and maximum (one instruction on sm_100 and later; the same value as two fminf / fmaxf) */
LH2G_DEV float fmax3f(float a, float b, float c) { float d; asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c)); return d; }
LH2G_DEV float fmin3f(float a, float b, float c) { float d; asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c)); return d; }

/* float -> integer conversions (cvt.rzi: truncation, saturation, NaN -> 0) */
LH2G_DEV uint32_t f2u(float x) { return __float2uint_rz(x); }
LH2G_DEV int f2i(float x) { return __float2int_rz(x); }
/* The float of an unsigned integer v < 2^23, exactly (float)v, without the conversion pipe (a quarter of the
 * FP32 rate and the bottleneck of code that unpacks many small fixed-point fields): 2^23 + v has the bit
 * pattern 0x4B000000 | v, and subtracting 2^23 is exact. */
LH2G_DEV float u2f23(uint32_t v) { return __uint_as_float(0x4B000000u | v) - 8388608.0f; }

/* ---- transcendental functions: Cody-Waite reduction + truncated Taylor series; atanh series for log2 ---- */
constexpr float CW_PIO2_1 = 1.5703125f, CW_PIO2_2 = 4.838705062866211e-4f, CW_PIO2_3 = -4.371138828673793e-8f;
constexpr float TWO_OVER_PI = 0.6366197466850281f;
constexpr float LN2_HI = 0.693145751953125f, LN2_LO = 1.428606765330187e-06f, LOG2E = 1.4426950216293335f;

LH2G_DEV void sincos_cw(float x, float* s, float* c) {
    const float kf = rintf(x * TWO_OVER_PI);
    float r = x - kf * CW_PIO2_1;
    r = r - kf * CW_PIO2_2;
    r = r - kf * CW_PIO2_3;
    const float r2 = r * r;
    const float sp = r + r * r2 * ((float)(-1.0 / 6.0) + r2 * ((float)(1.0 / 120.0) + r2 * ((float)(-1.0 / 5040.0) + r2 * (float)(1.0 / 362880.0))));
    const float cp = 1.0f + r2 * (-0.5f + r2 * ((float)(1.0 / 24.0) + r2 * ((float)(-1.0 / 720.0) + r2 * ((float)(1.0 / 40320.0) + r2 * (float)(-1.0 / 3628800.0)))));
    const int q = f2i(kf) & 3;
    if (q == 0) { *s = sp; *c = cp; }
    else if (q == 1) { *s = cp; *c = -sp; }
    else if (q == 2) { *s = -sp; *c = -cp; }
    else { *s = -cp; *c = sp; }
}

LH2G_DEV float exp_cw(float x) {
    if (x != x) return x;
    if (x > 88.72283f) return __int_as_float(0x7f800000);
    if (x < -87.33654f) return 0.0f;
    /* k = rint(x log2 e): |x log2 e| <= 128 here, so adding 1.5 * 2^23 rounds it to an integer (to nearest even,
     * as rintf does) in the low mantissa bits; no conversion instruction is needed for kf or k */
    const float shifted = x * LOG2E + 12582912.0f;
    const float kf = shifted - 12582912.0f;
    float r = x - kf * LN2_HI;
    r = r - kf * LN2_LO;
    const float p = 1.0f + r * (1.0f + r * (0.5f + r * ((float)(1.0 / 6.0) + r * ((float)(1.0 / 24.0) + r * ((float)(1.0 / 120.0) + r * ((float)(1.0 / 720.0) + r * (float)(1.0 / 5040.0)))))));
    const int k = __float_as_int(shifted) - 0x4B400000;
    if (k > 127) return p * __int_as_float(0x7f000000) * 2.0f;
    if (k < -126) return p * __int_as_float((k + 127 + 64) << 23) * __int_as_float(0x1f800000);
    return p * __int_as_float((k + 127) << 23);
}

LH2G_DEV float log2_at(float x) {
    if (x != x) return x;
    if (x < 0.0f) return __int_as_float(0x7fc00000);
    if (x == 0.0f) return __int_as_float(0xff800000);
    if (x == __int_as_float(0x7f800000)) return x;
    uint32_t b = __float_as_uint(x);
    int e = 0;
    if (b < 0x00800000u) { x = x * 8388608.0f; b = __float_as_uint(x); e = -23; }
    e += (int)((b >> 23) & 255u) - 127;
    float m = __uint_as_float((b & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    const float at = s + s * s2 * ((float)(1.0 / 3.0) + s2 * ((float)(1.0 / 5.0) + s2 * ((float)(1.0 / 7.0) + s2 * ((float)(1.0 / 9.0) + s2 * (float)(1.0 / 11.0)))));
    return (float)e + at * 2.885390043258667f;
}

/* natural logarithm: log2_at's reduction and atanh series, ln x = e ln 2 + 2 atanh(s) (ln 2 split in two so that
 * e ln 2 is exact) */
LH2G_DEV float log_at(float x) {
    if (x != x) return x;
    if (x < 0.0f) return __int_as_float(0x7fc00000);
    if (x == 0.0f) return __int_as_float(0xff800000);
    if (x == __int_as_float(0x7f800000)) return x;
    uint32_t b = __float_as_uint(x);
    int e = 0;
    if (b < 0x00800000u) { x = x * 8388608.0f; b = __float_as_uint(x); e = -23; }
    e += (int)((b >> 23) & 255u) - 127;
    float m = __uint_as_float((b & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    const float at = s + s * s2 * ((float)(1.0 / 3.0) + s2 * ((float)(1.0 / 5.0) + s2 * ((float)(1.0 / 7.0) + s2 * ((float)(1.0 / 9.0) + s2 * (float)(1.0 / 11.0)))));
    return (float)e * LN2_HI + ((float)e * LN2_LO + at * 2.0f);
}

/* x^y as exp(y ln x) for x > 0; 0^y = 0 (y > 0) or 1 (y = 0); NaN for x < 0 (the BSDFs raise squared roughness in
 * (0, 1) to a power in [0, 1]) */
LH2G_DEV float pow_at(float x, float y) {
    if (x != x || y != y) return x + y;
    if (x < 0.0f) return __int_as_float(0x7fc00000);
    if (y == 0.0f) return 1.0f;
    if (x == 0.0f) return y > 0.0f ? 0.0f : __int_as_float(0x7f800000);
    return exp_cw(y * log_at(x));
}

LH2G_DEV float atan_unit(float t) {
    float a = fabsf(t), off = 0.0f;
    if (a > 0.41421356f) { a = (a - 1.0f) / (a + 1.0f); off = 0.7853981852531433f; }
    const float a2 = a * a;
    const float p = a + a * a2 * ((float)(-1.0 / 3.0) + a2 * ((float)(1.0 / 5.0) + a2 * ((float)(-1.0 / 7.0) + a2 * ((float)(1.0 / 9.0) + a2 * ((float)(-1.0 / 11.0) + a2 * ((float)(1.0 / 13.0) + a2 * ((float)(-1.0 / 15.0) + a2 * ((float)(1.0 / 17.0) + a2 * ((float)(-1.0 / 19.0) + a2 * (float)(1.0 / 21.0))))))))));
    const float r = off + p;
    return t < 0.0f ? -r : r;
}

LH2G_DEV float atan2_at(float y, float x) {
    if (x != x || y != y) return x + y;
    const float ax = fabsf(x), ay = fabsf(y);
    float r;
    if (ax == 0.0f && ay == 0.0f) r = 0.0f;
    else if (ay <= ax) r = atan_unit(ay / ax);
    else r = 1.5707963705062866f - atan_unit(ax / ay);
    if (x < 0.0f) r = 3.1415927410125732f - r;
    return y < 0.0f ? -r : r;
}

LH2G_DEV float acos_at(float x) {
    x = x < -1.0f ? -1.0f : (x > 1.0f ? 1.0f : x);
    return atan2_at(sqrtf((1.0f - x) * (1.0f + x)), x);
}

/* ---- random numbers (the reference's WangHash seeding and Marsaglia xorshift32) ---- */
LH2G_DEV uint32_t WangHash(uint32_t s) { s = (s ^ 61u) ^ (s >> 16), s *= 9u, s = s ^ (s >> 4), s *= 0x27d4eb2du, s = s ^ (s >> 15); return s; }
LH2G_DEV uint32_t RandomInt(uint32_t& s) { s ^= s << 13, s ^= s >> 17, s ^= s << 5; return s; }
/* the n-th xorshift32 successor of x (RandomUInt applied n times) */
LH2G_DEV uint32_t xorshift_n(uint32_t x, const int n) {
    for (int i = 0; i < n; i++) x ^= x << 13, x ^= x >> 17, x ^= x << 5;
    return x;
}
LH2G_DEV float RandomFloat(uint32_t& s) { return __uint2float_rn(RandomInt(s)) * 2.3283064365387e-10f; }

LH2G_DEV float half2float(uint32_t h) { return __half2float(__ushort_as_half((unsigned short)h)); }

}  // namespace lh2g

/* lh2o.cpp - CPU ORACLE of the GB300 wavefront render core. TEST INFRASTRUCTURE ONLY (see lh2o.h).
 *
 * Build: g++ -O2 -std=c++17 -fPIC -shared -ffp-contract=off -fno-fast-math (oracle/Makefile).
 * -ffp-contract=off matters: the reference arithmetic is restated operation by operation, and a fused
 * multiply-add would change the rounding of the results the GPU is compared against.
 *
 * Evaluation order follows lib/CUDA/helper_math.h: dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z, vector
 * operators are component-wise, normalize(v) = v * (1/sqrt(dot(v,v))) (the host form of rsqrtf,
 * helper_math.h:63-66 and 1305-1318).
 */
#include "lh2o.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace {

typedef uint32_t uint;

/* ------------------------------------------------------------------------------------------------------
 * vector types and helpers in the reference's evaluation order
 * ---------------------------------------------------------------------------------------------------- */
struct f2 { float x, y; };
struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };

inline f2 mk2(float x, float y) { return {x, y}; }
inline f3 mk3(float x, float y, float z) { return {x, y, z}; }
inline f3 mk3(float s) { return {s, s, s}; }
inline f3 mk3(const f4& a) { return {a.x, a.y, a.z}; }
inline f3 ld3(const float* p) { return {p[0], p[1], p[2]}; }
inline f4 mk4(float x, float y, float z, float w) { return {x, y, z, w}; }
inline f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
inline f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline f3 operator*(f3 a, float b) { return {a.x * b, a.y * b, a.z * b}; }
inline f3 operator*(float b, f3 a) { return {b * a.x, b * a.y, b * a.z}; }
inline f3 operator/(f3 a, float b) { return {a.x / b, a.y / b, a.z / b}; }
inline f2 operator+(f2 a, f2 b) { return {a.x + b.x, a.y + b.y}; }
inline f2 operator*(f2 a, f2 b) { return {a.x * b.x, a.y * b.y}; }
inline f2 operator*(f2 a, float b) { return {a.x * b, a.y * b}; }
inline f4 operator+(f4 a, f4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline f4 operator*(f4 a, float b) { return {a.x * b, a.y * b, a.z * b, a.w * b}; }
inline f4 operator*(float b, f4 a) { return {b * a.x, b * a.y, b * a.z, b * a.w}; }
inline float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline f3 cross(f3 a, f3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float length(f3 v) { return sqrtf(dot(v, v)); }
inline f3 normalize(f3 v) { const float inv = 1.0f / sqrtf(dot(v, v)); return v * inv; }
inline f3 reflect(f3 i, f3 n) { return i - 2.0f * n * dot(n, i); }
inline float fmaxr(float a, float b) { return fmaxf(a, b); }  /* CUDA's max(float, float) */
inline float fminr(float a, float b) { return fminf(a, b); }
inline int imin(int a, int b) { return a < b ? a : b; }
inline int imax(int a, int b) { return a > b ? a : b; }

inline uint fbits(float f) { uint u; memcpy(&u, &f, 4); return u; }
inline float bitsf(uint u) { float f; memcpy(&f, &u, 4); return f; }

/* Float to integer conversions with the semantics of the GPU's cvt.rzi instructions: truncation,
 * saturation at the range ends, NaN -> 0. C leaves the out-of-range cases undefined. */
inline uint f2u(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xffffffffu;
    return (uint)x;
}
inline int f2i(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int)0x80000000u;
    return (int)x;
}

constexpr float PI = 3.14159265358979323846264f;      /* common_settings.h:47-50 */
constexpr float INVPI = 0.31830988618379067153777f;
constexpr float INV2PI = 0.15915494309189533576888f;
constexpr float TWOPI = 6.28318530717958647692528f;
constexpr float EPSILON = 0.0001f;                    /* common_settings.h:53 */
constexpr int MIPLEVELCOUNT = 5;                      /* common_settings.h:57 */
constexpr int NOHIT = -1;
constexpr uint S_SPECULAR = 1;                        /* RenderCore_PrimeRef/kernels/pathtracer.h:29 */

/* ------------------------------------------------------------------------------------------------------
 * Transcendental functions. The reference calls the CUDA library (sincosf, __sincosf, expf, __expf,
 * log2f, atan2, acos); to make host and device results identical both sides use these, written from the
 * mathematics: Cody-Waite argument reduction (Cody & Waite, "Software Manual for the Elementary
 * Functions", 1980) followed by truncated Taylor series, and the atanh series for the logarithm.
 * The device code carries the same formulas operation by operation.
 * ---------------------------------------------------------------------------------------------------- */
constexpr float CW_PIO2_1 = 1.5703125f;                     /* pi/2 split: 8 + 12 + 24 significant bits */
constexpr float CW_PIO2_2 = 4.838705062866211e-4f;
constexpr float CW_PIO2_3 = -4.371138828673793e-8f;
constexpr float TWO_OVER_PI = 0.6366197466850281f;

inline void lm_sincos(float x, float* s, float* c) {
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

constexpr float LN2_HI = 0.693145751953125f;
constexpr float LN2_LO = 1.428606765330187e-06f;
constexpr float LOG2E = 1.4426950216293335f;

inline float lm_expf(float x) {
    if (x != x) return x;
    if (x > 88.72283f) return bitsf(0x7f800000u);
    if (x < -87.33654f) return 0.0f; /* results below the normal range flush to zero */
    const float kf = rintf(x * LOG2E);
    float r = x - kf * LN2_HI;
    r = r - kf * LN2_LO;
    const float p = 1.0f + r * (1.0f + r * (0.5f + r * ((float)(1.0 / 6.0) + r * ((float)(1.0 / 24.0) + r * ((float)(1.0 / 120.0) + r * ((float)(1.0 / 720.0) + r * (float)(1.0 / 5040.0)))))));
    const int k = f2i(kf);
    if (k > 127) return p * bitsf(0x7f000000u) * 2.0f;
    if (k < -126) return p * bitsf((uint)(k + 127 + 64) << 23) * bitsf(0x1f800000u); /* 2^(k+64) * 2^-64 */
    return p * bitsf((uint)(k + 127) << 23);
}

inline float lm_log2f(float x) {
    if (x != x) return x;
    if (x < 0.0f) return bitsf(0x7fc00000u);
    if (x == 0.0f) return bitsf(0xff800000u);
    if (x == bitsf(0x7f800000u)) return x;
    uint b = fbits(x);
    int e = 0;
    if (b < 0x00800000u) { x = x * 8388608.0f; b = fbits(x); e = -23; }
    e += (int)((b >> 23) & 255u) - 127;
    float m = bitsf((b & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    const float at = s + s * s2 * ((float)(1.0 / 3.0) + s2 * ((float)(1.0 / 5.0) + s2 * ((float)(1.0 / 7.0) + s2 * ((float)(1.0 / 9.0) + s2 * (float)(1.0 / 11.0)))));
    return (float)e + at * 2.885390043258667f;
}

inline float lm_atan_unit(float t) { /* |t| <= 1 */
    float a = fabsf(t), off = 0.0f;
    if (a > 0.41421356f) { a = (a - 1.0f) / (a + 1.0f); off = 0.7853981852531433f; }
    const float a2 = a * a;
    const float p = a + a * a2 * ((float)(-1.0 / 3.0) + a2 * ((float)(1.0 / 5.0) + a2 * ((float)(-1.0 / 7.0) + a2 * ((float)(1.0 / 9.0) + a2 * ((float)(-1.0 / 11.0) + a2 * ((float)(1.0 / 13.0) + a2 * ((float)(-1.0 / 15.0) + a2 * ((float)(1.0 / 17.0) + a2 * ((float)(-1.0 / 19.0) + a2 * (float)(1.0 / 21.0))))))))));
    const float r = off + p;
    return t < 0.0f ? -r : r;
}

inline float lm_atan2f(float y, float x) {
    if (x != x || y != y) return x + y;
    const float ax = fabsf(x), ay = fabsf(y);
    float r;
    if (ax == 0.0f && ay == 0.0f) r = 0.0f;
    else if (ay <= ax) r = lm_atan_unit(ay / ax);
    else r = 1.5707963705062866f - lm_atan_unit(ax / ay);
    if (x < 0.0f) r = 3.1415927410125732f - r;
    return y < 0.0f ? -r : r;
}

inline float lm_acosf(float x) {
    x = x < -1.0f ? -1.0f : (x > 1.0f ? 1.0f : x);
    return lm_atan2f(sqrtf((1.0f - x) * (1.0f + x)), x);
}

/* ------------------------------------------------------------------------------------------------------
 * half precision conversions (exact half -> float, round-to-nearest-even float -> half)
 * ---------------------------------------------------------------------------------------------------- */
inline float half2float(uint h) {
    const uint sign = (h & 0x8000u) << 16, e = (h >> 10) & 31u, m = h & 1023u;
    if (e == 0) {
        const float f = (float)m * 5.9604644775390625e-8f;
        return sign ? -f : f;
    }
    if (e == 31) return bitsf(sign | 0x7f800000u | (m << 13));
    return bitsf(sign | ((e + 112u) << 23) | (m << 13));
}

inline uint16_t float2half(float f) {
    const uint x = fbits(f), sign = (x >> 16) & 0x8000u, ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);
    if (ax < 0x38800000u) {
        const uint e = ax >> 23;
        if (e < 102) return (uint16_t)sign;
        const uint m = (ax & 0x7fffffu) | 0x800000u, shift = 126 - e;
        uint h = m >> shift;
        const uint rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1u);
        if (rem > half || (rem == half && (h & 1u))) h++;
        return (uint16_t)(sign | h);
    }
    uint h = (ax >> 13) - (112u << 10);
    const uint rem = ax & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
    return (uint16_t)(sign | h);
}

/* ------------------------------------------------------------------------------------------------------
 * random numbers: tools_shared.h:60-62
 * ---------------------------------------------------------------------------------------------------- */
inline uint WangHash(uint s) { s = (s ^ 61u) ^ (s >> 16), s *= 9u, s = s ^ (s >> 4), s *= 0x27d4eb2du, s = s ^ (s >> 15); return s; }
inline uint RandomInt(uint& s) { s ^= s << 13, s ^= s >> 17, s ^= s << 5; return s; }
inline float RandomFloat(uint& s) { return (float)RandomInt(s) * 2.3283064365387e-10f; }

/* RandomBarycentrics: common_functions.h:52-71. The conversion to 0:32 fixed point saturates like the
 * GPU's float->uint conversion when r0 rounds up to 1.0. */
inline f3 RandomBarycentrics(const float r0) {
    const uint uf = f2u(r0 * 4294967296.0f);
    f2 A = mk2(1, 0), B = mk2(0, 1), C = mk2(0, 0);
    for (int i = 0; i < 16; ++i) {
        const int d = (int)((uf >> (2 * (15 - i))) & 0x3u);
        f2 An, Bn, Cn;
        switch (d) {
        case 0: An = (B + C) * 0.5f; Bn = (A + C) * 0.5f; Cn = (A + B) * 0.5f; break;
        case 1: An = A; Bn = (A + B) * 0.5f; Cn = (A + C) * 0.5f; break;
        case 2: An = (B + A) * 0.5f; Bn = B; Cn = (B + C) * 0.5f; break;
        default: An = (C + A) * 0.5f; Bn = (C + B) * 0.5f; Cn = C; break;
        }
        A = An, B = Bn, C = Cn;
    }
    const f2 r = (A + B + C) * 0.3333333f;
    return mk3(r.x, r.y, 1 - r.x - r.y);
}

/* tools_shared.h:101-120 */
inline uint PackNormal(const f3 N) {
    const float f = 65535.0f / fmaxf(sqrtf(8.0f * N.z + 8.0f), 0.0001f);
    return f2u(N.x * f + 32767.0f) + (f2u(N.y * f + 32767.0f) << 16);
}
inline f3 UnpackNormal(const uint p) {
    f4 nn = mk4((float)(p & 65535u) * (2.0f / 65535.0f), (float)(p >> 16) * (2.0f / 65535.0f), 0, 0);
    nn = nn + mk4(-1, -1, 1, -1);
    float l = dot(mk3(nn.x, nn.y, nn.z), mk3(-nn.x, -nn.y, -nn.w));
    nn.z = l, l = sqrtf(l), nn.x *= l, nn.y *= l;
    return mk3(nn.x, nn.y, nn.z) * 2.0f + mk3(0, 0, -1);
}

/* common_functions.h:73-116 */
inline void SetupTangentSpace(const f3& N, f3& T, f3& B) {
    const float sign = copysignf(1.0f, N.z);
    const float a = -1.0f / (sign + N.z);
    const float b = N.x * N.y * a;
    B = mk3(1.0f + sign * N.x * N.x * a, sign * b, -sign * N.x);
    T = mk3(b, sign + N.y * N.y * a, -N.y);
}
inline f3 Tangent2World(const f3& V, const f3& N) {
    f3 T, B;
    SetupTangentSpace(N, T, B);
    return V.x * T + V.y * B + V.z * N;
}
inline f3 DiffuseReflectionCosWeighted(const float r0, const float r1) {
    const float term1 = TWOPI * r0, term2 = sqrtf(1 - r1);
    float s, c;
    lm_sincos(term1, &s, &c);
    return mk3(c * term2, s * term2, sqrtf(r1));
}

/* tools_shared.h:213-216, 231-235, 266-280 */
inline float SurvivalProbability(const f3& albedo) { return fminr(1.0f, fmaxr(fmaxr(albedo.x, albedo.y), albedo.z)); }
inline f3 SafeOrigin(const f3& O, const f3& R, const f3& N, const float geoEpsilon) {
    return O + N * (dot(N, R) > 0 ? geoEpsilon : -geoEpsilon);
}
inline f3 ConsistentNormal(const f3& D, const f3& iN, const float alpha) {
    const float t = PI - 2 * alpha, q = (t * t) / (PI * (PI + (2 * PI - 4) * alpha));
    const float b = dot(D, iN), g = 1 + q * (b - 1), rho = sqrtf(q * (1 + g) / (1 + b));
    const f3 Rc = (g + rho * b) * iN - (rho * D);
    return normalize(D + Rc);
}

/* ------------------------------------------------------------------------------------------------------
 * scene
 * ---------------------------------------------------------------------------------------------------- */
struct BNode { float bmin[3]; uint first; float bmax[3]; uint count; };  /* count > 0: leaf */

struct BVH2 {
    std::vector<BNode> nodes;
    std::vector<uint> idx;
};

struct Mesh {
    std::vector<lh2g_core_tri> tris;
    std::vector<f3> v0, e1, e2;   /* intersection data: v0, v1 - v0, v2 - v0 from the vertex buffer */
    BVH2 bvh;
    float bmin[3], bmax[3];
};

struct Instance {
    int mesh;
    float T[16], inv[16];
    float wmin[3], wmax[3];
};

struct Sky { std::vector<f3> px; int w = 0, h = 0; float m[16]; };

}  // namespace

struct lh2o_scene {
    std::vector<Mesh> meshes;
    std::vector<Instance> inst;
    std::vector<lh2g_material> hostMats;
    std::vector<lh2g_gpu_material> mats;
    std::vector<uint> texels;
    std::vector<uint> texFirst, texWH;
    std::vector<lh2g_light_tri> triLights;
    std::vector<lh2g_point_light> pointLights;
    std::vector<lh2g_spot_light> spotLights;
    std::vector<lh2g_dir_light> dirLights;
    Sky sky;
    BVH2 top;
    bool finalized = false;
};

namespace {

/* mat4::Inverted (common_types.h:559-604): cofactor expansion. */
void invert4x4(const float* cell, float* out) {
    const float inv[16] = {
        cell[5] * cell[10] * cell[15] - cell[5] * cell[11] * cell[14] - cell[9] * cell[6] * cell[15] + cell[9] * cell[7] * cell[14] + cell[13] * cell[6] * cell[11] - cell[13] * cell[7] * cell[10],
        -cell[1] * cell[10] * cell[15] + cell[1] * cell[11] * cell[14] + cell[9] * cell[2] * cell[15] - cell[9] * cell[3] * cell[14] - cell[13] * cell[2] * cell[11] + cell[13] * cell[3] * cell[10],
        cell[1] * cell[6] * cell[15] - cell[1] * cell[7] * cell[14] - cell[5] * cell[2] * cell[15] + cell[5] * cell[3] * cell[14] + cell[13] * cell[2] * cell[7] - cell[13] * cell[3] * cell[6],
        -cell[1] * cell[6] * cell[11] + cell[1] * cell[7] * cell[10] + cell[5] * cell[2] * cell[11] - cell[5] * cell[3] * cell[10] - cell[9] * cell[2] * cell[7] + cell[9] * cell[3] * cell[6],
        -cell[4] * cell[10] * cell[15] + cell[4] * cell[11] * cell[14] + cell[8] * cell[6] * cell[15] - cell[8] * cell[7] * cell[14] - cell[12] * cell[6] * cell[11] + cell[12] * cell[7] * cell[10],
        cell[0] * cell[10] * cell[15] - cell[0] * cell[11] * cell[14] - cell[8] * cell[2] * cell[15] + cell[8] * cell[3] * cell[14] + cell[12] * cell[2] * cell[11] - cell[12] * cell[3] * cell[10],
        -cell[0] * cell[6] * cell[15] + cell[0] * cell[7] * cell[14] + cell[4] * cell[2] * cell[15] - cell[4] * cell[3] * cell[14] - cell[12] * cell[2] * cell[7] + cell[12] * cell[3] * cell[6],
        cell[0] * cell[6] * cell[11] - cell[0] * cell[7] * cell[10] - cell[4] * cell[2] * cell[11] + cell[4] * cell[3] * cell[10] + cell[8] * cell[2] * cell[7] - cell[8] * cell[3] * cell[6],
        cell[4] * cell[9] * cell[15] - cell[4] * cell[11] * cell[13] - cell[8] * cell[5] * cell[15] + cell[8] * cell[7] * cell[13] + cell[12] * cell[5] * cell[11] - cell[12] * cell[7] * cell[9],
        -cell[0] * cell[9] * cell[15] + cell[0] * cell[11] * cell[13] + cell[8] * cell[1] * cell[15] - cell[8] * cell[3] * cell[13] - cell[12] * cell[1] * cell[11] + cell[12] * cell[3] * cell[9],
        cell[0] * cell[5] * cell[15] - cell[0] * cell[7] * cell[13] - cell[4] * cell[1] * cell[15] + cell[4] * cell[3] * cell[13] + cell[12] * cell[1] * cell[7] - cell[12] * cell[3] * cell[5],
        -cell[0] * cell[5] * cell[11] + cell[0] * cell[7] * cell[9] + cell[4] * cell[1] * cell[11] - cell[4] * cell[3] * cell[9] - cell[8] * cell[1] * cell[7] + cell[8] * cell[3] * cell[5],
        -cell[4] * cell[9] * cell[14] + cell[4] * cell[10] * cell[13] + cell[8] * cell[5] * cell[14] - cell[8] * cell[6] * cell[13] - cell[12] * cell[5] * cell[10] + cell[12] * cell[6] * cell[9],
        cell[0] * cell[9] * cell[14] - cell[0] * cell[10] * cell[13] - cell[8] * cell[1] * cell[14] + cell[8] * cell[2] * cell[13] + cell[12] * cell[1] * cell[10] - cell[12] * cell[2] * cell[9],
        -cell[0] * cell[5] * cell[14] + cell[0] * cell[6] * cell[13] + cell[4] * cell[1] * cell[14] - cell[4] * cell[2] * cell[13] - cell[12] * cell[1] * cell[6] + cell[12] * cell[2] * cell[5],
        cell[0] * cell[5] * cell[10] - cell[0] * cell[6] * cell[9] - cell[4] * cell[1] * cell[10] + cell[4] * cell[2] * cell[9] + cell[8] * cell[1] * cell[6] - cell[8] * cell[2] * cell[5]};
    const float det = cell[0] * inv[0] + cell[1] * inv[4] + cell[2] * inv[8] + cell[3] * inv[12];
    for (int i = 0; i < 16; i++) out[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    if (det != 0) {
        const float invdet = 1.0f / det;
        for (int i = 0; i < 16; i++) out[i] = inv[i] * invdet;
    }
}

/* Object-space ray of an instance: O' = M O + m3, D' = M D with M the inverse transform (3x4). */
inline f3 xform_point(const float* m, f3 p) {
    return mk3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
               m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}
inline f3 xform_vector(const float* m, f3 v) {
    return mk3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z, m[8] * v.x + m[9] * v.y + m[10] * v.z);
}

/* Moller-Trumbore, returns u, v with hit point = (1-u-v) V0 + u V1 + v V2. */
inline bool isect_tri(const f3& O, const f3& D, const f3& v0, const f3& e1, const f3& e2, float& t, float& u, float& v) {
    const f3 p = cross(D, e2);
    const float det = dot(e1, p);
    if (det == 0.0f) return false;
    const float inv = 1.0f / det;
    const f3 s = O - v0;
    u = dot(s, p) * inv;
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    const f3 q = cross(s, e1);
    v = dot(D, q) * inv;
    if (!(v >= 0.0f && u + v <= 1.0f)) return false;
    t = dot(e2, q) * inv;
    return true;
}

/* --- binned SAH BVH2 build over boxes (16 bins, leaves of at most 4) --------------------------------- */
struct BuildPrim { float bmin[3], bmax[3], c[3]; };

inline float half_area(const float* mn, const float* mx) {
    const float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
    return dx * dy + dy * dz + dz * dx;
}

void build_bvh2(const std::vector<BuildPrim>& prims, BVH2& bvh) {
    const uint n = (uint)prims.size();
    bvh.nodes.clear();
    bvh.idx.resize(n);
    for (uint i = 0; i < n; i++) bvh.idx[i] = i;
    bvh.nodes.reserve(n ? 2 * n : 1);
    BNode root;
    for (int a = 0; a < 3; a++) root.bmin[a] = 1e30f, root.bmax[a] = -1e30f;
    root.first = 0, root.count = n;
    bvh.nodes.push_back(root);
    if (n == 0) { bvh.nodes[0].count = 0; return; }
    std::vector<uint> stack = {0};
    const int BINS = 16;
    while (!stack.empty()) {
        const uint ni = stack.back();
        stack.pop_back();
        BNode& node = bvh.nodes[ni];
        float cmin[3] = {1e30f, 1e30f, 1e30f}, cmax[3] = {-1e30f, -1e30f, -1e30f};
        for (int a = 0; a < 3; a++) node.bmin[a] = 1e30f, node.bmax[a] = -1e30f;
        for (uint i = node.first; i < node.first + node.count; i++) {
            const BuildPrim& p = prims[bvh.idx[i]];
            for (int a = 0; a < 3; a++) {
                node.bmin[a] = std::min(node.bmin[a], p.bmin[a]), node.bmax[a] = std::max(node.bmax[a], p.bmax[a]);
                cmin[a] = std::min(cmin[a], p.c[a]), cmax[a] = std::max(cmax[a], p.c[a]);
            }
        }
        if (node.count <= 2) continue;
        float bestCost = 1e30f;
        int bestAxis = -1, bestSplit = 0;
        for (int a = 0; a < 3; a++) {
            const float ext = cmax[a] - cmin[a];
            if (ext <= 0) continue;
            int cnt[BINS] = {0};
            float bmn[BINS][3], bmx[BINS][3];
            for (int b = 0; b < BINS; b++) for (int k = 0; k < 3; k++) bmn[b][k] = 1e30f, bmx[b][k] = -1e30f;
            const float scale = BINS / ext;
            for (uint i = node.first; i < node.first + node.count; i++) {
                const BuildPrim& p = prims[bvh.idx[i]];
                const int b = std::min(BINS - 1, (int)((p.c[a] - cmin[a]) * scale));
                cnt[b]++;
                for (int k = 0; k < 3; k++) bmn[b][k] = std::min(bmn[b][k], p.bmin[k]), bmx[b][k] = std::max(bmx[b][k], p.bmax[k]);
            }
            float rA[BINS], lmn[3] = {1e30f, 1e30f, 1e30f}, lmx[3] = {-1e30f, -1e30f, -1e30f};
            int rC[BINS];
            int c = 0;
            for (int b = BINS - 1; b > 0; b--) {
                c += cnt[b];
                for (int k = 0; k < 3; k++) lmn[k] = std::min(lmn[k], bmn[b][k]), lmx[k] = std::max(lmx[k], bmx[b][k]);
                rA[b] = c ? half_area(lmn, lmx) : 0.0f;
                rC[b] = c;
            }
            for (int k = 0; k < 3; k++) lmn[k] = 1e30f, lmx[k] = -1e30f;
            c = 0;
            for (int b = 0; b < BINS - 1; b++) {
                c += cnt[b];
                for (int k = 0; k < 3; k++) lmn[k] = std::min(lmn[k], bmn[b][k]), lmx[k] = std::max(lmx[k], bmx[b][k]);
                if (c == 0 || rC[b + 1] == 0) continue;
                const float cost = half_area(lmn, lmx) * c + rA[b + 1] * rC[b + 1];
                if (cost < bestCost) bestCost = cost, bestAxis = a, bestSplit = b;
            }
        }
        const float leafCost = half_area(node.bmin, node.bmax) * node.count;
        uint mid;
        if (bestAxis < 0) {
            if (node.count <= 4) continue;
            mid = node.first + node.count / 2; /* coincident centroids: split by count */
        } else {
            if (node.count <= 4 && bestCost >= leafCost) continue;
            const float ext = cmax[bestAxis] - cmin[bestAxis], scale = BINS / ext;
            uint* first = bvh.idx.data() + node.first;
            uint* last = first + node.count;
            uint* m = std::partition(first, last, [&](uint pi) {
                return std::min(BINS - 1, (int)((prims[pi].c[bestAxis] - cmin[bestAxis]) * scale)) <= bestSplit;
            });
            mid = (uint)(m - bvh.idx.data());
            if (mid == node.first || mid == node.first + node.count) mid = node.first + node.count / 2;
        }
        const uint first = node.first, count = node.count;
        const uint li = (uint)bvh.nodes.size();
        BNode l, r;
        l.first = first, l.count = mid - first;
        r.first = mid, r.count = first + count - mid;
        bvh.nodes[ni].first = li;
        bvh.nodes[ni].count = 0;
        bvh.nodes.push_back(l);
        bvh.nodes.push_back(r);
        stack.push_back(li + 1);
        stack.push_back(li);
    }
}

/* Conservative slab test: the interval is widened by a relative 2^-16 so that a box is never culled by
 * rounding when the triangle inside it is hit. */
constexpr float BOX_MARGIN = 1.52587890625e-05f;

inline bool box_hit(const float* bmin, const float* bmax, const f3& O, const f3& invD, float tmin, float tmax, float& tnear) {
    const float tx0 = (bmin[0] - O.x) * invD.x, tx1 = (bmax[0] - O.x) * invD.x;
    const float ty0 = (bmin[1] - O.y) * invD.y, ty1 = (bmax[1] - O.y) * invD.y;
    const float tz0 = (bmin[2] - O.z) * invD.z, tz1 = (bmax[2] - O.z) * invD.z;
    float tn = std::max(std::max(std::min(tx0, tx1), std::min(ty0, ty1)), std::min(tz0, tz1));
    float tf = std::min(std::min(std::max(tx0, tx1), std::max(ty0, ty1)), std::max(tz0, tz1));
    tn = tn - fabsf(tn) * BOX_MARGIN;
    tf = tf + fabsf(tf) * BOX_MARGIN;
    tn = std::max(tn, tmin);
    tf = std::min(tf, tmax);
    tnear = tn;
    return tn <= tf;
}

inline f3 safe_inv(const f3& D) {
    auto inv1 = [](float d) { return fabsf(d) < 1e-30f ? (d < 0 ? -1e30f : 1e30f) : 1.0f / d; };
    return mk3(inv1(D.x), inv1(D.y), inv1(D.z));
}

struct HitRec { float t, u, v; int inst, prim; bool found; };

inline bool better(const HitRec& h, float t, int inst, int prim) {
    if (!h.found) return true;
    if (t < h.t) return true;
    if (t > h.t) return false;
    return inst < h.inst || (inst == h.inst && prim < h.prim);
}

/* Closest (anyhit = false) or first (anyhit = true) hit inside one instance. Returns true on an any-hit. */
bool trace_blas(const lh2o_scene* s, int instIdx, const f3& Ow, const f3& Dw, float tmin, float tmax, bool anyhit, bool brute, HitRec& h) {
    const Instance& in = s->inst[instIdx];
    const Mesh& m = s->meshes[in.mesh];
    const f3 O = xform_point(in.inv, Ow), D = xform_vector(in.inv, Dw);
    auto test = [&](uint prim) -> bool {
        float t, u, v;
        if (!isect_tri(O, D, m.v0[prim], m.e1[prim], m.e2[prim], t, u, v)) return false;
        if (!(t > tmin && t < tmax)) return false;
        if (anyhit) return true;
        if (better(h, t, instIdx, (int)prim)) h.t = t, h.u = u, h.v = v, h.inst = instIdx, h.prim = (int)prim, h.found = true;
        return false;
    };
    if (brute) {
        for (uint p = 0; p < (uint)m.v0.size(); p++) if (test(p)) return true;
        return false;
    }
    if (m.bvh.nodes.empty() || m.v0.empty()) return false;
    const f3 invD = safe_inv(D);
    uint stack[128];
    int sp = 0;
    float tn;
    if (!box_hit(m.bvh.nodes[0].bmin, m.bvh.nodes[0].bmax, O, invD, tmin, tmax, tn)) return false;
    stack[sp++] = 0;
    while (sp > 0) {
        const BNode& node = m.bvh.nodes[stack[--sp]];
        const float limit = (!anyhit && h.found) ? h.t : tmax;
        if (node.count > 0) {
            for (uint i = node.first; i < node.first + node.count; i++) if (test(m.bvh.idx[i])) return true;
            continue;
        }
        float t0, t1;
        const BNode& a = m.bvh.nodes[node.first];
        const BNode& b = m.bvh.nodes[node.first + 1];
        const bool ha = box_hit(a.bmin, a.bmax, O, invD, tmin, limit, t0);
        const bool hb = box_hit(b.bmin, b.bmax, O, invD, tmin, limit, t1);
        if (ha && hb) {
            if (t0 <= t1) stack[sp++] = node.first + 1, stack[sp++] = node.first;
            else stack[sp++] = node.first, stack[sp++] = node.first + 1;
        } else if (ha) stack[sp++] = node.first;
        else if (hb) stack[sp++] = node.first + 1;
    }
    return false;
}

bool trace_scene(const lh2o_scene* s, const f3& O, const f3& D, float tmin, float tmax, bool anyhit, bool brute, HitRec& h) {
    h.found = false, h.t = tmax, h.inst = -1, h.prim = -1, h.u = h.v = 0;
    if (brute) {
        for (int i = 0; i < (int)s->inst.size(); i++) if (trace_blas(s, i, O, D, tmin, tmax, anyhit, true, h)) return true;
        return false;
    }
    if (s->inst.empty()) return false;
    const f3 invD = safe_inv(D);
    const BVH2& top = s->top;
    uint stack[64];
    int sp = 0;
    float tn;
    if (!box_hit(top.nodes[0].bmin, top.nodes[0].bmax, O, invD, tmin, tmax, tn)) return false;
    stack[sp++] = 0;
    while (sp > 0) {
        const BNode& node = top.nodes[stack[--sp]];
        if (node.count > 0) {
            for (uint i = node.first; i < node.first + node.count; i++) {
                const int ii = (int)top.idx[i];
                const float limit = (!anyhit && h.found) ? h.t : tmax;
                if (!box_hit(s->inst[ii].wmin, s->inst[ii].wmax, O, invD, tmin, limit, tn)) continue;
                if (trace_blas(s, ii, O, D, tmin, tmax, anyhit, false, h)) return true;
            }
            continue;
        }
        const float limit = (!anyhit && h.found) ? h.t : tmax;
        float t0, t1;
        const BNode& a = top.nodes[node.first];
        const BNode& b = top.nodes[node.first + 1];
        const bool ha = box_hit(a.bmin, a.bmax, O, invD, tmin, limit, t0);
        const bool hb = box_hit(b.bmin, b.bmax, O, invD, tmin, limit, t1);
        if (ha && hb) {
            if (t0 <= t1) stack[sp++] = node.first + 1, stack[sp++] = node.first;
            else stack[sp++] = node.first, stack[sp++] = node.first + 1;
        } else if (ha) stack[sp++] = node.first;
        else if (hb) stack[sp++] = node.first + 1;
    }
    return false;
}

inline lh2g_hit make_hit(const HitRec& h) {
    lh2g_hit r;
    if (!h.found) { r.bary = 0; r.inst = 0; r.prim = NOHIT; r.t = 1e34f; return r; }
    r.bary = f2u(65535.0f * h.u) + (f2u(65535.0f * h.v) << 16);  /* .optix.cu:180 */
    r.inst = h.inst, r.prim = h.prim, r.t = h.t;
    return r;
}

/* ------------------------------------------------------------------------------------------------------
 * materials, textures, shading data: material_shared.h:42-206, sampling_shared.h:29-104
 * ---------------------------------------------------------------------------------------------------- */
inline uint tochar(float a) { return f2u(a * 255.0f); }  /* TOCHAR, RenderCore_PrimeRef/rendercore.cpp:360 */
inline uint touint4(float a, float b, float c, float d) { return tochar(a) + (tochar(b) << 8) + (tochar(c) << 16) + (tochar(d) << 24); }

void pack_map(const lh2g_map_ref& r, const uint* first, const uint* wh, uint* out) {
    const uint w = wh[2 * r.texture], h = wh[2 * r.texture + 1];
    out[0] = (w & 0xffffu) | ((h & 0xffffu) << 16);
    out[1] = (uint)float2half(r.uvscale[0]) | ((uint)float2half(r.uvscale[1]) << 16);
    out[2] = (uint)float2half(r.uvoffset[0]) | ((uint)float2half(r.uvoffset[1]) << 16);
    out[3] = first[r.texture];
}

/* RenderCore::SetMaterials, RenderCore_PrimeRef/rendercore.cpp:362-402 */
void pack_material(const lh2g_material& m, const uint* first, const uint* wh, lh2g_gpu_material& g) {
    memset(&g, 0, sizeof(g));
    const float tr = 1 - m.absorption[0], tg = 1 - m.absorption[1], tb = 1 - m.absorption[2];
    g.base[0] = (uint)float2half(m.color[0]) | ((uint)float2half(m.color[1]) << 16);
    g.base[1] = (uint)float2half(m.color[2]) | ((uint)float2half(tr) << 16);
    g.base[2] = (uint)float2half(tg) | ((uint)float2half(tb) << 16);
    g.params[0] = touint4(m.metallic, m.subsurface, m.specular, m.roughness);
    g.params[1] = touint4(m.specularTint, m.anisotropic, m.sheen, m.sheenTint);
    g.params[2] = touint4(m.clearcoat, m.clearcoatGloss, m.transmission, 0);
    g.params[3] = fbits(m.eta);
    const lh2g_map_ref* refs[6] = {&m.color_map, &m.detail_color_map, &m.normal_map, &m.detail_normal_map, &m.specular_map, &m.roughness_map};
    for (int i = 0; i < 6; i++) if (refs[i]->texture >= 0) pack_map(*refs[i], first, wh, g.maps[i]);
    uint flags = (m.eta < 1 ? LH2G_MAT_ISDIELECTRIC : 0u);
    flags += m.color_map.texture >= 0 ? LH2G_MAT_HASDIFFUSEMAP : 0u;
    flags += m.normal_map.texture >= 0 ? LH2G_MAT_HASNORMALMAP : 0u;
    flags += m.specular_map.texture >= 0 ? LH2G_MAT_HASSPECULARITYMAP : 0u;
    flags += m.roughness_map.texture >= 0 ? LH2G_MAT_HASROUGHNESSMAP : 0u;
    flags += m.detail_normal_map.texture >= 0 ? LH2G_MAT_HAS2NDNORMALMAP : 0u;
    flags += m.detail_color_map.texture >= 0 ? LH2G_MAT_HAS2NDDIFFUSEMAP : 0u;
    flags += (m.flags & 1) ? LH2G_MAT_HASSMOOTHNORMALS : 0u;
    flags += (m.flags & 2) ? LH2G_MAT_HASALPHA : 0u;
    g.base[3] = flags;
}

struct ShadingData {
    f3 color; int flags;
    f3 transmittance; int matID;
    uint params[4];
};
inline float char2flt(uint a, int s) { return ((float)((a >> s) & 255u)) * (1.0f / 255.0f); }
inline float ROUGHNESS(const ShadingData& sd) { return fmaxr(0.001f, char2flt(sd.params[0], 24)); }
inline float TRANSMISSION(const ShadingData& sd) { return char2flt(sd.params[2], 16); }
inline float ETA(const ShadingData& sd) { return bitsf(sd.params[3]); }
inline bool IsEmissive(const ShadingData& sd) { return sd.color.x > 1.0f || sd.color.y > 1.0f || sd.color.z > 1.0f; }

inline f4 uchar4_to_float4(uint v) {
    const float r = 1.0f / 256.0f;
    return mk4((float)(v & 255u) * r, (float)((v >> 8) & 255u) * r, (float)((v >> 16) & 255u) * r, (float)(v >> 24) * r);
}

f4 FetchTexel(const lh2o_scene* s, const f2 texCoord, const int o, const int w, const int h) {
    const f2 tc = mk2((fmaxr(texCoord.x + 1000, 0.0f) * w) - 0.5f, (fmaxr(texCoord.y + 1000, 0.0f) * h) - 0.5f);
    const int iu = f2i(tc.x) % w;
    const int iv = f2i(tc.y) % h;
    const float fu = tc.x - floorf(tc.x);
    const float fv = tc.y - floorf(tc.y);
    const float w0 = (1 - fu) * (1 - fv);
    const float w1 = fu * (1 - fv);
    const float w2 = (1 - fu) * fv;
    const float w3 = 1 - (w0 + w1 + w2);
    const uint iu1 = (uint)((iu + 1) % w), iv1 = (uint)((iv + 1) % h);
    const uint* t = s->texels.data();
    const f4 p0 = uchar4_to_float4(t[o + iu + iv * w]);
    const f4 p1 = uchar4_to_float4(t[o + (int)iu1 + iv * w]);
    const f4 p2 = uchar4_to_float4(t[o + iu + (int)iv1 * w]);
    const f4 p3 = uchar4_to_float4(t[o + (int)iu1 + (int)iv1 * w]);
    return p0 * w0 + p1 * w1 + p2 * w2 + p3 * w3;
}

f4 FetchTexelTrilinear(const lh2o_scene* s, const float lambda, const f2 texCoord, const int offset, const int width, const int height) {
    int level0 = 0, level1 = 0;
    float f = 0;
    if (lambda >= 0) level0 = imin(MIPLEVELCOUNT - 1, f2i(lambda)), level1 = imin(MIPLEVELCOUNT - 1, level0 + 1), f = lambda - floorf(lambda);
    const float scale = (float)(width * height) * 1.3333333333f;
    const int o0 = offset + f2i(scale * (1 - bitsf((uint)(127 - 2 * level0) << 23)));
    const int o1 = offset + f2i(scale * (1 - bitsf((uint)(127 - 2 * level1) << 23)));
    const f4 p0 = FetchTexel(s, texCoord, o0, width >> level0, height >> level0);
    const f4 p1 = FetchTexel(s, texCoord, o1, width >> level1, height >> level1);
    return (1 - f) * p0 + f * p1;
}

inline f2 map_uvscale(const uint* m) { return mk2(half2float(m[1] & 0xffffu), half2float(m[1] >> 16)); }
inline f2 map_uvoffs(const uint* m) { return mk2(half2float(m[2] & 0xffffu), half2float(m[2] >> 16)); }

/* GetShadingData + SetupFrame, material_shared.h:42-206 (non-Prime barycentric convention: w V0 + u V1 + v V2,
 * CONSISTENTNORMALS on). Returns the three normals and the tangent. */
void GetShadingData(const lh2o_scene* s, const f3 D, const float u, const float v, const float coneWidth,
                    const lh2g_core_tri& tri, const int instIdx, ShadingData& sd, f3& N, f3& iN, f3& fN, f3& T) {
    const lh2g_gpu_material& mat = s->mats[tri.material];
    const uint part0 = mat.base[0], part1 = mat.base[1], part2 = mat.base[2], flags = mat.base[3];
    sd.color = mk3(half2float(part0 & 0xffffu), half2float(part0 >> 16), half2float(part1 & 0xffffu));
    sd.flags = 0;
    sd.transmittance = mk3(half2float(part1 >> 16), half2float(part2 & 0xffffu), half2float(part2 >> 16));
    sd.matID = 0;
    for (int i = 0; i < 4; i++) sd.params[i] = mat.params[i];
    /* SetupFrame */
    N = iN = fN = mk3(tri.Nx, tri.Ny, tri.Nz);
    T = ld3(tri.T);
    const float w = 1 - (u + v);
    if (flags & LH2G_MAT_HASSMOOTHNORMALS) iN = normalize(w * ld3(tri.vN0) + u * ld3(tri.vN1) + v * ld3(tri.vN2));
    const float* inv = s->inst[instIdx].inv;
    const f3 A = mk3(inv[0], inv[1], inv[2]), B = mk3(inv[4], inv[5], inv[6]), C = mk3(inv[8], inv[9], inv[10]);
    N = normalize(N.x * A + N.y * B + N.z * C);
    iN = normalize(iN.x * A + iN.y * B + iN.z * C);
    const bool backSide = dot(D, N) > 0;
    const float alpha = w * tri.alpha[0] + u * tri.alpha[1] + v * tri.alpha[2];
    iN = (backSide ? -1.0f : 1.0f) * ConsistentNormal(D * -1.0f, backSide ? (iN * -1.0f) : iN, alpha);
    fN = iN;
    /* texturing */
    float tu = 0, tv = 0;
    if (flags & (LH2G_MAT_HASDIFFUSEMAP | LH2G_MAT_HAS2NDDIFFUSEMAP | LH2G_MAT_HASSPECULARITYMAP | LH2G_MAT_HASNORMALMAP | LH2G_MAT_HAS2NDNORMALMAP | LH2G_MAT_HASROUGHNESSMAP)) {
        const float ww = 1 - (u + v);
        tu = ww * tri.u0 + u * tri.u1 + v * tri.u2;
        tv = ww * tri.v0 + u * tri.v1 + v * tri.v2;
    }
    if (flags & LH2G_MAT_HASDIFFUSEMAP) {
        const float lambda = tri.LOD + lm_log2f(coneWidth * (1.0f / fabsf(dot(D, N))));
        const uint* t0 = mat.maps[0];
        const f2 uvscale = map_uvscale(t0), uvoffs = map_uvoffs(t0);
        const f4 texel = FetchTexelTrilinear(s, lambda, uvscale * (uvoffs + mk2(tu, tv)), (int)t0[3], (int)(t0[0] & 0xffffu), (int)(t0[0] >> 16));
        if (texel.w < 0.5f) { sd.flags |= 1; return; }
        sd.color = sd.color * mk3(texel);
        if (flags & LH2G_MAT_HAS2NDDIFFUSEMAP) {
            const uint* t1 = mat.maps[1];
            const f2 uvscale1 = map_uvscale(t1), uvoffs1 = map_uvoffs(t1);
            sd.color = sd.color + (mk3(FetchTexel(s, uvscale1 * (uvoffs1 + mk2(tu, tv)), (int)t1[3], (int)(t1[0] & 0xffffu), (int)(t1[0] >> 16))) - mk3(0.5f));
        }
    }
    if (flags & LH2G_MAT_HASNORMALMAP) {
        const f3 Bt = ld3(tri.B);
        const uint* n0 = mat.maps[2];
        const uint part3 = mat.base[2];
        const float n0scale = copysignf(-0.0001f + 0.0001f * lm_expf(0.1f * fabsf((float)((part3 >> 8) & 255u) - 128.0f)), (float)((part3 >> 8) & 255u) - 128.0f);
        const f2 uvscale = map_uvscale(n0), uvoffs = map_uvoffs(n0);
        f3 sn = (mk3(FetchTexel(s, uvscale * (uvoffs + mk2(tu, tv)), (int)n0[3], (int)(n0[0] & 0xffffu), (int)(n0[0] >> 16))) - mk3(0.5f)) * 2.0f;
        sn.x *= n0scale, sn.y *= n0scale;
        if (flags & LH2G_MAT_HAS2NDNORMALMAP) {
            const uint* n1 = mat.maps[3];
            const float n1scale = copysignf(-0.0001f + 0.0001f * lm_expf(0.1f * ((float)((part3 >> 16) & 255u) - 128.0f)), (float)((part3 >> 16) & 255u) - 128.0f);
            const f2 uvscale1 = map_uvscale(n1), uvoffs1 = map_uvoffs(n1);
            f3 l1 = (mk3(FetchTexel(s, uvscale1 * (uvoffs1 + mk2(tu, tv)), (int)n1[3], (int)(n1[0] & 0xffffu), (int)(n1[0] >> 16))) - mk3(0.5f)) * 2.0f;
            l1.x *= n1scale, l1.y *= n1scale;
            sn = sn + l1;
        }
        sn = normalize(sn);
        fN = normalize(sn.x * T + sn.y * Bt + sn.z * iN);
    }
    if (flags & LH2G_MAT_HASROUGHNESSMAP) {
        const uint* rm = mat.maps[5];
        const f2 uvscale = map_uvscale(rm), uvoffs = map_uvoffs(rm);
        const f4 texel = FetchTexel(s, uvscale * (uvoffs + mk2(tu, tv)), (int)rm[3], (int)(rm[0] & 0xffffu), (int)(rm[0] >> 16));
        sd.params[0] = (sd.params[0] & 0x00ffffffu) + ((uint)f2i(texel.y * 255.0f) << 24);
        sd.params[0] = (sd.params[0] & 0xffffff00u) + (uint)f2i(texel.x * 255.0f);
    }
}

/* ------------------------------------------------------------------------------------------------------
 * Lambert BSDF with pure specular reflection and refraction: lib/sharedBSDFs/lambert.h:32-125
 * ---------------------------------------------------------------------------------------------------- */
inline float sqr(float x) { return x * x; }
float Fr_L(float VDotN, float eio) {
    if (VDotN < 0.0f) { eio = 1.0f / eio; VDotN = fabsf(VDotN); }
    const float SinThetaT2 = sqr(eio) * (1.0f - VDotN * VDotN);
    if (SinThetaT2 > 1.0f) return 1.0f;
    const float LDotN = sqrtf(1.0f - SinThetaT2);
    const float r1 = (VDotN - eio * LDotN) / (VDotN + eio * LDotN);
    const float r2 = (LDotN - eio * VDotN) / (LDotN + eio * VDotN);
    return 0.5f * (sqr(r1) + sqr(r2));
}
bool Refract_L(const f3 wi, const f3 n, const float eta, f3& wt) {
    const float cosThetaI = fabsf(dot(n, wi));
    const float sin2ThetaI = fmaxr(0.0f, 1.0f - cosThetaI * cosThetaI);
    const float sin2ThetaT = eta * eta * sin2ThetaI;
    if (sin2ThetaT >= 1) return false;
    const float cosThetaT = sqrtf(1.0f - sin2ThetaT);
    wt = eta * (wi * -1.0f) + (eta * cosThetaI - cosThetaT) * n;
    return true;
}
f3 EvaluateBSDF(const ShadingData& sd, const f3 iN, const f3 wi, float& pdf) {
    if (TRANSMISSION(sd) > 0.999f || ROUGHNESS(sd) <= 0.001f) { pdf = 0; return mk3(0); }
    pdf = fabsf(dot(wi, iN)) * INVPI;
    return sd.color * INVPI;
}
f3 SampleBSDF(const ShadingData& sd, f3 iN, const f3 N, const f3 wo, const float distance, const float r3, const float r4,
              f3& wi, float& pdf, bool& specular) {
    const float flip = (dot(wo, N) < 0) ? -1.0f : 1.0f;
    iN = iN * flip;
    specular = true, pdf = 1;
    f3 bsdf;
    const float TRANS = TRANSMISSION(sd);
    if (r4 < TRANS) {
        const float eio = flip < 0 ? (1.0f / ETA(sd)) : ETA(sd), F = Fr_L(dot(iN, wo), eio);
        f3 beer = mk3(1);
        beer.x = lm_expf(-sd.transmittance.x * distance * 2.0f);
        beer.y = lm_expf(-sd.transmittance.y * distance * 2.0f);
        beer.z = lm_expf(-sd.transmittance.z * distance * 2.0f);
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
            pdf = fmaxr(0.0f, dot(wi, iN)) * INVPI;
            specular = false;
            bsdf = sd.color * INVPI;
        }
    }
    if (dot(N * flip, wi) <= 0) pdf = 0;
    return bsdf;
}

/* ------------------------------------------------------------------------------------------------------
 * lights: lights_shared.h:37-105, 225-313 (ISLIGHTS importance selection over at most 64 lights)
 * ---------------------------------------------------------------------------------------------------- */
float PotentialTriLightContribution(const lh2o_scene* s, const int idx, const f3& O, const f3& N, const f3& I, const f3& bary) {
    const lh2g_light_tri& l = s->triLights[idx];
    f3 L = I;
    if (bary.x >= 0) L = bary.x * ld3(l.vertex0) + bary.y * ld3(l.vertex1) + bary.z * ld3(l.vertex2);
    L = L - O;
    const float att = 1.0f / dot(L, L);
    L = normalize(L);
    const float LNdotL = fmaxr(0.0f, -dot(ld3(l.N), L));
    const float NdotL = fmaxr(0.0f, dot(N, L));
    return l.energy * LNdotL * NdotL * att;
}
float PotentialPointLightContribution(const lh2o_scene* s, const int idx, const f3& I, const f3& N) {
    const lh2g_point_light& l = s->pointLights[idx];
    const f3 L = ld3(l.position) - I;
    const float NdotL = fmaxr(0.0f, dot(N, normalize(L)));
    const float att = 1.0f / dot(L, L);
    return l.energy * NdotL * att;
}
float PotentialSpotLightContribution(const lh2o_scene* s, const int idx, const f3& I, const f3& N) {
    const lh2g_spot_light& l = s->spotLights[idx];
    f3 L = ld3(l.position) - I;
    const float att = 1.0f / dot(L, L);
    L = normalize(L);
    const float d = (fmaxr(0.0f, -dot(L, ld3(l.direction))) - l.cosOuter) / (l.cosInner - l.cosOuter);
    const float NdotL = fmaxr(0.0f, dot(N, L));
    const float LNdotL = fmaxr(0.0f, fminr(1.0f, d));
    return (l.radiance[0] + l.radiance[1] + l.radiance[2]) * LNdotL * NdotL * att;
}
float PotentialDirectionalLightContribution(const lh2o_scene* s, const int idx, const f3& I, const f3& N) {
    (void)I;
    const lh2g_dir_light& l = s->dirLights[idx];
    const float LNdotL = fmaxr(0.0f, -(l.direction[0] * N.x + l.direction[1] * N.y + l.direction[2] * N.z));
    return l.energy * LNdotL;
}

f3 RandomPointOnLight(const lh2o_scene* s, float r0, float r1, const f3& I, const f3& N, float& pickProb, float& lightPdf, f3& lightColor) {
    const int ntri = (int)s->triLights.size(), npt = (int)s->pointLights.size();
    const int nspot = (int)s->spotLights.size(), ndir = (int)s->dirLights.size();
    const float lightCount = (float)(ntri + npt + nspot + ndir);
    const f3 bary = RandomBarycentrics(r0);
    float potential[64];
    float sum = 0, total = 0;
    int lights = 0, lightIdx = 0;
    for (int i = 0; i < ntri; i++) { float c = PotentialTriLightContribution(s, i, I, N, I, bary); potential[lights++] = c; sum += c; }
    for (int i = 0; i < npt; i++) { float c = PotentialPointLightContribution(s, i, I, N); potential[lights++] = c; sum += c; }
    for (int i = 0; i < nspot; i++) { float c = PotentialSpotLightContribution(s, i, I, N); potential[lights++] = c; sum += c; }
    for (int i = 0; i < ndir; i++) { float c = PotentialDirectionalLightContribution(s, i, I, N); potential[lights++] = c; sum += c; }
    if (sum <= 0) { lightPdf = 0; return mk3(1); }
    r1 *= sum;
    for (int i = 0; i < lights; i++) {
        total += potential[i];
        if (total >= r1) { lightIdx = i; break; }
    }
    pickProb = potential[lightIdx] / sum;
    lightIdx = imax(0, imin(lightIdx, f2i(lightCount) - 1));
    if (lightIdx < ntri) {
        const lh2g_light_tri& l = s->triLights[lightIdx];
        lightColor = ld3(l.radiance);
        const f3 P = bary.x * ld3(l.vertex0) + bary.y * ld3(l.vertex1) + bary.z * ld3(l.vertex2);
        f3 L = I - P;
        const float sqDist = dot(L, L);
        L = normalize(L);
        const float LNdotL = L.x * l.N[0] + L.y * l.N[1] + L.z * l.N[2];
        const float reciSolidAngle = sqDist / (l.area * LNdotL);
        lightPdf = (LNdotL > 0 && dot(L, N) < 0) ? reciSolidAngle : 0;
        return P;
    } else if (lightIdx < ntri + npt) {
        const lh2g_point_light& l = s->pointLights[lightIdx - ntri];
        const f3 P = ld3(l.position);
        const f3 L = P - I;
        const float sqDist = dot(L, L);
        lightColor = ld3(l.radiance) / sqDist;
        lightPdf = dot(L, N) > 0 ? 1.0f : 0.0f;
        return P;
    } else if (lightIdx < ntri + npt + nspot) {
        const lh2g_spot_light& l = s->spotLights[lightIdx - (ntri + npt)];
        const f3 P = ld3(l.position);
        f3 L = I - P;
        const float sqDist = dot(L, L);
        L = normalize(L);
        const float d = (fmaxr(0.0f, L.x * l.direction[0] + L.y * l.direction[1] + L.z * l.direction[2]) - l.cosOuter) / (l.cosInner - l.cosOuter);
        const float LNdotL = fminr(1.0f, d);
        lightPdf = (LNdotL > 0 && dot(L, N) < 0) ? (sqDist / LNdotL) : 0;
        lightColor = ld3(l.radiance);
        return P;
    } else {
        const lh2g_dir_light& l = s->dirLights[lightIdx - (ntri + npt + nspot)];
        const f3 L = ld3(l.direction);
        lightColor = ld3(l.radiance);
        const float NdotL = dot(L, N);
        lightPdf = NdotL < 0 ? 1.0f : 0.0f;
        return I - 1000.0f * L;
    }
}

/* SampleSkydome, tools_shared.h:185-202, with worldToSky.TransformVector (common_types.h:608-613). */
f3 SampleSkydome(const lh2o_scene* s, const f3& Dw) {
    if (s->sky.w <= 0 || s->sky.h <= 0) return mk3(0);
    const float* m = s->sky.m;
    const f3 D = -mk3(m[0] * Dw.x + m[1] * Dw.y + m[2] * Dw.z, m[4] * Dw.x + m[5] * Dw.y + m[6] * Dw.z, m[8] * Dw.x + m[9] * Dw.y + m[10] * Dw.z);
    float p = lm_atan2f(D.y, D.x);
    p = (p < 0) ? (p + 2 * PI) : p;
    const float theta = lm_acosf(D.z < -1.f ? -1.f : (D.z > 1.f ? 1.f : D.z));
    const uint u = f2u((float)s->sky.w * p * INV2PI - 0.5f);
    const uint v = f2u((float)s->sky.h * theta * INVPI - 0.5f);
    const uint idx = u + v * (uint)s->sky.w;
    return idx < (uint)(s->sky.w * s->sky.h) ? s->sky.px[idx] : mk3(0);
}

/* ------------------------------------------------------------------------------------------------------
 * one path, depth first: camera.h:39-68 + pathtracer.h:45-168 + connections.h:22-34
 * ---------------------------------------------------------------------------------------------------- */
struct Frame {
    const lh2o_scene* s;
    lh2g_view view;
    lh2g_render_params p;
    f3 right, up;
    long long P;
};

struct PathOut { float rgbw[4]; };

void trace_path(const Frame& F, const uint jobIndex, PathOut& out, std::vector<uint>& ext, std::vector<uint>& shad, lh2g_capture* cap) {
    const lh2o_scene* s = F.s;
    const lh2g_render_params& p = F.p;
    const int W = p.width, H = p.height;
    const float eps = p.geometryEpsilon;
    const bool nee = (p.flags & LH2G_RP_NEE) != 0;
    /* generateEyeRaysKernel */
    const uint x = jobIndex % (uint)W;
    uint y = jobIndex / (uint)W;
    y %= (uint)H;
    uint seed = WangHash(jobIndex + p.cameraR0);
    const float r0 = RandomFloat(seed), r1 = RandomFloat(seed);
    const float r2 = RandomFloat(seed), r3 = RandomFloat(seed);
    const f3 p1 = ld3(F.view.p1), pos = ld3(F.view.pos);
    const f3 posOnPixel = p1 + ((float)x + r0) * (F.right / (float)W) + ((float)y + r1) * (F.up / (float)H);
    f3 posOnLens;
    {   /* RandomPointOnLens, camera.h:22-33 */
        const float blade = (float)f2i(r2 * 9);
        float rr2 = (r2 - blade * (1.0f / 9.0f)) * 9.0f, rr1 = r3;
        float x1, y1, x2, y2;
        lm_sincos(blade * PI / 4.5f, &x1, &y1);
        lm_sincos((blade + 1.0f) * PI / 4.5f, &x2, &y2);
        if ((rr1 + rr2) > 1) rr1 = 1.0f - rr1, rr2 = 1.0f - rr2;
        const float xr = x1 * rr1 + x2 * rr2;
        const float yr = y1 * rr1 + y2 * rr2;
        posOnLens = pos + F.view.aperture * (F.right * xr + F.up * yr);
    }
    f3 O = posOnLens, D = normalize(posOnPixel - posOnLens);
    float tmin = eps;
    f3 throughput = mk3(1);
    uint FLAGS = S_SPECULAR;
    const uint pathIdx = jobIndex;
    out.rgbw[0] = out.rgbw[1] = out.rgbw[2] = out.rgbw[3] = 0;
    for (int pathLength = 1; pathLength <= p.maxDepth; pathLength++) {
        HitRec h;
        trace_scene(s, O, D, tmin, 1e34f, false, false, h);
        const lh2g_hit hit = make_hit(h);
        const long long capIdx = (long long)(pathLength - 1) * F.P + pathIdx;
        if (cap && cap->hits) cap->hits[capIdx] = hit;
        const uint R0 = (uint)p.samplesTaken * 7907u + (uint)pathLength * 91771u;
        if ((p.flags & LH2G_RP_DEPTH_W) && pathLength == 1) out.rgbw[3] += hit.prim == NOHIT ? 10000.0f : hit.t;
        if (hit.prim == NOHIT) {
            const f3 c = throughput * SampleSkydome(s, D);
            out.rgbw[0] += c.x, out.rgbw[1] += c.y, out.rgbw[2] += c.z;
            if (cap && cap->seeds) cap->seeds[capIdx] = 0;
            return;
        }
        const float HIT_U = (float)(hit.bary & 65535u) * (1.0f / 65535.0f);
        const float HIT_V = (float)(hit.bary >> 16) * (1.0f / 65535.0f);
        const float HIT_T = hit.t;
        const int INST = hit.inst, PRIM = hit.prim;
        const lh2g_core_tri& tri = s->meshes[s->inst[INST].mesh].tris[PRIM];
        ShadingData sd;
        f3 N, iN, fN, T;
        const f3 I = O + HIT_T * D;
        const float coneWidth = F.view.spreadAngle * HIT_T;
        GetShadingData(s, D, HIT_U, HIT_V, coneWidth, tri, INST, sd, N, iN, fN, T);
        if (IsEmissive(sd)) {
            const float DdotNL = -dot(D, N);
            if (DdotNL > 0) {
                const f3 c = throughput * sd.color;
                if (pathLength == 1 || (FLAGS & S_SPECULAR) || !nee) out.rgbw[0] += c.x, out.rgbw[1] += c.y, out.rgbw[2] += c.z;
            }
            if (cap && cap->seeds) cap->seeds[capIdx] = 0;
            return;
        }
        if (ROUGHNESS(sd) <= 0.001f || TRANSMISSION(sd) > 0.999f) FLAGS |= S_SPECULAR; else FLAGS &= ~S_SPECULAR;
        seed = WangHash(pathIdx * 17u + R0);
        const float faceDir = (dot(D, N) > 0) ? -1.0f : 1.0f;
        if (faceDir == 1) sd.transmittance = mk3(0);
        if ((FLAGS & S_SPECULAR) == 0 && nee) {
            const float q0 = RandomFloat(seed), q1 = RandomFloat(seed);
            float pickProb = 0, lightPdf = 0;
            f3 lightColor = mk3(0);
            f3 L = RandomPointOnLight(s, q0, q1, I, fN * faceDir, pickProb, lightPdf, lightColor) - I;
            const float dist = length(L);
            L = L * (1.0f / dist);
            const float NdotL = dot(L, fN * faceDir);
            if (NdotL > 0 && lightPdf > 0) {
                float bsdfPdf;
                const f3 sampledBSDF = EvaluateBSDF(sd, fN, L, bsdfPdf) * ROUGHNESS(sd);
                const f3 contribution = throughput * sampledBSDF * lightColor * (NdotL / (pickProb * lightPdf));
                shad[pathLength - 1]++;
                HitRec sh;
                const f3 SO = SafeOrigin(I, L, N, eps);
                if (!trace_scene(s, SO, L, 0.0f, dist - 2 * eps, true, false, sh))
                    out.rgbw[0] += contribution.x, out.rgbw[1] += contribution.y, out.rgbw[2] += contribution.z;
            }
        }
        f3 R;
        float newBsdfPdf;
        bool specular = false;
        const float q3 = RandomFloat(seed), q4 = RandomFloat(seed), q5 = RandomFloat(seed);
        const f3 bsdf = SampleBSDF(sd, fN, N, D * -1.0f, HIT_T, q3, q4, R, newBsdfPdf, specular);
        if (cap && cap->seeds) cap->seeds[capIdx] = seed;
        if (newBsdfPdf < EPSILON || std::isnan(newBsdfPdf)) return;
        if (specular) FLAGS |= S_SPECULAR;
        const float pr = pathLength == p.maxDepth ? 0.0f : (((FLAGS & S_SPECULAR) || pathLength < p.rrStartDepth) ? 1.0f : SurvivalProbability(bsdf));
        if (pr <= q5) return;
        throughput = throughput * (bsdf * fabsf(dot(fN, R)) / (pr * newBsdfPdf));
        ext[pathLength - 1]++;
        O = SafeOrigin(I, R, N, eps);
        D = R;
        tmin = 0.0f;
    }
}

void parallel_for(long long n, int nthreads, long long chunk, const std::function<void(long long, long long)>& fn) {
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<long long> next(0);
    auto worker = [&]() {
        for (;;) {
            const long long b = next.fetch_add(chunk);
            if (b >= n) break;
            fn(b, std::min(n, b + chunk));
        }
    };
    if (nthreads == 1) { worker(); return; }
    std::vector<std::thread> ts;
    for (int i = 0; i < nthreads; i++) ts.emplace_back(worker);
    for (auto& t : ts) t.join();
}

}  // namespace

/* ==========================================================================================================
 * C API
 * ======================================================================================================== */
extern "C" {

lh2o_scene* lh2o_create(void) { return new lh2o_scene(); }
void lh2o_destroy(lh2o_scene* s) { delete s; }

int lh2o_set_geometry(lh2o_scene* s, int meshIdx, const float* v4, int vertexCount, int triangleCount, const lh2g_core_tri* tris) {
    if (!s || meshIdx < 0 || meshIdx > (int)s->meshes.size() || vertexCount != 3 * triangleCount) return 1;
    if (meshIdx == (int)s->meshes.size()) s->meshes.emplace_back();
    Mesh& m = s->meshes[meshIdx];
    m.tris.assign(tris, tris + triangleCount);
    m.v0.resize(triangleCount), m.e1.resize(triangleCount), m.e2.resize(triangleCount);
    for (int a = 0; a < 3; a++) m.bmin[a] = 1e30f, m.bmax[a] = -1e30f;
    for (int i = 0; i < triangleCount; i++) {
        const float* a = v4 + 12 * i;
        const f3 p0 = mk3(a[0], a[1], a[2]), p1 = mk3(a[4], a[5], a[6]), p2 = mk3(a[8], a[9], a[10]);
        m.v0[i] = p0, m.e1[i] = p1 - p0, m.e2[i] = p2 - p0;
        const f3 ps[3] = {p0, p1, p2};
        for (const f3& q : ps) {
            m.bmin[0] = std::min(m.bmin[0], q.x), m.bmin[1] = std::min(m.bmin[1], q.y), m.bmin[2] = std::min(m.bmin[2], q.z);
            m.bmax[0] = std::max(m.bmax[0], q.x), m.bmax[1] = std::max(m.bmax[1], q.y), m.bmax[2] = std::max(m.bmax[2], q.z);
        }
    }
    s->finalized = false;
    return 0;
}

int lh2o_set_instance(lh2o_scene* s, int instIdx, int meshIdx, const float* T) {
    if (!s || instIdx < 0) return 1;
    if (meshIdx == -1) {
        if ((int)s->inst.size() > instIdx) s->inst.resize(instIdx);
        return 0;
    }
    if (instIdx > (int)s->inst.size()) return 1;
    if (instIdx == (int)s->inst.size()) s->inst.emplace_back();
    Instance& in = s->inst[instIdx];
    in.mesh = meshIdx;
    memcpy(in.T, T, 64);
    invert4x4(T, in.inv);
    s->finalized = false;
    return 0;
}

int lh2o_set_materials(lh2o_scene* s, const lh2g_material* mats, int count) {
    if (!s || count < 0) return 1;
    s->hostMats.assign(mats, mats + count);
    s->mats.resize(count);
    for (int i = 0; i < count; i++) pack_material(mats[i], s->texFirst.data(), s->texWH.data(), s->mats[i]);
    return 0;
}

int lh2o_set_textures(lh2o_scene* s, const lh2g_texture* tex, int count) {
    if (!s || count < 0) return 1;
    s->texels.clear(), s->texFirst.clear(), s->texWH.clear();
    for (int i = 0; i < count; i++) {
        s->texFirst.push_back((uint)s->texels.size());
        s->texWH.push_back(tex[i].width), s->texWH.push_back(tex[i].height);
        s->texels.insert(s->texels.end(), tex[i].texels, tex[i].texels + tex[i].pixelCount);
    }
    if (s->texels.size() < 16) s->texels.resize(16, 0);
    return 0;
}

int lh2o_set_lights(lh2o_scene* s, const lh2g_light_tri* tri, int ntri, const lh2g_point_light* pt, int npt,
                    const lh2g_spot_light* spot, int nspot, const lh2g_dir_light* dir, int ndir) {
    if (!s || ntri + npt + nspot + ndir > 64) return 1;
    s->triLights.assign(tri, tri + ntri);
    s->pointLights.assign(pt, pt + npt);
    s->spotLights.assign(spot, spot + nspot);
    s->dirLights.assign(dir, dir + ndir);
    return 0;
}

int lh2o_set_sky(lh2o_scene* s, const float* rgb, int w, int h, const float* m16) {
    if (!s || w < 0 || h < 0) return 1;
    s->sky.w = w, s->sky.h = h;
    s->sky.px.resize((size_t)w * h);
    for (size_t i = 0; i < (size_t)w * h; i++) s->sky.px[i] = mk3(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
    for (int i = 0; i < 16; i++) s->sky.m[i] = m16 ? m16[i] : ((i % 5 == 0) ? 1.0f : 0.0f);
    return 0;
}

int lh2o_finalize(lh2o_scene* s) {
    if (!s) return 1;
    parallel_for((long long)s->meshes.size(), 0, 1, [&](long long b, long long e) {
        for (long long mi = b; mi < e; mi++) {
            Mesh& m = s->meshes[mi];
            std::vector<BuildPrim> prims(m.v0.size());
            for (size_t i = 0; i < m.v0.size(); i++) {
                const f3 a = m.v0[i], bb = a + m.e1[i], c = a + m.e2[i];
                const f3 ps[3] = {a, bb, c};
                BuildPrim& p = prims[i];
                for (int k = 0; k < 3; k++) p.bmin[k] = 1e30f, p.bmax[k] = -1e30f;
                for (const f3& q : ps) {
                    const float qq[3] = {q.x, q.y, q.z};
                    for (int k = 0; k < 3; k++) p.bmin[k] = std::min(p.bmin[k], qq[k]), p.bmax[k] = std::max(p.bmax[k], qq[k]);
                }
                /* widen by 2^-20 of the magnitude: v0 + e1 is not exactly the vertex the test uses */
                for (int k = 0; k < 3; k++) {
                    p.bmin[k] -= fabsf(p.bmin[k]) * 9.5367431640625e-07f + 1e-30f;
                    p.bmax[k] += fabsf(p.bmax[k]) * 9.5367431640625e-07f + 1e-30f;
                    p.c[k] = (p.bmin[k] + p.bmax[k]) * 0.5f;
                }
            }
            build_bvh2(prims, m.bvh);
        }
    });
    std::vector<BuildPrim> ip(s->inst.size());
    for (size_t i = 0; i < s->inst.size(); i++) {
        Instance& in = s->inst[i];
        const Mesh& m = s->meshes[in.mesh];
        for (int k = 0; k < 3; k++) in.wmin[k] = 1e30f, in.wmax[k] = -1e30f;
        for (int c = 0; c < 8; c++) {
            const f3 q = mk3((c & 1) ? m.bmax[0] : m.bmin[0], (c & 2) ? m.bmax[1] : m.bmin[1], (c & 4) ? m.bmax[2] : m.bmin[2]);
            const f3 w = xform_point(in.T, q);
            const float ww[3] = {w.x, w.y, w.z};
            for (int k = 0; k < 3; k++) in.wmin[k] = std::min(in.wmin[k], ww[k]), in.wmax[k] = std::max(in.wmax[k], ww[k]);
        }
        for (int k = 0; k < 3; k++) {
            const float pad = (in.wmax[k] - in.wmin[k]) * 1e-5f + (fabsf(in.wmin[k]) + fabsf(in.wmax[k])) * 1e-6f + 1e-30f;
            in.wmin[k] -= pad, in.wmax[k] += pad;
            ip[i].bmin[k] = in.wmin[k], ip[i].bmax[k] = in.wmax[k], ip[i].c[k] = (in.wmin[k] + in.wmax[k]) * 0.5f;
        }
    }
    build_bvh2(ip, s->top);
    s->finalized = true;
    return 0;
}

int lh2o_trace(lh2o_scene* s, const lh2g_ray* rays, long long n, int mode, int brute, lh2g_hit* hits, uint32_t* occluded, int nthreads) {
    if (!s || !s->finalized) return 1;
    parallel_for(n, nthreads, 1024, [&](long long b, long long e) {
        for (long long i = b; i < e; i++) {
            const lh2g_ray& r = rays[i];
            HitRec h;
            const bool any = trace_scene(s, mk3(r.ox, r.oy, r.oz), mk3(r.dx, r.dy, r.dz), r.tmin, r.tmax, mode == 1, brute != 0, h);
            if (mode == 1) occluded[i] = any ? 1u : 0u;
            else hits[i] = make_hit(h);
        }
    });
    return 0;
}

int lh2o_trace_raw(lh2o_scene* s, const lh2g_ray* rays, long long n, float* t, int* inst, int* prim, float* u, float* v, int nthreads) {
    if (!s || !s->finalized) return 1;
    parallel_for(n, nthreads, 1024, [&](long long b, long long e) {
        for (long long i = b; i < e; i++) {
            const lh2g_ray& r = rays[i];
            HitRec h;
            trace_scene(s, mk3(r.ox, r.oy, r.oz), mk3(r.dx, r.dy, r.dz), r.tmin, r.tmax, false, false, h);
            t[i] = h.found ? h.t : 1e34f, inst[i] = h.found ? h.inst : 0, prim[i] = h.found ? h.prim : NOHIT;
            u[i] = h.found ? h.u : 0.0f, v[i] = h.found ? h.v : 0.0f;
        }
    });
    return 0;
}

int lh2o_render(lh2o_scene* s, const lh2g_view* view, const lh2g_render_params* p, float* pixelAccum, double* pixelAccum64,
                uint32_t* counters, lh2g_capture* capture, int nthreads) {
    if (!s || !s->finalized || !view || !p || p->width <= 0 || p->height <= 0 || p->spp <= 0 || p->maxDepth <= 0 || p->maxDepth > 64) return 1;
    Frame F;
    F.s = s, F.view = *view, F.p = *p;
    F.right = ld3(view->p2) - ld3(view->p1);
    F.up = ld3(view->p3) - ld3(view->p1);
    const long long WH = (long long)p->width * p->height;
    F.P = WH * p->spp;
    const int D = p->maxDepth;
    if (capture && capture->hits)
        for (long long i = 0; i < F.P * D; i++) capture->hits[i] = lh2g_hit{0, -1, -2, 0.0f};
    if (capture && capture->seeds) memset(capture->seeds, 0, sizeof(uint32_t) * F.P * D);
    std::vector<PathOut> paths(F.P);
    std::mutex mtx;
    std::vector<uint> extTot(D, 0), shadTot(D, 0);
    parallel_for(F.P, nthreads, 256, [&](long long b, long long e) {
        std::vector<uint> ext(D, 0), shad(D, 0);
        for (long long i = b; i < e; i++) trace_path(F, (uint)i, paths[i], ext, shad, capture);
        std::lock_guard<std::mutex> g(mtx);
        for (int d = 0; d < D; d++) extTot[d] += ext[d], shadTot[d] += shad[d];
    });
    /* per-pixel sums in sample order (deterministic) */
    for (long long px = 0; px < WH; px++) {
        for (int k = 0; k < 4; k++) {
            float acc = pixelAccum ? pixelAccum[px * 4 + k] : 0.0f;
            double acc64 = pixelAccum64 ? pixelAccum64[px * 4 + k] : 0.0;
            for (int smp = 0; smp < p->spp; smp++) {
                const float v = paths[smp * WH + px].rgbw[k];
                acc += v;
                acc64 += (double)v;
            }
            if (pixelAccum) pixelAccum[px * 4 + k] = acc;
            if (pixelAccum64) pixelAccum64[px * 4 + k] = acc64;
        }
    }
    if (counters) for (int d = 0; d < D; d++) counters[2 * d] = extTot[d], counters[2 * d + 1] = shadTot[d];
    return 0;
}

/* pure functions for the pinning tests */
uint32_t lh2o_wanghash(uint32_t v) { return WangHash(v); }
float lh2o_random_float(uint32_t* seed) { return RandomFloat(*seed); }
void lh2o_random_barycentrics(float r0, float* o) { const f3 b = RandomBarycentrics(r0); o[0] = b.x, o[1] = b.y, o[2] = b.z; }
uint32_t lh2o_pack_normal(const float* n) { return PackNormal(ld3(n)); }
void lh2o_unpack_normal(uint32_t p, float* o) { const f3 n = UnpackNormal(p); o[0] = n.x, o[1] = n.y, o[2] = n.z; }
void lh2o_diffuse_cos(float r0, float r1, float* o) { const f3 v = DiffuseReflectionCosWeighted(r0, r1); o[0] = v.x, o[1] = v.y, o[2] = v.z; }
void lh2o_tangent2world(const float* v, const float* n, float* o) { const f3 r = Tangent2World(ld3(v), ld3(n)); o[0] = r.x, o[1] = r.y, o[2] = r.z; }
void lh2o_consistent_normal(const float* d, const float* in, float alpha, float* o) { const f3 r = ConsistentNormal(ld3(d), ld3(in), alpha); o[0] = r.x, o[1] = r.y, o[2] = r.z; }
void lh2o_sincos(float x, float* s, float* c) { lm_sincos(x, s, c); }
float lh2o_expf(float x) { return lm_expf(x); }
float lh2o_log2f(float x) { return lm_log2f(x); }
float lh2o_atan2f(float y, float x) { return lm_atan2f(y, x); }
float lh2o_acosf(float x) { return lm_acosf(x); }
uint16_t lh2o_float2half(float f) { return float2half(f); }
float lh2o_half2float(uint16_t h) { return half2float(h); }
void lh2o_pack_material(const lh2g_material* m, const uint32_t* first, const uint32_t* wh, lh2g_gpu_material* out) { pack_material(*m, first, wh, *out); }
void lh2o_invert4x4(const float* m, float* o) { invert4x4(m, o); }

}  // extern "C"


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
inline f3 operator+(f3 a, float b) { return {a.x + b, a.y + b, a.z + b}; }
inline f3 operator+(float b, f3 a) { return {b + a.x, b + a.y, b + a.z}; }
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
constexpr uint S_BOUNCED = 2;                         /* RenderCore_Optix7Filter/kernels/pathtracer.h:30-31 */
constexpr uint S_VIASPECULAR = 4;

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

/* natural logarithm: lm_log2f's reduction and atanh series, ln x = e ln 2 + 2 atanh(s) (ln 2 split so e ln 2 is exact) */
inline float lm_logf(float x) {
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
    return (float)e * LN2_HI + ((float)e * LN2_LO + at * 2.0f);
}

/* x^y as exp(y ln x) for x > 0; 0^y = 0 (y > 0) or 1 (y = 0); NaN for x < 0 */
inline float lm_powf(float x, float y) {
    if (x != x || y != y) return x + y;
    if (x < 0.0f) return bitsf(0x7fc00000u);
    if (y == 0.0f) return 1.0f;
    if (x == 0.0f) return y > 0.0f ? 0.0f : bitsf(0x7f800000u);
    return lm_expf(y * lm_logf(x));
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
    std::vector<f3> pos;          /* the vertex buffer, 3 per triangle (the rasteriser transforms it) */
    std::vector<f3> v0, e1, e2;   /* intersection data: v0, v1 - v0, v2 - v0 from the vertex buffer */
    BVH2 bvh;
    float bmin[3], bmax[3];
};

struct Instance {
    int mesh;
    float T[16], inv[16];
    float wmin[3], wmax[3];
};

/* the sky and its 64x scaled-down copy (the average of each 64 x 64 tile, RenderCore::SetSkyData,
 * lib/rendercore_optix7/rendercore.cpp:716-740), which the OptiX 7 estimator samples after a diffuse bounce */
struct Sky { std::vector<f3> px; int w = 0, h = 0; float m[16]; std::vector<f3> small; };

}  // namespace

/* one record of the light tree (the device LightCluster, common_classes.h:522-527; the parent in the normal's w) */
struct LtCluster { int light, left, right; float intensity; float bmin[4], bmax[4]; float N[3]; int parent; };
static_assert(sizeof(LtCluster) == 64, "the device record");

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
    std::vector<LtCluster> lightTree;   /* built by lh2o_set_lights (the light tree) */
    Sky sky;
    BVH2 top;
    bool finalized = false;
    /* blue-noise tables expanded to one uint per entry as rendercore_optix7/rendercore.cpp:247-256 does: Sobol
     * 256 x 256 at 0, scrambling 128 x 128 x 8 at 65536, ranking 128 x 128 x 8 at 3 * 65536; then 64 zero entries,
     * which the ranking reads of deep path lengths at the last tile pixel reach (the reference reads past its
     * buffer there). Empty: no tables, every sample uses xorshift numbers. */
    std::vector<uint> blueNoise;
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
    f4 tint;   /* the Disney BSDF's tint (xyz) and luminance (w) of the base colour, when GetShadingData is asked */
};
/* material_shared.h:19-35,118-119: the base colour's tint through CIE XYZ */
inline f4 tint_of(const f3 rgb) {
    const f3 xyz = mk3(fmaxf(0.0f, 0.412453f * rgb.x + 0.357580f * rgb.y + 0.180423f * rgb.z),
                       fmaxf(0.0f, 0.212671f * rgb.x + 0.715160f * rgb.y + 0.072169f * rgb.z),
                       fmaxf(0.0f, 0.019334f * rgb.x + 0.119193f * rgb.y + 0.950227f * rgb.z));
    if (!(xyz.y > 0)) return {1.0f, 1.0f, 1.0f, xyz.y};
    const f3 n = xyz * (1.0f / xyz.y);
    return {fmaxf(0.0f, 3.240479f * n.x - 1.537150f * n.y - 0.498535f * n.z), fmaxf(0.0f, -0.969256f * n.x + 1.875992f * n.y + 0.041556f * n.z),
            fmaxf(0.0f, 0.055648f * n.x - 0.204043f * n.y + 1.057311f * n.z), xyz.y};
}
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
                    const lh2g_core_tri& tri, const int instIdx, ShadingData& sd, f3& N, f3& iN, f3& fN, f3& T, const bool withTint = false) {
    const lh2g_gpu_material& mat = s->mats[tri.material];
    const uint part0 = mat.base[0], part1 = mat.base[1], part2 = mat.base[2], flags = mat.base[3];
    sd.color = mk3(half2float(part0 & 0xffffu), half2float(part0 >> 16), half2float(part1 & 0xffffu));
    sd.flags = 0;
    sd.transmittance = mk3(half2float(part1 >> 16), half2float(part2 & 0xffffu), half2float(part2 >> 16));
    sd.matID = 0;
    for (int i = 0; i < 4; i++) sd.params[i] = mat.params[i];
    if (withTint) sd.tint = tint_of(sd.color);
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
 * The Disney principled BSDF (the OptiX 7 / PrimeAdaptive cores' default kernels/bsdf.h branch):
 * lib/sharedBSDFs/disney.h, ggxmdf.h (CUDA branches of the samplers) and frosted.h, restated in their operation
 * order with this file's transcendentals (lm_sincos, lm_expf, lm_logf, lm_powf). Values the reference leaves unset
 * on measure-zero paths (a direction exactly in the tangent plane) are zero here.
 * ---------------------------------------------------------------------------------------------------- */
namespace dis {
inline float METALLIC(const ShadingData& s) { return char2flt(s.params[0], 0); }
inline float SUBSURFACE(const ShadingData& s) { return char2flt(s.params[0], 8); }
inline float SPECULAR(const ShadingData& s) { return char2flt(s.params[0], 16); }
inline float SPECTINT(const ShadingData& s) { return char2flt(s.params[1], 0); }
inline float ANISOTROPIC(const ShadingData& s) { return char2flt(s.params[1], 8); }
inline float SHEEN(const ShadingData& s) { return char2flt(s.params[1], 16); }
inline float SHEENTINT(const ShadingData& s) { return char2flt(s.params[1], 24); }
inline float CLEARCOAT(const ShadingData& s) { return char2flt(s.params[2], 0); }
inline float CLEARCOATGLOSS(const ShadingData& s) { return char2flt(s.params[2], 8); }
inline f3 TINT(const ShadingData& s) { return mk3(s.tint.x, s.tint.y, s.tint.z); }
inline float LUMINANCE(const ShadingData& s) { return s.tint.w; }
inline float sqr(float x) { return x * x; }
inline float saturate(float x) { return fmaxr(0.0f, fminr(1.0f, x)); }
inline float lerp(float a, float b, float t) { return a + t * (b - a); }
inline float mix(float a, float b, float x) { return x <= 0 ? a : x >= 1 ? b : lerp(a, b, x); }
inline float clampv(float f, float a, float b) { return fmaxr(a, fminr(f, b)); }
inline f3 w2t(const f3 V, const f3 N, const f3 T, const f3 B) { return mk3(dot(V, T), dot(V, B), dot(V, N)); }
inline f3 t2w(const f3 V, const f3 N, const f3 T, const f3 B) { return V.x * T + V.y * B + V.z * N; }
inline f3 cos_sample(const float r0, const float r1, const f3 N, const f3 T, const f3 B) {   /* common_functions.h:118-124 */
    const float term1 = TWOPI * r0, term2 = sqrtf(1 - r1);
    float sn, cs;
    lm_sincos(term1, &sn, &cs);
    return (cs * term2 * T) + (sn * term2) * B + sqrtf(r1) * N;
}
/* ggxmdf.h */
inline float ggx_D(const f3 m, const float ax, const float ay) {
    if (m.z == 0) return sqr(ax) * INVPI;
    const float c2 = sqr(m.z), sinT = sqrtf(fmaxr(0.0f, 1 - c2)), tan2 = (1.0f - c2) / c2;
    const float st = (ax == ay || sinT == 0.0f) ? 1.0f / sqr(ax) : sqr(m.x / (sinT * ax)) + sqr(m.y / (sinT * ay));
    return 1.0f / (PI * ax * ay * sqr(c2) * sqr(1.0f + tan2 * st));
}
inline float ggx_lambda(const f3 v, const float ax, const float ay) {
    if (v.z == 0) return 0;
    const float c2 = v.z * v.z, sinT = sqrtf(fmaxr(0.0f, 1 - c2));
    const float proj = (ax == ay || sinT == 0.0f) ? ax : sqrtf(sqr((v.x * ax) / sinT) + sqr((v.y * ay) / sinT));
    const float tan2 = sqr(sinT) / c2, a2rcp = sqr(proj) * tan2;
    return (-1.0f + sqrtf(1.0f + a2rcp)) * 0.5f;
}
inline float ggx_G(const f3 wi, const f3 wo, const float ax, const float ay) { return 1.0f / (1.0f + ggx_lambda(wo, ax, ay) + ggx_lambda(wi, ax, ay)); }
inline float ggx_G1(const f3 v, const float ax, const float ay) { return 1.0f / (1.0f + ggx_lambda(v, ax, ay)); }
inline f3 ggx_sample(const f3 v, const float r0, const float r1, const float ax, const float ay) {
    const float sgn = v.z < 0.0f ? -1.0f : 1.0f;
    const f3 st = normalize(mk3(sgn * v.x * ax, sgn * v.y * ay, sgn * v.z));
    const f3 t1 = v.z < 0.9999f ? normalize(cross(st, mk3(0, 0, 1))) : mk3(1, 0, 0);
    const f3 t2 = cross(t1, st);
    const float a = 1.0f / (1.0f + st.z), r = sqrtf(r0);
    const float phi = r1 < a ? (r1 / a * PI) : (PI + (r1 - a) / (1.0f - a) * PI);
    float p1, p2;
    lm_sincos(phi, &p2, &p1);
    p1 *= r;
    p2 *= r * (r1 < a ? 1.0f : st.z);
    const f3 h = p1 * t1 + p2 * t2 + sqrtf(fmaxr(0.0f, 1.0f - p1 * p1 - p2 * p2)) * st;
    return normalize(mk3(h.x * ax, h.y * ay, fmaxr(0.0f, h.z)));
}
inline float ggx_pdf(const f3 v, const f3 m, const float ax, const float ay) {
    if (v.z == 0.0f) return 0;
    return ggx_G1(v, ax, ay) * fabsf(dot(v, m)) * ggx_D(m, ax, ay) / fabsf(v.z);
}
inline float gtr1_D(const f3 m, const float ax) {
    const float alpha = clampv(ax, 0.001f, 0.999f), a2 = sqr(alpha);
    const float a = (a2 - 1.0f) / (PI * lm_logf(a2)), b = (1 / (1 + (a2 - 1) * sqr(m.z)));
    return a * b;
}
inline float gtr1_lambda(const f3 v, const float ax) {
    if (v.z == 0) return 0;
    const float c2 = sqr(v.z), sinT = sqrtf(fmaxr(0.0f, 1.0f - c2));
    if (sinT == 0) return 0;
    const float cot2 = c2 / sqr(sinT), cot = sqrtf(cot2), alpha2 = sqr(clampv(ax, 0.001f, 0.999f));
    const float a = sqrtf(cot2 + alpha2), b = sqrtf(cot2 + 1.0f), c = lm_logf(cot + b), d = lm_logf(cot + a);
    return (a - b + cot * (c - d)) / (cot * lm_logf(alpha2));
}
inline float gtr1_G(const f3 wi, const f3 wo, const float ax) { return 1.0f / (1.0f + gtr1_lambda(wo, ax) + gtr1_lambda(wi, ax)); }
inline f3 gtr1_sample(const float r0, const float r1, const float ax) {
    const float alpha = clampv(ax, 0.001f, 0.999f), a2 = sqr(alpha);
    const float c2 = (1.0f - lm_powf(a2, 1.0f - r0)) / (1.0f - a2), sinT = sqrtf(fmaxr(0.0f, 1.0f - c2));
    float sp, cp;
    lm_sincos(TWOPI * r1, &sp, &cp);
    return mk3(cp * sinT, sp * sinT, sqrtf(c2));
}
inline float gtr1_pdf(const f3 m, const float ax) { return gtr1_D(m, ax) * fabsf(m.z); }
inline void alpha_from_roughness(const float roughness, const float anisotropy, float& ax, float& ay) {
    const float sq = roughness * roughness, aspect = sqrtf(1.0f + anisotropy * (anisotropy < 0 ? 0.9f : -0.9f));
    ax = fmaxr(0.001f, sq / aspect), ay = fmaxr(0.001f, sq * aspect);
}
/* frosted.h */
inline float fresnel_dielectric(const float eta, const float ci, const float ct) {
    if (ci == 0 && ct == 0) return 1;
    const float k0 = eta * ct, k1 = eta * ci;
    return 0.5f * (sqr((ci - k0) / (ci + k0)) + sqr((ct - k1) / (ct + k1)));
}
inline float fresnel_reflectance(const float ci, const float eta, float& ct) {
    const float st2 = (1 - sqr(ci)) * sqr(eta);
    if (st2 > 1) { ct = 0; return 1; }
    ct = fminr(sqrtf(fmaxr(1 - st2, 0.0f)), 1.0f);
    return fresnel_dielectric(eta, fabsf(ci), ct);
}
inline f3 refracted_direction(const f3 wo, const f3 m, const float cwm, const float ct, const float rcpEta) {
    const f3 wi = cwm > 0 ? (rcpEta * cwm - ct) * m - rcpEta * wo : (rcpEta * cwm + ct) * m - rcpEta * wo;
    return wi * ((3 - dot(wi, wi)) * 0.5f);
}
inline float choose_reflection(const float F) { const float r = F * 1, t = (1 - F) * 1, sum = r + t; return sum != 0 ? r / sum : 1; }
inline f3 half_reflection(const f3 wo, const f3 wi) { const f3 h = normalize(wi + wo); return h.z < 0 ? (h * -1) : h; }
inline f3 half_refraction(const f3 wo, const f3 wi, const float eta) { const f3 h = normalize(wo + eta * wi); return h.z < 0 ? (h * -1) : h; }
inline f3 eval_reflection(const f3 color, const f3 wo, const f3 wi, const f3 m, const float ax, const float ay, const float F) {
    const float denom = fabsf(4 * wo.z * wi.z);
    if (denom == 0) return mk3(0);
    const float D = ggx_D(m, ax, ay), G = ggx_G(wi, wo, ax, ay);
    return color * (F * D * G / denom);
}
inline f3 eval_refraction(const float eta, const f3 color, const f3 wo, const f3 wi, const f3 m, const float ax, const float ay, const float Tr) {
    if (wo.z == 0 || wi.z == 0) return mk3(0);
    const float cih = dot(m, wi), coh = dot(m, wo), dots = (cih * coh) / (wi.z * wo.z), sd = coh + eta * cih;
    if (fabsf(sd) < 1.0e-6f) return mk3(0);
    const float D = ggx_D(m, ax, ay), G = ggx_G(wi, wo, ax, ay);
    float mult = fabsf(dots) * Tr * D * G / sqr(sd);
    mult *= sqr(eta);
    return color * mult;
}
inline float reflection_jacobian(const float coh) { return coh == 0 ? 0.0f : 1 / (4 * fabsf(coh)); }
inline float refraction_jacobian(const f3 wo, const f3 wi, const f3 m, const float eta) {
    const float cih = dot(m, wi), coh = dot(m, wo), sd = coh + eta * cih;
    if (fabsf(sd) < 1.0e-6f) return 0;
    return fabsf(cih) * sqr(eta / sd);
}
/* disney.h */
inline float schlick(const float u) { const float m = saturate(1.0f - u), m2 = sqr(m), m4 = sqr(m2); return m4 * m; }
inline float clearcoat_roughness(const ShadingData& s) { return mix(0.1f, 0.001f, CLEARCOATGLOSS(s)); }
inline f3 specular_fresnel(const ShadingData& s, const f3 o, const f3 h) {
    const float st = SPECTINT(s), M = METALLIC(s);
    f3 v = (1.0f - st) + st * TINT(s);
    v = v * (SPECULAR(s) * 0.08f);
    v = (1.0f - M) * v + M * s.color;
    const float f = schlick(fabsf(dot(o, h)));
    return (1.0f - f) * v + f;
}
inline f3 clearcoat_fresnel(const ShadingData& s, const f3 o, const f3 h) { return mk3(mix(0.04f, 1.0f, schlick(fabsf(dot(o, h)))) * 0.25f * CLEARCOAT(s)); }
template <bool GTR1>
inline void sample_mf(const ShadingData& s, const float r0, const float r1, const float ax, const float ay, const f3 wol, f3& wil, float& pdf, f3& value) {
    if (wol.z == 0) { value = mk3(0); pdf = 0; return; }
    const f3 m = GTR1 ? gtr1_sample(r0, r1, ax) : ggx_sample(wol, r0, r1, ax, ay);
    wil = reflect(wol * -1.0f, m);
    if (wil.z == 0) return;
    const float coh = dot(wol, m);
    pdf = (GTR1 ? gtr1_pdf(m, ax) : ggx_pdf(wol, m, ax, ay)) / fabsf(4.0f * coh);
    if (pdf < 1.0e-6f) return;
    const float D = GTR1 ? gtr1_D(m, ax) : ggx_D(m, ax, ay);
    const float G = GTR1 ? gtr1_G(wil, wol, ax) : ggx_G(wil, wol, ax, ay);
    value = GTR1 ? clearcoat_fresnel(s, wol, m) : specular_fresnel(s, wol, m);
    value = value * (D * G);
}
template <bool GTR1>
inline float evaluate_mf(const ShadingData& s, const float ax, const float ay, const f3 wol, const f3 wil, const f3 m, f3& bsdf) {
    if (wol.z == 0 || wil.z == 0) return 0;
    const float coh = dot(wol, m);
    if (coh == 0) return 0;
    const float D = GTR1 ? gtr1_D(m, ax) : ggx_D(m, ax, ay);
    const float G = GTR1 ? gtr1_G(wil, wol, ax) : ggx_G(wil, wol, ax, ay);
    bsdf = GTR1 ? clearcoat_fresnel(s, wol, m) : specular_fresnel(s, wol, m);
    bsdf = bsdf * (D * G / fabsf(4.0f * wol.z * wil.z));
    return (GTR1 ? gtr1_pdf(m, ax) : ggx_pdf(wol, m, ax, ay)) / fabsf(4.0f * coh);
}
inline float evaluate_diffuse(const ShadingData& s, const f3 iN, const f3 wow, const f3 wiw, const f3 m, f3& value) {
    const float con = dot(iN, wow), cin = dot(iN, wiw), cih = dot(wiw, m);
    const float fl = schlick(cin), fv = schlick(con), R = ROUGHNESS(s), SS = SUBSURFACE(s);
    float fd = 0;
    if (SS != 1.0f) {
        const float fd90 = 0.5f + 2.0f * sqr(cih) * R;
        fd = mix(1.0f, fd90, fl) * mix(1.0f, fd90, fv);
    }
    if (SS > 0) {
        const float fss90 = sqr(cih) * R, fss = mix(1.0f, fss90, fl) * mix(1.0f, fss90, fv);
        const float ss = 1.25f * (fss * (1.0f / (fabsf(con) + fabsf(cin)) - 0.5f) + 0.5f);
        fd = mix(fd, ss, SS);
    }
    value = s.color * fd * INVPI * (1.0f - METALLIC(s));
    return fabsf(cin) * INVPI;
}
inline float evaluate_sheen(const ShadingData& s, const f3 wiw, const f3 m, f3& value) {
    const float fh = schlick(dot(wiw, m)), st = SHEENTINT(s);
    value = (1.0f - st) + st * TINT(s);
    value = value * (fh * SHEEN(s) * (1.0f - METALLIC(s)));
    return 1.0f / (2 * PI);
}
inline f4 weights_of(const ShadingData& s) {
    const float M = METALLIC(s);
    f4 w = {lerp(LUMINANCE(s), 0, M), lerp(SHEEN(s), 0, M), lerp(SPECULAR(s), 1, M), CLEARCOAT(s) * 0.25f};
    return w * (1.0f / (w.x + w.y + w.z + w.w));
}
f3 SampleBSDF(const ShadingData& s, f3 iN, const f3 N, const f3 iT, const f3 wow, const float distance, const float r0, const float r1,
              const float r2, f3& wiw, float& pdf, bool& specular) {
    const float flip = (dot(wow, N) < 0) ? -1.0f : 1.0f;
    iN = iN * flip;
    const f3 B = normalize(cross(iN, iT)), T = normalize(cross(iN, B));
    const float TR = TRANSMISSION(s);
    if (r0 < TR) {
        specular = true;
        const float r3 = r0 / TR;
        const f3 wol = w2t(wow, iN, T, B);
        const float eta = flip < 0 ? (1 / ETA(s)) : ETA(s);
        if (eta == 1) return mk3(0);
        const f3 beer = mk3(lm_expf(-s.transmittance.x * distance * 2.0f), lm_expf(-s.transmittance.y * distance * 2.0f),
                            lm_expf(-s.transmittance.z * distance * 2.0f));
        float ax, ay;
        alpha_from_roughness(ROUGHNESS(s), ANISOTROPIC(s), ax, ay);
        const f3 m = ggx_sample(wol, r1, r3, ax, ay);
        const float rcpEta = 1 / eta, cwm = clampv(dot(wol, m), -1.0f, 1.0f);
        float ct, jac;
        const float F = fresnel_reflectance(cwm, eta, ct);
        f3 wil, ret;
        if (r2 < F) {
            wil = reflect(wol * -1.0f, m);
            if (wil.z * wol.z <= 0) return mk3(0);
            ret = eval_reflection(s.color, wol, wil, m, ax, ay, F);
            pdf = F, jac = reflection_jacobian(cwm);
        } else {
            wil = refracted_direction(wol, m, cwm, ct, eta);
            if (wil.z * wol.z > 0) return mk3(0);
            ret = eval_refraction(rcpEta, s.color, wol, wil, m, ax, ay, 1 - F);
            pdf = 1 - F, jac = refraction_jacobian(wol, wil, m, rcpEta);
        }
        pdf *= jac * ggx_pdf(wol, m, ax, ay);
        if (pdf > 1.0e-6f) wiw = t2w(wil, iN, T, B);
        return ret * beer;
    }
    const float r3 = (r0 - TR) / (1 - TR);
    f4 w = weights_of(s);
    const f4 cdf = {w.x, w.x + w.y, w.x + w.y + w.z, 0};
    float probability, cpdf = 0;
    f3 contrib = mk3(0), value = mk3(0);
    if (r3 < cdf.y) {
        const float r2b = r3 / cdf.y;
        wiw = cos_sample(r2b, r1, iN, T, B);
        const f3 m = normalize(wiw + wow);
        if (r3 < cdf.x) cpdf = evaluate_diffuse(s, iN, wow, wiw, m, value), probability = w.x * cpdf, w.x = 0;
        else cpdf = evaluate_sheen(s, wiw, m, value), probability = w.y * cpdf, w.y = 0;
    } else {
        const f3 wol = w2t(wow, iN, T, B);
        f3 wil = mk3(0);
        if (r3 < cdf.z) {
            const float r2b = (r3 - cdf.y) / (cdf.z - cdf.y);
            float ax, ay;
            alpha_from_roughness(ROUGHNESS(s), ANISOTROPIC(s), ax, ay);
            sample_mf<false>(s, r2b, r1, ax, ay, wol, wil, cpdf, value);
            probability = w.z * cpdf, w.z = 0;
        } else {
            const float r2b = (r3 - cdf.z) / (1 - cdf.z), a = clearcoat_roughness(s);
            sample_mf<true>(s, r2b, r1, a, a, wol, wil, cpdf, value);
            probability = w.w * cpdf, w.w = 0;
        }
        value = value * (1.0f / fabsf(4.0f * wol.z * wil.z));
        wiw = t2w(wil, iN, T, B);
    }
    if (w.x + w.y > 0) {
        const f3 m = normalize(wiw + wow);
        if (w.x > 0) probability += w.x * evaluate_diffuse(s, iN, wow, wiw, m, contrib), value = value + contrib;
        if (w.y > 0) probability += w.y * evaluate_sheen(s, wiw, m, contrib), value = value + contrib;
    }
    if (w.z + w.w > 0) {
        const f3 wol = w2t(wow, iN, T, B), wil = w2t(wiw, iN, T, B), m = normalize(wol + wil);
        if (w.z > 0) {
            float ax, ay;
            alpha_from_roughness(ROUGHNESS(s), ANISOTROPIC(s), ax, ay);
            probability += w.z * evaluate_mf<false>(s, ax, ay, wol, wil, m, contrib);
            value = value + contrib;
        }
        if (w.w > 0) {
            const float a = clearcoat_roughness(s);
            probability += w.w * evaluate_mf<true>(s, a, a, wol, wil, m, contrib);
            value = value + contrib;
        }
    }
    pdf = probability > 1.0e-6f ? probability : 0;
    return value;
}
f3 EvaluateBSDF(const ShadingData& s, const f3 iN, const f3 iT, const f3 wow, const f3 wiw, float& pdf) {
    if (TRANSMISSION(s) > 0.5f) {
        const f3 B = normalize(cross(iN, iT)), T = normalize(cross(iN, B));
        const f3 wol = w2t(wow, iN, T, B), wil = w2t(wiw, iN, T, B);
        const float eta = wol.z > 0 ? ETA(s) : (1.0f / ETA(s));
        if (eta == 1) { pdf = 0; return mk3(0); }
        float ax, ay, jac;
        alpha_from_roughness(ROUGHNESS(s), ANISOTROPIC(s), ax, ay);
        f3 ret, m;
        float ct;
        if (wil.z * wol.z >= 0) {
            m = half_reflection(wol, wil);
            const float cwm = dot(wol, m), F = fresnel_reflectance(cwm, 1 / eta, ct);
            ret = eval_reflection(s.color, wol, wil, m, ax, ay, F);
            pdf = choose_reflection(F), jac = reflection_jacobian(cwm);
        } else {
            m = half_refraction(wol, wil, eta);
            const float cwm = dot(wol, m), F = fresnel_reflectance(cwm, 1 / eta, ct);
            ret = eval_refraction(eta, s.color, wol, wil, m, ax, ay, 1 - F);
            pdf = 1 - choose_reflection(F), jac = refraction_jacobian(wol, wil, m, eta);
        }
        pdf *= jac * ggx_pdf(wol, m, ax, ay);
        return ret;
    }
    if (ROUGHNESS(s) <= 0.001f) { pdf = 0; return mk3(0); }
    const f3 B = normalize(cross(iN, iT)), T = normalize(cross(iN, B));
    const f4 w = weights_of(s);
    pdf = 0;
    f3 value = mk3(0);
    if (w.x + w.y > 0) {
        const f3 m = normalize(wiw + wow);
        if (w.x > 0) pdf += w.x * evaluate_diffuse(s, iN, wow, wiw, m, value);
        if (w.y > 0) pdf += w.y * evaluate_sheen(s, wiw, m, value);   /* overwrites the diffuse value, as disney.h does */
    }
    if (w.z + w.w > 0) {
        const f3 wol = w2t(wow, iN, T, B), wil = w2t(wiw, iN, T, B), m = normalize(wol + wil);
        if (w.z > 0) {
            float ax, ay;
            alpha_from_roughness(ROUGHNESS(s), ANISOTROPIC(s), ax, ay);
            f3 c = mk3(0);
            const float sp = evaluate_mf<false>(s, ax, ay, wol, wil, m, c);
            if (sp > 0) pdf += w.z * sp, value = value + c;
        }
        if (w.w > 0) {
            const float a = clearcoat_roughness(s);
            f3 c = mk3(0);
            const float cp = evaluate_mf<true>(s, a, a, wol, wil, m, c);
            if (cp > 0) pdf += w.w * cp, value = value + c;
        }
    }
    return value;
}
}  // namespace dis

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
    lh2o_features feat;        /* LH2G_RP_FILTER: SVGF feature buffers (W*H entries each) */
    uint bandPix = 0;          /* a band of rows (lh2g_render_params rowBegin / rowCount): its pixels; 0: the whole frame */
    /* the index in the whole frame of the band's path l */
    uint global(uint l) const {
        if (!bandPix) return l;
        return (l / bandPix) * ((uint)p.width * (uint)p.height) + (uint)p.rowBegin * (uint)p.width + l % bandPix;
    }
};

/* Radiance of one path: rgbw[0] = the direct half (and the primary distance in w), rgbw[1] = the indirect
 * half (only LH2G_RP_FILTER frames route radiance there). */
struct PathOut { float rgbw[2][4]; };

/* ------------------------------------------------------------------------------------------------------
 * SVGF feature packing (lib/CUDA/shared_kernel_code/tools_shared.h:122-136, 157-183, 282-304)
 * ---------------------------------------------------------------------------------------------------- */
inline uint umin(uint a, uint b) { return a < b ? a : b; }
inline uint umax(uint a, uint b) { return a > b ? a : b; }
/* PackNormal2: 10 bits per component at bits 2, 12, 22; bits 0-1 stay free for the specular flag */
inline uint PackNormal2(const f3 N) {
    const uint x = umin(f2u((N.x + 1) * 511), 1023u);
    const uint y = umin(f2u((N.y + 1) * 511), 1023u);
    const uint z = umin(f2u((N.z + 1) * 511), 1023u);
    return (x << 2u) + (y << 12u) + (z << 22u);
}
inline f3 UnpackNormal2(const uint pi) {
    const uint x = (pi >> 2u) & 1023u, y = (pi >> 12u) & 1023u, z = pi >> 22u;
    return mk3((float)x * (1.0f / 511.0f) - 1, (float)y * (1.0f / 511.0f) - 1, (float)z * (1.0f / 511.0f) - 1);
}
/* HDRtoRGB32: 10:11:11 unsigned fixed point of min(1, c) */
inline uint HDRtoRGB32(const f3& c) {
    const uint r = f2u(1023.0f * fminr(1.0f, c.x));
    const uint g = f2u(2047.0f * fminr(1.0f, c.y));
    const uint b = f2u(2047.0f * fminr(1.0f, c.z));
    return (r << 22) + (g << 11) + b;
}
inline f3 RGB32toHDR(const uint c) {
    return mk3((float)(c >> 22) * (1.0f / 1023.0f), (float)((c >> 11) & 2047) * (1.0f / 2047.0f), (float)(c & 2047) * (1.0f / 2047.0f));
}
inline f3 RGB32toHDRmin1(const uint c) {
    return mk3((float)umax(1u, c >> 22) * (1.0f / 1023.0f), (float)umax(1u, (c >> 11) & 2047) * (1.0f / 2047.0f),
               (float)umax(1u, c & 2047) * (1.0f / 2047.0f));
}
/* PackFeatures (RenderCore_Optix7Filter/kernels/pathtracer.h:44-47): the history count in w & 15 survives */
inline void PackFeatures(uint* f, const uint albedo, const uint packedNormal, const float t, const uint isSpecular, const uint matid) {
    const uint w = (isSpecular << 4) + (matid << 6) + (f[3] & 15);
    f[0] = albedo, f[1] = packedNormal, f[2] = fbits(t), f[3] = w;
}
inline void store4(float* d, float x, float y, float z, float w) { d[0] = x, d[1] = y, d[2] = z, d[3] = w; }
/* calculateDepthDerivatives (RenderCore_Optix7Filter/kernels/pathtracer.h:48-57): depth change of the rays
 * through the pixels right of and below (x, y) where they meet the plane of the hit. The plane is the one
 * through the hit point I with the world-space geometric normal N; the reference takes vertex 0 and the face
 * normal of the object-space triangle, the same plane when the instance transform is the identity. */
inline void DepthDerivatives(const int x, const int y, const int w, const int h, const float depth, const f3& I, const f3& N,
                             const f3& p1, const f3& p2, const f3& p3, const f3& pos, float* out) {
    const f3 rayDXDir = normalize((p1 + (float)(x + 0.5f + 1) * (1.0f / w) * p2 + (float)(y + 0.5f) * (1.0f / h) * p3) - pos);
    const float rayDXDepth = dot(I - pos, N) / dot(N, rayDXDir);
    const f3 rayDYDir = normalize((p1 + (float)(x + 0.5f) * (1.0f / w) * p2 + (float)(y + 0.5f + 1) * (1.0f / h) * p3) - pos);
    const float rayDYDepth = dot(I - pos, N) / dot(N, rayDYDir);
    store4(out, 0, 0, rayDXDepth - depth, rayDYDepth - depth);
}

void trace_path(const Frame& F, const uint jobIndex, PathOut& out, std::vector<uint>& ext, std::vector<uint>& shad, lh2g_capture* cap) {
    const lh2o_scene* s = F.s;
    const lh2g_render_params& p = F.p;
    const int W = p.width, H = p.height;
    const float eps = p.geometryEpsilon;
    const bool nee = (p.flags & LH2G_RP_NEE) != 0;
    const bool filt = (p.flags & LH2G_RP_FILTER) != 0;
    const uint WH = (uint)W * (uint)H;
    /* generateEyeRaysKernel (a band's paths take their index in the whole frame) */
    const uint gIdx = F.global(jobIndex);
    const uint x = gIdx % (uint)W;
    uint y = gIdx / (uint)W;
    y %= (uint)H;
    uint seed = WangHash(gIdx + p.cameraR0);
    const float r0 = RandomFloat(seed), r1 = RandomFloat(seed);
    const float r2 = RandomFloat(seed), r3 = RandomFloat(seed);
    const f3 p1 = ld3(F.view.p1), pos = ld3(F.view.pos);
    f3 O, D;
    if (filt) {
        /* filter core: pixel corner of the jittered view, no lens (RenderCore_Optix7Filter/optix/.optix.cu:66-100) */
        const float u = (float)x * (1.0f / (float)W), v = (float)y * (1.0f / (float)H);
        const f3 posOnPixel = p1 + u * F.right + v * F.up;
        O = pos, D = normalize(posOnPixel - pos);
    } else {
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
        O = posOnLens, D = normalize(posOnPixel - posOnLens);
    }
    float tmin = eps;
    f3 throughput = mk3(1);
    uint FLAGS = S_SPECULAR;
    const uint pathIdx = jobIndex;
    for (int h = 0; h < 2; h++) out.rgbw[h][0] = out.rgbw[h][1] = out.rgbw[h][2] = out.rgbw[h][3] = 0;
    /* filter data of sample 0 (RenderCore_Optix7Filter/kernels/pathtracer.h:95-104) */
    const uint sampleIdx = pathIdx / WH + (uint)p.samplesTaken;
    uint* feat = filt && sampleIdx == 0 && F.feat.features ? F.feat.features + 4 * (size_t)pathIdx : nullptr;
    float* wpos = feat ? F.feat.worldPos + 4 * (size_t)pathIdx : nullptr;
    float* ddep = feat ? F.feat.deltaDepth + 4 * (size_t)pathIdx : nullptr;
    const f3 vp2 = F.right, vp3 = F.up;   /* p2 - p1, p3 - p1 of the view */
    for (int pathLength = 1; pathLength <= p.maxDepth; pathLength++) {
        HitRec h;
        trace_scene(s, O, D, tmin, 1e34f, false, false, h);
        const lh2g_hit hit = make_hit(h);
        const long long capIdx = (long long)(pathLength - 1) * F.P + pathIdx;
        if (cap && cap->hits) cap->hits[capIdx] = hit;
        const uint R0 = filt ? p.frameSeed + (uint)pathLength * 91771u : (uint)p.samplesTaken * 7907u + (uint)pathLength * 91771u;
        /* radiance goes to the indirect half once the path has bounced off a diffuse vertex */
        float* acc = out.rgbw[filt && (FLAGS & S_BOUNCED) ? 1 : 0];
        const bool firstHitToBeStored = feat && (FLAGS & S_BOUNCED) == 0;
        const uint isSpecular = (FLAGS & S_VIASPECULAR) ? 1 : 0;
        if (pathLength == 1 && firstHitToBeStored) {
            PackFeatures(feat, 0, 0, 1e34f, 0, 0);
            store4(wpos, 0, 0, 0, bitsf(0));
            store4(ddep, 0, 0, 0, 0);
        }
        if ((p.flags & LH2G_RP_DEPTH_W) && pathLength == 1) acc[3] += hit.prim == NOHIT ? 10000.0f : hit.t;
        if (hit.prim == NOHIT) {
            const f3 c = throughput * SampleSkydome(s, D);
            acc[0] += c.x, acc[1] += c.y, acc[2] += c.z;
            if (firstHitToBeStored) {
                const uint packedNormal = PackNormal2(D * -1.0f) + isSpecular;
                PackFeatures(feat, HDRtoRGB32(c), packedNormal, hit.t, isSpecular, 0);
                const f3 far = O + 50000 * D;
                store4(wpos, far.x, far.y, far.z, bitsf(packedNormal));
                store4(ddep, 0, 0, 0, 0);
            }
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
        const uint matID = std::min<uint>(tri.material, (uint)s->mats.size() - 1);   /* ShadingData::matID is never assigned in the reference; the material index is what it names */
        if (IsEmissive(sd)) {
            const float DdotNL = -dot(D, N);
            if (DdotNL > 0) {
                const f3 c = throughput * sd.color;
                if (pathLength == 1 || (FLAGS & S_SPECULAR) || !nee) acc[0] += c.x, acc[1] += c.y, acc[2] += c.z;
            }
            if (firstHitToBeStored) {
                const uint packedNormal = PackNormal2(N) + isSpecular;
                PackFeatures(feat, HDRtoRGB32(sd.color), packedNormal, HIT_T, isSpecular, matID);
                store4(wpos, I.x, I.y, I.z, bitsf(packedNormal));
                DepthDerivatives((int)(pathIdx % (uint)W), (int)(pathIdx / (uint)W), W, H, HIT_T, I, N, p1, vp2, vp3, pos, ddep);
            }
            if (cap && cap->seeds) cap->seeds[capIdx] = 0;
            return;
        }
        if (ROUGHNESS(sd) <= 0.001f || TRANSMISSION(sd) > 0.999f) FLAGS |= S_SPECULAR; else FLAGS &= ~S_SPECULAR;
        seed = WangHash(gIdx * 17u + R0);
        if (firstHitToBeStored) {
            if (FLAGS & S_SPECULAR) {
                feat[0] = HDRtoRGB32(sd.color);   /* modulated by the first diffuse vertex later */
            } else {
                f3 albedo = sd.color;
                if (FLAGS & S_VIASPECULAR) albedo = albedo * RGB32toHDR(feat[0]);
                /* the reference writes flip ? -fN : fN with flip = +-1, which always takes the first branch */
                const uint packedNormal = PackNormal2(fN * -1.0f) + isSpecular;
                PackFeatures(feat, HDRtoRGB32(albedo), packedNormal, HIT_T, isSpecular, matID);
                store4(wpos, I.x, I.y, I.z, bitsf(packedNormal));
                DepthDerivatives((int)(pathIdx % (uint)W), (int)(pathIdx / (uint)W), W, H, HIT_T, I, N, p1, vp2, vp3, pos, ddep);
            }
        }
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
                    acc[0] += contribution.x, acc[1] += contribution.y, acc[2] += contribution.z;
            }
        }
        if (pathLength == p.maxDepth && firstHitToBeStored) {
            /* the path ends here before its first diffuse bounce (RenderCore_Optix7Filter/kernels/pathtracer.h:288-299) */
            const uint packedNormal = PackNormal2(N) + isSpecular;
            PackFeatures(feat, 0, packedNormal, HIT_T, isSpecular, 0);
            store4(wpos, I.x, I.y, I.z, bitsf(packedNormal));
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
        if (!(FLAGS & S_SPECULAR)) FLAGS |= S_BOUNCED; else FLAGS |= S_VIASPECULAR;
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

/* ------------------------------------------------------------------------------------------------------
 * SVGF, lib/CUDA/shared_kernel_code/finalize_shared.h:169-600, one pixel per call, in the kernels' order
 * ---------------------------------------------------------------------------------------------------- */
inline f4 ld4(const float* p) { return {p[0], p[1], p[2], p[3]}; }
inline f4 operator-(f4 a, f4 b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
inline float dot4(f4 a, f4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline f3 fmin3(float a, f3 b) { return mk3(fminr(a, b.x), fminr(a, b.y), fminr(a, b.z)); }
inline f3 fmin3(f3 a, float b) { return mk3(fminr(a.x, b), fminr(a.y, b), fminr(a.z, b)); }
inline f3 fmax3(float a, f3 b) { return mk3(fmaxr(a, b.x), fmaxr(a, b.y), fmaxr(a, b.z)); }
inline float clampf(float f, float a, float b) { return fmaxr(a, fminr(f, b)); }
inline f3 clamp3(f3 v, f3 a, f3 b) { return mk3(clampf(v.x, a.x, b.x), clampf(v.y, a.y, b.y), clampf(v.z, a.z, b.z)); }

inline float Luminance(const f3 rgb) { return 0.299f * fminr(rgb.x, 10.0f) + 0.587f * fminr(rgb.y, 10.0f) + 0.114f * fminr(rgb.z, 10.0f); }
inline f3 RGBToYCoCg(const f3 RGB) {
    const f3 rgb = fmin3(4.0f, RGB);
    const float Y = dot(rgb, mk3(1, 2, 1)) * 0.25f;
    const float Co = dot(rgb, mk3(2, 0, -2)) * 0.25f + (0.5f * 256.0f / 255.0f);
    const float Cg = dot(rgb, mk3(-1, 2, -1)) * 0.25f + (0.5f * 256.0f / 255.0f);
    return mk3(Y, Co, Cg);
}
inline f3 YCoCgToRGB(const f3 c) {
    const float Y = c.x, Co = c.y - (0.5f * 256.0f / 255.0f), Cg = c.z - (0.5f * 256.0f / 255.0f);
    return mk3(Y + Co - Cg, Y + Cg, Y - Co - Cg);
}
/* two non-negative rgb triples as 5:11 unsigned fixed point in the bits of one float4 */
inline void CombineToFloat4(const f3& A, const f3& B, float* out) {
    const uint Ar = f2u(fminr(A.x, 31.999f) * 2048.0f), Ag = f2u(fminr(A.y, 31.999f) * 2048.0f), Ab = f2u(fminr(A.z, 31.999f) * 2048.0f);
    const uint Br = f2u(fminr(B.x, 31.999f) * 2048.0f), Bg = f2u(fminr(B.y, 31.999f) * 2048.0f), Bb = f2u(fminr(B.z, 31.999f) * 2048.0f);
    out[0] = bitsf((Ar << 16) + Ag), out[1] = bitsf(Ab), out[2] = bitsf((Br << 16) + Bg), out[3] = bitsf(Bb);
}
inline f3 GetDirect(const float* X) {
    const uint v0 = fbits(X[0]), v1 = fbits(X[1]);
    return mk3((float)(v0 >> 16) * (1.0f / 2048.0f), (float)(v0 & 65535) * (1.0f / 2048.0f), (float)v1 * (1.0f / 2048.0f));
}
inline f3 GetIndirect(const float* X) {
    const uint v2 = fbits(X[2]), v3 = fbits(X[3]);
    return mk3((float)(v2 >> 16) * (1.0f / 2048.0f), (float)(v2 & 65535) * (1.0f / 2048.0f), (float)v3 * (1.0f / 2048.0f));
}
/* 2^-p for p in [0, 126] from the exponent bits (tools_shared.h:86) */
inline float oneoverpow2(const int p) { return bitsf((uint)(127 - p) << 23); }
/* x^128 by seven squarings; the reference calls powf(x, 128) */
inline float pow128(float x) { for (int i = 0; i < 7; i++) x = x * x; return x; }
inline float MitchellNetravali(const float v) {   /* sampling_shared.h:22-27, B = C = 1/3 */
    const float B = 1.0f / 3.0f, C = 1.0f / 3.0f, x = fabsf(v), x2 = x * x, x3 = x2 * x;
    if (x < 1) return (1.0f / 6.0f) * ((12 - 9 * B - 6 * C) * x3 + (-18 + 12 * B + 6 * C) * x2 + (6 - 2 * B));
    else if (x < 2) return 1.0f / 6.0f * ((-B - 6 * C) * x3 + (6 * B + 30 * C) * x2 + (-12 * B - 48 * C) * x + (8 * B + 24 * C));
    return 0.0f;
}

struct SvgfView { f4 prevPos, prevE, prevRight, prevUp; };
/* host part of prepareFilter (finalize_shared.h:293-314): the previous camera as a plane and two screen axes */
SvgfView svgf_view(const lh2g_view& v, int h) {
    const f3 pos = ld3(v.pos), p1 = ld3(v.p1), p2 = ld3(v.p2), p3 = ld3(v.p3);
    const f3 centre = 0.5f * (p2 + p3);
    const f3 direction = normalize(centre - pos);
    const f3 right = normalize(p2 - p1);
    const f3 up = normalize(p3 - p1);
    const float screenSize = length(p3 - p1);
    const float lenReci = (float)h / screenSize;
    SvgfView r;
    r.prevPos = mk4(pos.x, pos.y, pos.z, -(dot(pos, direction) - dot(centre, direction)));
    r.prevE = mk4(direction.x, direction.y, direction.z, 0);
    const f3 rr = right * lenReci, uu = up * lenReci;
    r.prevRight = mk4(rr.x, rr.y, rr.z, dot(p1, right) * lenReci);
    r.prevUp = mk4(uu.x, uu.y, uu.z, dot(p1, up) * lenReci);
    return r;
}

struct Svgf {
    int w, h;
    const lh2o_svgf* b;
    f4 world(const float* buf, int x, int y) const {   /* ReadWorldPos */
        if (x >= 0 && y >= 0 && x < w && y < h) return ld4(buf + 4 * ((size_t)x + (size_t)y * w));
        return mk4(1e20f, 1e20f, 1e20f, bitsf(0));
    }
    float WorldDistance(int px, int py, const f4& cur) const {
        const f4 p = world(b->prevWorldPos, px, py);
        const f3 localNormal = UnpackNormal2(fbits(cur.w)), prevNormal = UnpackNormal2(fbits(p.w));
        if ((fbits(p.w) & 3) != 1) return 1e21f;            /* only specular pixels are searched */
        if (dot(localNormal, prevNormal) < 0.85f) return 1e21f;
        return length(mk3(cur - p));
    }
    float FineWorldDistance(const f2 pixel, const f4& cur) const {
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
    int RefineHistoryPos(f2& pos, const f2 offset, const f4& cur, float& bestDist, const float step) const {
        int bestTap = 0;
        const f2 c0 = mk2(pos.x - step, pos.y), c1 = mk2(pos.x + step, pos.y), c2 = mk2(pos.x, pos.y - step), c3 = mk2(pos.x, pos.y + step);
        float d;
        d = FineWorldDistance(c0 + offset, cur); if (d < bestDist) bestDist = d, pos = c0, bestTap = 1;
        d = FineWorldDistance(c1 + offset, cur); if (d < bestDist) bestDist = d, pos = c1, bestTap = 2;
        d = FineWorldDistance(c2 + offset, cur); if (d < bestDist) bestDist = d, pos = c2, bestTap = 3;
        d = FineWorldDistance(c3 + offset, cur); if (d < bestDist) bestDist = d, pos = c3, bestTap = 4;
        return bestTap;
    }
    /* ReadTexelConsistent (sampling_shared.h:136-175): bilinear history read whose taps must agree in normal
     * (dot >= 0.95) and specularity with the pixel; out.x = -1 when no tap qualifies */
    f4 ReadConsistent(const float* buf, const f4& localPos, const f3& localNormal, float u, float v) const {
        const int iu1 = f2i(floorf(u)), iv1 = f2i(floorf(v)), iu0 = imax(0, iu1 - 1), iv0 = imax(0, iv1 - 1);
        if (iu1 >= w || iv1 >= h || iu1 < 0 || iv1 < 0) return mk4(-1, -1, -1, -1);
        const float fu = u - floorf(u), fv = v - floorf(v);
        const size_t a0 = (size_t)iu0 + (size_t)iv0 * w, a1 = (size_t)iu1 + (size_t)iv0 * w;
        const size_t a2 = (size_t)iu0 + (size_t)iv1 * w, a3 = (size_t)iu1 + (size_t)iv1 * w;
        const f4 p0 = ld4(buf + 4 * a0), p1 = ld4(buf + 4 * a1), p2 = ld4(buf + 4 * a2), p3 = ld4(buf + 4 * a3);
        const uint n0 = fbits(b->prevWorldPos[4 * a0 + 3]), n1 = fbits(b->prevWorldPos[4 * a1 + 3]);
        const uint n2 = fbits(b->prevWorldPos[4 * a2 + 3]), n3 = fbits(b->prevWorldPos[4 * a3 + 3]);
        const uint spec = fbits(localPos.w) & 3;
        float w0 = (1 - fu) * (1 - fv), w1 = fu * (1 - fv), w2 = (1 - fu) * fv, w3 = 1 - (w0 + w1 + w2);
        if (dot(UnpackNormal2(n0), localNormal) < 0.95f || (n0 & 3) != spec) w0 = 0;
        if (dot(UnpackNormal2(n1), localNormal) < 0.95f || (n1 & 3) != spec) w1 = 0;
        if (dot(UnpackNormal2(n2), localNormal) < 0.95f || (n2 & 3) != spec) w2 = 0;
        if (dot(UnpackNormal2(n3), localNormal) < 0.95f || (n3 & 3) != spec) w3 = 0;
        const float sum = w0 + w1 + w2 + w3;
        if (sum == 0) return mk4(-1, -1, -1, -1);
        return (w0 * p0 + w1 * p1 + w2 * p2 + w3 * p3) * (1.0f / sum);
    }
    /* ReadTexelConsistent2 (sampling_shared.h:177-220): the same for packed direct + indirect light, dot >= 0.975 */
    bool ReadConsistent2(const float* buf, const f4& localPos, const f3& localNormal, float u, float v, f3& direct, f3& indirect) const {
        const int iu1 = f2i(floorf(u)), iv1 = f2i(floorf(v)), iu0 = imax(0, iu1 - 1), iv0 = imax(0, iv1 - 1);
        if (iu1 >= w || iv1 >= h || iu1 < 0 || iv1 < 0) return false;
        const float fu = u - floorf(u), fv = v - floorf(v);
        const size_t a[4] = {(size_t)iu0 + (size_t)iv0 * w, (size_t)iu1 + (size_t)iv0 * w, (size_t)iu0 + (size_t)iv1 * w,
                             (size_t)iu1 + (size_t)iv1 * w};
        const uint spec = fbits(localPos.w) & 3;
        float wt[4];
        wt[0] = (1 - fu) * (1 - fv), wt[1] = fu * (1 - fv), wt[2] = (1 - fu) * fv, wt[3] = 1 - (wt[0] + wt[1] + wt[2]);
        for (int k = 0; k < 4; k++) {
            const uint n = fbits(b->prevWorldPos[4 * a[k] + 3]);
            if (dot(UnpackNormal2(n), localNormal) < 0.975f || (n & 3) != spec) wt[k] = 0;
        }
        const float sum = wt[0] + wt[1] + wt[2] + wt[3];
        if (sum == 0) return false;
        f3 d = wt[0] * GetDirect(buf + 4 * a[0]), in = wt[0] * GetIndirect(buf + 4 * a[0]);
        for (int k = 1; k < 4; k++) d = d + wt[k] * GetDirect(buf + 4 * a[k]), in = in + wt[k] * GetIndirect(buf + 4 * a[k]);
        direct = d * (1.0f / sum), indirect = in * (1.0f / sum);
        return true;
    }

    /* prepareFilterKernel (finalize_shared.h:217-291) */
    void prepare(int x, int y, const float* accum, const SvgfView& V, const lh2g_filter_params& fp, float scale) const {
        const size_t px = (size_t)x + (size_t)y * w, WH = (size_t)w * h;
        uint* feature = b->features + 4 * px;
        const f3 direct = mk3(ld4(accum + 4 * px)) * scale;
        const f4 localWorldPos = ld4(b->worldPos + 4 * px);
        const f3 albedo = RGB32toHDRmin1(feature[0]);
        const f3 indirect = mk3(ld4(accum + 4 * (px + WH))) * scale;
        const f3 reciAlbedo = mk3(1.0f / albedo.x, 1.0f / albedo.y, 1.0f / albedo.z);
        const f3 directLight = fmin3(direct * reciAlbedo, fp.clampDirect);
        const f3 indirectLight = fmin3(indirect * reciAlbedo, fp.clampIndirect);
        CombineToFloat4(directLight, indirectLight, b->shading + 4 * px);
        float lumDirect = Luminance(directLight), lumDirect2 = lumDirect * lumDirect;
        float lumIndirect = Luminance(indirectLight), lumIndirect2 = lumIndirect * lumIndirect;
        f2 prevPixelPos;
        if (((feature[3] >> 4) & 3) == 0) {
            /* diffuse: project the world position into the previous camera */
            const f3 dd = normalize(mk3(localWorldPos - V.prevPos));
            const f4 D = mk4(dd.x, dd.y, dd.z, 0);
            const f3 ss = mk3(V.prevPos) + mk3(D) * (V.prevPos.w / dot4(V.prevE, D));
            const f4 S = mk4(ss.x, ss.y, ss.z, 0);
            prevPixelPos = mk2(dot4(S, V.prevRight) - V.prevRight.w - fp.j0, dot4(S, V.prevUp) - V.prevUp.w - fp.j1);
        } else {
            prevPixelPos = mk2((float)x, (float)y);
            if (!fp.camIsStationary) {
                /* specular: diamond search for the position in the previous frame's world positions */
                float bestDist = length(mk3(localWorldPos - ld4(b->prevWorldPos + 4 * px))), stepSize = 5.0f;
                const f2 offset = mk2(fp.j0 - fp.prevj0, fp.j1 - fp.prevj1);
                int iter = 0;
                for (;;) {
                    const int tap = RefineHistoryPos(prevPixelPos, offset, localWorldPos, bestDist, stepSize);
                    if (tap == 0) { stepSize *= 0.45f; if (stepSize < 0.05f) break; }
                    if (++iter == 25) break;
                }
            }
        }
        prevPixelPos = prevPixelPos + mk2(0.5f, 0.5f);
        const float ppx = prevPixelPos.x, ppy = prevPixelPos.y;
        bool hit = false;
        if (ppx >= 0 && ppx < (float)w && ppy >= 0 && ppy < (float)h) {
            const f3 localNormal = UnpackNormal2(feature[1]);
            const f4 history = ReadConsistent(b->prevMoments, localWorldPos, localNormal, ppx, ppy);
            if (history.x > -1) {
                lumDirect = 0.2f * lumDirect + 0.8f * history.x;
                lumDirect2 = 0.2f * lumDirect2 + 0.8f * history.y;
                lumIndirect = 0.2f * lumIndirect + 0.8f * history.z;
                lumIndirect2 = 0.2f * lumIndirect2 + 0.8f * history.w;
                if ((feature[3] & 15) < 15) feature[3]++;
                hit = true;
            }
        }
        if (!hit) feature[3] &= 0xfffffff0u;   /* reset the history count */
        b->motion[2 * px] = prevPixelPos.x, b->motion[2 * px + 1] = prevPixelPos.y;
        store4(b->moments + 4 * px, lumDirect, lumDirect2, lumIndirect, lumIndirect2);
    }

    /* applyFilterKernel (finalize_shared.h:320-476): 5x5 a-trous (corners cut) at step 2^(phase-1) with normal,
     * depth, material and luminance stops; phase 1 blends with the clamped history, the last pass remodulates */
    void apply(int x, int y, const float* A, const float* B, float* C, int phase, bool lastPass) const {
        const size_t px = (size_t)x + (size_t)y * w;
        const uint* lf = b->features + 4 * px;
        const f4 localPos = ld4(b->worldPos + 4 * px);
        const f3 localNormal = UnpackNormal2(lf[1]);
        const f3 localColor = RGB32toHDR(lf[0]);
        const uint localMatID = lf[3] >> 4;
        float directWeightSum = 1, indirectWeightSum = 1;
        f3 directSum = directWeightSum * GetDirect(A + 4 * px);
        f3 indirectSum = indirectWeightSum * GetIndirect(A + 4 * px);
        const float localDirect = Luminance(GetDirect(A + 4 * px));
        const float localIndirect = Luminance(GetIndirect(A + 4 * px));
        const float localDepth = bitsf(lf[2]);
        const float localDdx = b->deltaDepth[4 * px + 2], localDdy = b->deltaDepth[4 * px + 3];
        const float sigma = 10.0f * oneoverpow2(phase - 1);
        const float factor = (lf[3] & 15) == 0 ? 400.0f : 1.0f;
        const f4 m = ld4(b->moments + 4 * px);
        const float var_dir = m.y - m.x * m.x, var_ind = m.w - m.z * m.z;
        const float rdir = -1.0f / (sigma * factor * sqrtf(var_dir + 0.00001f) + 0.00001f);
        const float rind = -1.0f / (sigma * factor * sqrtf(var_ind + 0.00001f) + 0.00001f);
        const int step = 1 << (phase - 1);
        for (int vv = -2; vv <= 2; vv++) {
            const int v = vv * step + y;
            const int r = (vv == 2 || vv == -2) ? 1 : 2;
            if (v < 0 || v >= h) continue;
            for (int uu = -r; uu <= r; uu++) {
                if (uu == 0 && vv == 0) continue;
                const int u = std::min(std::max(uu * step + x, 0), w - 1);
                const size_t q = (size_t)u + (size_t)v * w;
                const uint* nf = b->features + 4 * q;
                const float w_dist = (float)(uu * uu + vv * vv) * (-1.0f / 7.5f);
                const f3 nDirect = GetDirect(A + 4 * q), nIndirect = GetIndirect(A + 4 * q);
                float w_normal = pow128(fmaxr(0.0f, dot(UnpackNormal2(nf[1]), localNormal)));
                const float expected = localDepth + localDdx * (float)(uu * step) + localDdy * (float)(vv * step);
                const float depthError = fabsf(expected - bitsf(nf[2]));
                const float expectedDifference = fabsf(expected - localDepth);
                const float w_depth = depthError / fmaxr(0.00001f, (0.5f + (float)phase * 0.5f) * expectedDifference);
                /* the reference's ternary mixes the double literal 0.0001 with a float: the product is formed in double */
                if ((nf[3] >> 4) != localMatID) w_normal = (float)((double)w_normal * 0.0001);
                else w_normal = w_normal * dot(localColor, RGB32toHDR(nf[0]));
                float w_dir = w_normal * lm_expf(fabsf(localDirect - Luminance(nDirect)) * rdir + w_dist - w_depth);
                float w_ind = w_normal * lm_expf(fabsf(localIndirect - Luminance(nIndirect)) * rind + w_dist - w_depth);
                if (!std::isfinite(w_dir)) w_dir = 0;
                if (!std::isfinite(w_ind)) w_ind = 0;
                directSum = directSum + nDirect * w_dir, directWeightSum += w_dir;
                indirectSum = indirectSum + nIndirect * w_ind, indirectWeightSum += w_ind;
            }
        }
        f3 directFiltered = directSum * (1.0f / fmaxr(0.0001f, directWeightSum));
        f3 indirectFiltered = indirectSum * (1.0f / fmaxr(0.0001f, indirectWeightSum));
        if (phase == 1) {
            const float mx = b->motion[2 * px], my = b->motion[2 * px + 1];
            const int ix = f2i(mx), iy = f2i(my);
            f3 prevDirect, prevIndirect;
            if (ix >= 0 && ix < w && iy >= 0 && iy < h && ReadConsistent2(B, localPos, localNormal, mx, my, prevDirect, prevIndirect)) {
                /* neighbourhood clamp in YCoCg, +-0.75 sigma over the 3x3 block of the unfiltered input */
                prevDirect = RGBToYCoCg(prevDirect), prevIndirect = RGBToYCoCg(prevIndirect);
                f3 dirAvg = RGBToYCoCg(directFiltered), dirVar = dirAvg * dirAvg;
                f3 indAvg = RGBToYCoCg(indirectFiltered), indVar = indAvg * indAvg;
                auto add = [&](size_t q) {
                    const f3 f = RGBToYCoCg(GetDirect(A + 4 * q)), g = RGBToYCoCg(GetIndirect(A + 4 * q));
                    dirAvg = dirAvg + f, dirVar = dirVar + f * f, indAvg = indAvg + g, indVar = indVar + g * g;
                };
                if (x > 1) {
                    if (y > 1) add(px - w - 1);
                    add(px - 1);
                    if (y < h - 1) add(px + w - 1);
                }
                if (y > 1) add(px - w);
                if (y < h - 1) add(px + w);
                if (x < w - 1) {
                    if (y > 1) add(px + 1 - w);
                    add(px + 1);
                    if (y < h - 1) add(px + 1 + w);
                }
                dirAvg = dirAvg * (1.0f / 9.0f), dirVar = dirVar * (1.0f / 9.0f), indAvg = indAvg * (1.0f / 9.0f), indVar = indVar * (1.0f / 9.0f);
                f3 sd = fmax3(0.0f, dirVar - dirAvg * dirAvg), si = fmax3(0.0f, indVar - indAvg * indAvg);
                sd = mk3(sqrtf(sd.x), sqrtf(sd.y), sqrtf(sd.z)), si = mk3(sqrtf(si.x), sqrtf(si.y), sqrtf(si.z));
                prevDirect = clamp3(prevDirect, dirAvg - 0.75f * sd, dirAvg + 0.75f * sd);
                prevIndirect = clamp3(prevIndirect, indAvg - 0.75f * si, indAvg + 0.75f * si);
                directFiltered = directFiltered * 0.1f + YCoCgToRGB(prevDirect) * 0.9f;
                indirectFiltered = indirectFiltered * 0.1f + YCoCgToRGB(prevIndirect) * 0.9f;
            }
        }
        if (lastPass) {
            const f3 c = (directFiltered + indirectFiltered) * RGB32toHDR(lf[0]);
            store4(C + 4 * px, sqrtf(c.x), sqrtf(c.y), sqrtf(c.z), 1);
        } else {
            CombineToFloat4(directFiltered, indirectFiltered, C + 4 * px);
        }
    }

    /* TAApassKernel (finalize_shared.h:498-539); reads 'pixels', writes 'out' */
    void taa(int x, int y, const float* pixels, const float* prev, float* out) const {
        const size_t px = (size_t)x + (size_t)y * w;
        f3 pixel = mk3(ld4(pixels + 4 * px));
        const float ppx = b->motion[2 * px] - 0.5f, ppy = b->motion[2 * px + 1] - 0.5f;
        if (ppx >= 0 && ppx < (float)w && ppy >= 0 && ppy < (float)h) {
            const f3 newPixel = RGBToYCoCg(pixel);
            /* ReadTexelBmitchellNetravali (sampling_shared.h:117-134) */
            const int x1 = f2i(ppx - 2.0f), y1 = f2i(ppy - 2.0f);
            float totalWeight = 0;
            f4 total = mk4(0, 0, 0, 0);
            for (int yy = y1; yy < y1 + 4; yy++)
                for (int xx = x1; xx < x1 + 4; xx++)
                    if (xx >= 0 && yy > 0 && xx < w && yy < h) {
                        const float weight = MitchellNetravali((float)xx - ppx) * MitchellNetravali((float)yy - ppy);
                        total = total + ld4(prev + 4 * ((size_t)xx + (size_t)yy * w)) * weight;
                        totalWeight += weight;
                    }
            f3 history = RGBToYCoCg(mk3(total * (1.0f / totalWeight)));
            f3 colorAvg = newPixel, colorVar = newPixel * newPixel;
            auto add = [&](size_t q) { const f3 f = RGBToYCoCg(mk3(ld4(pixels + 4 * q))); colorAvg = colorAvg + f, colorVar = colorVar + f * f; };
            if (x > 1) {
                if (y > 1) add(px - w - 1);
                add(px - 1);
                if (y < h - 1) add(px + w - 1);
            }
            if (y > 1) add(px - w);
            if (y < h - 1) add(px + w);
            if (x < w - 1) {
                if (y > 1) add(px + 1 - w);
                add(px + 1);
                if (y < h - 1) add(px + 1 + w);
            }
            colorAvg = colorAvg * (1.0f / 9.0f), colorVar = colorVar * (1.0f / 9.0f);
            f3 sigma = fmax3(0.0f, colorVar - colorAvg * colorAvg);
            sigma = mk3(sqrtf(sigma.x), sqrtf(sigma.y), sqrtf(sigma.z));
            history = clamp3(history, colorAvg - 1.25f * sigma, colorAvg + 1.25f * sigma);
            pixel = YCoCgToRGB(newPixel * 0.1f + history * 0.9f);
            if (std::isnan(pixel.x + pixel.y + pixel.z)) pixel = YCoCgToRGB(newPixel);
        }
        const f3 c = fmin3(10.0f, pixel);
        store4(out + 4 * px, c.x, c.y, c.z, 0);
    }
    /* unsharpenTAAKernel (finalize_shared.h:553-576): sharpen, then square (the gamma is applied again later) */
    void unsharpen(int x, int y, const float* pixels, float* target) const {
        if (x == 0 || y == 0 || x >= w - 1 || y >= h - 1) return;
        auto P = [&](int xx, int yy) { return ld4(pixels + 4 * ((size_t)xx + (size_t)yy * w)); };
        const f4 p0 = P(x - 1, y - 1), p1 = P(x, y - 1), p2 = P(x + 1, y - 1), p3 = P(x + 1, y);
        const f4 p4 = P(x + 1, y + 1), p5 = P(x, y + 1), p6 = P(x - 1, y + 1), p7 = P(x - 1, y);
        const f4 c = P(x, y);
        const f4 blur = 0.35f * p0 + 0.5f * p1 + 0.35f * p2 + 0.5f * p3 + 0.35f * p4 + 0.5f * p5 + 0.35f * p6 + 0.5f * p7;
        const f4 sharp = c * 2.7f - 0.5f * blur;
        const f4 pixel = mk4(fmaxr(c.x, sharp.x), fmaxr(c.y, sharp.y), fmaxr(c.z, sharp.z), fmaxr(c.w, sharp.w));
        store4(target + 4 * ((size_t)x + (size_t)y * w), pixel.x * pixel.x, pixel.y * pixel.y, pixel.z * pixel.z, 0);
    }
    /* finalizeNoTAAKernel (finalize_shared.h:587-595) */
    void finalize_no_taa(int x, int y, const float* pixels, float* target) const {
        if (x == 0 || y == 0 || x >= w - 1 || y >= h - 1) return;
        const f4 p = ld4(pixels + 4 * ((size_t)x + (size_t)y * w));
        store4(target + 4 * ((size_t)x + (size_t)y * w), sqrtf(p.x), sqrtf(p.y), sqrtf(p.z), 0);
    }
};

/* ------------------------------------------------------------------------------------------------------
 * radiance cache (no reference counterpart): the encoding, the network and its gradients with the rounding
 * points of the GPU kernels - fp16 grid features, bf16 weights, activations and loss gradients - and sums in
 * double; and one Adam step
 * ---------------------------------------------------------------------------------------------------- */
constexpr int NRC_IN = 64, NRC_HID = 64, NRC_LEVELS = 12, NRC_T = 1 << 19;
inline float bf16r(float x) {   /* round to bfloat16, nearest even */
    uint b = fbits(x);
    if ((b & 0x7f800000u) == 0x7f800000u) return x;
    b = (b + 0x7fffu + ((b >> 16) & 1u)) & 0xffff0000u;
    return bitsf(b);
}
inline float f16r(float x) { return half2float(float2half(x)); }
inline void one_blob4(float x, float* out) {
    for (int i = 0; i < 4; i++) out[i] = fmaxr(0.0f, 1.0f - fabsf(x * 4.0f - ((float)i + 0.5f)));
}
inline void sph01(f3 d, float& th, float& ph) {
    th = lm_acosf(fminr(fmaxr(d.z, -1.0f), 1.0f)) * INVPI;
    ph = lm_atan2f(d.y, d.x) * INV2PI + 0.5f;
}
struct NrcCell { uint i, j, k; float fx, fy, fz; };
inline f3 nrc_unit(const lh2o_nrc_spec& S, const float* q) {
    float u[3];
    for (int a = 0; a < 3; a++) u[a] = fminr(fmaxr((q[a] - S.bmin[a]) * S.inv[a], 0.0f), 1.0f);
    return mk3(u[0], u[1], u[2]);
}
inline NrcCell nrc_cell(const lh2o_nrc_spec& S, int l, f3 p) {
    const float r = (float)S.res[l];
    const float x = p.x * r, y = p.y * r, z = p.z * r;
    NrcCell c;
    c.i = (uint)imin(f2i(floorf(x)), S.res[l] - 1), c.j = (uint)imin(f2i(floorf(y)), S.res[l] - 1), c.k = (uint)imin(f2i(floorf(z)), S.res[l] - 1);
    c.fx = x - (float)c.i, c.fy = y - (float)c.j, c.fz = z - (float)c.k;
    return c;
}
inline uint nrc_index(const lh2o_nrc_spec& S, int l, uint x, uint y, uint z) {
    if (S.dense[l]) {
        const uint r1 = (uint)S.res[l] + 1u;
        return x + r1 * (y + r1 * z);
    }
    return ((x * 1u) ^ (y * 2654435761u) ^ (z * 805459861u)) & (uint)(NRC_T - 1);
}
inline float nrc_weight(const NrcCell& c, int corner) {
    return ((corner & 1) ? c.fx : 1.0f - c.fx) * ((corner & 2) ? c.fy : 1.0f - c.fy) * ((corner & 4) ? c.fz : 1.0f - c.fz);
}
void nrc_encode(const lh2o_nrc_spec& S, const float* grid, const float* q, float* e, bool emulate = true) {
    const f3 p = nrc_unit(S, q);
    for (int l = 0; l < NRC_LEVELS; l++) {
        const NrcCell c = nrc_cell(S, l, p);
        float f0 = 0.0f, f1 = 0.0f;
        for (int corner = 0; corner < 8; corner++) {
            const uint idx = nrc_index(S, l, c.i + (corner & 1), c.j + ((corner >> 1) & 1), c.k + (corner >> 2));
            const size_t at = ((size_t)l * NRC_T + idx) * 2;
            const float w = nrc_weight(c, corner);
            const float g0 = emulate ? f16r(grid[at]) : grid[at], g1 = emulate ? f16r(grid[at + 1]) : grid[at + 1];
            f0 = f0 + w * g0, f1 = f1 + w * g1;
        }
        e[2 * l] = f0, e[2 * l + 1] = f1;
    }
    float th, ph;
    sph01(mk3(q[4], q[5], q[6]), th, ph);
    one_blob4(th, e + 24), one_blob4(ph, e + 28);
    sph01(mk3(q[8], q[9], q[10]), th, ph);
    one_blob4(th, e + 32), one_blob4(ph, e + 36);
    one_blob4(fminr(fmaxr(q[3], 0.0f), 1.0f), e + 40);
    e[44] = q[12], e[45] = q[13], e[46] = q[14], e[47] = 1.0f;
    for (int i = 48; i < NRC_IN; i++) e[i] = 0.0f;
}
/* forward of one sample: act[0..4] (bf16 values when emulating), y[3] */
void nrc_forward1(const float* mlp, const float* e, float act[5][64], double* y, bool emulate) {
    for (int k = 0; k < NRC_IN; k++) act[0][k] = emulate ? bf16r(e[k]) : e[k];
    for (int j = 0; j < 5; j++) {
        const int rows = j < 4 ? NRC_HID : 3;
        const float* W = mlp + (size_t)j * NRC_HID * NRC_IN;
        for (int n = 0; n < rows; n++) {
            double z = 0.0;
            for (int k = 0; k < NRC_IN; k++) z += (double)act[j][k] * (double)(emulate ? bf16r(W[n * NRC_IN + k]) : W[n * NRC_IN + k]);
            if (j < 4) act[j + 1][n] = emulate ? bf16r(fmaxr((float)z, 0.0f)) : (float)std::max(z, 0.0);
            else y[n] = emulate ? (double)(float)z : z;
        }
    }
}


/* ------------------------------------------------------------------------------------------------------
 * The OptiX 7 core's estimator (lib/rendercore_optix7/kernels/pathtracer.h:54-238, ray generation of
 * optix/.optix.cu:71-129) and the PrimeAdaptive core's variant of it (lib/RenderCore_PrimeAdaptive/kernels/
 * pathtracer.h:52-238, camera.h:39-139), both with the Lambert BSDF of lib/sharedBSDFs/lambert.h (the alternative
 * their kernels/bsdf.h offers). Run per path depth first: every random number depends on (path, depth) only.
 * ---------------------------------------------------------------------------------------------------- */
constexpr uint S_BOUNCEDTWICE = 8;                   /* rendercore_optix7/kernels/pathtracer.h:31 */
constexpr int MIS_OPTIX7 = 1, MIS_ADAPTIVE = 2;

/* RayTarget, lib/RenderSystem/common_functions.h:29-50 (atan2f, sinf, cosf by the oracle's own functions) */
inline f3 RayTarget(const int sx, const int sy, const float r0, const float r1, const int W, const int H, const float distortion,
                    const f3 p1, const f3 right, const f3 up) {
    if (distortion == 0) {
        const float u = ((float)sx + r0) * (1.0f / W);
        const float v = ((float)sy + r1) * (1.0f / H);
        return p1 + u * right + v * up;
    }
    const float tx = sx / (float)W - 0.5f, ty = sy / (float)H - 0.5f;
    const float rr = tx * tx + ty * ty;
    const float rq = sqrtf(rr) * (1.0f + distortion * rr + distortion * rr * rr);
    const float theta = lm_atan2f(tx, ty);
    float st, ct;
    lm_sincos(theta, &st, &ct);
    const float bx = (st * rq + 0.5f) * W;
    const float by = (ct * rq + 0.5f) * H;
    return p1 + (bx + r0) * (right / (float)W) + (by + r1) * (up / (float)H);
}

/* RandomPointOnLens, optix/.optix.cu:71-83 and RenderCore_PrimeAdaptive/kernels/camera.h:22-33 */
inline f3 RandomPointOnLens(const float r0, float r1, const f3 pos, const float aperture, const f3 right, const f3 up) {
    const float blade = (float)f2i(r0 * 9);
    float r2 = (r0 - blade * (1.0f / 9.0f)) * 9.0f;
    float x1, y1, x2, y2;
    lm_sincos(blade * PI / 4.5f, &x1, &y1);
    lm_sincos((blade + 1.0f) * PI / 4.5f, &x2, &y2);
    if ((r1 + r2) > 1) r1 = 1.0f - r1, r2 = 1.0f - r2;
    const float xr = x1 * r1 + x2 * r2;
    const float yr = y1 * r1 + y2 * r2;
    return pos + aperture * (right * xr + up * yr);
}

/* blueNoiseSampler4, lib/CUDA/shared_kernel_code/tools_shared.h:324-337 */
inline f4 blueNoiseSampler4(const uint* bn, int x, int y, int sampleIndex, int sampleDimension) {
    const uint* r = bn + sampleDimension + (x + y * 128) * 8 + 65536 * 3;
    const int rsi1 = (sampleIndex ^ (int)r[0]) & 255, rsi2 = (sampleIndex ^ (int)r[1]) & 255;
    const int rsi3 = (sampleIndex ^ (int)r[2]) & 255, rsi4 = (sampleIndex ^ (int)r[3]) & 255;
    const int v1 = (int)bn[sampleDimension + 0 + rsi1 * 256];
    const int v2 = (int)bn[sampleDimension + 1 + rsi2 * 256];
    const int v3 = (int)bn[sampleDimension + 2 + rsi3 * 256];
    const int v4 = (int)bn[sampleDimension + 3 + rsi4 * 256];
    const uint* b = bn + (sampleDimension & 7) + (x + y * 128) * 8 + 65536;
    return mk4((0.5f + (float)(v1 ^ (int)b[0])) * (1.0f / 256.0f), (0.5f + (float)(v2 ^ (int)b[1])) * (1.0f / 256.0f),
               (0.5f + (float)(v3 ^ (int)b[2])) * (1.0f / 256.0f), (0.5f + (float)(v4 ^ (int)b[3])) * (1.0f / 256.0f));
}

/* SampleSmallSkydome, tools_shared.h:204-211, on the 64x scaled-down sky */
f3 SampleSmallSkydome(const lh2o_scene* s, const f3& Dw) {
    const uint w = (uint)s->sky.w >> 6, h = (uint)s->sky.h >> 6;
    if (w == 0 || h == 0) return mk3(0);
    const float* m = s->sky.m;
    const f3 D = -mk3(m[0] * Dw.x + m[1] * Dw.y + m[2] * Dw.z, m[4] * Dw.x + m[5] * Dw.y + m[6] * Dw.z, m[8] * Dw.x + m[9] * Dw.y + m[10] * Dw.z);
    float p = lm_atan2f(D.y, D.x);
    p = (p < 0) ? (p + 2 * PI) : p;
    const float theta = lm_acosf(D.z < -1.f ? -1.f : (D.z > 1.f ? 1.f : D.z));
    const uint u = f2u((float)w * p * INV2PI - 0.5f);
    const uint v = f2u((float)h * theta * INVPI - 0.5f);
    const uint idx = u + v * w;
    return idx < w * h ? s->sky.small[idx] : mk3(0);
}

/* CalculateLightPDF and LightPickProb, lights_shared.h:111-117, 158-177 */
inline float CalculateLightPDF(const f3& D, const float t, const float lightArea, const f3 lightNormal) {
    return (t * t) / (fabsf(dot(D, lightNormal)) * lightArea);
}
float LightPickProb(const lh2o_scene* s, int idx, const f3& O, const f3& N, const f3& I) {
    float potential[64];
    float sum = 0;
    int lights = 0;
    for (size_t i = 0; i < s->triLights.size(); i++) { const float c = PotentialTriLightContribution(s, (int)i, O, N, I, mk3(-1)); potential[lights++] = c; sum += c; }
    for (size_t i = 0; i < s->pointLights.size(); i++) { const float c = PotentialPointLightContribution(s, (int)i, O, N); potential[lights++] = c; sum += c; }
    for (size_t i = 0; i < s->spotLights.size(); i++) { const float c = PotentialSpotLightContribution(s, (int)i, O, N); potential[lights++] = c; sum += c; }
    for (size_t i = 0; i < s->dirLights.size(); i++) { const float c = PotentialDirectionalLightContribution(s, (int)i, O, N); potential[lights++] = c; sum += c; }
    if (sum <= 0) return 0;
    return (idx >= 0 && idx < lights) ? potential[idx] / sum : 0.0f;
}

/* ------------------------------------------------------------------------------------------------------
 * the stochastic-lightcuts light tree (LH2G_RP_LIGHTTREE)
 * build: RenderCore::UpdateLightTree / FindBestMatch / UpdateLightTreeNormals, rendercore_optix7/rendercore.cpp:571-680,
 *   with the LightCluster constructors and Cost of common_classes.h:487-514; a leaf box starts empty (the
 *   reference grows a box nothing initialised);
 * use: CalculateChildNodeWeights, LightPickProbLTree, RandomPointOnLightLTree, lights_shared.h:120-156, 198-217,
 *   322-395 (the three point draws of a child box in x, y, z order, as the CUDA compiler evaluates make_float3's
 *   arguments); a parentless leaf (a one-light tree) ends LightPickProbLTree's walk.
 * ---------------------------------------------------------------------------------------------------- */

static LtCluster lt_cluster(int light, float intensity) {
    LtCluster c;
    c.light = light, c.left = -1, c.right = -1, c.intensity = intensity;
    for (int k = 0; k < 4; k++) c.bmin[k] = 1e34f, c.bmax[k] = -1e34f;   /* aabb::Reset */
    c.N[0] = c.N[1] = c.N[2] = 0, c.parent = -1;
    return c;
}
/* aabb::Grow: _mm_min_ps(bmin, p) / _mm_max_ps(bmax, p), lane by lane, p's w 0 */
static void lt_grow(LtCluster& c, const float* lo, const float* hi) {
    for (int k = 0; k < 4; k++) {
        c.bmin[k] = c.bmin[k] < lo[k] ? c.bmin[k] : lo[k];
        c.bmax[k] = c.bmax[k] > hi[k] ? c.bmax[k] : hi[k];
    }
}
static void lt_grow_p(LtCluster& c, float x, float y, float z) { const float p[4] = {x, y, z, 0}; lt_grow(c, p, p); }
static float lt_cost(const LtCluster& c) {
    const f3 d = mk3(c.bmax[0] - c.bmin[0], c.bmax[1] - c.bmin[1], c.bmax[2] - c.bmin[2]);
    return c.intensity * dot(d, d);
}
static int lt_find_best_match(const std::vector<LtCluster>& t, const int* todo, int idx, int n) {
    float bestCost = 1e34f;
    int bestIdx = 0;
    for (int i = 0; i < n; i++)
        if (i != idx) {
            LtCluster tmp = t[todo[idx]];
            lt_grow(tmp, t[todo[i]].bmin, t[todo[i]].bmax);
            tmp.intensity += t[todo[i]].intensity;
            const float cost = lt_cost(tmp);
            if (cost < bestCost) bestCost = cost, bestIdx = i;
        }
    return bestIdx;
}
static void lt_normals(std::vector<LtCluster>& t, const lh2o_scene* s, int node) {
    LtCluster& c = t[node];
    if (c.left > -1) {
        lt_normals(t, s, c.left);
        lt_normals(t, s, c.right);
        const f3 Nl = ld3(t[c.left].N), Nr = ld3(t[c.right].N);
        const f3 n = dot(Nl, Nr) > 0.9f ? normalize(Nl + Nr) : mk3(0);
        c.N[0] = n.x, c.N[1] = n.y, c.N[2] = n.z;
        t[c.left].parent = t[c.right].parent = node;
    } else if (c.light & ((1 << 30) + (1 << 29))) {
        c.N[0] = c.N[1] = c.N[2] = 0;
    } else {
        memcpy(c.N, s->triLights[c.light].N, sizeof c.N);
    }
}
static std::vector<LtCluster> lt_build(const lh2o_scene* s) {
    const int Nt = (int)s->triLights.size(), M = (int)s->pointLights.size(), O = (int)s->spotLights.size();
    std::vector<LtCluster> t((size_t)(Nt + M + O) * 2, lt_cluster(-1, 0));
    if (Nt + M + O == 0) return t;
    std::vector<int> todo((size_t)(Nt + M + O));
    for (int i = 0; i < Nt; i++) {
        const lh2g_light_tri& l = s->triLights[i];
        LtCluster c = lt_cluster(i, l.energy);
        lt_grow_p(c, l.vertex0[0], l.vertex0[1], l.vertex0[2]);
        lt_grow_p(c, l.vertex1[0], l.vertex1[1], l.vertex1[2]);
        lt_grow_p(c, l.vertex2[0], l.vertex2[1], l.vertex2[2]);
        t[i + 1] = c, todo[i] = i + 1;
    }
    for (int i = 0; i < M; i++) {
        const float* p = s->pointLights[i].position;
        LtCluster c = lt_cluster(i | (1 << 30), s->pointLights[i].energy);
        lt_grow_p(c, p[0] - 0.001f, p[1] - 0.001f, p[2] - 0.001f);
        lt_grow_p(c, p[0] + 0.001f, p[1] + 0.001f, p[2] + 0.001f);
        t[i + 1 + Nt] = c, todo[i + Nt] = i + 1 + Nt;
    }
    for (int i = 0; i < O; i++) {
        const lh2g_spot_light& l = s->spotLights[i];
        LtCluster c = lt_cluster(i | (1 << 29), l.radiance[0] + l.radiance[1] + l.radiance[2]);
        lt_grow_p(c, l.position[0] - 0.001f, l.position[1] - 0.001f, l.position[2] - 0.001f);
        lt_grow_p(c, l.position[0] + 0.001f, l.position[1] + 0.001f, l.position[2] + 0.001f);
        t[i + 1 + Nt + M] = c, todo[i + Nt + M] = i + 1 + Nt + M;
    }
    int remaining = Nt + M + O, N = Nt + M + O;
    int A = 0, B = lt_find_best_match(t, todo.data(), A, remaining);
    while (remaining > 1) {
        const int C = lt_find_best_match(t, todo.data(), B, remaining);
        if (A == C) {
            t[N + 1] = t[todo[A]];
            lt_grow(t[N + 1], t[todo[B]].bmin, t[todo[B]].bmax);
            t[N + 1].intensity += t[todo[B]].intensity;
            t[N + 1].left = todo[A], t[N + 1].right = todo[B];
            for (int i = A; i < remaining - 1; i++) todo[i] = todo[i + 1];
            if (B > A) B--;
            for (int i = B; i < remaining - 2; i++) todo[i] = todo[i + 1];
            remaining -= 2;
            todo[remaining] = ++N;
            A = remaining++;
            B = lt_find_best_match(t, todo.data(), A, remaining);
        } else {
            A = B, B = C;
        }
    }
    t[0] = t[todo[0]];
    lt_normals(t, s, 0);
    return t;
}

static f3 lt_min3(const LtCluster& c) { return mk3(c.bmin[0], c.bmin[1], c.bmin[2]); }
static f3 lt_max3(const LtCluster& c) { return mk3(c.bmax[0], c.bmax[1], c.bmax[2]); }
float CalculateChildNodeWeights(const std::vector<LtCluster>& tree, const int node, const f3& I, const f3& N, uint& seed) {
    const int left = tree[node].left, right = tree[node].right;
    const f3 b1j = lt_min3(tree[left]), b1k = lt_min3(tree[right]);
    const f3 b2j = lt_max3(tree[left]), b2k = lt_max3(tree[right]);
    const f3 diag_j = b2j - b1j, diag_k = b2k - b1k;
    const f3 LN = ld3(tree[node].N);
    const f3 Bj = 0.5f * diag_j, Bk = 0.5f * diag_k;
    const f3 Cj = (b1j + b2j) * 0.5f, Ck = (b1k + b2k) * 0.5f;
    const f3 Dj = Cj - I, Dk = Ck - I;
    const f3 min_j = mk3(fmaxr(Dj.x - Bj.x, 0.0f), fmaxr(Dj.y - Bj.y, 0.0f), fmaxr(Dj.z - Bj.z, 0.0f));
    const f3 min_k = mk3(fmaxr(Dk.x - Bk.x, 0.0f), fmaxr(Dk.y - Bk.y, 0.0f), fmaxr(Dk.z - Bk.z, 0.0f));
    const float dist2j = dot(min_j, min_j), dist2k = dot(min_k, min_k);
    const f3 max_j = Dj + Bj, max_k = Dk + Bk;
    const float dist2j_max = dot(max_j, max_j), dist2k_max = dot(max_k, max_k);
    const float Ij = tree[left].intensity, Ik = tree[right].intensity;
    const float a0 = RandomFloat(seed), a1 = RandomFloat(seed), a2 = RandomFloat(seed);
    const f3 Rj = b1j + (b2j - b1j) * mk3(a0, a1, a2);
    const float c0 = RandomFloat(seed), c1 = RandomFloat(seed), c2 = RandomFloat(seed);
    const f3 Rk = b1k + (b2k - b1k) * mk3(c0, c1, c2);
    const f3 Lj = normalize(Rj - I), Lk = normalize(Rk - I);
    float Fj = fmaxr(0.001f, dot(N, Lj)), Fk = fmaxr(0.001f, dot(N, Lk));
    if (dot(LN, LN) > 0.001f) Fj *= fmaxr(0.001f, dot(LN, Lj * -1.0f)), Fk *= fmaxr(0.001f, dot(LN, Lk * -1.0f));
    const bool insideBoth = dist2j == 0 && dist2k == 0;
    const float wmin_j = (Fj * Ij) / (insideBoth ? 1.0f : fmaxr(0.0001f, dist2j));
    const float wmin_k = (Fk * Ik) / (insideBoth ? 1.0f : fmaxr(0.0001f, dist2k));
    const float wmax_j = (Fj * Ij) / fmaxr(0.0001f, dist2j_max);
    const float wmax_k = (Fj * Ij) / fmaxr(0.0001f, dist2k_max);   /* sic: the left child's F and I */
    const float pmin_j = wmin_j / (wmin_j + wmin_k);
    const float pmax_j = wmax_j / (wmax_j + wmax_k);
    return 0.5f * (pmin_j + pmax_j);
}
float LightPickProbLTree(const std::vector<LtCluster>& tree, int idx, const f3& N, const f3& I, uint& seed) {
    int node = idx + 1;
    float pickProb = 1;
    while (node != 0) {
        const int parent = tree[node].parent;
        if (parent < 0) break;
        const float p = CalculateChildNodeWeights(tree, parent, I, N, seed);
        if (tree[parent].left == node) pickProb *= p; else pickProb *= 1 - p;
        node = parent;
    }
    return pickProb;
}
f3 RandomPointOnLightLTree(const lh2o_scene* s, const std::vector<LtCluster>& tree, float r0, float r1, uint& seed, const f3& I, const f3& N,
                           float& pickProb, float& lightPdf, f3& lightColor) {
    pickProb = 1;
    if (tree.empty()) { lightPdf = 0; return mk3(1); }
    int node = 0, lightIdx = 0;
    while (true) {
        if (tree[node].left == -1) { lightIdx = tree[node].light; break; }
        const float p_j = CalculateChildNodeWeights(tree, node, I, N, seed);
        if (r1 < p_j) node = tree[node].left, r1 *= 1.0f / p_j, pickProb *= p_j;
        else node = tree[node].right, r1 = (r1 - p_j) / (1 - p_j), pickProb *= 1 - p_j;
    }
    if (lightIdx & (1 << 30)) {
        const lh2g_point_light& l = s->pointLights[lightIdx - (1 << 30)];
        const f3 P = ld3(l.position);
        const f3 L = P - I;
        const float sqDist = dot(L, L);
        lightColor = ld3(l.radiance) / sqDist;
        lightPdf = dot(L, N) > 0 ? 1.0f : 0.0f;
        return P;
    } else if (lightIdx & (1 << 29)) {
        const lh2g_spot_light& l = s->spotLights[lightIdx - (1 << 29)];
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
        const f3 bary = RandomBarycentrics(r0);
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
    }
}

inline void add4(float* a, const f4& v) { a[0] += v.x, a[1] += v.y, a[2] += v.z, a[3] += v.w; }

/* CLAMPINTENSITY (core_settings.h:191-194) and FIXNAN_FLOAT3 (common_settings.h:66) */
inline void clamp_intensity(f3& c, const float clampValue) {
    const float v = fmaxr(c.x, fmaxr(c.y, c.z));
    if (v > clampValue) { const float m = clampValue / v; c.x *= m, c.y *= m, c.z *= m; }
}
inline void fix_nan(f3& a) { if (!std::isfinite(a.x + a.y + a.z)) a = mk3(0); }

/* Radiance of one path of these estimators, summed in the order the path produces it: per path length its sky or
 * emitter term, then the contribution of its light connection when that is unoccluded. (The reference adds the
 * connections to the pixel after the wave loop, and the paths of a pixel race on it; the order here is fixed, and
 * the sums agree with the reference's within float rounding.) w: the connections' count (OptiX 7) or the sample
 * count (PrimeAdaptive). */
struct MisPath { f4 acc; };

/* pathIdx: the path as the shading sees it (pixel + layer * W*H); pass: the 'pass' of the shading kernel;
 * R0(d) is the shading seed of path length d; O, D, tmin: the primary ray. feat (PrimeAdaptive, may be null):
 * this path's float4 feature (albedo, packed normal). capIdx: the path's slot in capture arrays (-1: none). */
template <typename R0Fn>
void trace_path_mis(const Frame& F, const int flavor, const uint pathIdx, const uint pass, const R0Fn& R0, f3 O, f3 D, float tmin,
                    MisPath& out, std::vector<uint>& ext, std::vector<uint>& shad, lh2g_capture* cap, long long capIdx, float* feat) {
    const lh2o_scene* s = F.s;
    const lh2g_render_params& p = F.p;
    const int W = p.width, H = p.height;
    const float eps = p.geometryEpsilon;
    const bool nee = (p.flags & LH2G_RP_NEE) != 0;
    const uint* bn = s->blueNoise.empty() ? nullptr : s->blueNoise.data();
    out.acc = mk4(0, 0, 0, flavor == MIS_ADAPTIVE ? 1.0f : 0.0f);   /* accumulator[pathIdx].w += 1 at path length 1 */
    f3 throughput = mk3(1);
    float bsdfPdf = 1;
    uint FLAGS = S_SPECULAR, packedNormal = 0;
    const uint sampleIdx = pathIdx / ((uint)W * (uint)H) + pass;
    for (int pathLength = 1; pathLength <= p.maxDepth; pathLength++) {
        HitRec h;
        trace_scene(s, O, D, tmin, 1e34f, false, false, h);
        const lh2g_hit hit = make_hit(h);
        const long long ci = capIdx < 0 ? -1 : (long long)(pathLength - 1) * F.P + capIdx;
        if (cap && cap->hits && ci >= 0) cap->hits[ci] = hit;
        auto capSeed = [&](uint v) { if (cap && cap->seeds && ci >= 0) cap->seeds[ci] = v; };
        const bool firstHitToBeStored = feat && (FLAGS & S_BOUNCED) == 0;
        if (hit.prim == NOHIT) {
            const f3 skyPixel = (FLAGS & S_BOUNCED) ? SampleSmallSkydome(s, D) : SampleSkydome(s, D);
            f3 contribution = throughput * skyPixel * (1.0f / bsdfPdf);
            clamp_intensity(contribution, p.clampValue);
            fix_nan(contribution);
            out.acc.x += contribution.x, out.acc.y += contribution.y, out.acc.z += contribution.z;
            if (firstHitToBeStored) store4(feat, contribution.x, contribution.y, contribution.z, bitsf(PackNormal2(D * -1.0f)));
            capSeed(0);
            return;
        }
        const float HIT_U = (float)(hit.bary & 65535u) * (1.0f / 65535.0f);
        const float HIT_V = (float)(hit.bary >> 16) * (1.0f / 65535.0f);
        const float HIT_T = hit.t;
        const lh2g_core_tri& tri = s->meshes[s->inst[hit.inst].mesh].tris[hit.prim];
        ShadingData sd;
        f3 N, iN, fN, T;
        const f3 I = O + HIT_T * D;
        const bool disney = (p.flags & LH2G_RP_DISNEY) != 0;   /* kernels/bsdf.h's default branch */
        GetShadingData(s, D, HIT_U, HIT_V, F.view.spreadAngle * HIT_T, tri, hit.inst, sd, N, iN, fN, T, disney);
        if (firstHitToBeStored) store4(feat, sd.color.x, sd.color.y, sd.color.z, bitsf(PackNormal2(iN)));
        if (sd.flags & 1) {   /* alpha: the ray continues behind the surface */
            capSeed(0);
            if (pathLength >= p.maxDepth) return;
            ext[pathLength - 1]++;
            fix_nan(throughput);
            if (flavor == MIS_OPTIX7) {
                O = I + D * eps;   /* flags, direction, packed normal and pdf carry over */
                tmin = eps;
            } else {
                O = I;
                tmin = EPSILON;
                packedNormal = 0;
            }
            continue;
        }
        if (IsEmissive(sd)) {
            const float DdotNL = -dot(D, N);
            if (DdotNL > 0) {
                f3 contribution = mk3(0);
                if (pathLength == 1 || (FLAGS & S_SPECULAR) || !nee) {
                    contribution = sd.color;   /* the reference leaves the throughput out here */
                } else {
                    const f3 lastN = UnpackNormal(packedNormal);
                    const float lightPdf = CalculateLightPDF(D, HIT_T, tri.area, N);
                    float pickProb;
                    if (p.flags & LH2G_RP_LIGHTTREE) {   /* the shading seed, drawn before this branch in the reference */
                        uint seed = WangHash(pathIdx * 17u + R0(pathLength));
                        pickProb = LightPickProbLTree(s->lightTree, tri.ltriIdx, lastN, I, seed);
                    } else {
                        pickProb = LightPickProb(s, tri.ltriIdx, O, lastN, I);
                    }
                    if ((bsdfPdf + lightPdf * pickProb) > 0) contribution = throughput * sd.color * (1.0f / (bsdfPdf + lightPdf * pickProb));
                }
                clamp_intensity(contribution, p.clampValue);
                fix_nan(contribution);
                out.acc.x += contribution.x, out.acc.y += contribution.y, out.acc.z += contribution.z;
            }
            capSeed(0);
            return;
        }
        if (FLAGS & S_BOUNCED) sd.params[0] |= 255u << 24;   /* path regularisation: roughness 1 after a bounce */
        if (ROUGHNESS(sd) <= 0.001f || TRANSMISSION(sd) > 0.5f) FLAGS |= S_SPECULAR; else FLAGS &= ~S_SPECULAR;
        const float faceDir = (dot(D, N) > 0) ? -1.0f : 1.0f;
        if (faceDir == 1) sd.transmittance = mk3(0);
        throughput = throughput * (1.0f / bsdfPdf);
        uint seed = WangHash(pathIdx * 17u + R0(pathLength));
        f4 r4;
        if (sampleIdx < 64 && bn) {
            const uint x = ((pathIdx % (uint)W) + (p.shift & 127u)) & 127u;
            const uint y = ((pathIdx / (uint)W) + (p.shift >> 24)) & 127u;
            r4 = blueNoiseSampler4(bn, (int)x, (int)y, (int)sampleIdx, 4 * pathLength - 4);
        } else {
            r4.x = RandomFloat(seed), r4.y = RandomFloat(seed);
            r4.z = RandomFloat(seed), r4.w = RandomFloat(seed);
        }
        if ((FLAGS & S_SPECULAR) == 0 && nee) {
            float pickProb = 0, lightPdf = 0;
            f3 lightColor = mk3(0);
            f3 L = ((p.flags & LH2G_RP_LIGHTTREE) ? RandomPointOnLightLTree(s, s->lightTree, r4.x, r4.y, seed, I, fN * faceDir, pickProb, lightPdf, lightColor)
                                                  : RandomPointOnLight(s, r4.x, r4.y, I, fN * faceDir, pickProb, lightPdf, lightColor)) - I;
            const float dist = length(L);
            L = L * (1.0f / dist);
            const float NdotL = dot(L, fN * faceDir);
            if (NdotL > 0 && lightPdf > 0) {
                float lbsdfPdf;
                /* lambert.h's BSDF_HAS_PURE_SPECULARS scales the value by ROUGHNESS (pathtracer.h:194-198) */
                const f3 sampledBSDF = disney ? dis::EvaluateBSDF(sd, fN, T, D * -1.0f, L, lbsdfPdf) : EvaluateBSDF(sd, fN, L, lbsdfPdf) * ROUGHNESS(sd);
                if (lbsdfPdf > 0) {
                    f3 contribution = throughput * sampledBSDF * lightColor * (NdotL / (pickProb * lightPdf + lbsdfPdf));
                    fix_nan(contribution);
                    clamp_intensity(contribution, p.clampValue);
                    shad[pathLength - 1]++;
                    HitRec sh;
                    const f3 SO = SafeOrigin(I, L, N, eps);
                    const bool occluded = trace_scene(s, SO, L, flavor == MIS_OPTIX7 ? eps : 0.0f, dist - 2 * eps, true, false, sh);
                    if (!occluded) {
                        out.acc.x += contribution.x, out.acc.y += contribution.y, out.acc.z += contribution.z;
                        if (flavor == MIS_OPTIX7) out.acc.w += 1.0f;
                    }
                }
            }
        }
        /* one diffuse bounce at most (ENOUGH_BOUNCES = S_BOUNCED), or the maximum path length */
        if ((FLAGS & S_BOUNCED) || pathLength == p.maxDepth) { capSeed(seed); return; }
        f3 R = mk3(0);
        float newBsdfPdf = 0.0f;   /* the Disney sampler leaves it unset on its early exits: the path ends there */
        bool specular = false;
        const float r5 = RandomFloat(seed);   /* lambert.h's SampleBSDF draws it and does not use it */
        const f3 bsdf = disney ? dis::SampleBSDF(sd, fN, N, T, D * -1.0f, HIT_T, r4.z, r4.w, r5, R, newBsdfPdf, specular)
                               : SampleBSDF(sd, fN, N, D * -1.0f, HIT_T, r4.z, r4.w, R, newBsdfPdf, specular);
        if (newBsdfPdf < EPSILON || std::isnan(newBsdfPdf)) { capSeed(seed); return; }
        if (specular) FLAGS |= S_SPECULAR;
        const float pr = ((FLAGS & S_SPECULAR) || (FLAGS & S_BOUNCED) == 0) ? 1.0f : SurvivalProbability(bsdf);
        if (pr < RandomFloat(seed)) { capSeed(seed); return; }
        throughput = throughput * (1 / pr);
        capSeed(seed);
        ext[pathLength - 1]++;
        packedNormal = PackNormal(fN * faceDir);
        if (!(FLAGS & S_SPECULAR)) FLAGS |= (FLAGS & S_BOUNCED) ? S_BOUNCEDTWICE : S_BOUNCED; else FLAGS |= S_VIASPECULAR;
        O = SafeOrigin(I, R, N, eps);
        D = R;
        fix_nan(throughput);
        throughput = throughput * bsdf * fabsf(dot(fN, R));
        bsdfPdf = newBsdfPdf;
        tmin = flavor == MIS_OPTIX7 ? eps : 0.0f;
    }
}

/* the primary ray of the OptiX 7 core, optix/.optix.cu:85-129 (setupPrimaryRay, generateEyeRay) */
inline void primary_optix7(const Frame& F, const uint pathIdx, f3& O, f3& D) {
    const lh2g_render_params& p = F.p;
    const uint W = (uint)p.width, H = (uint)p.height;
    const uint pixelIdx = pathIdx % (W * H);
    const uint sampleIdx = pathIdx / (W * H) + (uint)p.samplesTaken;
    uint seed = WangHash(pathIdx * 16789u + (uint)p.samplesTaken * 1791u);
    const int sx = (int)(pixelIdx % W), sy = (int)(pixelIdx / W);
    f4 r4;
    if (sampleIdx < 64 && !F.s->blueNoise.empty()) {
        r4 = blueNoiseSampler4(F.s->blueNoise.data(), (sx + (int)(p.shift & 127u)) & 127, (sy + (int)(p.shift >> 24)) & 127, (int)sampleIdx, 0);
    } else {
        r4.x = RandomFloat(seed), r4.y = RandomFloat(seed);
        r4.z = RandomFloat(seed), r4.w = RandomFloat(seed);
    }
    O = RandomPointOnLens(r4.x, r4.z, ld3(F.view.pos), F.view.aperture, F.right, F.up);
    const f3 posOnPixel = RayTarget(sx, sy, r4.y, r4.w, (int)W, (int)H, F.view.distortion, ld3(F.view.p1), F.right, F.up);
    D = normalize(posOnPixel - O);
}

/* the primary ray of the PrimeAdaptive core for pixel (sx, sy) and sample index sampleIdx: blue noise (no tile
 * shift) below 64, else xorshift numbers from WangHash(thread + R0) (camera.h:39-80, 96-139) */
inline void primary_adaptive(const Frame& F, const int sx, const int sy, const uint sampleIdx, const uint thread, const uint R0, f3& O, f3& D) {
    f4 r4;
    if (sampleIdx < 64 && !F.s->blueNoise.empty()) {
        r4 = blueNoiseSampler4(F.s->blueNoise.data(), sx & 127, sy & 127, (int)sampleIdx, 0);
    } else {
        uint seed = WangHash(thread + R0);
        r4.x = RandomFloat(seed), r4.y = RandomFloat(seed);
        r4.z = RandomFloat(seed), r4.w = RandomFloat(seed);
    }
    O = RandomPointOnLens(r4.x, r4.z, ld3(F.view.pos), F.view.aperture, F.right, F.up);
    const f3 posOnPixel = RayTarget(sx, sy, r4.y, r4.w, F.p.width, F.p.height, F.view.distortion, ld3(F.view.p1), F.right, F.up);
    D = normalize(posOnPixel - O);
}

/* estimateVarianceKernel, lib/CUDA/shared_kernel_code/finalize_shared.h:97-151 (powf(x, 2) as x * x) */
float estimate_variance(const float* frameAcc, const float* features, const int x, const int y, const int W, const int H, const int spp) {
    const long long WH = (long long)W * H;
    const float x1 = (float)imax(0, x - 4), y1 = (float)imax(0, y - 4), x2 = (float)imin(W - 1, x + 4), y2 = (float)imin(H - 1, y + 4);
    f3 total = mk3(0);
    float weightSum = 0;
    for (int i = 0; i < spp; i++) {
        const f3 Nlocal = UnpackNormal2(fbits(features[4 * (x + (long long)y * W + i * WH) + 3]));
        for (int v = (int)y1; v <= y2; v++)
            for (int u = (int)x1; u <= x2; u++) {
                const long long a = u + (long long)v * W + i * WH;
                const float* feature = features + 4 * a;
                const f3 normal = UnpackNormal2(fbits(feature[3]));
                const f3 albedo = ld3(feature);
                const f3 smp = ld3(frameAcc + 4 * a);
                const f3 lighting = mk3(smp.x / fmaxr(albedo.x, 0.001f), smp.y / fmaxr(albedo.y, 0.001f), smp.z / fmaxr(albedo.z, 0.001f));
                const uint dx = (uint)std::abs(x - u), dy = (uint)std::abs(y - v);
                const float xweight = dx == 1 ? 0.9f : (dx == 2 ? 0.75f : (dx == 3 ? 0.55f : (dx == 4 ? 0.35f : 1.0f)));
                const float yweight = dy == 1 ? 0.9f : (dy == 2 ? 0.75f : (dy == 3 ? 0.55f : (dy == 4 ? 0.35f : 1.0f)));
                const float c = fmaxr(0.0001f, dot(normal, Nlocal));
                const float weight = xweight * yweight * (c * c);
                weightSum += weight;
                total = total + lighting * weight;
            }
    }
    const f3 average = total * (1.0f / weightSum);
    float variance = 0;
    for (int i = 0; i < spp; i++) {
        const long long a = x + (long long)y * W + i * WH;
        const f3 albedo = ld3(features + 4 * a);
        const f3 smp = ld3(frameAcc + 4 * a);
        const f3 lighting = mk3(smp.x / fmaxr(albedo.x, 0.001f), smp.y / fmaxr(albedo.y, 0.001f), smp.z / fmaxr(albedo.z, 0.001f));
        const float d = Luminance(lighting) - Luminance(average);
        variance += d * d;
    }
    variance /= 3.0f * spp;
    return (variance + EPSILON) / (Luminance(average) + EPSILON);
}

/* samples S = 1..24 a pixel asks for (generateEyeRaysKernelAdaptive: sample S when !(S > deviation)) */
inline int adaptive_wanted(const float d) {
    int c = 0;
    for (int S = 1; S <= 24; S++) if (!((float)S > d)) c = S;
    return c;
}

}  // namespace

/* ==========================================================================================================
 * C API
 * ======================================================================================================== */
namespace {

/* ======================================================================================================
 * SoftRasterizer core (lib/RenderCore_SoftRasterizer): z-buffered scanline rasterisation of every instance,
 * restated from rasterizer.cpp:66-171 (Mesh::Render), :201-215 (Rasterizer::Reinit), :225-240
 * (Rasterizer::Render) and rendercore.cpp:55-185,213-222 (SetGeometry / SetInstance / SetMaterials / Render).
 * Sequential, in the reference's order: instances, then triangles, then edges, then rows and spans; a fragment
 * replaces the pixel when its interpolated 1/z is below the z-buffer's (which starts at 0).
 *
 * Conversions the C++ source leaves to the platform are fixed here, and the GPU core does the same:
 * float -> int truncates and saturates (NaN -> 0), as Arm and the GPU do (x86 returns INT_MIN out of range);
 * float -> unsigned (the texel coordinates and the shade) truncates to a 64-bit integer and keeps its low 32
 * bits, as x86-64 compilers emit it (0 for NaN and beyond the 64-bit range).
 * Two guards the reference lacks, both unreachable for finite input: a span whose left end lies at x <= -1 is dropped
 * (the reference would write into the previous row; clipping against the left plane keeps spans at x >= 0.5 up to
 * rounding), and a fragment whose 1/z is NaN is dropped (the reference's z-test lets it through).
 * ==================================================================================================== */
struct RsMesh4 { float m[16]; };

inline int rs_f2i(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int)0x80000000u;
    return (int)x;
}
inline uint rs_f2u(float x) {
    if (!(x > -9223372036854775808.0f && x < 9223372036854775808.0f)) return 0u;
    return (uint)(uint64_t)(int64_t)x;
}
/* operator*(mat4, mat4), lib/platform/system.cpp:57-68 */
inline RsMesh4 rs_mul(const float* a, const float* b) {
    RsMesh4 r;
    for (int i = 0; i < 16; i += 4)
        for (int j = 0; j < 4; j++) r.m[i + j] = a[i] * b[j] + a[i + 1] * b[j + 4] + a[i + 2] * b[j + 8] + a[i + 3] * b[j + 12];
    return r;
}
/* operator*(mat4, float4), system.cpp:90-96 (the xyz rows) */
inline f3 rs_xform(const float* a, float x, float y, float z, float w) {
    return mk3(a[0] * x + a[1] * y + a[2] * z + a[3] * w, a[4] * x + a[5] * y + a[6] * z + a[7] * w, a[8] * x + a[9] * y + a[10] * z + a[11] * w);
}
/* ScaleColor, rasterizer.cpp:20-25 */
inline uint rs_scale_color(uint c, uint scale) {
    const uint rb = (((c & 0xff00ffu) * scale) >> 8) & 0xff00ffu;
    const uint g = (((c & 0xff00u) * scale) >> 8) & 0xff00u;
    return rb + g;
}

/* Rasterizer::Reinit's frustum planes (rasterizer.cpp:205-214) for a w x h target */
void rs_frustum(int w, int h, f4* fr) {
    const float C = -1.0f, x1 = 0.5f, x2 = w - 1.5f, y1 = 0.5f, y2 = h - 1.5f;
    const f3 p0 = mk3(0.0f, 0.0f, 0.0f);
    const f3 p1 = mk3(((x1 - w * 0.5f) * C) / w, ((y1 - h * 0.5f) * C) / w, 1.0f);
    const f3 p2 = mk3(((x2 - w * 0.5f) * C) / w, ((y1 - h * 0.5f) * C) / w, 1.0f);
    const f3 p3 = mk3(((x2 - w * 0.5f) * C) / w, ((y2 - h * 0.5f) * C) / w, 1.0f);
    const f3 p4 = mk3(((x1 - w * 0.5f) * C) / w, ((y2 - h * 0.5f) * C) / w, 1.0f);
    fr[0] = {0.0f, 0.0f, -1.0f, 0.2f};
    const f3 a = normalize(cross(p1 - p0, p4 - p1)), b = normalize(cross(p2 - p0, p1 - p2));
    const f3 c = normalize(cross(p3 - p0, p2 - p3)), d = normalize(cross(p4 - p0, p3 - p4));
    fr[1] = {a.x, a.y, a.z, 0.0f}, fr[2] = {b.x, b.y, b.z, 0.0f}, fr[3] = {c.x, c.y, c.z, 0.0f}, fr[4] = {d.x, d.y, d.z, 0.0f};
}

/* RenderCore::Render's camera transform (rendercore.cpp:215-222), inverted as Rasterizer::Render does
 * (rasterizer.cpp:239), times the scene root's identity transform (SGNode::Render, rasterizer.cpp:187) */
RsMesh4 rs_view(const lh2g_view* v) {
    const f3 pos = ld3(v->pos), p1 = ld3(v->p1), p2 = ld3(v->p2), p3 = ld3(v->p3);
    const f3 X = normalize(p2 - p1), Y = normalize(p1 - p3), Z = normalize(pos - 0.5f * (p2 + p3));
    float R[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    R[0] = X.x, R[4] = X.y, R[8] = X.z;
    R[1] = Y.x, R[5] = Y.y, R[9] = Y.z;
    R[2] = Z.x, R[6] = Z.y, R[10] = Z.z;
    const float Tr[16] = {1, 0, 0, pos.x, 0, 1, 0, pos.y, 0, 0, 1, pos.z, 0, 0, 0, 1};
    const RsMesh4 cam = rs_mul(Tr, R);
    float inv[16];
    invert4x4(cam.m, inv);
    const float I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    return rs_mul(inv, I);
}

/* RenderCore::SetMaterials' colour (rendercore.cpp:175-181) */
uint rs_diffuse(const lh2g_material& m) {
    return ((uint)rs_f2i(m.color[2] * 255.0f) << 16) + ((uint)rs_f2i(m.color[1] * 255.0f) << 8) + (uint)rs_f2i(m.color[0] * 255.0f);
}

struct RsTables { std::vector<float> xl, xr, ul, ur, vl, vr, zl, zr; };

/* Mesh::Render (rasterizer.cpp:66-171) for one instance; returns the fragments that passed the depth test */
uint64_t rs_mesh(const lh2o_scene& s, const Mesh& mesh, const float* T, const f4* fr, int W, int H, RsTables& tb, uint* pixels, float* zbuffer) {
    /* cull the mesh against the five planes (:69-75) */
    f3 c[8];
    for (int i = 0; i < 8; i++) c[i] = rs_xform(T, (i & 1) ? mesh.bmax[0] : mesh.bmin[0], ((i >> 1) & 1) ? mesh.bmax[1] : mesh.bmin[1], (i >> 2) ? mesh.bmax[2] : mesh.bmin[2], 1.0f);
    for (int p = 0; p < 5; p++) {
        int i = 0;
        for (; i < 8; i++)
            if ((dot(mk3(fr[p].x, fr[p].y, fr[p].z), c[i]) - fr[p].w) > 0) break;
        if (i == 8) return 0;
    }
    uint64_t frags = 0;
    const size_t nt = mesh.tris.size();
    for (size_t i = 0; i < nt; i++) {
        const lh2g_core_tri& ct = mesh.tris[i];
        const lh2g_material& mat = s.hostMats[ct.material];
        const int tex = mat.color_map.texture;
        const uint diffuse = rs_diffuse(mat);
        const uint* src = tex >= 0 ? s.texels.data() + s.texFirst[tex] : &diffuse;
        const float tw = tex >= 0 ? (float)s.texWH[2 * tex] : 1.0f, th = tex >= 0 ? (float)s.texWH[2 * tex + 1] : 1.0f;
        const int umask = (int)tw, vmask = (int)th;
        f3 tpos[3];
        for (int v = 0; v < 3; v++) tpos[v] = rs_xform(T, mesh.pos[3 * i + v].x, mesh.pos[3 * i + v].y, mesh.pos[3 * i + v].z, 1.0f);
        /* back faces (:86-87) */
        const f3 Nt = rs_xform(T, ct.Nx, ct.Ny, ct.Nz, 0.0f);
        if (dot(tpos[0], Nt) > 0) continue;
        /* clip against the near and left planes (:89-106) */
        f3 cpos[2][8];
        f2 cuv[2][8];
        int nin = 3, nout = 0, from = 0, to = 1;
        const float us[3] = {ct.u0, ct.u1, ct.u2}, vs[3] = {ct.v0, ct.v1, ct.v2};
        for (int v = 0; v < 3; v++) cpos[0][v] = tpos[v], cuv[0][v] = {us[v], vs[v]};
        for (int p = 0; p < 2; p++, from = 1 - from, to = 1 - to, nin = nout, nout = 0)
            for (int v = 0; v < nin; v++) {
                const f3 A = cpos[from][v], B = cpos[from][(v + 1) % nin];
                const f2 Auv = cuv[from][v], Buv = cuv[from][(v + 1) % nin];
                const f3 pn = mk3(fr[p].x, fr[p].y, fr[p].z);
                const float t1 = dot(pn, A) - fr[p].w, t2 = dot(pn, B) - fr[p].w;
                if (t1 < 0 && t2 >= 0) {
                    const float f = t1 / (t1 - t2);
                    cuv[to][nout] = {Auv.x + (Buv.x - Auv.x) * f, Auv.y + (Buv.y - Auv.y) * f}, cpos[to][nout++] = A + f * (B - A);
                    cuv[to][nout] = Buv, cpos[to][nout++] = B;
                } else if (t1 >= 0 && t2 >= 0) {
                    cuv[to][nout] = Buv, cpos[to][nout++] = B;
                } else if (t1 >= 0 && t2 < 0) {
                    const float f = t1 / (t1 - t2);
                    cuv[to][nout] = {Auv.x + (Buv.x - Auv.x) * f, Auv.y + (Buv.y - Auv.y) * f}, cpos[to][nout++] = A + f * (B - A);
                }
            }
        if (nin == 0) continue;
        /* project (:109-112) */
        f3* pos = cpos[from];
        const f2* tuv = cuv[from];
        for (int v = 0; v < nin; v++)
            pos[v].x = ((pos[v].x * W) / -pos[v].z) + (float)(W / 2), pos[v].y = ((pos[v].y * W) / pos[v].z) + (float)(H / 2);
        /* edges into the outline tables (:114-137) */
        const uint shade = rs_f2u((ct.Nz + 1) * 64.0f + 127.9f);
        int miny = H - 1, maxy = 0;
        for (int j = 0; j < nin; j++) {
            int vert0 = j, vert1 = (j + 1) % nin;
            if (pos[vert0].y > pos[vert1].y) std::swap(vert0, vert1);
            const float y0 = pos[vert0].y, y1 = pos[vert1].y, rydiff = 1.0f / (y1 - y0);
            if (y0 == y1 || y0 >= H || y1 < 1) continue;
            const int iy0 = std::max(1, rs_f2i(y0) + 1), iy1 = std::min(H - 2, rs_f2i(y1));
            float x0 = pos[vert0].x, dx = (pos[vert1].x - x0) * rydiff;
            float z0 = 1.0f / pos[vert0].z, z1 = 1.0f / pos[vert1].z, dz = (z1 - z0) * rydiff;
            float u0 = tuv[vert0].x * z0, du = (tuv[vert1].x * z1 - u0) * rydiff;
            float v0 = tuv[vert0].y * z0, dv = (tuv[vert1].y * z1 - v0) * rydiff;
            const float f = (float)iy0 - y0;
            x0 += dx * f, u0 += du * f, v0 += dv * f, z0 += dz * f;
            for (int y = iy0; y <= iy1; y++) {
                if (x0 < tb.xl[y]) tb.xl[y] = x0, tb.ul[y] = u0, tb.vl[y] = v0, tb.zl[y] = z0;
                if (x0 > tb.xr[y]) tb.xr[y] = x0, tb.ur[y] = u0, tb.vr[y] = v0, tb.zr[y] = z0;
                x0 += dx, u0 += du, v0 += dv, z0 += dz;
            }
            miny = std::min(miny, iy0), maxy = std::max(maxy, iy1);
        }
        /* spans (:138-169), resetting the tables' rows behind them */
        for (int y = miny; y <= maxy; tb.xl[y] = (float)(W - 1), tb.xr[y++] = 0.0f) {
            const float x0 = tb.xl[y], x1 = tb.xr[y], rxdiff = 1.0f / (x1 - x0);
            float u0 = tb.ul[y], du = (tb.ur[y] - u0) * rxdiff;
            float v0 = tb.vl[y], dv = (tb.vr[y] - v0) * rxdiff;
            float z0 = tb.zl[y], dz = (tb.zr[y] - z0) * rxdiff;
            const int ix0 = rs_f2i(x0) + 1, ix1 = std::min(W - 2, rs_f2i(x1));
            if (ix0 < 1) continue;
            const float f = (float)ix0 - x0;
            u0 += f * du, v0 += f * dv, z0 += f * dz;
            uint* dest = pixels + (size_t)y * W;
            float* zbuf = zbuffer + (size_t)y * W;
            for (int x = ix0; x <= ix1; x++, u0 += du, v0 += dv, z0 += dz) {
                if (!(z0 < zbuf[x])) continue;
                const float z = 1.0f / z0;
                const uint u = rs_f2u(u0 * z * tw) % (uint)umask, v = rs_f2u(v0 * z * th) % (uint)vmask;
                dest[x] = rs_scale_color(src[u + v * (uint)umask], shade), zbuf[x] = z0;
                frags++;
            }
        }
    }
    return frags;
}

}  // namespace

extern "C" {

lh2o_scene* lh2o_create(void) { return new lh2o_scene(); }
void lh2o_destroy(lh2o_scene* s) { delete s; }

int lh2o_set_geometry(lh2o_scene* s, int meshIdx, const float* v4, int vertexCount, int triangleCount, const lh2g_core_tri* tris) {
    if (!s || meshIdx < 0 || meshIdx > (int)s->meshes.size() || vertexCount != 3 * triangleCount) return 1;
    if (meshIdx == (int)s->meshes.size()) s->meshes.emplace_back();
    Mesh& m = s->meshes[meshIdx];
    m.tris.assign(tris, tris + triangleCount);
    m.v0.resize(triangleCount), m.e1.resize(triangleCount), m.e2.resize(triangleCount), m.pos.resize((size_t)3 * triangleCount);
    for (int a = 0; a < 3; a++) m.bmin[a] = 1e30f, m.bmax[a] = -1e30f;
    for (int i = 0; i < triangleCount; i++) {
        const float* a = v4 + 12 * i;
        const f3 p0 = mk3(a[0], a[1], a[2]), p1 = mk3(a[4], a[5], a[6]), p2 = mk3(a[8], a[9], a[10]);
        m.v0[i] = p0, m.e1[i] = p1 - p0, m.e2[i] = p2 - p0;
        m.pos[3 * i] = p0, m.pos[3 * i + 1] = p1, m.pos[3 * i + 2] = p2;
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
    if (!s || ntri < 0 || npt < 0 || nspot < 0 || ndir < 0 || (long long)ntri + npt + nspot > (1 << 16) || ndir > 64) return 1;
    s->triLights.assign(tri, tri + ntri);
    s->pointLights.assign(pt, pt + npt);
    s->spotLights.assign(spot, spot + nspot);
    s->dirLights.assign(dir, dir + ndir);
    s->lightTree = lt_build(s);
    return 0;
}

/* the light tree of the scene's lights: 2 * (area + point + spot lights) records of 16 words (the device
 * LightCluster); returns the record count (out null: only the count), or -1 when out holds fewer than that
 * (capacity in records) */
int lh2o_light_tree(const lh2o_scene* s, void* out, int capacity) {
    if (!s) return -1;
    if (!out) return (int)s->lightTree.size();
    if (capacity < (int)s->lightTree.size()) return -1;
    if (!s->lightTree.empty()) memcpy(out, s->lightTree.data(), sizeof(LtCluster) * s->lightTree.size());
    return (int)s->lightTree.size();
}

int lh2o_set_sky(lh2o_scene* s, const float* rgb, int w, int h, const float* m16) {
    if (!s || w < 0 || h < 0) return 1;
    s->sky.w = w, s->sky.h = h;
    s->sky.px.resize((size_t)w * h);
    for (size_t i = 0; i < (size_t)w * h; i++) s->sky.px[i] = mk3(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
    for (int i = 0; i < 16; i++) s->sky.m[i] = m16 ? m16[i] : ((i % 5 == 0) ? 1.0f : 0.0f);
    const int sw = w >> 6, sh = h >> 6;
    s->sky.small.assign((size_t)sw * sh, mk3(0));
    for (int y = 0; y < sh; y++)
        for (int x = 0; x < sw; x++) {
            f3 total = mk3(0);
            for (int v = 0; v < 64; v++)
                for (int u = 0; u < 64; u++) total = total + s->sky.px[(size_t)(x * 64 + u) + (size_t)(y * 64 + v) * w];
            s->sky.small[(size_t)x + (size_t)y * sw] = total * (1.0f / (64 * 64));
        }
    return 0;
}

int lh2o_set_blue_noise(lh2o_scene* s, const uint8_t* sobol, const uint8_t* scrambling, const uint8_t* ranking) {
    if (!s) return 1;
    if (!sobol || !scrambling || !ranking) { s->blueNoise.clear(); return 0; }
    s->blueNoise.assign(65536 * 5 + 64, 0u);
    for (int i = 0; i < 65536; i++) s->blueNoise[i] = sobol[i];
    for (int i = 0; i < 128 * 128 * 8; i++) s->blueNoise[i + 65536] = scrambling[i], s->blueNoise[i + 3 * 65536] = ranking[i];
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

/* A frame of the OptiX 7 core's estimator: per path its terminal term and connections; per pixel the terms of the
 * frame's samples in sample order, then their connections (first, then second) in sample order. */
static int render_optix7(lh2o_scene* s, const lh2g_view* view, const lh2g_render_params* p, float* pixelAccum, double* pixelAccum64,
                         uint32_t* counters, lh2g_capture* capture, int nthreads) {
    Frame F;
    F.s = s, F.view = *view, F.p = *p;
    F.right = ld3(view->p2) - ld3(view->p1);
    F.up = ld3(view->p3) - ld3(view->p1);
    memset(&F.feat, 0, sizeof(F.feat));
    const long long WH = (long long)p->width * p->height;
    F.P = WH * p->spp;
    const int D = p->maxDepth;
    if (capture && capture->hits)
        for (long long i = 0; i < F.P * D; i++) capture->hits[i] = lh2g_hit{0, -1, -2, 0.0f};
    if (capture && capture->seeds) memset(capture->seeds, 0, sizeof(uint32_t) * F.P * D);
    /* shading seed of wave d: the d-th RandomUInt(camRNGseed) of the frame (cameraR0 is the first) + d * 91771 */
    uint draws[65];
    draws[1] = p->cameraR0;
    for (int d = 2; d <= D; d++) { uint x = draws[d - 1]; draws[d] = RandomInt(x); }
    auto R0 = [&](int d) { return draws[d] + (uint)d * 91771u; };
    std::vector<MisPath> paths(F.P);
    std::mutex mtx;
    std::vector<uint> extTot(D, 0), shadTot(D, 0);
    parallel_for(F.P, nthreads, 256, [&](long long b, long long e) {
        std::vector<uint> ext(D, 0), shad(D, 0);
        for (long long i = b; i < e; i++) {
            f3 O, Dd;
            primary_optix7(F, (uint)i, O, Dd);
            trace_path_mis(F, MIS_OPTIX7, (uint)i, (uint)p->samplesTaken, R0, O, Dd, p->geometryEpsilon, paths[i], ext, shad, capture, i, nullptr);
        }
        std::lock_guard<std::mutex> g(mtx);
        for (int d = 0; d < D; d++) extTot[d] += ext[d], shadTot[d] += shad[d];
    });
    for (long long px = 0; px < WH; px++)
        for (int smp = 0; smp < p->spp; smp++) {
            const f4& v = paths[smp * WH + px].acc;
            if (pixelAccum) add4(pixelAccum + 4 * px, v);
            if (pixelAccum64) {
                double* a64 = pixelAccum64 + 4 * px;
                a64[0] += v.x, a64[1] += v.y, a64[2] += v.z, a64[3] += v.w;
            }
        }
    if (counters) for (int d = 0; d < D; d++) counters[2 * d] = extTot[d], counters[2 * d + 1] = shadTot[d];
    return 0;
}

int lh2o_render_ex(lh2o_scene* s, const lh2g_view* view, const lh2g_render_params* p, float* pixelAccum, double* pixelAccum64,
                   uint32_t* counters, lh2g_capture* capture, const lh2o_features* feat, int nthreads) {
    if (!s || !s->finalized || !view || !p || p->width <= 0 || p->height <= 0 || p->spp <= 0 || p->maxDepth <= 0 || p->maxDepth > 64) return 1;
    const size_t lights = s->triLights.size() + s->pointLights.size() + s->spotLights.size() + s->dirLights.size();
    if ((p->flags & LH2G_RP_LIGHTTREE) ? !(p->flags & LH2G_RP_OPTIX7) : lights > 64) return 1;   /* 64 potentials at most */
    if (p->flags & LH2G_RP_OPTIX7) {
        if ((p->flags & (LH2G_RP_FILTER | LH2G_RP_NRC | LH2G_RP_ADAPTIVE)) || p->rowCount != 0) return 1;
        return render_optix7(s, view, p, pixelAccum, pixelAccum64, counters, capture, nthreads);
    }
    const bool filt = (p->flags & LH2G_RP_FILTER) != 0;
    const bool band = p->rowCount > 0;
    if (band && (filt || (p->flags & LH2G_RP_NRC) || p->rowBegin < 0 || p->rowBegin + p->rowCount > p->height)) return 1;
    Frame F;
    F.s = s, F.view = *view, F.p = *p;
    F.right = ld3(view->p2) - ld3(view->p1);
    F.up = ld3(view->p3) - ld3(view->p1);
    memset(&F.feat, 0, sizeof(F.feat));
    if (filt && feat) F.feat = *feat;
    /* WH: the pixels rendered (a band's rows, or the frame); the accumulator holds them */
    const long long WH = (long long)p->width * (band ? p->rowCount : p->height);
    if (band) F.bandPix = (uint)WH;
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
    /* per-pixel sums in sample order (deterministic); LH2G_RP_FILTER frames have a second, indirect half */
    for (int half = 0; half < (filt ? 2 : 1); half++)
        for (long long px = 0; px < WH; px++) {
            const long long o = (half * WH + px) * 4;
            for (int k = 0; k < 4; k++) {
                float acc = pixelAccum ? pixelAccum[o + k] : 0.0f;
                double acc64 = pixelAccum64 ? pixelAccum64[o + k] : 0.0;
                for (int smp = 0; smp < p->spp; smp++) {
                    const float v = paths[smp * WH + px].rgbw[half][k];
                    acc += v;
                    acc64 += (double)v;
                }
                if (pixelAccum) pixelAccum[o + k] = acc;
                if (pixelAccum64) pixelAccum64[o + k] = acc64;
            }
        }
    if (counters) for (int d = 0; d < D; d++) counters[2 * d] = extTot[d], counters[2 * d + 1] = shadTot[d];
    return 0;
}

int lh2o_render(lh2o_scene* s, const lh2g_view* view, const lh2g_render_params* p, float* pixelAccum, double* pixelAccum64,
                uint32_t* counters, lh2g_capture* capture, int nthreads) {
    return lh2o_render_ex(s, view, p, pixelAccum, pixelAccum64, counters, capture, nullptr, nthreads);
}

int lh2o_render_adaptive(lh2o_scene* s, const lh2g_view* view, const lh2g_render_params* p, float* accum, float* frame, float* devScale,
                         uint32_t* counters, uint32_t* adaptivePaths, float* frameAccOut, float* featuresOut, float* deviationOut,
                         lh2g_capture* capture, int nthreads) {
    if (!s || !s->finalized || !view || !p || !accum || !devScale || p->width <= 0 || p->height <= 0 || p->spp <= 0 || p->maxDepth <= 0 ||
        p->maxDepth > 32 || (p->flags & (LH2G_RP_FILTER | LH2G_RP_NRC | LH2G_RP_OPTIX7)) || p->rowCount != 0)
        return 1;
    Frame F;
    F.s = s, F.view = *view, F.p = *p;
    F.right = ld3(view->p2) - ld3(view->p1);
    F.up = ld3(view->p3) - ld3(view->p1);
    memset(&F.feat, 0, sizeof(F.feat));
    const int W = p->width, H = p->height, spp = p->spp, D = p->maxDepth;
    const long long WH = (long long)W * H, P = WH * spp;
    F.P = P;
    const uint pass = (uint)p->samplesTaken;
    if (capture && capture->hits)
        for (long long i = 0; i < P * D; i++) capture->hits[i] = lh2g_hit{0, -1, -2, 0.0f};
    if (capture && capture->seeds) memset(capture->seeds, 0, sizeof(uint32_t) * P * D);
    std::vector<float> frameAcc(4 * P, 0.0f), feat(4 * P, 0.0f);
    std::vector<MisPath> paths(P);
    std::mutex mtx;
    std::vector<uint> extTot(2 * D, 0), shadTot(2 * D, 0);
    /* first wave: spp samples per pixel (RenderCore_PrimeAdaptive/rendercore.cpp:606-658) */
    auto R0a = [&](int d) { return pass * 7907u + (uint)d * 91771u; };
    parallel_for(P, nthreads, 256, [&](long long b, long long e) {
        std::vector<uint> ext(D, 0), shad(D, 0);
        for (long long j = b; j < e; j++) {
            const int sx = (int)(j % W);
            const uint row = (uint)(j / W);
            const uint sampleIdx = pass + row / (uint)H;
            f3 O, Dd;
            primary_adaptive(F, sx, (int)(row % (uint)H), sampleIdx, (uint)j, p->cameraR0, O, Dd);
            trace_path_mis(F, MIS_ADAPTIVE, (uint)j, pass, R0a, O, Dd, p->geometryEpsilon, paths[j], ext, shad, capture, j, &feat[4 * j]);
        }
        std::lock_guard<std::mutex> g(mtx);
        for (int d = 0; d < D; d++) extTot[d] += ext[d], shadTot[d] += shad[d];
    });
    for (long long j = 0; j < P; j++) add4(&frameAcc[4 * j], paths[j].acc);
    /* variance estimate, the samples each pixel asks for, the budget (rendercore.cpp:663-680) */
    std::vector<float> dev(WH);
    std::vector<int> want(WH);
    const float scale = *devScale;
    parallel_for(WH, nthreads, 1024, [&](long long b, long long e) {
        for (long long px = b; px < e; px++) {
            dev[px] = estimate_variance(frameAcc.data(), feat.data(), (int)(px % W), (int)(px / W), W, H, spp) * scale;
            want[px] = adaptive_wanted(dev[px]);
        }
    });
    unsigned long long total = 0;
    for (long long px = 0; px < WH; px++) total += (unsigned long long)want[px];
    const float budget = (float)(W * H * spp);
    uint pathCount = (uint)total;
    if ((float)pathCount > budget) pathCount = (uint)budget;
    if ((float)pathCount > 0.98f * budget) *devScale *= 0.92f;
    else if ((float)pathCount > 0.96f * budget) *devScale *= 0.98f;
    else if ((float)pathCount < 0.91f * budget) *devScale *= 1.08f;
    else if ((float)pathCount < 0.94f * budget) *devScale *= 1.02f;
    /* the samples kept: the first `budget` in the order of the generating threads (thread = pixel + (S - 1) * W*H),
     * i.e. all with S below S*, and those with S = S* of the first r pixels that ask for S* */
    std::vector<int> kept(WH);
    {
        long long room = (long long)pathCount;
        for (long long px = 0; px < WH; px++) kept[px] = 0;
        for (int S = 1; S <= 24 && room > 0; S++)
            for (long long px = 0; px < WH && room > 0; px++)
                if (want[px] >= S) kept[px] = S, room--;
    }
    if (adaptivePaths) *adaptivePaths = pathCount;
    /* second wave (rendercore.cpp:682-713): slots in pixel order, S ascending within a pixel */
    std::vector<long long> first(WH + 1, 0);
    for (long long px = 0; px < WH; px++) first[px + 1] = first[px] + kept[px];
    const long long n2 = first[WH];
    std::vector<MisPath> extra(n2);
    auto R0b = [&](int d) { return pass * 59071u + (uint)d * 31771u; };
    parallel_for(WH, nthreads, 64, [&](long long b, long long e) {
        std::vector<uint> ext(D, 0), shad(D, 0);
        for (long long px = b; px < e; px++)
            for (int S = 1; S <= kept[px]; S++) {
                const uint thread = (uint)(px + (long long)(S - 1) * WH);
                const uint pathIdx = (uint)(px + (long long)(S % spp) * WH);
                f3 O, Dd;
                primary_adaptive(F, (int)(px % W), (int)(px / W), (uint)S + (uint)spp + pass, thread, p->frameSeed, O, Dd);
                trace_path_mis(F, MIS_ADAPTIVE, pathIdx, pass + (uint)spp, R0b, O, Dd, p->geometryEpsilon, extra[first[px] + S - 1], ext, shad,
                               nullptr, -1, nullptr);
            }
        std::lock_guard<std::mutex> g(mtx);
        for (int d = 0; d < D; d++) extTot[D + d] += ext[d], shadTot[D + d] += shad[d];
    });
    /* into the layers: the second-wave paths of layer i are those with S % spp == i, added in S order */
    for (long long px = 0; px < WH; px++)
        for (int S = 1; S <= kept[px]; S++) add4(&frameAcc[4 * (px + (S % spp) * WH)], extra[first[px] + S - 1].acc);
    /* finalizeASRenderKernel (finalize_shared.h:71-93) after samplesTaken += spp */
    const int frames = (p->samplesTaken + spp) / spp;
    const float pixelValueScale = 1.0f / (float)frames;
    for (long long px = 0; px < WH; px++) {
        f4 q = mk4(0, 0, 0, 0);
        for (int i = 0; i < spp; i++) q = q + ld4(&frameAcc[4 * (px + i * WH)]);
        const f4 add = q * (1.0f / q.w);
        float* a = accum + 4 * px;
        add4(a, add);
        if (frame) for (int k = 0; k < 4; k++) frame[4 * px + k] = a[k] * pixelValueScale;
    }
    if (counters) for (int d = 0; d < 2 * D; d++) counters[2 * d] = extTot[d], counters[2 * d + 1] = shadTot[d];
    if (frameAccOut) memcpy(frameAccOut, frameAcc.data(), sizeof(float) * 4 * P);
    if (featuresOut) memcpy(featuresOut, feat.data(), sizeof(float) * 4 * P);
    if (deviationOut) memcpy(deviationOut, dev.data(), sizeof(float) * WH);
    return 0;
}

int lh2o_svgf_frame(lh2o_svgf* f, const float* accum, const lh2g_filter_params* fp, int nthreads) {
    if (!f || !accum || !fp || f->width <= 0 || f->height <= 0 || fp->samplesTaken <= 0) return 1;
    Svgf S;
    S.w = f->width, S.h = f->height, S.b = f;
    const SvgfView V = svgf_view(fp->prevView, f->height);
    const float scale = 1.0f / (float)fp->samplesTaken;
    auto rows = [&](const std::function<void(int, int)>& fn) {
        parallel_for(S.h, nthreads, 4, [&](long long b, long long e) {
            for (long long y = b; y < e; y++)
                for (int x = 0; x < S.w; x++) fn(x, (int)y);
        });
    };
    rows([&](int x, int y) { S.prepare(x, y, accum, V, *fp, scale); });
    rows([&](int x, int y) { S.apply(x, y, f->shading, f->filteredIN, f->filteredOUT, 1, false); });
    rows([&](int x, int y) { S.apply(x, y, f->filteredOUT, nullptr, f->filteredIN, 2, false); });
    rows([&](int x, int y) { S.apply(x, y, f->filteredIN, nullptr, f->shading, 3, true); });
    if (fp->taa) {
        rows([&](int x, int y) { S.taa(x, y, f->shading, f->prevPixels, f->taaPixels); });
        rows([&](int x, int y) { S.unsharpen(x, y, f->taaPixels, f->target); });
        std::swap(f->taaPixels, f->prevPixels);
    } else {
        rows([&](int x, int y) { S.finalize_no_taa(x, y, f->shading, f->target); });
        std::swap(f->shading, f->prevPixels);
    }
    std::swap(f->filteredIN, f->filteredOUT);
    std::swap(f->prevWorldPos, f->worldPos);
    std::swap(f->moments, f->prevMoments);
    return 0;
}

void lh2o_nrc_encode(const lh2o_nrc_spec* S, const float* grid, const float* q, float* e64) { nrc_encode(*S, grid, q, e64); }

int lh2o_nrc_forward(const lh2o_nrc_spec* S, const float* grid, const float* mlp, const float* queries, long long n, float* out4, int emulate,
                     int nthreads) {
    if (!S || !grid || !mlp || !queries || !out4 || n < 0) return 1;
    parallel_for(n, nthreads, 256, [&](long long b, long long e) {
        float enc[64], act[5][64];
        double y[3];
        for (long long i = b; i < e; i++) {
            nrc_encode(*S, grid, queries + 16 * i, enc, emulate != 0);
            nrc_forward1(mlp, enc, act, y, emulate != 0);
            out4[4 * i] = (float)y[0], out4[4 * i + 1] = (float)y[1], out4[4 * i + 2] = (float)y[2], out4[4 * i + 3] = 0.0f;
        }
    });
    return 0;
}

int lh2o_nrc_forward64(const lh2o_nrc_spec* S, const float* grid, const float* mlp, const float* queries, long long n, double* out3) {
    if (!S || !grid || !mlp || !queries || !out3 || n < 0) return 1;
    float enc[64], act[5][64];
    for (long long i = 0; i < n; i++) {
        nrc_encode(*S, grid, queries + 16 * i, enc, false);
        nrc_forward1(mlp, enc, act, out3 + 3 * i, false);
    }
    return 0;
}

int lh2o_nrc_gradients(const lh2o_nrc_spec* S, const float* grid, const float* mlp, const float* queries, const float* targets, long long n,
                       int emulate, double* gMlp, double* gGrid, double* loss) {
    if (!S || !grid || !mlp || !queries || !targets || !gMlp || n <= 0) return 1;
    const double inv = 1.0 / (3.0 * (double)n);
    double L = 0.0;
    float enc[64], act[5][64];
    double y[3];
    for (long long i = 0; i < n; i++) {
        const float* q = queries + 16 * i;
        nrc_encode(*S, grid, q, enc, emulate != 0);
        nrc_forward1(mlp, enc, act, y, emulate != 0);
        /* relative L2: (y - t)^2 / (y^2 + 0.01), y constant in the denominator */
        double delta[64] = {0};
        for (int c = 0; c < 3; c++) {
            const float yf = (float)y[c];
            const double den = emulate ? (double)(yf * yf + 0.01f) : y[c] * y[c] + 0.01;
            const double e = y[c] - (double)targets[4 * i + c];
            L += e * e / den * inv;
            const double d = 2.0 * e / den * inv;
            delta[c] = emulate ? (double)bf16r((float)d) : d;
        }
        for (int j = 4; j >= 0; j--) {
            const int rows = j < 4 ? NRC_HID : 3;
            const float* W = mlp + (size_t)j * NRC_HID * NRC_IN;
            double* gW = gMlp + (size_t)j * NRC_HID * NRC_IN;
            for (int nn = 0; nn < rows; nn++)
                for (int k = 0; k < NRC_IN; k++) gW[nn * NRC_IN + k] += delta[nn] * (double)act[j][k];
            double g[64];
            for (int k = 0; k < NRC_IN; k++) {
                double sum = 0.0;
                for (int nn = 0; nn < rows; nn++) sum += delta[nn] * (double)(emulate ? bf16r(W[nn * NRC_IN + k]) : W[nn * NRC_IN + k]);
                g[k] = sum;
            }
            if (j > 0) {
                for (int k = 0; k < NRC_IN; k++) {
                    const double m = act[j][k] > 0.0f ? g[k] : 0.0;
                    delta[k] = emulate ? (double)bf16r((float)m) : m;
                }
            } else if (gGrid) {
                const f3 p = nrc_unit(*S, q);
                for (int l = 0; l < NRC_LEVELS; l++) {
                    const NrcCell c = nrc_cell(*S, l, p);
                    for (int corner = 0; corner < 8; corner++) {
                        const uint idx = nrc_index(*S, l, c.i + (corner & 1), c.j + ((corner >> 1) & 1), c.k + (corner >> 2));
                        const double w = nrc_weight(c, corner);
                        gGrid[((size_t)l * NRC_T + idx) * 2] += w * g[2 * l];
                        gGrid[((size_t)l * NRC_T + idx) * 2 + 1] += w * g[2 * l + 1];
                    }
                }
            }
        }
    }
    if (loss) *loss = L;
    return 0;
}

void lh2o_nrc_adam(float* p, float* m, float* v, const float* g, long long n, float lr, long long step) {
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-15f;
    const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)step))), c2 = (float)(1.0 / (1.0 - std::pow(0.99, (double)step)));
    for (long long i = 0; i < n; i++) {
        const float mi = b1 * m[i] + (1.0f - b1) * g[i];
        const float vi = b2 * v[i] + (1.0f - b2) * (g[i] * g[i]);
        p[i] = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        m[i] = mi, v[i] = vi;
    }
}

/* pure functions for the pinning tests */
uint32_t lh2o_pack_normal2(const float* n) { return PackNormal2(ld3(n)); }
void lh2o_unpack_normal2(uint32_t p, float* o) { const f3 n = UnpackNormal2(p); o[0] = n.x, o[1] = n.y, o[2] = n.z; }
uint32_t lh2o_hdr_to_rgb32(const float* c) { return HDRtoRGB32(ld3(c)); }
void lh2o_rgb32_to_hdr(uint32_t c, int min1, float* o) { const f3 v = min1 ? RGB32toHDRmin1(c) : RGB32toHDR(c); o[0] = v.x, o[1] = v.y, o[2] = v.z; }
void lh2o_combine_to_float4(const float* a, const float* b, float* o) { CombineToFloat4(ld3(a), ld3(b), o); }
void lh2o_split_float4(const float* x, float* d, float* i) {
    const f3 a = GetDirect(x), b = GetIndirect(x);
    d[0] = a.x, d[1] = a.y, d[2] = a.z, i[0] = b.x, i[1] = b.y, i[2] = b.z;
}
void lh2o_rgb_to_ycocg(const float* c, float* o) { const f3 v = RGBToYCoCg(ld3(c)); o[0] = v.x, o[1] = v.y, o[2] = v.z; }
void lh2o_ycocg_to_rgb(const float* c, float* o) { const f3 v = YCoCgToRGB(ld3(c)); o[0] = v.x, o[1] = v.y, o[2] = v.z; }
float lh2o_luminance(const float* c) { return Luminance(ld3(c)); }
float lh2o_mitchell_netravali(float v) { return MitchellNetravali(v); }
void lh2o_svgf_view(const lh2g_view* v, int h, float* out16) {
    const SvgfView r = svgf_view(*v, h);
    const f4 q[4] = {r.prevPos, r.prevE, r.prevRight, r.prevUp};
    for (int k = 0; k < 4; k++) out16[4 * k] = q[k].x, out16[4 * k + 1] = q[k].y, out16[4 * k + 2] = q[k].z, out16[4 * k + 3] = q[k].w;
}
uint32_t lh2o_wanghash(uint32_t v) { return WangHash(v); }
void lh2o_bluenoise4(const uint32_t* bn, int x, int y, int sampleIndex, int sampleDimension, float* out4) {
    const f4 r = blueNoiseSampler4(bn, x, y, sampleIndex, sampleDimension);
    out4[0] = r.x, out4[1] = r.y, out4[2] = r.z, out4[3] = r.w;
}
float lh2o_random_float(uint32_t* seed) { return RandomFloat(*seed); }
void lh2o_random_barycentrics(float r0, float* o) { const f3 b = RandomBarycentrics(r0); o[0] = b.x, o[1] = b.y, o[2] = b.z; }
uint32_t lh2o_pack_normal(const float* n) { return PackNormal(ld3(n)); }
void lh2o_unpack_normal(uint32_t p, float* o) { const f3 n = UnpackNormal(p); o[0] = n.x, o[1] = n.y, o[2] = n.z; }
void lh2o_diffuse_cos(float r0, float r1, float* o) { const f3 v = DiffuseReflectionCosWeighted(r0, r1); o[0] = v.x, o[1] = v.y, o[2] = v.z; }
void lh2o_tangent2world(const float* v, const float* n, float* o) { const f3 r = Tangent2World(ld3(v), ld3(n)); o[0] = r.x, o[1] = r.y, o[2] = r.z; }
void lh2o_consistent_normal(const float* d, const float* in, float alpha, float* o) { const f3 r = ConsistentNormal(ld3(d), ld3(in), alpha); o[0] = r.x, o[1] = r.y, o[2] = r.z; }
void lh2o_sincos(float x, float* s, float* c) { lm_sincos(x, s, c); }
float lh2o_logf(float x) { return lm_logf(x); }
float lh2o_powf(float x, float y) { return lm_powf(x, y); }
float lh2o_expf(float x) { return lm_expf(x); }
float lh2o_log2f(float x) { return lm_log2f(x); }
float lh2o_atan2f(float y, float x) { return lm_atan2f(y, x); }
float lh2o_acosf(float x) { return lm_acosf(x); }
uint16_t lh2o_float2half(float f) { return float2half(f); }
float lh2o_half2float(uint16_t h) { return half2float(h); }
void lh2o_pack_material(const lh2g_material* m, const uint32_t* first, const uint32_t* wh, lh2g_gpu_material* out) { pack_material(*m, first, wh, *out); }
void lh2o_invert4x4(const float* m, float* o) { invert4x4(m, o); }

int lh2o_raster(lh2o_scene* s, const lh2g_view* view, int W, int H, uint32_t* pixels, float* zbuffer, uint64_t* fragments) {
    if (!s || !view || !pixels || W < 3 || H < 3 || W > 8192 || H > 8192) return 1;
    for (const Instance& in : s->inst)
        for (const lh2g_core_tri& t : s->meshes[in.mesh].tris)
            if (t.material >= s->hostMats.size()) return 1;
    std::vector<float> zb;
    if (!zbuffer) zb.resize((size_t)W * H), zbuffer = zb.data();
    memset(pixels, 0, sizeof(uint) * (size_t)W * H);
    memset(zbuffer, 0, sizeof(float) * (size_t)W * H);
    f4 fr[5];
    rs_frustum(W, H, fr);
    RsTables tb;
    for (std::vector<float>* t : {&tb.xl, &tb.xr, &tb.ul, &tb.ur, &tb.vl, &tb.vr, &tb.zl, &tb.zr}) t->assign(H, 0.0f);
    for (int y = 0; y < H; y++) tb.xl[y] = (float)(W - 1), tb.xr[y] = 0.0f;
    const RsMesh4 root = rs_view(view);
    /* instances that share a mesh share its scene-graph node, whose transform is the one set last
     * (rendercore.cpp:118-131: the Mesh object is the child node and holds localTransform) */
    std::vector<const float*> meshT(s->meshes.size(), nullptr);
    for (const Instance& in : s->inst) meshT[in.mesh] = in.T;
    uint64_t frags = 0;
    for (const Instance& in : s->inst) {
        const RsMesh4 M = rs_mul(root.m, meshT[in.mesh]);
        frags += rs_mesh(*s, s->meshes[in.mesh], M.m, fr, W, H, tb, pixels, zbuffer);
    }
    if (fragments) *fragments = frags;
    return 0;
}

}  // extern "C"


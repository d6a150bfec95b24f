/* traverse.cuh - two-level BVH8 traversal (TLAS over instances, one BLAS per mesh).
 *
 * Replaces the closed OptiX / OptiX Prime ray queries of the reference (optixTrace,
 * lib/rendercore_optix7/optix/.optix.cu:125,136,148; rtpQueryExecute, lib/RenderCore_PrimeRef/rendercore.cpp:573,605).
 *
 * Results are independent of the tree: the closest hit is the smallest t among all triangles passing the
 * Moller-Trumbore test, ties broken by the lowest (instance, primitive); box tests only cull and are widened
 * (planes rounded outward at build time, t-interval widened by a relative 2^-16 here) so that they never
 * reject a box holding an accepted hit. The triangle test itself is the exact arithmetic of the oracle.
 *
 * Stack entries are (code, tnear): code bits 31..30 = 00 node index, 01 leaf (bits 29..28 = count - 1,
 * bits 27..0 = first slot), 10 instance index; 0xffffffff marks the return from an instance to the TLAS.
 */
#pragma once
#include "core_types.cuh"
#include "device_math.cuh"

namespace lh2g {

#ifndef LH2G_STACK
#define LH2G_STACK 80
#endif
constexpr float BOX_MARGIN = 1.52587890625e-05f;
constexpr uint32_t ENTRY_MARKER = 0xffffffffu;
constexpr uint32_t MAX_STEPS = 1u << 20;   /* far beyond any traversal of a well-formed tree */

struct HitRec { float t, u, v; int inst, prim; };

LH2G_DEV float safe_rcp(float d) { return fabsf(d) < 1e-30f ? (d < 0.0f ? -1e30f : 1e30f) : 1.0f / d; }

LH2G_DEV float3 xform_point(const float* m, float3 p) {
    return make_float3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
                       m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}
LH2G_DEV float3 xform_vector(const float* m, float3 v) {
    return make_float3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z, m[8] * v.x + m[9] * v.y + m[10] * v.z);
}

/* Moller-Trumbore, identical operation order to the oracle. */
LH2G_DEV bool isect_tri(const float3 O, const float3 D, const float4 a, const float4 b, const float4 c, float& t, float& u, float& v) {
    const float3 v0 = xyz(a), e1 = xyz(b), e2 = xyz(c);
    const float3 p = cross(D, e2);
    const float det = dot(e1, p);
    if (det == 0.0f) return false;
    const float inv = 1.0f / det;
    const float3 s = O - v0;
    u = dot(s, p) * inv;
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    const float3 q = cross(s, e1);
    v = dot(D, q) * inv;
    if (!(v >= 0.0f && u + v <= 1.0f)) return false;
    t = dot(e2, q) * inv;
    return true;
}

LH2G_DEV uint32_t byte_of(uint32_t w0, uint32_t w1, int i) { return ((i < 4 ? w0 : w1) >> ((i & 3) * 8)) & 255u; }

/* Resumable traversal state of one ray (one lane). step() processes the current stack entry and pops the
 * next one; it returns false once the ray is finished. Kernels interleave step() with per-lane refills of
 * finished rays, so a warp keeps all lanes busy instead of waiting for its slowest ray. */
struct Traversal {
    uint2 stack[LH2G_STACK];
    float3 Ow, Dw, O, D, invD;
    float tmin, tmax;
    int sp, curInst;
    uint32_t entry, steps;
    bool found;
    HitRec best;

    __device__ __forceinline__ void begin(const SceneGPU& S, const float3 o, const float3 d, const float t0, const float t1) {
        Ow = O = o, Dw = D = d, tmin = t0, tmax = t1;
        invD = make_float3(safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
        best.t = t1, best.u = best.v = 0.0f, best.inst = -1, best.prim = NOHIT;
        found = false, sp = 0, curInst = -1, steps = 0;
        entry = S.tlasRoot;
    }

    /* returns true while the ray has work left; anyHitDone is set when an any-hit query found an occluder */
    template <bool ANYHIT>
    __device__ __forceinline__ bool step(const SceneGPU& S, uint32_t& status, bool& anyHitDone) {
        if (entry == 0xffffffffu && sp == 0 && curInst < 0 && steps == 0) return false;   /* empty scene */
        if (++steps > MAX_STEPS) { status |= LH2G_STATUS_TRAVERSAL_LIMIT; return false; }
        const uint32_t kind = entry >> 30;
        if (entry == ENTRY_MARKER) {
            O = Ow, D = Dw;
            invD = make_float3(safe_rcp(Dw.x), safe_rcp(Dw.y), safe_rcp(Dw.z));
            curInst = -1;
        } else if (kind == 0u) {
            const uint4* np = S.nodes + (size_t)entry * 5;
            const uint4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3), n4 = __ldg(np + 4);
            const float px = __uint_as_float(n0.x), py = __uint_as_float(n0.y), pz = __uint_as_float(n0.z);
            const float sx = __uint_as_float((n0.w & 255u) << 23), sy = __uint_as_float(((n0.w >> 8) & 255u) << 23),
                        sz = __uint_as_float(((n0.w >> 16) & 255u) << 23);
            const float limit = (!ANYHIT && found) ? best.t : tmax;
            uint32_t keys[8], codes[8];
            uint32_t hitmask = 0;
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const uint32_t meta = byte_of(n1.z, n1.w, i);
                keys[i] = 0xffffffffu, codes[i] = 0;
                if (meta == 0u) continue;
                const float lx = fmaf((float)byte_of(n2.x, n2.y, i), sx, px), hx = fmaf((float)byte_of(n3.z, n3.w, i), sx, px);
                const float ly = fmaf((float)byte_of(n2.z, n2.w, i), sy, py), hy = fmaf((float)byte_of(n4.x, n4.y, i), sy, py);
                const float lz = fmaf((float)byte_of(n3.x, n3.y, i), sz, pz), hz = fmaf((float)byte_of(n4.z, n4.w, i), sz, pz);
                const float tx0 = (lx - O.x) * invD.x, tx1 = (hx - O.x) * invD.x;
                const float ty0 = (ly - O.y) * invD.y, ty1 = (hy - O.y) * invD.y;
                const float tz0 = (lz - O.z) * invD.z, tz1 = (hz - O.z) * invD.z;
                float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
                float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
                tn = fmaf(-fabsf(tn), BOX_MARGIN, tn);
                tf = fmaf(fabsf(tf), BOX_MARGIN, tf);
                tn = fmaxf(tn, tmin);
                tf = fminf(tf, limit);
                if (!(tn <= tf)) continue;
                hitmask |= 1u << i;
                keys[i] = __float_as_uint(fmaxf(tn, 0.0f));
                if (meta & 0x80u) codes[i] = n1.x + (meta & 7u);
                else {
                    const uint32_t first = n1.y + (meta & 31u), cnt = meta >> 5;
                    codes[i] = (curInst < 0 ? 0x80000000u : 0x40000000u) | ((cnt - 1u) << 28) | first;
                }
            }
            const int nh = __popc(hitmask);
            if (sp + nh > LH2G_STACK) status |= LH2G_STATUS_STACK_OVERFLOW;
            if (ANYHIT) {
                /* any hit: order does not matter */
#pragma unroll
                for (int i = 0; i < 8; i++)
                    if ((hitmask & (1u << i)) && sp < LH2G_STACK) stack[sp++] = make_uint2(codes[i], keys[i]);
            } else {
                /* closest hit: nearest child on top */
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    if (!(hitmask & (1u << i))) continue;
                    int rank = 0;
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        if (j == i || !(hitmask & (1u << j))) continue;
                        rank += (keys[j] < keys[i] || (keys[j] == keys[i] && j < i)) ? 1 : 0;
                    }
                    const int slot = sp + (nh - 1 - rank);
                    if (slot < LH2G_STACK) stack[slot] = make_uint2(codes[i], keys[i]);
                }
                sp = min(sp + nh, LH2G_STACK);
            }
        } else if (kind == 1u) {
            const uint32_t first = entry & 0x0fffffffu, cnt = ((entry >> 28) & 3u) + 1u;
            for (uint32_t k = 0; k < cnt; k++) {
                const float4* td = S.triData + (size_t)(first + k) * 3;
                const float4 a = __ldg(td), b = __ldg(td + 1), c = __ldg(td + 2);
                float t, u, v;
                if (!isect_tri(O, D, a, b, c, t, u, v)) continue;
                if (!(t > tmin && t < tmax)) continue;
                if (ANYHIT) { anyHitDone = true; return false; }
                const int prim = __float_as_int(a.w);
                if (!found || t < best.t || (t == best.t && (curInst < best.inst || (curInst == best.inst && prim < best.prim)))) {
                    best.t = t, best.u = u, best.v = v, best.inst = curInst, best.prim = prim;
                    found = true;
                }
            }
        } else {
            const uint32_t first = entry & 0x0fffffffu, cnt = ((entry >> 28) & 3u) + 1u;
            if (cnt > 1u && sp < LH2G_STACK) stack[sp++] = make_uint2(0x80000000u | ((cnt - 2u) << 28) | (first + 1u), 0u);
            const int ii = (int)__ldg(S.tlasPrims + first);
            const InstanceGPU* in = S.inst + ii;
            const uint32_t root = __ldg(&in->blasRoot);
            if (root != 0xffffffffu && sp < LH2G_STACK) {
                float m[12];
#pragma unroll
                for (int k = 0; k < 12; k++) m[k] = __ldg(&in->inv[k]);
                O = xform_point(m, Ow), D = xform_vector(m, Dw);
                invD = make_float3(safe_rcp(D.x), safe_rcp(D.y), safe_rcp(D.z));
                curInst = ii;
                stack[sp++] = make_uint2(ENTRY_MARKER, 0u);
                entry = root;
                return true;
            }
        }
        for (;;) {
            if (sp == 0) return false;
            const uint2 e = stack[--sp];
            entry = e.x;
            if (entry == ENTRY_MARKER || ANYHIT || (entry >> 30) == 2u) return true;
            if (!found || __uint_as_float(e.y) <= best.t) return true;
        }
    }
};

/* Single-ray form (used where lanes do not refill). */
template <bool ANYHIT>
LH2G_DEV bool trace_ray(const SceneGPU& S, const float3 Ow, const float3 Dw, const float tmin, const float tmax, HitRec& best, uint32_t& status) {
    Traversal tr;
    tr.begin(S, Ow, Dw, tmin, tmax);
    bool any = false;
    if (S.tlasRoot != 0xffffffffu)
        while (tr.step<ANYHIT>(S, status, any)) {}
    best = tr.best;
    return ANYHIT ? any : tr.found;
}

/* Persistent, self-refilling loop of a warp: every lane traverses its own ray; a lane whose ray finished takes
 * the next one from the queue (one atomic per warp per refill round, ballot + popc to hand out indices).
 * fetch is a 32-bit work counter; count the number of rays; onFinish(i, tr, anyHit) writes the result. */
template <bool ANYHIT, typename Load, typename Finish>
LH2G_DEV void trace_queue(const SceneGPU& S, uint32_t* fetch, const uint32_t count, uint32_t& status, Load load, Finish onFinish) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t lanemask_lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lanemask_lt));
    Traversal tr;
    uint32_t ray = 0;
    bool active = false, exhausted = false;
    if (S.tlasRoot == 0xffffffffu) {
        /* no geometry: every ray misses */
        for (;;) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(fetch, 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= count) return;
            const uint32_t i = base + lane;
            if (i < count) {
                float3 o, d;
                float t0, t1;
                load(i, o, d, t0, t1);
                tr.begin(S, o, d, t0, t1);
                onFinish(i, tr, false);
            }
        }
    }
    for (;;) {
        if (!exhausted) {
            const uint32_t need = __ballot_sync(0xffffffffu, !active);
            if (need) {
                const int leader = __ffs(need) - 1;
                uint32_t base = 0;
                if ((int)lane == leader) base = atomicAdd(fetch, (uint32_t)__popc(need));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (base + (uint32_t)__popc(need) >= count) exhausted = true;
                if (!active) {
                    const uint32_t i = base + __popc(need & lanemask_lt);
                    if (i < count) {
                        float3 o, d;
                        float t0, t1;
                        load(i, o, d, t0, t1);
                        tr.begin(S, o, d, t0, t1);
                        ray = i;
                        active = true;
                    }
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) return;
        if (active) {
            bool anyHit = false;
            if (!tr.step<ANYHIT>(S, status, anyHit)) {
                onFinish(ray, tr, anyHit);
                active = false;
            }
        }
    }
}

}  // namespace lh2g

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
 * With LH2G_GROUP_STACK an entry holds a node's remaining hit children instead (see there).
 */
#pragma once
#include "core_types.cuh"
#include "device_math.cuh"

namespace lh2g {

#ifndef LH2G_STACK
#define LH2G_STACK 80
#endif
/* Traversal strategy (tuning switches, all give identical results):
 *   LH2G_COOP        1: 8 lanes per ray (warp-cooperative), 0: one lane per ray
 *   LH2G_WHILE_WHILE 1: a lane descends interior nodes until it holds a leaf before leaf work; 0: one entry per step
 *   LH2G_REFILL      1: a lane takes a new ray as soon as its ray finishes; 0: a warp takes 32 rays at a time */
#ifndef LH2G_COOP
#define LH2G_COOP 0
#endif
#ifndef LH2G_WHILE_WHILE
#define LH2G_WHILE_WHILE 0
#endif
#ifndef LH2G_REFILL
#define LH2G_REFILL 0
#endif
/* LH2G_SPECULATIVE 1: a lane that reaches a triangle leaf while other lanes of its warp still visit interior
 * nodes sets the leaf aside and visits nodes too; it tests the leaf with the next one it reaches, before it leaves
 * the instance, or at the end of the ray (Aila and Laine's speculative traversal). 0: one entry per step. */
#ifndef LH2G_SPECULATIVE
#define LH2G_SPECULATIVE 0
#endif
/* LH2G_SORT_CHILDREN 1: a node's hit children go on the stack sorted by entry distance; 0: the nearest is visited
 * next, the others are pushed unsorted */
#ifndef LH2G_SORT_CHILDREN
#define LH2G_SORT_CHILDREN 1
#endif
/* LH2G_SORT_ANYHIT 1: any-hit queries push their hit children sorted too (nearest first); 0: in slot order */
#ifndef LH2G_SORT_ANYHIT
#define LH2G_SORT_ANYHIT 0
#endif
/* LH2G_GROUP_STACK 1: a node's hit children other than the one visited next go on the stack as ONE group entry
 * (child base, leaf base, the meta bytes of the children not yet taken) instead of one entry each; a pop takes the
 * group's lowest remaining slot and writes the rest back (after Ylitie, Karras and Laine, "Efficient Incoherent Ray
 * Traversal on GPUs Through Compressed Wide BVHs", HPG 2017). Closest-hit queries visit the nearest hit child
 * first and keep one entry distance per group, that of the nearest child, a lower bound of the others' for culling
 * on pop; any-hit queries take children in slot order, as with LH2G_SORT_ANYHIT 0. No sorting network, no
 * per-child push. LH2G_GSTACK entries of 20 B (one per level of the descent, plus instance markers). */
#ifndef LH2G_GROUP_STACK
#define LH2G_GROUP_STACK 0
#endif
#ifndef LH2G_GSTACK
#define LH2G_GSTACK 32
#endif
/* LH2G_SHORT_STACK K (a power of two, 0: off): the top K entries of a lane's stack live in shared memory, a ring of
 * K slots strided by the block size; older entries spill to the local-memory stack when the ring is full and are
 * popped back from there. Every kernel that traverses with it runs LH2G_TRAV_BLOCK threads per block. */
#ifndef LH2G_SHORT_STACK
#define LH2G_SHORT_STACK 0
#endif
#if LH2G_GROUP_STACK && (LH2G_COOP || LH2G_SHORT_STACK)
#error "LH2G_GROUP_STACK is a variant of the one-lane-per-ray traversal with the local-memory stack"
#endif
constexpr int LH2G_TRAV_BLOCK = 128;
/* tuning switch: resident CTAs per SM the traversal kernels (k_extend, k_connect and the serving loop's) are compiled
 * for, a register cap; 0 leaves it to the compiler (56 registers, 9 CTAs). 10 gives 48 registers without spills in
 * k_extend: 1867 against 1817 Mrays/s on the 1080p frame (11 and 12: 40 registers with spills, 1846 at 12). */
#ifndef LH2G_TRAV_MINBLOCKS
#define LH2G_TRAV_MINBLOCKS 10
#endif
#if LH2G_TRAV_MINBLOCKS > 0
#define LH2G_TRAV_BOUNDS __launch_bounds__(LH2G_TRAV_BLOCK, LH2G_TRAV_MINBLOCKS)
#else
#define LH2G_TRAV_BOUNDS __launch_bounds__(LH2G_TRAV_BLOCK)
#endif
/* the any-hit kernels' own cap (default: the same) */
#ifndef LH2G_CONNECT_MINBLOCKS
#define LH2G_CONNECT_MINBLOCKS LH2G_TRAV_MINBLOCKS
#endif
#if LH2G_CONNECT_MINBLOCKS > 0
#define LH2G_CONNECT_BOUNDS __launch_bounds__(LH2G_TRAV_BLOCK, LH2G_CONNECT_MINBLOCKS)
#else
#define LH2G_CONNECT_BOUNDS __launch_bounds__(LH2G_TRAV_BLOCK)
#endif
/* tuning switch: the plain core's wave traversal kernels' (k_extend, k_connect) preferred shared-memory carveout,
 * in percent of the SM's unified L1 / shared storage (-1: the driver's choice); they use no shared memory.
 * 0 (all of it L1): 1941-1947 against 1862-1868 Mrays/s on the 1080p frame with six frames in flight, where those
 * kernels run beside other frames' shading kernels (50: 1864); a kernel alone is a little slower with it
 * (k_extend of frames rendered one at a time 1.64 against 1.60 ms), so the ray-query and serving kernels keep
 * the driver's choice (with the hint: incoherent closest-hit queries -2.6 %, the small serving mix -2.5 %). */
#ifndef LH2G_TRAV_CARVEOUT
#define LH2G_TRAV_CARVEOUT 0
#endif
/* the same for the shading kernels (k_shade, k_tail), which hold the light potentials in dynamic shared memory
 * (100, all of it shared: 1897 Mrays/s, both kernels slower; 0: 1391-1397, k_shade 2.04 against 0.62 ms with fewer
 * CTAs resident; -1 stays) */
#ifndef LH2G_SHADE_CARVEOUT
#define LH2G_SHADE_CARVEOUT -1
#endif
/* LH2G_STAGE_RAYS 1: in the warp-batch loop (LH2G_REFILL 0, LH2G_COOP 0) the next 32 rays' path-state records
 * (the SoA arrays a kernel names: origins, directions, ...) are copied into the warp's shared-memory slot by bulk
 * asynchronous copies (cp.async.bulk, completion on an mbarrier) while the warp traces the current 32; 0 (the
 * default, measured faster): every lane loads its ray from global memory when its batch starts. The slots (4-6 KB
 * per CTA, 36-54 KB per SM) move the SM's shared-memory carve-out up and take that much L1 from the node and
 * triangle reads, and other warps already hide the direct loads' latency: k_extend took 2.00 ms per 1080p frame
 * with staging against 1.66 ms without (k_connect 1.40 against 1.32). */
#ifndef LH2G_STAGE_RAYS
#define LH2G_STAGE_RAYS 0
#endif
/* with LH2G_REFILL: idle lanes of a warp take new rays once at least this many are idle (or all are) */
#ifndef LH2G_REFILL_MIN
#define LH2G_REFILL_MIN 1
#endif
constexpr float BOX_MARGIN = 1.52587890625e-05f;
constexpr float SLAB_MARGIN = 1.71661376953125e-05f;   /* 2^-16 + 2^-19 */
constexpr uint32_t ENTRY_MARKER = 0xffffffffu;
constexpr uint32_t MAX_STEPS = 1u << 20;   /* far beyond any traversal of a well-formed tree */

struct HitRec { float t, u, v; int inst, prim; };

/* A NaN in a ray's origin, direction or interval makes it a miss without traversal: the box tests ignore NaN
 * operands (min / max return the other one), so such a ray would visit every box along its other axes, and with
 * an all-NaN direction the whole tree. The triangle test accepts no hit for it either way. */
LH2G_DEV bool ray_has_nan(const float3 o, const float3 d, const float t0, const float t1) {
    return o.x != o.x || o.y != o.y || o.z != o.z || d.x != d.x || d.y != d.y || d.z != d.z || t0 != t0 || t1 != t1;
}

/* 1 / d for the box tests, which only cull: the hardware reciprocal (at most 1 ulp off, which the slab margins
 * cover); |d| below 1e-30 (no denormal reaches rcp) gives +-1e30 */
LH2G_DEV float safe_rcp(float d) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(d));
    return fabsf(d) < 1e-30f ? (d < 0.0f ? -1e30f : 1e30f) : r;
}

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
/* byte i & 3 of w as a float, exactly: one byte permute builds the bits of 2^23 + byte (0x4B0000bb), one FADD
 * removes 2^23 (an integer-to-float conversion would run on the quarter-rate conversion pipe, 48 times per node) */
LH2G_DEV float plane_byte(uint32_t w, int i) { return __uint_as_float(__byte_perm(w, 0x4Bu, 0x4550u | (uint32_t)(i & 3))) - 8388608.0f; }
/* 1 + (byte i & 3 of w) * 2^-15, exactly: one byte permute builds the bits 0x3F80bb00 */
LH2G_DEV float plane_unit(uint32_t w, int i) { return __uint_as_float(__byte_perm(w, 0x3F80u, 0x5406u | ((uint32_t)(i & 3) << 4))); }

/* Compare-exchange for the sorting network. */
LH2G_DEV void cx(uint32_t& a, uint32_t& b) { const uint32_t lo = min(a, b), hi = max(a, b); a = lo, b = hi; }

/* Resumable traversal state of one ray (one lane). step() runs the interior-node loop until the lane holds a
 * leaf, an instance or a return marker (so a warp executes node work and leaf work in separate phases), handles
 * that entry and pops the next; it returns false once the ray is finished. Kernels interleave step() with
 * per-lane refills of finished rays. */
struct Traversal {
#if LH2G_GROUP_STACK
    static constexpr int CAP = LH2G_GSTACK;
    uint4 stack[LH2G_GSTACK];   /* group {child base, leaf base, meta bytes lo, hi}; single entry {code, 0, 0, 0} */
    float gnear[LH2G_GSTACK];   /* closest hit: a group's entry distance bound */
#else
    static constexpr int CAP = LH2G_STACK;
    uint2 stack[LH2G_STACK];
#endif
    float3 Ow, Dw, O, D, invD;
    float tmin, tmax;
    int sp, curInst;
#if LH2G_SHORT_STACK
    int base;   /* entries [0, base) are in the local stack, [base, sp) in the lane's shared ring */
    /* the lane's ring: slot j at ring()[j * LH2G_TRAV_BLOCK] (one ring per lane, shared by the lane's traversals) */
    static __device__ __forceinline__ uint2* ring() {
        __shared__ uint2 shortStack[LH2G_SHORT_STACK * LH2G_TRAV_BLOCK];
        return shortStack + threadIdx.x;
    }
#endif
    /* pushes one entry; the caller has checked sp < CAP */
    __device__ __forceinline__ void push(const uint2 e) {
#if LH2G_SHORT_STACK
        uint2* r = ring();
        if (sp - base == LH2G_SHORT_STACK) {
            stack[base] = r[(base & (LH2G_SHORT_STACK - 1)) * LH2G_TRAV_BLOCK];
            base++;
        }
        r[(sp & (LH2G_SHORT_STACK - 1)) * LH2G_TRAV_BLOCK] = e;
        sp++;
#elif LH2G_GROUP_STACK
        stack[sp++] = make_uint4(e.x, 0u, 0u, 0u);
#else
        stack[sp++] = e;
#endif
    }
    /* removes and returns the top entry; the caller has checked sp > 0 */
    __device__ __forceinline__ uint2 take() {
#if LH2G_SHORT_STACK
        if (sp == base) {
            base = --sp;
            return stack[sp];
        }
        --sp;
        return ring()[(sp & (LH2G_SHORT_STACK - 1)) * LH2G_TRAV_BLOCK];
#elif LH2G_GROUP_STACK
        return make_uint2(stack[--sp].x, 0u);
#else
        return stack[--sp];
#endif
    }
    uint32_t entry, steps, nodes, tris;
    uint32_t postponed;   /* LH2G_SPECULATIVE: a triangle leaf set aside (0: none) */
    bool found;
    HitRec best;

    __device__ __forceinline__ void begin(const SceneGPU& S, const float3 o, const float3 d, const float t0, const float t1) {
        Ow = O = o, Dw = D = d, tmin = t0, tmax = t1;
        invD = make_float3(safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
        best.t = t1, best.u = best.v = 0.0f, best.inst = -1, best.prim = NOHIT;
        found = false, sp = 0, curInst = -1, steps = 0, nodes = 0, tris = 0;
#if LH2G_SHORT_STACK
        base = 0;
#endif
        entry = ray_has_nan(o, d, t0, t1) ? ENTRY_MARKER : S.tlasRoot;   /* the marker step ends a NaN ray */
        postponed = 0u;
    }

    /* the triangles of a leaf entry; false when an any-hit query found an occluder */
    template <bool ANYHIT>
    __device__ __forceinline__ bool leaf(const SceneGPU& S, const uint32_t code, bool& anyHitDone) {
        const uint32_t first = code & 0x0fffffffu, cnt = ((code >> 28) & 3u) + 1u;
        for (uint32_t k = 0; k < cnt; k++) {
            const float4* td = S.triData + (size_t)(first + k) * 3;
            const float4 a = __ldg(td), b = __ldg(td + 1), c = __ldg(td + 2);
            float t, u, v;
            tris++;
            if (!isect_tri(O, D, a, b, c, t, u, v)) continue;
            if (!(t > tmin && t < tmax)) continue;
            if (ANYHIT) { anyHitDone = true; return false; }
            const int prim = __float_as_int(a.w);
            if (!found || t < best.t || (t == best.t && (curInst < best.inst || (curInst == best.inst && prim < best.prim)))) {
                best.t = t, best.u = u, best.v = v, best.inst = curInst, best.prim = prim;
                found = true;
            }
        }
        return true;
    }

    /* tests a set-aside leaf; false when an any-hit query found an occluder */
    template <bool ANYHIT>
    __device__ __forceinline__ bool flush(const SceneGPU& S, bool& anyHitDone) {
        if (!postponed) return true;
        const uint32_t p = postponed;
        postponed = 0u;
        return leaf<ANYHIT>(S, p, anyHitDone);
    }

    /* pops the next entry that can still hold a closer hit; false when the stack is empty */
    template <bool ANYHIT>
    __device__ __forceinline__ bool pop() {
#if LH2G_GROUP_STACK
        for (;;) {
            if (sp == 0) return false;
            const uint4 e = stack[sp - 1];
            if ((e.z | e.w) == 0u) {   /* a single entry: an instance marker or the rest of a TLAS leaf */
                sp--;
                entry = e.x;
                return true;
            }
            if (!ANYHIT && found && gnear[sp - 1] > fmaxf(best.t, 0.0f)) { sp--; continue; }
            /* the group's lowest remaining slot: its meta byte, then the rest written back (or the group dropped) */
            const bool lo = e.z != 0u;
            const uint32_t w = lo ? e.z : e.w;
            const uint32_t sh = (uint32_t)(__ffs(w) - 1) & ~7u;
            const uint32_t m = (w >> sh) & 255u, rest = w & ~(255u << sh);
            if ((rest | (lo ? e.w : 0u)) == 0u) sp--;
            else if (lo) stack[sp - 1].z = rest;
            else stack[sp - 1].w = rest;
            entry = (m & 0x80u) ? e.x + (m & 7u) : e.y + ((m >> 5) << 28) + (m & 31u);
            return true;
        }
#else
        for (;;) {
            if (sp == 0) return false;
            const uint2 e = take();
            entry = e.x;
            if (entry == ENTRY_MARKER || ANYHIT || (entry >> 30) == 2u) return true;
            /* e.y is the entry distance clamped to 0 and rounded down, a lower bound of the hits behind the entry
             * once both sides are clamped: with a negative tmin the best hit may lie behind the origin */
            if (!found || __uint_as_float(e.y) <= fmaxf(best.t, 0.0f)) return true;
        }
#endif
    }

    /* tests the 8 children of interior node `entry`. LH2G_SORT_CHILDREN 1: pushes the hit ones, nearest on top,
     * and returns false (the caller pops); 0: makes the nearest hit child the current entry, pushes the others
     * unsorted and returns true (false when nothing was hit). Either order visits every box the ray may hit. */
    template <bool ANYHIT>
    __device__ __forceinline__ bool visit_node(const SceneGPU& S, uint32_t& status) {
        const uint4* np = S.nodes + (size_t)entry * 5;
        const uint4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3), n4 = __ldg(np + 4);
        /* slab distances in the form t(q) = q * a + b, a = 2^e * invD (exact), b = (p - O) * invD */
        const float ax = __uint_as_float((n0.w & 255u) << 23) * invD.x, ay = __uint_as_float(((n0.w >> 8) & 255u) << 23) * invD.y,
                    az = __uint_as_float(((n0.w >> 16) & 255u) << 23) * invD.z;
        const float bx = (__uint_as_float(n0.x) - O.x) * invD.x, by = (__uint_as_float(n0.y) - O.y) * invD.y,
                    bz = (__uint_as_float(n0.z) - O.z) * invD.z;
        /* A plane byte q enters as v = 1 + q 2^-15, so t = q a + b = v A + (b - A) with A = 2^15 a (exact): one FMA
         * per plane. Widening folded into the offset, per axis: M = |b| + 255 |a| bounds |t| of every plane of the
         * axis; the rounding of the distances is below 2^-21 M + 2^-8 |a| (a few ulp of the operands, the roundings
         * of b - A - m (below 2^-23 (|b| + |A| + m)) and of the FMA); the margin wanted is 2^-16 |t|.
         * m = (2^-16 + 2^-19) M + 2^-7 |a| covers all of it. t - 2^-16 |t| is increasing in t, so the margin taken per
         * axis before the max (min) is the margin of the entry (exit) distance; a bound per axis, not the largest of
         * the three, keeps rays almost parallel to a plane (one huge |b|) from widening their other two slabs. An
         * overflowing A makes both distances of its axis NaN, which the min / max ignore: the box is kept. */
        const float Ax = ax * 32768.0f, Ay = ay * 32768.0f, Az = az * 32768.0f;
        const float mx = fmaf(fabsf(ax), 0.0078125f, fmaf(255.0f, fabsf(ax), fabsf(bx)) * SLAB_MARGIN),
                    my = fmaf(fabsf(ay), 0.0078125f, fmaf(255.0f, fabsf(ay), fabsf(by)) * SLAB_MARGIN),
                    mz = fmaf(fabsf(az), 0.0078125f, fmaf(255.0f, fabsf(az), fabsf(bz)) * SLAB_MARGIN);
        const float cx0 = bx - Ax, cy0 = by - Ay, cz0 = bz - Az;
        const float bxl = cx0 - mx, bxh = cx0 + mx, byl = cy0 - my, byh = cy0 + my, bzl = cz0 - mz, bzh = cz0 + mz;
        /* near / far plane words per axis, swapped for negative directions */
        const bool nx = invD.x < 0.0f, ny = invD.y < 0.0f, nz = invD.z < 0.0f;
        const uint32_t nlx0 = nx ? n3.z : n2.x, nlx1 = nx ? n3.w : n2.y, nhx0 = nx ? n2.x : n3.z, nhx1 = nx ? n2.y : n3.w;
        const uint32_t nly0 = ny ? n4.x : n2.z, nly1 = ny ? n4.y : n2.w, nhy0 = ny ? n2.z : n4.x, nhy1 = ny ? n2.w : n4.y;
        const uint32_t nlz0 = nz ? n4.z : n3.x, nlz1 = nz ? n4.w : n3.y, nhz0 = nz ? n3.x : n4.z, nhz1 = nz ? n3.y : n4.w;
        const float limit = (!ANYHIT && found) ? best.t : tmax;
        uint32_t key[8];
        const uint32_t metaLo = n1.z, metaHi = n1.w;
        uint32_t hlo = 0u, hhi = 0u;   /* LH2G_GROUP_STACK: 0xff in the bytes of the hit children */
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const uint32_t sel = 0x4440u | (uint32_t)(i & 3);
            const uint32_t meta = __byte_perm(i < 4 ? metaLo : metaHi, 0u, sel);
            const float txn = fmaf(plane_unit(i < 4 ? nlx0 : nlx1, i), Ax, bxl);
            const float txf = fmaf(plane_unit(i < 4 ? nhx0 : nhx1, i), Ax, bxh);
            const float tyn = fmaf(plane_unit(i < 4 ? nly0 : nly1, i), Ay, byl);
            const float tyf = fmaf(plane_unit(i < 4 ? nhy0 : nhy1, i), Ay, byh);
            const float tzn = fmaf(plane_unit(i < 4 ? nlz0 : nlz1, i), Az, bzl);
            const float tzf = fmaf(plane_unit(i < 4 ? nhz0 : nhz1, i), Az, bzh);
            const float tn = fmaxf(fmax3f(txn, tyn, tzn), tmin);
            const float tf = fminf(fmin3f(txf, tyf, tzf), limit);
            const bool hit = meta != 0u && tn <= tf;
            /* key: distance with the low 3 bits replaced by the slot (rounded down: culling stays conservative) */
            key[i] = hit ? ((__float_as_uint(fmaxf(tn, 0.0f)) & ~7u) | (uint32_t)i) : 0xffffffffu;
            if (LH2G_GROUP_STACK && hit) {
                if (i < 4) hlo |= 0xffu << (8 * (i & 3));
                else hhi |= 0xffu << (8 * (i & 3));
            }
        }
        /* leaf code = kind | (count - 1) << 28 | first slot; the fields do not overlap, so it is a sum */
        const uint32_t leafBase = (curInst < 0 ? 0x80000000u : 0x40000000u) - (1u << 28) + n1.y;
#if LH2G_GROUP_STACK
        nodes++;
        /* the hit children's meta bytes (a child's byte is never 0) */
        uint32_t glo = metaLo & hlo, ghi = metaHi & hhi;
        if ((glo | ghi) == 0u) return false;
        uint32_t first, near = 0u;
        if (ANYHIT) {
            first = glo ? (uint32_t)(__ffs(glo) - 1) >> 3 : 4u + ((uint32_t)(__ffs(ghi) - 1) >> 3);
        } else {
            const uint32_t b = min(min(min(key[0], key[1]), min(key[2], key[3])), min(min(key[4], key[5]), min(key[6], key[7])));
            first = b & 7u, near = b & ~7u;
        }
        const uint32_t sh = (first & 3u) * 8u;
        const uint32_t m = ((first < 4u ? glo : ghi) >> sh) & 255u;
        if (first < 4u) glo &= ~(255u << sh);
        else ghi &= ~(255u << sh);
        entry = (m & 0x80u) ? n1.x + (m & 7u) : leafBase + ((m >> 5) << 28) + (m & 31u);
        if ((glo | ghi) != 0u) {
            if (sp < LH2G_GSTACK) {
                stack[sp] = make_uint4(n1.x, leafBase, glo, ghi);
                if (!ANYHIT) gnear[sp] = __uint_as_float(near);
                sp++;
            } else {
                status |= LH2G_STATUS_STACK_OVERFLOW;
            }
        }
        return true;
#elif !LH2G_SORT_CHILDREN
        const uint32_t best = min(min(min(key[0], key[1]), min(key[2], key[3])), min(min(key[4], key[5]), min(key[6], key[7])));
        nodes++;
        if (best == 0xffffffffu) return false;
        {
            const uint32_t meta = __byte_perm(metaLo, metaHi, best & 7u) & 255u;
            entry = (meta & 0x80u) ? n1.x + (meta & 7u) : leafBase + ((meta >> 5) << 28) + (meta & 31u);
        }
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const uint32_t kk = key[k];
            if (kk == 0xffffffffu || kk == best) continue;
            const uint32_t meta = __byte_perm(metaLo, metaHi, kk & 7u) & 255u;
            const uint32_t code = (meta & 0x80u) ? n1.x + (meta & 7u) : leafBase + ((meta >> 5) << 28) + (meta & 31u);
            if (sp < LH2G_STACK) push(make_uint2(code, kk & ~7u));
            else status |= LH2G_STATUS_STACK_OVERFLOW;
        }
        return true;
#else
        if (!ANYHIT || LH2G_SORT_ANYHIT) {
            cx(key[0], key[1]), cx(key[2], key[3]), cx(key[4], key[5]), cx(key[6], key[7]);
            cx(key[0], key[2]), cx(key[1], key[3]), cx(key[4], key[6]), cx(key[5], key[7]);
            cx(key[1], key[2]), cx(key[5], key[6]);
            cx(key[0], key[4]), cx(key[1], key[5]), cx(key[2], key[6]), cx(key[3], key[7]);
            cx(key[2], key[4]), cx(key[3], key[5]);
            cx(key[1], key[2]), cx(key[3], key[4]), cx(key[5], key[6]);
        }
        if (sp + 8 <= LH2G_STACK) {
#pragma unroll
            for (int k = 7; k >= 0; k--) {
                const uint32_t kk = key[k];
                if (kk == 0xffffffffu) continue;
                const uint32_t meta = __byte_perm(metaLo, metaHi, kk & 7u) & 255u;   /* byte (slot) of the 8 meta bytes */
                const uint32_t code = (meta & 0x80u) ? n1.x + (meta & 7u) : leafBase + ((meta >> 5) << 28) + (meta & 31u);
                push(make_uint2(code, kk & ~7u));
            }
        } else {
#pragma unroll
            for (int k = 7; k >= 0; k--) {
                const uint32_t kk = key[k];
                if (kk == 0xffffffffu) continue;
                const uint32_t meta = __byte_perm(metaLo, metaHi, kk & 7u) & 255u;
                const uint32_t code = (meta & 0x80u) ? n1.x + (meta & 7u) : leafBase + ((meta >> 5) << 28) + (meta & 31u);
                if (sp < LH2G_STACK) push(make_uint2(code, kk & ~7u));
                else status |= LH2G_STATUS_STACK_OVERFLOW;
            }
        }
        nodes++;
        return false;
#endif
    }

    /* returns true while the ray has work left; anyHitDone is set when an any-hit query found an occluder */
    template <bool ANYHIT>
    __device__ __forceinline__ bool step(const SceneGPU& S, uint32_t& status, bool& anyHitDone) {
#if LH2G_WHILE_WHILE
        /* node phase: descend until the current entry is a leaf, an instance or a marker */
        while ((entry >> 30) == 0u) {
            if (++steps > MAX_STEPS) { status |= LH2G_STATUS_TRAVERSAL_LIMIT; return false; }
            if (!visit_node<ANYHIT>(S, status) && !pop<ANYHIT>()) return false;
        }
#elif LH2G_SPECULATIVE
        /* lanes of the warp that are at interior nodes now (a lane at a leaf joins them instead of idling) */
        const uint32_t atNode = __ballot_sync(__activemask(), (entry >> 30) == 0u);
        if ((entry >> 30) == 0u) {
            if (++steps > MAX_STEPS) { status |= LH2G_STATUS_TRAVERSAL_LIMIT; return false; }
            if (visit_node<ANYHIT>(S, status) || pop<ANYHIT>()) return true;
            flush<ANYHIT>(S, anyHitDone);   /* the stack is empty: the set-aside leaf ends the ray */
            return false;
        }
        if ((entry >> 30) == 1u) {
            if (++steps > MAX_STEPS) { status |= LH2G_STATUS_TRAVERSAL_LIMIT; return false; }
            if (!postponed && atNode) {
                postponed = entry;
            } else if (!leaf<ANYHIT>(S, entry, anyHitDone) || !flush<ANYHIT>(S, anyHitDone)) {
                return false;
            }
            if (pop<ANYHIT>()) return true;
            flush<ANYHIT>(S, anyHitDone);
            return false;
        }
        /* a marker or an instance changes the ray's space: the set-aside leaf (of the current space) goes first */
        if (!flush<ANYHIT>(S, anyHitDone)) return false;
#else
        if ((entry >> 30) == 0u) {
            if (++steps > MAX_STEPS) { status |= LH2G_STATUS_TRAVERSAL_LIMIT; return false; }
            return visit_node<ANYHIT>(S, status) || pop<ANYHIT>();
        }
#endif
        if (++steps > MAX_STEPS) { status |= LH2G_STATUS_TRAVERSAL_LIMIT; return false; }
        const uint32_t kind = entry >> 30;
        if (entry == ENTRY_MARKER) {
            O = Ow, D = Dw;
            invD = make_float3(safe_rcp(Dw.x), safe_rcp(Dw.y), safe_rcp(Dw.z));
            curInst = -1;
        } else if (kind == 1u) {
            if (!leaf<ANYHIT>(S, entry, anyHitDone)) return false;
        } else {
            const uint32_t first = entry & 0x0fffffffu, cnt = ((entry >> 28) & 3u) + 1u;
            /* a full stack drops work: the status word says so (the hit record may then be wrong) */
            if (cnt > 1u) {
                if (sp < CAP) push(make_uint2(0x80000000u | ((cnt - 2u) << 28) | (first + 1u), 0u));
                else status |= LH2G_STATUS_STACK_OVERFLOW;
            }
            const int ii = (int)__ldg(S.tlasPrims + first);
            /* an InstanceGPU is four aligned float4: the three rows of the inverse transform, then blasRoot */
            const float4* in = reinterpret_cast<const float4*>(S.inst + ii);
            const uint32_t root = __float_as_uint(__ldg(in + 3).x);
            if (root != 0xffffffffu && sp >= CAP) status |= LH2G_STATUS_STACK_OVERFLOW;
            if (root != 0xffffffffu && sp < CAP) {
                const float4 r0 = __ldg(in), r1 = __ldg(in + 1), r2 = __ldg(in + 2);
                const float m[12] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w};
                O = xform_point(m, Ow), D = xform_vector(m, Dw);
                invD = make_float3(safe_rcp(D.x), safe_rcp(D.y), safe_rcp(D.z));
                curInst = ii;
                push(make_uint2(ENTRY_MARKER, 0u));
                entry = root;
                return true;
            }
        }
        return pop<ANYHIT>();
    }
};

/* ======================================================================================================
 * Warp-cooperative traversal: a group of 8 lanes traces one ray, lane g testing child slot g of the current
 * 8-wide node (and triangle g of a leaf). The ray state is replicated in the group's lanes (identical
 * arithmetic, so all 8 copies agree and the group's control flow is uniform); the stack is shared by the group
 * and lives in shared memory. A finished group takes the next ray from the queue (one atomic per group).
 * ==================================================================================================== */
constexpr int COOP = 8;                      /* lanes per ray */
constexpr int COOP_STACK = 64;               /* shared-memory stack entries per group */

struct CoopRay {
    float3 Ow, Dw, O, D, invD, invDw;
    float tmin, tmax;
    int sp, curInst;
    uint32_t entry, steps, nodes, tris;
    bool found;
    HitRec best;
};

template <bool ANYHIT>
LH2G_DEV bool coop_pop(CoopRay& r, const uint2* stk) {
    for (;;) {
        if (r.sp == 0) return false;
        const uint2 e = stk[--r.sp];
        r.entry = e.x;
        if (e.x == ENTRY_MARKER || ANYHIT || (e.x >> 30) == 2u) return true;
        if (!r.found || __uint_as_float(e.y) <= fmaxf(r.best.t, 0.0f)) return true;   /* clamped like the key */
    }
}

/* One entry of the group's ray. g = lane within the group, gmask = the group's lanes. Returns false when the ray
 * is finished (anyHit set when an any-hit query found an occluder). */
template <bool ANYHIT>
LH2G_DEV bool coop_step(const SceneGPU& S, CoopRay& r, uint2* stk, const int g, const uint32_t gmask, uint32_t& status, bool& anyHit) {
    if (++r.steps > MAX_STEPS) { status |= LH2G_STATUS_TRAVERSAL_LIMIT; return false; }
    const uint32_t entry = r.entry, kind = entry >> 30;
    if (entry == ENTRY_MARKER) {
        r.O = r.Ow, r.D = r.Dw, r.invD = r.invDw, r.curInst = -1;
    } else if (kind == 0u) {
        const uint4* np = S.nodes + (size_t)entry * 5;
        const uint4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3), n4 = __ldg(np + 4);
        const float3 invD = r.invD, O = r.O;
        const float ax = __uint_as_float((n0.w & 255u) << 23) * invD.x, ay = __uint_as_float(((n0.w >> 8) & 255u) << 23) * invD.y,
                    az = __uint_as_float(((n0.w >> 16) & 255u) << 23) * invD.z;
        const float bx = (__uint_as_float(n0.x) - O.x) * invD.x, by = (__uint_as_float(n0.y) - O.y) * invD.y,
                    bz = (__uint_as_float(n0.z) - O.z) * invD.z;
        const float err = (fmaxf(fmaxf(fabsf(bx), fabsf(by)), fabsf(bz)) + 255.0f * fmaxf(fmaxf(fabsf(ax), fabsf(ay)), fabsf(az))) * 9.5367431640625e-07f;
        const uint32_t sel = 0x4440u | (uint32_t)(g & 3), hi = g >= 4;
        const uint32_t meta = __byte_perm(hi ? n1.w : n1.z, 0u, sel);
        const float qlx = plane_byte(hi ? n2.y : n2.x, g), qhx = plane_byte(hi ? n3.w : n3.z, g);
        const float qly = plane_byte(hi ? n2.w : n2.z, g), qhy = plane_byte(hi ? n4.y : n4.x, g);
        const float qlz = plane_byte(hi ? n3.y : n3.x, g), qhz = plane_byte(hi ? n4.w : n4.z, g);
        const float tx0 = fmaf(qlx, ax, bx), tx1 = fmaf(qhx, ax, bx);
        const float ty0 = fmaf(qly, ay, by), ty1 = fmaf(qhy, ay, by);
        const float tz0 = fmaf(qlz, az, bz), tz1 = fmaf(qhz, az, bz);
        float tn = fmax3f(fminf(tx0, tx1), fminf(ty0, ty1), fminf(tz0, tz1));
        float tf = fmin3f(fmaxf(tx0, tx1), fmaxf(ty0, ty1), fmaxf(tz0, tz1));
        tn = fmaf(-fabsf(tn), BOX_MARGIN, tn) - err;
        tf = fmaf(fabsf(tf), BOX_MARGIN, tf) + err;
        tn = fmaxf(tn, r.tmin);
        tf = fminf(tf, (!ANYHIT && r.found) ? r.best.t : r.tmax);
        const bool hit = meta != 0u && tn <= tf;
        const uint32_t key = hit ? ((__float_as_uint(fmaxf(tn, 0.0f)) & ~7u) | (uint32_t)g) : 0xffffffffu;
        const uint32_t bal = __ballot_sync(gmask, hit);
        const int nh = __popc(bal);
        int rank;
        if (ANYHIT) {
            rank = __popc(bal & gmask & ((1u << (threadIdx.x & 31)) - 1u));
        } else {
            rank = 0;
#pragma unroll
            for (int j = 0; j < COOP; j++) rank += __shfl_sync(gmask, key, j, COOP) < key ? 1 : 0;
        }
        if (r.sp + nh > COOP_STACK) status |= LH2G_STATUS_STACK_OVERFLOW;
        if (hit) {
            uint32_t code;
            if (meta & 0x80u) code = n1.x + (meta & 7u);
            else code = (r.curInst < 0 ? 0x80000000u : 0x40000000u) | (((meta >> 5) - 1u) << 28) | (n1.y + (meta & 31u));
            const int slot = r.sp + nh - 1 - rank;
            if (slot < COOP_STACK) stk[slot] = make_uint2(code, key & ~7u);
        }
        __syncwarp(gmask);
        r.sp = min(r.sp + nh, COOP_STACK);
        r.nodes++;
    } else if (kind == 1u) {
        const uint32_t first = entry & 0x0fffffffu, cnt = ((entry >> 28) & 3u) + 1u;
        float t = 0.0f, u = 0.0f, v = 0.0f;
        bool ok = false;
        int prim = 0x7fffffff;
        if ((uint32_t)g < cnt) {
            const float4* td = S.triData + (size_t)(first + g) * 3;
            const float4 a = __ldg(td), b = __ldg(td + 1), c = __ldg(td + 2);
            ok = isect_tri(r.O, r.D, a, b, c, t, u, v) && t > r.tmin && t < r.tmax;
            prim = __float_as_int(a.w);
        }
        r.tris += cnt;
        if (ANYHIT) {
            if (__ballot_sync(gmask, ok)) { anyHit = true; return false; }
        } else {
            /* closest among the group's triangles (t, then primitive), then against the best so far */
            if (!ok) t = __int_as_float(0x7f800000), prim = 0x7fffffff;
#pragma unroll
            for (int off = 1; off < COOP; off <<= 1) {
                const float ot = __shfl_xor_sync(gmask, t, off, COOP), ou = __shfl_xor_sync(gmask, u, off, COOP), ov = __shfl_xor_sync(gmask, v, off, COOP);
                const int op = __shfl_xor_sync(gmask, prim, off, COOP);
                const bool ook = __shfl_xor_sync(gmask, ok ? 1 : 0, off, COOP) != 0;
                if (ook && (!ok || ot < t || (ot == t && op < prim))) t = ot, u = ou, v = ov, prim = op, ok = true;
            }
            if (ok && (!r.found || t < r.best.t || (t == r.best.t && (r.curInst < r.best.inst || (r.curInst == r.best.inst && prim < r.best.prim))))) {
                r.best.t = t, r.best.u = u, r.best.v = v, r.best.inst = r.curInst, r.best.prim = prim;
                r.found = true;
            }
        }
    } else {
        const uint32_t first = entry & 0x0fffffffu, cnt = ((entry >> 28) & 3u) + 1u;
        if (cnt > 1u && r.sp < COOP_STACK) {
            if (g == 0) stk[r.sp] = make_uint2(0x80000000u | ((cnt - 2u) << 28) | (first + 1u), 0u);
            __syncwarp(gmask);
            r.sp++;
        } else if (cnt > 1u) {
            status |= LH2G_STATUS_STACK_OVERFLOW;
        }
        const int ii = (int)__ldg(S.tlasPrims + first);
        const InstanceGPU* in = S.inst + ii;
        const uint32_t root = __ldg(&in->blasRoot);
        if (root != 0xffffffffu && r.sp >= COOP_STACK) status |= LH2G_STATUS_STACK_OVERFLOW;
        if (root != 0xffffffffu && r.sp < COOP_STACK) {
            float m[12];
#pragma unroll
            for (int k = 0; k < 12; k++) m[k] = __ldg(&in->inv[k]);
            r.O = xform_point(m, r.Ow), r.D = xform_vector(m, r.Dw);
            r.invD = make_float3(safe_rcp(r.D.x), safe_rcp(r.D.y), safe_rcp(r.D.z));
            r.curInst = ii;
            if (g == 0) stk[r.sp] = make_uint2(ENTRY_MARKER, 0u);
            __syncwarp(gmask);
            r.sp++;
            r.entry = root;
            return true;
        }
    }
    return coop_pop<ANYHIT>(r, stk);
}

/* Persistent queue loop of a warp with 4 cooperative groups. stackBase: the block's shared stack storage
 * (COOP_STACK entries per group). load(i, o, d, t0, t1) reads ray i; onFinish(i, r, anyHit) is called by every
 * lane of the group (write from one lane). */
template <bool ANYHIT, typename Load, typename Finish>
LH2G_DEV void trace_queue_coop(const SceneGPU& S, uint32_t* fetch, const uint32_t count, uint32_t& status, uint2* stackBase, Load load,
                               Finish onFinish, unsigned long long* stats = nullptr) {
    const int lane = threadIdx.x & 31, g = lane & (COOP - 1), grp = lane / COOP;
    const uint32_t gmask = 0xffu << (grp * COOP);
    uint2* stk = stackBase + (threadIdx.x / COOP) * COOP_STACK;
    unsigned long long nodeSum = 0, triSum = 0;
    CoopRay r;
    uint32_t ray = 0;
    bool active = false, exhausted = false;
    for (;;) {
        if (!active && !exhausted) {
            uint32_t i = 0;
            if (g == 0) i = atomicAdd(fetch, 1u);
            i = __shfl_sync(gmask, i, 0, COOP);
            if (i < count) {
                float3 o, d;
                float t0, t1;
                load(i, o, d, t0, t1);
                r.Ow = r.O = o, r.Dw = r.D = d, r.tmin = t0, r.tmax = t1;
                r.invDw = r.invD = make_float3(safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
                r.best.t = t1, r.best.u = r.best.v = 0.0f, r.best.inst = -1, r.best.prim = NOHIT;
                r.found = false, r.sp = 0, r.curInst = -1, r.steps = 0, r.nodes = 0, r.tris = 0;
                r.entry = S.tlasRoot;
                ray = i;
                active = true;
                if (S.tlasRoot == 0xffffffffu || ray_has_nan(o, d, t0, t1)) { onFinish(ray, r, false); active = false; }
            } else {
                exhausted = true;
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (active) {
            bool anyHit = false;
            if (!coop_step<ANYHIT>(S, r, stk, g, gmask, status, anyHit)) {
                onFinish(ray, r, anyHit);
                if (g == 0) nodeSum += r.nodes, triSum += r.tris;
                active = false;
            }
        }
    }
    if (stats) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) nodeSum += __shfl_xor_sync(0xffffffffu, nodeSum, off), triSum += __shfl_xor_sync(0xffffffffu, triSum, off);
        if (lane == 0) atomicAdd(stats, nodeSum), atomicAdd(stats + 1, triSum);
    }
}

/* ---- the warp-batch loop with path-state records staged by bulk copies ----
 * trace_queue's warp-batch form (a warp takes 32 consecutive rays, the first batch by its index, later ones from
 * the shared counter) with the loads moved off the warps: while a warp traces batch k, lane 0 has already fetched
 * the index of batch k + 1 and issued one cp.async.bulk per named SoA array (32 x 16 bytes, or fewer at the
 * queue's end) into the warp's slot, completing on the warp's mbarrier. A batch's records are read from the slot
 * into registers before the next copy into it is issued, so one slot per warp suffices. The rays and their results
 * are those of trace_queue (every index below count traced once, results written by index).
 * Waits are bounded: a copy not complete after STAGE_WAIT_LIMIT polls sets LH2G_STATUS_COPY_TIMEOUT, the batch is
 * skipped, the warp waits (bounded again) for the copy and leaves the loop. */
constexpr uint32_t STAGE_WAIT_LIMIT = 1u << 22;
constexpr int STAGE_WARPS = LH2G_TRAV_BLOCK / 32;

LH2G_DEV uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
LH2G_DEV bool stage_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t k = 0; k < STAGE_WAIT_LIMIT; k++) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}
/* lane 0: the records [base, base + n) of each array into the slot, n = min(32, count - base) */
template <int NARR>
LH2G_DEV void stage_issue(const float4* const (&src)[NARR], float4 (*slot)[32], uint32_t bar, uint32_t base, uint32_t n) {
    const uint32_t bytes = n * 16u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   /* the slot's earlier reads before the copy's writes */
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes * NARR) : "memory");
#pragma unroll
    for (int a = 0; a < NARR; a++)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(smem_u32(slot[a])), "l"((unsigned long long)__cvta_generic_to_global(src[a] + base)), "r"(bytes), "r"(bar)
                     : "memory");
}

/* conv(i, v, o, d, t0, t1): the ray of index i from its NARR records v[0..NARR-1] (src[a][i] each) */
template <bool ANYHIT, int NARR, typename Conv, typename Finish>
LH2G_DEV void trace_queue_staged(const SceneGPU& S, uint32_t* fetch, const uint32_t count, uint32_t& status, const float4* const (&src)[NARR],
                                 Conv conv, Finish onFinish, unsigned long long* stats = nullptr) {
    __shared__ __align__(128) float4 slots[STAGE_WARPS][NARR][32];
    __shared__ __align__(8) uint64_t bars[STAGE_WARPS];
    unsigned long long nodeSum = 0, triSum = 0;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    float4 (*slot)[32] = slots[warp];
    const uint32_t bar = smem_u32(&bars[warp]);
    if (lane == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    const uint32_t firstRound = gridDim.x * blockDim.x;
    uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u, parity = 0;
    if (base < count && lane == 0) stage_issue<NARR>(src, slot, bar, base, min(32u, count - base));
    Traversal tr;
    while (base < count) {   /* warp-uniform */
        if (!__all_sync(0xffffffffu, stage_wait(bar, parity))) {   /* (the warp leaves together) */
            status |= LH2G_STATUS_COPY_TIMEOUT;
            stage_wait(bar, parity);   /* the copy may still write the slot */
            break;
        }
        parity ^= 1u;
        const uint32_t i = base + lane;
        float3 o, d;
        float t0 = 0.0f, t1 = 0.0f;
        if (i < count) {
            float4 v[NARR];
#pragma unroll
            for (int a = 0; a < NARR; a++) v[a] = slot[a][lane];
            conv(i, v, o, d, t0, t1);
        }
        __syncwarp();   /* every lane holds its records: the slot is free */
        uint32_t next = count;
        if (firstRound < count) {
            if (lane == 0) next = firstRound + atomicAdd(fetch, 32u);
            next = __shfl_sync(0xffffffffu, next, 0);
        }
        if (next < count && lane == 0) stage_issue<NARR>(src, slot, bar, next, min(32u, count - next));
        if (i < count) {
            tr.begin(S, o, d, t0, t1);
            bool anyHit = false;
            if (S.tlasRoot != 0xffffffffu)
                while (tr.step<ANYHIT>(S, status, anyHit)) {}
            onFinish(i, tr, anyHit);
            nodeSum += tr.nodes, triSum += tr.tris;
        }
        __syncwarp();
        base = next;
    }
    if (stats) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) nodeSum += __shfl_xor_sync(0xffffffffu, nodeSum, off), triSum += __shfl_xor_sync(0xffffffffu, triSum, off);
        if (lane == 0) atomicAdd(stats, nodeSum), atomicAdd(stats + 1, triSum);
    }
}

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
LH2G_DEV void trace_queue(const SceneGPU& S, uint32_t* fetch, const uint32_t count, uint32_t& status, Load load, Finish onFinish,
                          unsigned long long* stats = nullptr) {
    unsigned long long nodeSum = 0, triSum = 0;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t lanemask_lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lanemask_lt));
    Traversal tr;
    uint32_t ray = 0;
    bool active = false, exhausted = false;
    if (S.tlasRoot == 0xffffffffu || !LH2G_REFILL) {
        /* a warp takes 32 rays at a time and traces each to the end (also used when there is no geometry). The
         * first 32 rays of a warp are fixed by its index, later ones come from the shared counter: a short queue
         * costs no atomics at all, a long one is still balanced dynamically. */
        const uint32_t firstRound = gridDim.x * blockDim.x;
        uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
        for (bool first = true;; first = false) {
            if (!first) {
                if (firstRound >= count) break;
                if (lane == 0) base = firstRound + atomicAdd(fetch, 32u);
                base = __shfl_sync(0xffffffffu, base, 0);
            }
            if (base >= count) break;   /* warp-uniform */
            const uint32_t i = base + lane;
            if (i < count) {
                float3 o, d;
                float t0, t1;
                load(i, o, d, t0, t1);
                tr.begin(S, o, d, t0, t1);
                bool anyHit = false;
                if (S.tlasRoot != 0xffffffffu)
                    while (tr.step<ANYHIT>(S, status, anyHit)) {}
                onFinish(i, tr, anyHit);
                nodeSum += tr.nodes, triSum += tr.tris;
            }
        }
        if (stats) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) nodeSum += __shfl_xor_sync(0xffffffffu, nodeSum, off), triSum += __shfl_xor_sync(0xffffffffu, triSum, off);
            if (lane == 0) atomicAdd(stats, nodeSum), atomicAdd(stats + 1, triSum);
        }
        return;
    }
    for (;;) {
        if (!exhausted) {
            const uint32_t need = __ballot_sync(0xffffffffu, !active);
            if (need && (__popc(need) >= LH2G_REFILL_MIN || need == 0xffffffffu)) {
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
        if (!__any_sync(0xffffffffu, active)) break;
        if (active) {
            bool anyHit = false;
            if (!tr.step<ANYHIT>(S, status, anyHit)) {
                onFinish(ray, tr, anyHit);
                nodeSum += tr.nodes, triSum += tr.tris;
                active = false;
            }
        }
    }
    if (stats) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) nodeSum += __shfl_xor_sync(0xffffffffu, nodeSum, off), triSum += __shfl_xor_sync(0xffffffffu, triSum, off);
        if (lane == 0) atomicAdd(stats, nodeSum), atomicAdd(stats + 1, triSum);
    }
}

/* The queue loop of the configured strategy. */
template <bool ANYHIT, typename Load, typename FinishT, typename FinishC>
LH2G_DEV void trace_queue_any(const SceneGPU& S, uint32_t* fetch, const uint32_t count, uint32_t& status, uint2* stackBase, Load load,
                              FinishT finishThread, FinishC finishCoop, unsigned long long* stats) {
#if LH2G_COOP
    trace_queue_coop<ANYHIT>(S, fetch, count, status, stackBase, load, finishCoop, stats);
#else
    trace_queue<ANYHIT>(S, fetch, count, status, load, finishThread, stats);
#endif
}

}  // namespace lh2g

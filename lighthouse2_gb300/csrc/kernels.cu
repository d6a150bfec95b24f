/* kernels.cu - wavefront path-tracing stages and ray-query kernels of the GB300 render core.
 *
 * Stage structure of the reference's wave loop (lib/RenderCore_PrimeRef/rendercore.cpp:551-611,
 * lib/rendercore_optix7/rendercore.cpp:878-922), rebuilt for one GB300:
 *   generate  primary rays (lib/RenderCore_PrimeRef/kernels/camera.h:39-68)
 *   extend    closest hit of every ray in the current queue (persistent warps fetching 32 rays at a time)
 *   shade     one thread per path (lib/RenderCore_PrimeRef/kernels/pathtracer.h:45-168); extension rays and
 *             connections are compacted into the next queues by warp ballot + popc with one atomic per warp
 *   connect   any hit of every connection; unoccluded ones add their contribution (connections.h:22-34)
 *   finalize  per-pixel sum of the frame's samples in sample order, scaled by 1 / samples (finalize_shared.h:29-45)
 *   tail      from a chosen path length on, the few remaining paths run to their end in one persistent kernel
 * Queue sizes live in device counters; no stage waits for the host, so a frame is a fixed launch sequence.
 * Radiance is accumulated per path (each path is owned by exactly one thread per stage), so the result does
 * not depend on the order in which the queues were filled.
 */
#include "kernels.cuh"
#include "wavefront.cuh"

namespace lh2g {

namespace {


/* -------------------------------------------------------------------------------------------------- */
__global__ void __launch_bounds__(256) k_generate(const FrameGPU F, const WaveBuffers B) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F.P) return;
    const uint32_t p = primary_slot_path(F, (uint32_t)i);
    float3 O, D;
    primary_ray(F, p, O, D);
    B.O[0][i] = make_float4(O.x, O.y, O.z, __uint_as_float(p));
    B.D[0][i] = make_float4(D.x, D.y, D.z, __uint_as_float(S_SPECULAR));
    B.T[0][i] = make_float4(1.0f, 1.0f, 1.0f, F.eps);
    B.pathAcc[p] = make_float4(0, 0, 0, 0);
    if (F.flags & LH2G_RP_FILTER) B.pathAcc[p + F.P] = make_float4(0, 0, 0, 0);
    if (F.flags & LH2G_RP_NRC) B.nrcRec[p + 4 * F.P] = make_float4(0, 0, 0, 0);   /* no cache query yet */
}
/* primary rays of the OptiX 7 estimator, or the first wave of a PrimeAdaptive frame (sample layers of W*H paths) */
__global__ void __launch_bounds__(256) k_generate_mis(const SceneGPU S, const FrameGPU F, const WaveBuffers B) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F.P) return;
    float3 O, D;
    const bool adaptive = (F.flags & LH2G_RP_ADAPTIVE) != 0;
    uint32_t p = (uint32_t)i;   /* the path's slot (adaptive frames keep path order: their second wave maps slots to layers) */
    if (adaptive) {
        const uint32_t row = (uint32_t)i / (uint32_t)F.W;
        primary_adaptive(S, F, (int)((uint32_t)i % (uint32_t)F.W), (int)(row % (uint32_t)F.H), F.pass + row / (uint32_t)F.H, (uint32_t)i, F.cameraR0, O, D);
    } else {
        p = primary_slot_path(F, (uint32_t)i);
        primary_optix7(S, F, p, O, D);
    }
    B.O[0][i] = make_float4(O.x, O.y, O.z, __uint_as_float((p << 6) | S_SPECULAR | MIS_TMIN_EPS));
    B.D[0][i] = make_float4(D.x, D.y, D.z, __uint_as_float(0u));
    B.T[0][i] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    B.pathAcc[p] = make_float4(0.0f, 0.0f, 0.0f, adaptive ? 1.0f : 0.0f);   /* PrimeAdaptive: w counts the pixel's samples */
}
__device__ __forceinline__ uint32_t queue_count(const FrameGPU& F, const WaveBuffers& B, const Counters* C, int depth) {
    return depth == 1 ? (B.firstCount ? *B.firstCount : (uint32_t)F.P) : C->extension[depth - 2];
}

/* -------------------------------------------------------------------------------------------------- */
template <bool MIS>
__global__ void LH2G_TRAV_BOUNDS k_extend(const SceneGPU S, const FrameGPU F, const WaveBuffers B, const int depth) {
    Counters* C = B.counters;
    const uint32_t count = queue_count(F, B, C, depth);
    const int q = (depth - 1) & 1;
    const float4* __restrict__ O4 = B.O[q];
    const float4* __restrict__ D4 = B.D[q];
    const float4* __restrict__ T4 = B.T[q];
    uint32_t status = 0;
    __shared__ uint2 stackBase[LH2G_COOP ? 128 / COOP * COOP_STACK : 1];
    auto write = [&](uint32_t i, bool found, const HitRec& best) {
        float4 rec;
        if (found) rec = make_float4(__uint_as_float(f2u(65535.0f * best.u) + (f2u(65535.0f * best.v) << 16)), __int_as_float(best.inst),
                                     __int_as_float(best.prim), best.t);
        else rec = make_float4(__uint_as_float(0u), __int_as_float(0), __int_as_float(NOHIT), 1e34f);
        B.hits[i] = rec;
        if (B.capHits) {
            const uint32_t pathIdx = MIS ? __float_as_uint(O4[i].w) >> 6 : __float_as_uint(O4[i].w);
            lh2g_hit c;
            c.bary = __float_as_uint(rec.x), c.inst = __float_as_int(rec.y), c.prim = __float_as_int(rec.z), c.t = rec.w;
            B.capHits[(size_t)(depth - 1) * F.P + pathIdx] = c;
        }
    };
#if LH2G_STAGE_RAYS && !LH2G_COOP && !LH2G_REFILL
    (void)stackBase;
    if constexpr (MIS) {   /* origins (w: path slot and flags, tmin) and directions */
        const float4* const src[2] = {O4, D4};
        trace_queue_staged<false, 2>(S, &C->fetch[depth - 1], count, status, src,
            [&](uint32_t, const float4 (&v)[2], float3& o, float3& d, float& t0, float& t1) {
                o = xyz(v[0]), d = xyz(v[1]), t0 = mis_tmin(__float_as_uint(v[0].w), F.eps), t1 = 1e34f;
            },
            [&](uint32_t i, const Traversal& tr, bool) { write(i, tr.found, tr.best); }, C->travStats);
    } else {   /* origins, directions, throughput (w: tmin) */
        const float4* const src[3] = {O4, D4, T4};
        trace_queue_staged<false, 3>(S, &C->fetch[depth - 1], count, status, src,
            [&](uint32_t, const float4 (&v)[3], float3& o, float3& d, float& t0, float& t1) {
                o = xyz(v[0]), d = xyz(v[1]), t0 = v[2].w, t1 = 1e34f;
            },
            [&](uint32_t i, const Traversal& tr, bool) { write(i, tr.found, tr.best); }, C->travStats);
    }
#else
    trace_queue_any<false>(S, &C->fetch[depth - 1], count, status, stackBase,
        [&](uint32_t i, float3& o, float3& d, float& t0, float& t1) {
            if (MIS) {
                const float4 a = O4[i];
                o = xyz(a), d = xyz(D4[i]), t0 = mis_tmin(__float_as_uint(a.w), F.eps), t1 = 1e34f;
            } else {
                o = xyz(O4[i]), d = xyz(D4[i]), t0 = T4[i].w, t1 = 1e34f;
            }
        },
        [&](uint32_t i, const Traversal& tr, bool) { write(i, tr.found, tr.best); },
        [&](uint32_t i, const CoopRay& tr, bool) { if ((threadIdx.x & (COOP - 1)) == 0) write(i, tr.found, tr.best); },
        C->travStats);
#endif
    if (status) atomicOr(&C->status, status);
}

/* -------------------------------------------------------------------------------------------------- */
template <bool MIS>
__device__ __forceinline__ void shade_path(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, const int depth, const uint32_t i, ShadeOut& out,
                                           float* pot) {
    const int q = (depth - 1) & 1;
    if (MIS) shade_mis(S, F, B, depth, B.O[q][i], B.D[q][i], B.T[q][i], B.hits[i], out, pot);
    else shade_core(S, F, B, depth, B.O[q][i], B.D[q][i], B.T[q][i], B.hits[i], out, pot);
}

/* the shading order of the extension queue of path length `depth` (partition_queue) */
__global__ void __launch_bounds__(PART_TILE) k_partition(const FrameGPU F, const WaveBuffers B, const int depth) {
    Counters* C = B.counters;
    partition_queue(B.hits, queue_count(F, B, C, depth), B.order, &C->hitCount[depth - 1], &C->missCount[depth - 1]);
}

/* tuning switch: resident CTAs per SM the shading kernel is compiled for (register cap; 6: 80 registers and a
 * few spills, 24 warps per SM where the compiler's 128 registers allowed 16); 0 leaves it to the compiler */
#ifndef LH2G_SHADE_MINBLOCKS
#define LH2G_SHADE_MINBLOCKS 6
#endif
#if LH2G_SHADE_MINBLOCKS > 0
template <bool MIS>
__global__ void __launch_bounds__(WAVE_BLOCK, LH2G_SHADE_MINBLOCKS) k_shade(const SceneGPU S, const FrameGPU F, const WaveBuffers B, const int depth) {
#else
template <bool MIS>
__global__ void __launch_bounds__(WAVE_BLOCK) k_shade(const SceneGPU S, const FrameGPU F, const WaveBuffers B, const int depth) {
#endif
    Counters* C = B.counters;
    const uint32_t count = queue_count(F, B, C, depth);
    const int nq = depth & 1;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    extern __shared__ float potential[];   /* light-selection potentials, (lights) x 128 threads, sized at launch */
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += stride) {
        const uint32_t i = base + threadIdx.x;
        ShadeOut out;
        out.ext = out.shadow = false;
        if (i < count) shade_path<MIS>(S, F, B, depth, B.order ? __ldg(B.order + i) : i, out, potential + threadIdx.x);
        const uint32_t em = __ballot_sync(0xffffffffu, out.ext);
        if (em) {
            const int leader = __ffs(em) - 1;
            uint32_t slot = 0;
            if ((int)lane == leader) slot = atomicAdd(&C->extension[depth - 1], (uint32_t)__popc(em));
            slot = __shfl_sync(0xffffffffu, slot, leader) + __popc(em & lanemask_lt());
            if (out.ext) B.O[nq][slot] = out.eO, B.D[nq][slot] = out.eD, B.T[nq][slot] = out.eT;
        }
        const uint32_t sm = __ballot_sync(0xffffffffu, out.shadow);
        if (sm) {
            const int leader = __ffs(sm) - 1;
            uint32_t slot = 0;
            if ((int)lane == leader) slot = atomicAdd(&C->shadow[depth - 1], (uint32_t)__popc(sm));
            slot = __shfl_sync(0xffffffffu, slot, leader) + __popc(sm & lanemask_lt());
            if (out.shadow) B.shO[slot] = out.sO, B.shD[slot] = out.sD, B.shE[slot] = out.sE;
        }
    }
}

/* -------------------------------------------------------------------------------------------------- */
/* The tail of the wave loop: the paths still alive when path length `startDepth` begins are few, and tracing
 * them wave by wave would cost one launch and the latency of the slowest ray per remaining path length. Here a
 * persistent thread takes one path at a time from the queue and runs it to its end: closest hit, shading,
 * the connection's any-hit query and its contribution, the next segment. Every per-path quantity (RNG states,
 * hit records, radiance and its order of accumulation, queue counts per path length) is the one the wave loop
 * produces. */
/* tuning switch: resident CTAs per SM the tail kernel is compiled for (register cap); 0 leaves it to the compiler */
#ifndef LH2G_TAIL_MINBLOCKS
#define LH2G_TAIL_MINBLOCKS 0
#endif
#if LH2G_TAIL_MINBLOCKS > 0
#define LH2G_TAIL_BOUNDS __launch_bounds__(WAVE_BLOCK, LH2G_TAIL_MINBLOCKS)
#else
#define LH2G_TAIL_BOUNDS __launch_bounds__(WAVE_BLOCK)
#endif
template <bool MIS>
__global__ void LH2G_TAIL_BOUNDS k_tail(const SceneGPU S, const FrameGPU F, const WaveBuffers B, const int startDepth) {
    Counters* C = B.counters;
    const uint32_t count = queue_count(F, B, C, startDepth);
    const int q = (startDepth - 1) & 1;
    extern __shared__ float potential[];   /* light-selection potentials, (lights) x 128 threads, sized at launch */
    float* pot = potential + threadIdx.x;
    uint32_t status = 0;
    unsigned long long cn = 0, ct = 0, an = 0, at = 0;
    /* the first path of a thread is fixed by its index; later ones come from the shared counter */
    const uint32_t firstRound = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i = firstRound < count ? firstRound + atomicAdd(&C->fetch[3 * 64], 1u) : count) {
        float4 o4 = B.O[q][i], d4 = B.D[q][i], t4 = B.T[q][i];
        for (int depth = startDepth; depth <= F.maxDepth; depth++) {
            Traversal tr;
            tr.begin(S, xyz(o4), xyz(d4), MIS ? mis_tmin(__float_as_uint(o4.w), F.eps) : t4.w, 1e34f);
            bool any = false;
            if (S.tlasRoot != 0xffffffffu)
                while (tr.step<false>(S, status, any)) {}
            cn += tr.nodes, ct += tr.tris;
            const float4 hit = hit_record(tr.found, tr.best);
            if (B.capHits) {
                lh2g_hit c;
                c.bary = __float_as_uint(hit.x), c.inst = __float_as_int(hit.y), c.prim = __float_as_int(hit.z), c.t = hit.w;
                B.capHits[(size_t)(depth - 1) * F.P + (MIS ? __float_as_uint(o4.w) >> 6 : __float_as_uint(o4.w))] = c;
            }
            ShadeOut out;
            out.ext = out.shadow = false;
            if (MIS) shade_mis(S, F, B, depth, o4, d4, t4, hit, out, pot);
            else shade_core(S, F, B, depth, o4, d4, t4, hit, out, pot);
            if (out.shadow) {
                atomicAdd(&C->shadow[depth - 1], 1u);
                Traversal sh;
                sh.begin(S, xyz(out.sO), xyz(out.sD), (MIS && (F.flags & LH2G_RP_OPTIX7)) ? F.eps : 0.0f, out.sD.w);
                bool occluded = false;
                if (S.tlasRoot != 0xffffffffu)
                    while (sh.step<true>(S, status, occluded)) {}
                an += sh.nodes, at += sh.tris;
                if (!occluded) {
                    float4* accP = B.pathAcc + ((__float_as_uint(out.sE.w) & 1u) ? F.P : 0) + __float_as_uint(out.sO.w);
                    float4 acc = *accP;
                    acc.x += out.sE.x, acc.y += out.sE.y, acc.z += out.sE.z;
                    if (MIS && (F.flags & LH2G_RP_OPTIX7)) acc.w += 1.0f;   /* the OptiX 7 core counts connections in w */
                    *accP = acc;
                }
            }
            if (!out.ext) break;
            atomicAdd(&C->extension[depth - 1], 1u);
            o4 = out.eO, d4 = out.eD, t4 = out.eT;
        }
    }
    if (status) atomicOr(&C->status, status);
    if (cn | ct) atomicAdd(&C->travStats[0], cn), atomicAdd(&C->travStats[1], ct);
    if (an | at) atomicAdd(&C->travStats[2], an), atomicAdd(&C->travStats[3], at);
}

/* -------------------------------------------------------------------------------------------------- */
__global__ void LH2G_CONNECT_BOUNDS k_connect(const SceneGPU S, const FrameGPU F, const WaveBuffers B, const int depth) {
    Counters* C = B.counters;
    const uint32_t count = C->shadow[depth - 1];
    uint32_t status = 0;
    __shared__ uint2 stackBase[LH2G_COOP ? 128 / COOP * COOP_STACK : 1];
    const bool optix7 = (F.flags & LH2G_RP_OPTIX7) != 0;   /* tmin epsilon, and a count of the connections in w */
    auto add = [&](uint32_t i) {
        const float4 e = B.shE[i];
        const uint32_t pathIdx = __float_as_uint(B.shO[i].w);
        float4* accP = B.pathAcc + ((__float_as_uint(e.w) & 1u) ? F.P : 0) + pathIdx;   /* e.w bit 0: indirect half */
        float4 acc = *accP;
        acc.x += e.x, acc.y += e.y, acc.z += e.z;
        if (optix7) acc.w += 1.0f;
        *accP = acc;
    };
#if LH2G_STAGE_RAYS && !LH2G_COOP && !LH2G_REFILL
    (void)stackBase;
    const float4* const src[2] = {B.shO, B.shD};   /* origins and directions (w: distance to the light) */
    trace_queue_staged<true, 2>(S, &C->fetch[64 + depth - 1], count, status, src,
        [&](uint32_t, const float4 (&v)[2], float3& o, float3& d, float& t0, float& t1) {
            o = xyz(v[0]), d = xyz(v[1]), t0 = optix7 ? F.eps : 0.0f, t1 = v[1].w;
        },
        [&](uint32_t i, const Traversal&, bool occluded) { if (!occluded) add(i); }, C->travStats + 2);
#else
    trace_queue_any<true>(S, &C->fetch[64 + depth - 1], count, status, stackBase,
        [&](uint32_t i, float3& o, float3& d, float& t0, float& t1) {
            const float4 d4 = B.shD[i];
            o = xyz(B.shO[i]), d = xyz(d4), t0 = optix7 ? F.eps : 0.0f, t1 = d4.w;
        },
        [&](uint32_t i, const Traversal&, bool occluded) { if (!occluded) add(i); },
        [&](uint32_t i, const CoopRay&, bool occluded) { if (!occluded && (threadIdx.x & (COOP - 1)) == 0) add(i); },
        C->travStats + 2);
#endif
    if (status) atomicOr(&C->status, status);
}

/* --------------------------------------------------------------------------------------------------
 * Connections grouped by light: a counting sort over the light index the shading stage keeps in E.w bits 1..6.
 * Shadow rays towards one light from neighbouring points visit much of the same tree, so a warp of them
 * diverges less. Within a light, each warp's connections stay together and in their order; the warps' runs follow
 * one another in the order their atomics arrive. */
__global__ void k_conn_count(const WaveBuffers B, const int depth) {
    __shared__ uint32_t h[64];
    if (threadIdx.x < 64) h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t n = B.counters->shadow[depth - 1];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&h[(__float_as_uint(B.shE[i].w) >> 1) & 63u], 1u);
    __syncthreads();
    if (threadIdx.x < 64 && h[threadIdx.x]) atomicAdd(&B.connBins[threadIdx.x], h[threadIdx.x]);
}
/* one block of 64 threads: running offsets of the bins, counts cleared for the next wave */
__global__ void k_conn_scan(const WaveBuffers B) {
    __shared__ uint32_t v[64];
    const uint32_t t = threadIdx.x;
    v[t] = B.connBins[t];
    __syncthreads();
    if (t == 0) {
        uint32_t run = 0;
        for (int k = 0; k < 64; k++) {
            const uint32_t c = v[k];
            v[k] = run;
            run += c;
        }
    }
    __syncthreads();
    B.connBins[64 + t] = v[t];
    B.connBins[t] = 0;
}
__global__ void k_conn_scatter(const WaveBuffers B, const int depth) {
    const uint32_t n = B.counters->shadow[depth - 1];
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w0 < n; w0 += gridDim.x * blockDim.x) {
        const uint32_t i = w0 + lane;
        const bool valid = i < n;
        const float4 e = valid ? B.shE[i] : make_float4(0, 0, 0, 0);
        const uint32_t bin = valid ? (__float_as_uint(e.w) >> 1) & 63u : 64u;
        const uint32_t peers = __match_any_sync(0xffffffffu, bin);
        const uint32_t leader = (uint32_t)__ffs(peers) - 1u;
        uint32_t base = 0;
        if (valid && lane == leader) base = atomicAdd(&B.connBins[64 + bin], (uint32_t)__popc(peers));
        base = __shfl_sync(0xffffffffu, base, (int)leader);
        if (valid) {
            const uint32_t pos = base + (uint32_t)__popc(peers & lanemask_lt());
            B.sortO[pos] = B.shO[i], B.sortD[pos] = B.shD[i], B.sortE[pos] = e;
        }
    }
}

/* Connections grouped by light within chunks of CONN_CHUNK consecutive queue entries (setting "sortConnections" 2):
 * a counting sort in shared memory per chunk. The queue is in shading order, which follows the primary rays' pixel
 * tiles, so a chunk's connections start from one region of the image; grouped by light, a warp's shadow rays then
 * share both their origin region and their target and visit much the same nodes. Entries do not leave their chunk. */
constexpr uint32_t CONN_CHUNK = 1024;
__global__ void __launch_bounds__(256) k_conn_local(const WaveBuffers B, const int depth) {
    __shared__ uint32_t cnt[64], off[64];
    const uint32_t n = B.counters->shadow[depth - 1];
    for (uint32_t c0 = blockIdx.x * CONN_CHUNK; c0 < n; c0 += gridDim.x * CONN_CHUNK) {
        if (threadIdx.x < 64) cnt[threadIdx.x] = 0;
        __syncthreads();
        uint32_t bin[4], rank[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint32_t i = c0 + threadIdx.x + 256u * k;
            bin[k] = 64u, rank[k] = 0;
            if (i < n) bin[k] = (__float_as_uint(B.shE[i].w) >> 1) & 63u, rank[k] = atomicAdd(&cnt[bin[k]], 1u);
        }
        __syncthreads();
        if (threadIdx.x < 32) {   /* exclusive prefix over the 64 bins, two per lane */
            const uint32_t lane = threadIdx.x, a = cnt[2 * lane], b = cnt[2 * lane + 1];
            uint32_t sum = a + b;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, sum, d);
                if (lane >= (uint32_t)d) sum += v;
            }
            const uint32_t excl = sum - (a + b);
            off[2 * lane] = excl, off[2 * lane + 1] = excl + a;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (bin[k] == 64u) continue;
            const uint32_t i = c0 + threadIdx.x + 256u * k, pos = c0 + off[bin[k]] + rank[k];
            B.sortO[pos] = B.shO[i], B.sortD[pos] = B.shD[i], B.sortE[pos] = B.shE[i];
        }
        __syncthreads();
    }
}

/* --------------------------------------------------------------------------------------------------
 * Extension rays grouped by direction octant before a bounce wave's closest-hit queries (setting "sortRays"): a
 * counting sort over 8 bins of the queue into sortO/D/E; within a bin, each warp's rays stay together and in order,
 * so neighbouring pixels' rays stay neighbours. A warp of rays heading into one octant visits more of the same
 * nodes. Results do not change (everything per path follows the path, not its queue slot). */
__device__ __forceinline__ uint32_t ray_octant(const float4 d) {
    return (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
}
__global__ void k_ray_count(const WaveBuffers B, const int depth) {
    __shared__ uint32_t h[8];
    if (threadIdx.x < 8) h[threadIdx.x] = 0;
    __syncthreads();
    const int q = (depth - 1) & 1;
    const uint32_t n = B.counters->extension[depth - 2];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) atomicAdd(&h[ray_octant(B.D[q][i])], 1u);
    __syncthreads();
    if (threadIdx.x < 8 && h[threadIdx.x]) atomicAdd(&B.connBins[threadIdx.x], h[threadIdx.x]);
}
__global__ void k_ray_scatter(const WaveBuffers B, const int depth) {
    const int q = (depth - 1) & 1;
    const uint32_t n = B.counters->extension[depth - 2];
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t w0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w0 < n; w0 += gridDim.x * blockDim.x) {
        const uint32_t i = w0 + lane;
        const bool valid = i < n;
        const float4 d = valid ? B.D[q][i] : make_float4(0, 0, 0, 0);
        const uint32_t bin = valid ? ray_octant(d) : 64u;
        const uint32_t peers = __match_any_sync(0xffffffffu, bin);
        const uint32_t leader = (uint32_t)__ffs(peers) - 1u;
        uint32_t base = 0;
        if (valid && lane == leader) base = atomicAdd(&B.connBins[64 + bin], (uint32_t)__popc(peers));
        base = __shfl_sync(0xffffffffu, base, (int)leader);
        if (valid) {
            const uint32_t pos = base + (uint32_t)__popc(peers & lanemask_lt());
            B.sortO[pos] = B.O[q][i], B.sortD[pos] = d, B.sortE[pos] = B.T[q][i];
        }
    }
}

/* -------------------------------------------------------------------------------------------------- */
/* radiance cache: the queries of the paths that ended at their cache vertex (state 1) and the training samples of
 * the paths that went on (state 2: target = radiance gathered from the vertex on / throughput into it) */
__global__ void k_nrc_collect(const FrameGPU F, const WaveBuffers B, float4* __restrict__ queries, uint32_t* __restrict__ qPath,
                              float4* __restrict__ trainQ, float4* __restrict__ trainT, uint32_t* counts, const uint32_t trainCap) {
    const int64_t P = F.P;
    const uint32_t lane = threadIdx.x & 31u;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < P; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = base + threadIdx.x;
        const float state = p < P ? B.nrcRec[4 * P + p].w : 0.0f;
        const uint32_t qm = __ballot_sync(0xffffffffu, state == 1.0f), tm = __ballot_sync(0xffffffffu, state == 2.0f);
        uint32_t qb = 0, tb = 0;
        if (lane == 0) {
            if (qm) qb = atomicAdd(&counts[0], (uint32_t)__popc(qm));
            if (tm) tb = atomicAdd(&counts[1], (uint32_t)__popc(tm));
        }
        qb = __shfl_sync(0xffffffffu, qb, 0) + __popc(qm & lanemask_lt());
        tb = __shfl_sync(0xffffffffu, tb, 0) + __popc(tm & lanemask_lt());
        if (state == 1.0f) {
            for (int k = 0; k < 4; k++) queries[4 * (size_t)qb + k] = B.nrcRec[k * P + p];
            qPath[qb] = (uint32_t)p;
        } else if (state == 2.0f && tb < trainCap) {
            const float4 T = B.nrcRec[4 * P + p], pre = B.nrcRec[5 * P + p], L = B.pathAcc[p];
            const float tx = T.x > 1e-8f ? (L.x - pre.x) / T.x : 0.0f, ty = T.y > 1e-8f ? (L.y - pre.y) / T.y : 0.0f;
            const float tz = T.z > 1e-8f ? (L.z - pre.z) / T.z : 0.0f;
            for (int k = 0; k < 4; k++) trainQ[4 * (size_t)tb + k] = B.nrcRec[k * P + p];
            trainT[tb] = make_float4(tx, ty, tz, 0.0f);
        }
    }
}

/* the cache's prediction, times the throughput into the vertex, completes each path that ended there */
__global__ void k_nrc_apply(const FrameGPU F, const WaveBuffers B, const float4* __restrict__ pred, const uint32_t* __restrict__ qPath,
                            const uint32_t* counts) {
    const uint32_t n = counts[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = qPath[i];
        const float4 T = B.nrcRec[4 * F.P + p], y = pred[i];
        float4 acc = B.pathAcc[p];
        acc.x += T.x * fmaxf(y.x, 0.0f), acc.y += T.y * fmaxf(y.y, 0.0f), acc.z += T.z * fmaxf(y.z, 0.0f);
        B.pathAcc[p] = acc;
    }
}

/* -------------------------------------------------------------------------------------------------- */
/* overwrite: the accumulator starts from zero (a frame that does not accumulate) instead of its stored sum */
__global__ void k_finalize(const FrameGPU F, const WaveBuffers B, const float scale, const int overwrite) {
    const int64_t px = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t WH = F.bandPix ? (int64_t)F.bandPix : (int64_t)F.W * F.H;   /* the pixels rendered (a band's) */
    if (px >= WH) return;
    const bool filt = (F.flags & LH2G_RP_FILTER) != 0;
    for (int half = 0; half < (filt ? 2 : 1); half++) {
        float4 acc = overwrite ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : B.accum[half * WH + px];
        for (int s = 0; s < F.spp; s++) {
            const float4 v = B.pathAcc[half * F.P + s * WH + px];
            acc.x += v.x, acc.y += v.y, acc.z += v.z, acc.w += v.w;
        }
        B.accum[half * WH + px] = acc;
        /* LH2G_RP_FILTER frames are presented by the filter */
        if (!filt) B.frame[px] = make_float4(acc.x * scale, acc.y * scale, acc.z * scale, acc.w * scale);
    }
}

/* -------------------------------------------------------------------------------------------------- */
template <int MODE>
__global__ void __launch_bounds__(128) k_trace(const SceneGPU S, const lh2g_ray* __restrict__ rays, void* __restrict__ out, const long long n,
                                               uint32_t* fetch, uint32_t* statusOut) {
    uint32_t status = 0;
    __shared__ uint2 stackBase[LH2G_COOP ? 128 / COOP * COOP_STACK : 1];
    auto write = [&](uint32_t i, bool found, const HitRec& best, bool any) {
        if (MODE == 1) ((uint32_t*)out)[i] = any ? 1u : 0u;
        else {
            uint4 rec;
            if (found) rec = make_uint4(f2u(65535.0f * best.u) + (f2u(65535.0f * best.v) << 16), (uint32_t)best.inst, (uint32_t)best.prim,
                                        __float_as_uint(best.t));
            else rec = make_uint4(0u, 0u, (uint32_t)NOHIT, __float_as_uint(1e34f));
            ((uint4*)out)[i] = rec;
        }
    };
    /* queries of more than 2^31 rays are processed in chunks by the host */
    trace_queue_any<MODE == 1>(S, fetch, (uint32_t)n, status, stackBase,
        [&](uint32_t i, float3& o, float3& d, float& t0, float& t1) {
            const float4* r = (const float4*)(rays + i);
            const float4 a = __ldg(r), b = __ldg(r + 1);
            o = xyz(a), d = xyz(b), t0 = a.w, t1 = b.w;
        },
        [&](uint32_t i, const Traversal& tr, bool any) { write(i, tr.found, tr.best, any); },
        [&](uint32_t i, const CoopRay& tr, bool any) { if ((threadIdx.x & (COOP - 1)) == 0) write(i, tr.found, tr.best, any); },
        nullptr);
    if (status) atomicOr(statusOut, status);
}

/* -------------------------------------------------------------------------------------------------- */
__global__ void k_tri_prep(const float4* __restrict__ verts, uint32_t n, uint32_t seg, float4* __restrict__ triData, float4* __restrict__ lo,
                           float4* __restrict__ hi, uint32_t* __restrict__ segOf) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = verts[3 * i], b = verts[3 * i + 1], c = verts[3 * i + 2];
    const float3 v0 = xyz(a), e1 = xyz(b) - v0, e2 = xyz(c) - v0;
    triData[3 * i] = make_float4(v0.x, v0.y, v0.z, __int_as_float((int)i));
    triData[3 * i + 1] = make_float4(e1.x, e1.y, e1.z, 0.0f);
    triData[3 * i + 2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
    const float3 v1 = v0 + e1, v2 = v0 + e2;
    float3 mn = make_float3(fminf(fminf(v0.x, v1.x), v2.x), fminf(fminf(v0.y, v1.y), v2.y), fminf(fminf(v0.z, v1.z), v2.z));
    float3 mx = make_float3(fmaxf(fmaxf(v0.x, v1.x), v2.x), fmaxf(fmaxf(v0.y, v1.y), v2.y), fmaxf(fmaxf(v0.z, v1.z), v2.z));
    /* widen by 2^-20 of the magnitude (covers the rounding of v0 + e1 and of dequantised planes) */
    const float k = 9.5367431640625e-07f;
    mn = make_float3(mn.x - (fabsf(mn.x) * k + 1e-30f), mn.y - (fabsf(mn.y) * k + 1e-30f), mn.z - (fabsf(mn.z) * k + 1e-30f));
    mx = make_float3(mx.x + (fabsf(mx.x) * k + 1e-30f), mx.y + (fabsf(mx.y) * k + 1e-30f), mx.z + (fabsf(mx.z) * k + 1e-30f));
    lo[i] = make_float4(mn.x, mn.y, mn.z, 0.0f);
    hi[i] = make_float4(mx.x, mx.y, mx.z, 0.0f);
    segOf[i] = seg;
}

__global__ void k_gather_tris(const float4* __restrict__ triIn, const uint32_t* __restrict__ leafPrim, uint32_t n, float4* __restrict__ triOut) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t p = leafPrim[i];
    triOut[3 * i] = triIn[3 * p], triOut[3 * i + 1] = triIn[3 * p + 1], triOut[3 * i + 2] = triIn[3 * p + 2];
}

int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

}  // namespace

int persistent_blocks_trace(int mode) {
    int per = 0;
    if (mode == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_trace<1>, 128, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_trace<0>, 128, 0);
    return sm_count() * (per > 0 ? per : 1);
}

int persistent_blocks_wave(int which) {
    int per = 0;
    if (LH2G_TRAV_CARVEOUT >= 0 && which <= 1) {   /* on the current device, before the occupancy query */
        cudaFuncSetAttribute(k_extend<false>, cudaFuncAttributePreferredSharedMemoryCarveout, LH2G_TRAV_CARVEOUT);
        cudaFuncSetAttribute(k_extend<true>, cudaFuncAttributePreferredSharedMemoryCarveout, LH2G_TRAV_CARVEOUT);
        cudaFuncSetAttribute(k_connect, cudaFuncAttributePreferredSharedMemoryCarveout, LH2G_TRAV_CARVEOUT);
    }
    if (LH2G_SHADE_CARVEOUT >= 0 && which >= 2) {
        cudaFuncSetAttribute(k_shade<false>, cudaFuncAttributePreferredSharedMemoryCarveout, LH2G_SHADE_CARVEOUT);
        cudaFuncSetAttribute(k_shade<true>, cudaFuncAttributePreferredSharedMemoryCarveout, LH2G_SHADE_CARVEOUT);
        cudaFuncSetAttribute(k_tail<false>, cudaFuncAttributePreferredSharedMemoryCarveout, LH2G_SHADE_CARVEOUT);
        cudaFuncSetAttribute(k_tail<true>, cudaFuncAttributePreferredSharedMemoryCarveout, LH2G_SHADE_CARVEOUT);
    }
    if (which == 0) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_extend<false>, 128, 0);
    else if (which == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_connect, 128, 0);
    else if (which == 2) {
        /* the grid the registers allow; the potentials' shared memory grows with the scene's lights, and as the
         * shading loop is grid-stride, blocks beyond what shared memory lets reside simply start later */
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_shade<false>, WAVE_BLOCK, WAVE_BLOCK * sizeof(float));
    }
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_tail<false>, WAVE_BLOCK, WAVE_BLOCK * sizeof(float));
    return sm_count() * (per > 0 ? per : 1);
}

constexpr int MIS_FLAGS = LH2G_RP_OPTIX7 | LH2G_RP_ADAPTIVE;
void launch_generate(const FrameGPU& F, const WaveBuffers& B, cudaStream_t st) {
    k_generate<<<(unsigned)((F.P + 255) / 256), 256, 0, st>>>(F, B);
}
void launch_generate_mis(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, cudaStream_t st) {
    k_generate_mis<<<(unsigned)((F.P + 255) / 256), 256, 0, st>>>(S, F, B);
}
void launch_extend(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, int depth, int blocks, cudaStream_t st) {
    if (F.flags & MIS_FLAGS) k_extend<true><<<blocks, 128, 0, st>>>(S, F, B, depth);
    else k_extend<false><<<blocks, 128, 0, st>>>(S, F, B, depth);
}
void launch_shade(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, int depth, int blocks, cudaStream_t st) {
    if (B.order) k_partition<<<sm_count() * 4, PART_TILE, 0, st>>>(F, B, depth);
    /* at most 64 lights select by potential (render validation); light-tree frames keep no potentials */
    const int lights = (F.flags & LH2G_RP_LIGHTTREE) ? 1 : std::max(1, S.nTri + S.nPoint + S.nSpot + S.nDir);
    if (F.flags & MIS_FLAGS) k_shade<true><<<blocks, WAVE_BLOCK, (size_t)lights * WAVE_BLOCK * sizeof(float), st>>>(S, F, B, depth);
    else k_shade<false><<<blocks, WAVE_BLOCK, (size_t)lights * WAVE_BLOCK * sizeof(float), st>>>(S, F, B, depth);
}
void launch_connect(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, int depth, int blocks, cudaStream_t st) {
    k_connect<<<blocks, 128, 0, st>>>(S, F, B, depth);
}
void launch_tail(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, int startDepth, int blocks, cudaStream_t st) {
    /* the potentials' shared memory as in launch_shade; the loop takes paths from a counter, so blocks beyond what
     * shared memory lets reside start later */
    const int lights = (F.flags & LH2G_RP_LIGHTTREE) ? 1 : std::max(1, S.nTri + S.nPoint + S.nSpot + S.nDir);
    const size_t smem = (size_t)lights * WAVE_BLOCK * sizeof(float);
    if (F.flags & MIS_FLAGS) k_tail<true><<<blocks, WAVE_BLOCK, smem, st>>>(S, F, B, startDepth);
    else k_tail<false><<<blocks, WAVE_BLOCK, smem, st>>>(S, F, B, startDepth);
}
void launch_nrc_collect(const FrameGPU& F, const WaveBuffers& B, float4* queries, uint32_t* qPath, float4* trainQ, float4* trainT, uint32_t* counts,
                        uint32_t trainCap, cudaStream_t st) {
    k_nrc_collect<<<sm_count() * 8, 256, 0, st>>>(F, B, queries, qPath, trainQ, trainT, counts, trainCap);
}
void launch_nrc_apply(const FrameGPU& F, const WaveBuffers& B, const float4* pred, const uint32_t* qPath, const uint32_t* counts, cudaStream_t st) {
    k_nrc_apply<<<sm_count() * 8, 256, 0, st>>>(F, B, pred, qPath, counts);
}
void launch_sort_connections(const WaveBuffers& B, int depth, cudaStream_t st) {
    k_conn_count<<<sm_count() * 4, 256, 0, st>>>(B, depth);
    k_conn_scan<<<1, 64, 0, st>>>(B);
    k_conn_scatter<<<sm_count() * 8, 256, 0, st>>>(B, depth);
}
void launch_sort_connections_local(const WaveBuffers& B, int depth, cudaStream_t st) {
    k_conn_local<<<sm_count() * 8, 256, 0, st>>>(B, depth);
}
/* Extension rays grouped by direction octant within chunks of RAY_CHUNK consecutive queue entries (setting "sortRays"
 * 2): the queue follows the primary rays' pixel tiles, so a chunk's rays start from one region of the image; grouped
 * by octant within it, a warp's rays share origin region and direction octant. */
constexpr uint32_t RAY_CHUNK = 1024;
__global__ void __launch_bounds__(256) k_ray_local(const WaveBuffers B, const int depth) {
    __shared__ uint32_t cnt[8], off[8];
    const int q = (depth - 1) & 1;
    const uint32_t n = B.counters->extension[depth - 2];
    for (uint32_t c0 = blockIdx.x * RAY_CHUNK; c0 < n; c0 += gridDim.x * RAY_CHUNK) {
        if (threadIdx.x < 8) cnt[threadIdx.x] = 0;
        __syncthreads();
        uint32_t bin[4], rank[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint32_t i = c0 + threadIdx.x + 256u * k;
            bin[k] = 8u, rank[k] = 0;
            if (i < n) bin[k] = ray_octant(B.D[q][i]), rank[k] = atomicAdd(&cnt[bin[k]], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t acc = 0;
            for (int b = 0; b < 8; b++) off[b] = acc, acc += cnt[b];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (bin[k] == 8u) continue;
            const uint32_t i = c0 + threadIdx.x + 256u * k, pos = c0 + off[bin[k]] + rank[k];
            B.sortO[pos] = B.O[q][i], B.sortD[pos] = B.D[q][i], B.sortE[pos] = B.T[q][i];
        }
        __syncthreads();
    }
}
void launch_sort_rays_local(const WaveBuffers& B, int depth, cudaStream_t st) {
    k_ray_local<<<sm_count() * 8, 256, 0, st>>>(B, depth);
}
void launch_sort_rays(const WaveBuffers& B, int depth, cudaStream_t st) {
    k_ray_count<<<sm_count() * 4, 256, 0, st>>>(B, depth);
    k_conn_scan<<<1, 64, 0, st>>>(B);
    k_ray_scatter<<<sm_count() * 8, 256, 0, st>>>(B, depth);
}
void launch_finalize(const FrameGPU& F, const WaveBuffers& B, float scale, int overwrite, cudaStream_t st) {
    const int64_t WH = F.bandPix ? (int64_t)F.bandPix : (int64_t)F.W * F.H;
    k_finalize<<<(unsigned)((WH + 255) / 256), 256, 0, st>>>(F, B, scale, overwrite);
}
void launch_trace(const SceneGPU& S, const lh2g_ray* rays, void* out, long long n, int mode, uint32_t* fetch, uint32_t* status, int blocks, cudaStream_t st) {
    if (mode == 1) k_trace<1><<<blocks, 128, 0, st>>>(S, rays, out, n, fetch, status);
    else k_trace<0><<<blocks, 128, 0, st>>>(S, rays, out, n, fetch, status);
}
void launch_tri_prep(const float4* verts, uint32_t n, uint32_t seg, float4* triData, float4* lo, float4* hi, uint32_t* segOf, cudaStream_t st) {
    if (n) k_tri_prep<<<(n + 255) / 256, 256, 0, st>>>(verts, n, seg, triData, lo, hi, segOf);
}
void launch_gather_tris(const float4* triIn, const uint32_t* leafPrim, uint32_t n, float4* triOut, cudaStream_t st) {
    if (n) k_gather_tris<<<(n + 255) / 256, 256, 0, st>>>(triIn, leafPrim, n, triOut);
}

}  // namespace lh2g

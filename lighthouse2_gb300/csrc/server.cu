/* server.cu - the serving loop: render and ray-query jobs of several resident scenes, continuously batched.
 *
 * No counterpart in the reference, whose closest analogue is the asynchronous Render / WaitForRender of one core
 * (lib/rendercore_optix7/rendercore.cpp:803-847, 945-957): one frame at a time per core. Here jobs of different
 * scenes, resolutions, sample counts and depths share one set of wavefront queues:
 *
 *   tick      one CUDA graph, replayed: generate the primary rays of the jobs admitted since the last tick and
 *             append them to the current queue; extend (closest hit) every ray in the queue; shade every path
 *             vertex, compacting extension rays into the other queue and connections into the shadow queue;
 *             connect (any hit); swap the queues; copy the per-job counts of live paths to the host.
 *             A path carries its job slot (bits 8..15) and its own path length (bits 16..22) in its flag word,
 *             so paths of jobs admitted at different ticks, and at different depths, are processed together.
 *   admission a job is admitted when its paths fit in the queue capacity (path memory, counted from the live
 *             paths of the jobs in flight) and a
 *             slot is free: the smallest pending job first, the oldest one once it has waited longer than a bound.
 *             Its paths enter the queues in ranges, at most a tick budget of new paths per tick, so that a large
 *             job does not stretch the ticks every small job needs. A job whose live-path count reached zero is
 *             finalized (its per-path radiance summed per pixel, in sample order), its slot and memory released,
 *             and its image copied to the caller's host buffer by a worker thread.
 *   ray queries run on the worker thread's own stream, concurrently with the render ticks.
 *
 * Every per-path quantity (RNG seeds, hit records, radiance and its order of accumulation) is the one the
 * plain core computes for the same job: a job's image does not depend on what else is in flight.
 * Queue sizes never leave the device; the host reads only the live-path counts, one tick behind.
 */
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "lh2g.h"
#include "wavefront.cuh"

namespace lh2g {
int context_scene(lh2g_context* ctx, SceneGPU* scene, int* device, int* blocks4, int* tailDepth);
FrameGPU frame_of(const lh2g_view* view, const lh2g_render_params* p);
void launch_trace(const SceneGPU& S, const lh2g_ray* rays, void* out, long long n, int mode, uint32_t* fetch, uint32_t* status,
                  int persistentBlocks, cudaStream_t st);
int persistent_blocks_trace(int mode);
}  // namespace lh2g

using namespace lh2g;

namespace lh2g {
namespace srv {

constexpr int MAX_SLOTS = 256;         /* job slots: 8 bits of the flag word */
constexpr int MAX_NEW = 64;            /* path ranges admitted per tick */
constexpr int MAX_SCENES = 16;         /* scene records travel as a kernel parameter */
constexpr int MAX_EXPRESS = 64;        /* express jobs admitted per tick */
constexpr uint32_t SLOT_SHIFT = 8, DEPTH_SHIFT = 16;

struct JobGPU {
    FrameGPU F;                        /* F.P = paths of the job */
    int scene;
    float4* pathAcc;                   /* F.P entries */
    float4* out;                       /* W*H: per-pixel sums over the job's samples */
};

struct ServerState {
    uint32_t cur;                      /* queue the next tick extends */
    uint32_t qCount[2];
    uint32_t shadowCount;
    uint32_t fetch[4];
    uint32_t status;
    uint32_t newCount, newTotal;       /* path ranges admitted for the next tick and their paths */
    uint32_t newSlot[MAX_NEW];
    uint32_t newStart[MAX_NEW];        /* first path (index within its job) of each range */
    uint32_t newPrefix[MAX_NEW + 1];
    uint32_t expCount, expTotal;       /* express jobs of this tick (whole jobs) and their paths */
    uint32_t expSlot[MAX_EXPRESS];
    uint32_t expPrefix[MAX_EXPRESS + 1];
    unsigned long long rays;           /* rays traced over all ticks */
    unsigned long long ticks;
    uint32_t hitCount, missCount;      /* slots placed in this tick's shading order */
};

struct SceneTable { SceneGPU s[MAX_SCENES]; };

struct Queues {
    float4* O[2];
    float4* D[2];
    float4* T[2];
    float4* hits;
    float4* shO;
    float4* shD;
    float4* shE;
    uint32_t* order;                   /* shading order of the current queue (partition_queue) */
    uint32_t cap;                      /* slots of each queue */
};

__device__ __forceinline__ uint32_t slot_of(const float4& d4) { return (__float_as_uint(d4.w) >> SLOT_SHIFT) & 255u; }

/* primary rays of the jobs admitted for this tick, appended to the current queue */
__global__ void __launch_bounds__(256) k_srv_generate(const JobGPU* __restrict__ jobs, ServerState* st, const Queues Q) {
    const uint32_t total = st->newTotal, n = st->newCount;
    if (total == 0) return;
    const uint32_t cur = st->cur, base = st->qCount[cur];
    /* admission keeps base + total within the queue; should it not, the paths that do not fit are left out and
     * the tick reports it instead of writing past the queue */
    if (base + total > Q.cap && blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&st->status, LH2G_STATUS_QUEUE_OVERFLOW);
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total && base + g < Q.cap; g += gridDim.x * blockDim.x) {
        uint32_t j = 0;
        while (j + 1 < n && st->newPrefix[j + 1] <= g) j++;
        const uint32_t slot = st->newSlot[j];
        const JobGPU& J = jobs[slot];
        /* a job's ranges run over its primary queue order (pixel tiles, as the plain core queues them); the path
         * of that position is generated */
        const uint32_t i = primary_slot_path(J.F, st->newStart[j] + (g - st->newPrefix[j]));
        float3 O, D;
        primary_ray(J.F, i, O, D);
        Q.O[cur][base + g] = make_float4(O.x, O.y, O.z, __uint_as_float(i));
        Q.D[cur][base + g] = make_float4(D.x, D.y, D.z, __uint_as_float(S_SPECULAR | (slot << SLOT_SHIFT) | (1u << DEPTH_SHIFT)));
        Q.T[cur][base + g] = make_float4(1.0f, 1.0f, 1.0f, J.F.eps);
        J.pathAcc[i] = make_float4(0, 0, 0, 0);
    }
}

/* closest hit of every ray in the current queue, each against the scene of its job */
__global__ void LH2G_TRAV_BOUNDS k_srv_extend(const __grid_constant__ SceneTable scenes, const JobGPU* __restrict__ jobs, ServerState* st,
                                                    const Queues Q) {
    const uint32_t cur = st->cur, count = st->qCount[cur] + st->newTotal;
    const uint32_t lane = threadIdx.x & 31u, firstRound = gridDim.x * blockDim.x;
    uint32_t status = 0;
    uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    for (bool first = true;; first = false) {
        if (!first) {
            if (firstRound >= count) break;
            if (lane == 0) base = firstRound + atomicAdd(&st->fetch[0], 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
        }
        if (base >= count) break;
        const uint32_t i = base + lane;
        if (i < count) {
            const float4 o4 = Q.O[cur][i], d4 = Q.D[cur][i], t4 = Q.T[cur][i];
            const SceneGPU& S = scenes.s[jobs[slot_of(d4)].scene];
            Traversal tr;
            tr.begin(S, xyz(o4), xyz(d4), t4.w, 1e34f);
            bool any = false;
            if (S.tlasRoot != 0xffffffffu)
                while (tr.step<false>(S, status, any)) {}
            Q.hits[i] = hit_record(tr.found, tr.best);
        }
    }
    if (status) atomicOr(&st->status, status);
}

/* one vertex of every path in the current queue: extension rays to the other queue, connections to the shadow
 * queue (warp ballot + popc, one atomic per warp), finished paths leave their job's live count */
/* register cap as the plain core's shading kernel: 6 CTAs per SM, with the light potentials in dynamic shared
 * memory sized to the largest light count of the resident scenes */
__global__ void __launch_bounds__(WAVE_BLOCK, 6) k_srv_shade(const __grid_constant__ SceneTable scenes, const JobGPU* __restrict__ jobs,
                                                         ServerState* st, const Queues Q, int* alive) {
    const uint32_t cur = st->cur, nq = cur ^ 1u, count = st->qCount[cur] + st->newTotal;
    const uint32_t lane = threadIdx.x & 31u;
    extern __shared__ float potential[];   /* (largest light count of the scenes) x 128 threads */
    for (uint32_t b0 = blockIdx.x * blockDim.x; b0 < count; b0 += gridDim.x * blockDim.x) {
        const uint32_t j = b0 + threadIdx.x;
        ShadeOut out;
        out.ext = out.shadow = false;
        uint32_t slot = 0;
        if (j < count) {
            const uint32_t i = __ldg(Q.order + j);
            const float4 o4 = Q.O[cur][i], d4 = Q.D[cur][i], t4 = Q.T[cur][i], hit = Q.hits[i];
            slot = slot_of(d4);
            const int depth = (int)((__float_as_uint(d4.w) >> DEPTH_SHIFT) & 127u);
            const JobGPU& J = jobs[slot];
            WaveBuffers B;
            memset(&B, 0, sizeof(B));
            B.pathAcc = J.pathAcc;
            shade_core(scenes.s[J.scene], J.F, B, depth, o4, d4, t4, hit, out, potential + threadIdx.x);
            if (out.ext) out.eD.w = __uint_as_float(__float_as_uint(out.eD.w) + (1u << DEPTH_SHIFT));
            if (out.shadow) out.sE.w = __uint_as_float(__float_as_uint(out.sE.w) | (slot << SLOT_SHIFT));
        }
        /* paths that end here leave their job's live count: one atomic per job and warp (one per path would
         * serialise on the few counters of the jobs in flight) */
        const uint32_t endSlot = (j < count && !out.ext) ? slot : 0xffffffffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, endSlot);
        if (endSlot != 0xffffffffu && lane == (uint32_t)(__ffs(peers) - 1)) atomicSub(&alive[endSlot], __popc(peers));
        const uint32_t em = __ballot_sync(0xffffffffu, out.ext);
        if (em) {
            const int leader = __ffs(em) - 1;
            uint32_t s = 0;
            if ((int)lane == leader) s = atomicAdd(&st->qCount[nq], (uint32_t)__popc(em));
            s = __shfl_sync(0xffffffffu, s, leader) + __popc(em & lanemask_lt());
            if (out.ext) Q.O[nq][s] = out.eO, Q.D[nq][s] = out.eD, Q.T[nq][s] = out.eT;
        }
        const uint32_t sm = __ballot_sync(0xffffffffu, out.shadow);
        if (sm) {
            const int leader = __ffs(sm) - 1;
            uint32_t s = 0;
            if ((int)lane == leader) s = atomicAdd(&st->shadowCount, (uint32_t)__popc(sm));
            s = __shfl_sync(0xffffffffu, s, leader) + __popc(sm & lanemask_lt());
            if (out.shadow) Q.shO[s] = out.sO, Q.shD[s] = out.sD, Q.shE[s] = out.sE;
        }
    }
}

/* the shading order of this tick's queue: hits first, misses last */
__global__ void __launch_bounds__(PART_TILE) k_srv_partition(ServerState* st, const Queues Q) {
    partition_queue(Q.hits, st->qCount[st->cur] + st->newTotal, Q.order, &st->hitCount, &st->missCount);
}

/* any hit of every connection; unoccluded ones add their contribution to their path */
__global__ void LH2G_CONNECT_BOUNDS k_srv_connect(const __grid_constant__ SceneTable scenes, const JobGPU* __restrict__ jobs, ServerState* st,
                                                     const Queues Q) {
    const uint32_t count = st->shadowCount;
    const uint32_t lane = threadIdx.x & 31u, firstRound = gridDim.x * blockDim.x;
    uint32_t status = 0;
    uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u;
    for (bool first = true;; first = false) {
        if (!first) {
            if (firstRound >= count) break;
            if (lane == 0) base = firstRound + atomicAdd(&st->fetch[1], 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
        }
        if (base >= count) break;
        const uint32_t i = base + lane;
        if (i < count) {
            const float4 e = Q.shE[i], o4 = Q.shO[i], d4 = Q.shD[i];
            const uint32_t tag = __float_as_uint(e.w), slot = (tag >> SLOT_SHIFT) & 255u;
            const JobGPU& J = jobs[slot];
            const SceneGPU& S = scenes.s[J.scene];
            Traversal tr;
            tr.begin(S, xyz(o4), xyz(d4), 0.0f, d4.w);
            bool occluded = false;
            if (S.tlasRoot != 0xffffffffu)
                while (tr.step<true>(S, status, occluded)) {}
            if (!occluded) {
                float4* accP = J.pathAcc + ((tag & 1u) ? J.F.P : 0) + __float_as_uint(o4.w);
                float4 acc = *accP;
                acc.x += e.x, acc.y += e.y, acc.z += e.z;
                *accP = acc;
            }
        }
    }
    if (status) atomicOr(&st->status, status);
}

/* Express jobs: every path of the small jobs admitted this tick, from its primary ray to its end, one thread per
 * path (the loop of the plain core's tail kernel), beside the tick's wave kernels. A small job so finishes within
 * one tick instead of one tick per bounce. Per-path work is the plain core's, as in the waves. */
__global__ void __launch_bounds__(WAVE_BLOCK) k_srv_express(const __grid_constant__ SceneTable scenes, const JobGPU* __restrict__ jobs,
                                                           ServerState* st, int* alive) {
    const uint32_t total = st->expTotal, n = st->expCount;
    if (total == 0) return;
    __shared__ float potential[64 * WAVE_BLOCK];
    float* pot = potential + threadIdx.x;
    uint32_t status = 0;
    unsigned long long rays = 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    /* whole warps go round the loop together, so that the warp-aggregated live-count update sees all lanes */
    for (uint32_t g0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); g0 < total; g0 += stride) {
        const uint32_t g = g0 + (threadIdx.x & 31u);
        uint32_t slot = 0xffffffffu;
        if (g < total) {
            uint32_t j = 0;
            while (j + 1 < n && st->expPrefix[j + 1] <= g) j++;
            slot = st->expSlot[j];
            const uint32_t i = g - st->expPrefix[j];
            const JobGPU& J = jobs[slot];
            const SceneGPU& S = scenes.s[J.scene];
            WaveBuffers B;
            memset(&B, 0, sizeof(B));
            B.pathAcc = J.pathAcc;
            float3 O, D;
            primary_ray(J.F, i, O, D);
            float4 o4 = make_float4(O.x, O.y, O.z, __uint_as_float(i));
            float4 d4 = make_float4(D.x, D.y, D.z, __uint_as_float(S_SPECULAR | (slot << SLOT_SHIFT) | (1u << DEPTH_SHIFT)));
            float4 t4 = make_float4(1.0f, 1.0f, 1.0f, J.F.eps);
            J.pathAcc[i] = make_float4(0, 0, 0, 0);
            for (int depth = 1; depth <= J.F.maxDepth; depth++) {
                Traversal tr;
                tr.begin(S, xyz(o4), xyz(d4), t4.w, 1e34f);
                bool any = false;
                if (S.tlasRoot != 0xffffffffu)
                    while (tr.step<false>(S, status, any)) {}
                rays++;
                ShadeOut out;
                out.ext = out.shadow = false;
                shade_core(S, J.F, B, depth, o4, d4, t4, hit_record(tr.found, tr.best), out, pot);
                if (out.shadow) {
                    rays++;
                    Traversal sh;
                    sh.begin(S, xyz(out.sO), xyz(out.sD), 0.0f, out.sD.w);
                    bool occluded = false;
                    if (S.tlasRoot != 0xffffffffu)
                        while (sh.step<true>(S, status, occluded)) {}
                    if (!occluded) {
                        float4* accP = J.pathAcc + ((__float_as_uint(out.sE.w) & 1u) ? J.F.P : 0) + __float_as_uint(out.sO.w);
                        float4 acc = *accP;
                        acc.x += out.sE.x, acc.y += out.sE.y, acc.z += out.sE.z;
                        *accP = acc;
                    }
                }
                if (!out.ext) break;
                o4 = out.eO, d4 = out.eD, t4 = out.eT;
                d4.w = __uint_as_float(__float_as_uint(d4.w) + (1u << DEPTH_SHIFT));
            }
        }
        /* the finished paths leave their job's live count: one atomic per job and warp */
        const uint32_t peers = __match_any_sync(0xffffffffu, slot);
        if (slot != 0xffffffffu && (threadIdx.x & 31u) == (uint32_t)(__ffs(peers) - 1)) atomicSub(&alive[slot], __popc(peers));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) rays += __shfl_xor_sync(0xffffffffu, rays, off);
    if ((threadIdx.x & 31u) == 0 && rays) atomicAdd(&st->rays, rays);
    if (status) atomicOr(&st->status, status);
}

/* closes a tick: swap the queues, count the rays, clear the per-tick state */
__global__ void k_srv_end(ServerState* st) {
    const uint32_t cur = st->cur;
    st->rays += (unsigned long long)(st->qCount[cur] + st->newTotal) + st->shadowCount;
    st->ticks++;
    st->qCount[cur] = 0;
    st->cur = cur ^ 1u;
    st->shadowCount = 0;
    st->fetch[0] = st->fetch[1] = 0;
    st->newCount = st->newTotal = 0;
    st->expCount = st->expTotal = 0;
    st->hitCount = st->missCount = 0;
}

/* ---- the device-side tick loop (setting "deviceLoop") ----
 * The tick graph's body runs inside a conditional WHILE node: one graph launch runs tick after tick on the device,
 * and k_srv_loop_end decides at the end of each tick whether another follows. It admits the next ranges of the jobs
 * whose paths are still entering the queues (the host's admitted-job list, in admission order, within the tick
 * budget), and ends the launch when a job's live count reached zero (the host finalizes it), when the host has
 * work waiting (a job submitted since the launch: a mapped host word it reads once per tick, no spinning), when no
 * work is left, or after `limit` ticks. The host admits new jobs and finalizes finished ones between launches. */
struct LoopState {
    uint32_t ticks;                    /* ticks run by the current launch */
    uint32_t limit;                    /* at most this many per launch */
    uint32_t budget;                   /* new paths per tick */
    uint32_t nPart;                    /* jobs with paths still to enter the queues, in admission order */
    uint32_t partSlot[MAX_SLOTS], partNext[MAX_SLOTS], partEnd[MAX_SLOTS];
    uint32_t active[MAX_SLOTS];        /* 1: the slot holds a job the host has not finalized */
    const int* doorbell;               /* mapped host word, nonzero while jobs wait for the host */
};

__global__ void __launch_bounds__(MAX_SLOTS) k_srv_loop_end(ServerState* st, LoopState* L, const int* __restrict__ alive,
                                                          cudaGraphConditionalHandle handle) {
    const int k = threadIdx.x;
    const int anyDone = __syncthreads_or(L->active[k] && alive[k] <= 0);
    if (k != 0) return;
    L->ticks++;
    bool go = !anyDone && L->ticks < L->limit && *(const volatile int*)L->doorbell == 0;
    if (go) {
        uint32_t n = 0, total = 0, budget = L->budget;
        for (uint32_t p = 0; p < L->nPart && budget > 0 && n < (uint32_t)MAX_NEW; p++) {
            const uint32_t rem = L->partEnd[p] - L->partNext[p];
            if (!rem) continue;
            const uint32_t c = min(rem, budget);
            st->newSlot[n] = L->partSlot[p], st->newStart[n] = L->partNext[p], st->newPrefix[n] = total;
            total += c, budget -= c, n++;
            L->partNext[p] += c;
        }
        st->newPrefix[n] = total, st->newCount = n, st->newTotal = total;
        go = st->qCount[st->cur] > 0 || total > 0;   /* paths in flight or entering */
    }
    cudaGraphSetConditional(handle, go ? 1u : 0u);
}

/* per-pixel sums of a finished job's paths in sample order (as the plain core's finalize) */
__global__ void k_srv_finalize(const JobGPU J) {
    const int64_t px = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t WH = (int64_t)J.F.W * J.F.H;
    if (px >= WH) return;
    float4 acc = make_float4(0, 0, 0, 0);
    for (int s = 0; s < J.F.spp; s++) {
        const float4 v = J.pathAcc[s * WH + px];
        acc.x += v.x, acc.y += v.y, acc.z += v.z, acc.w += v.w;
    }
    J.out[px] = acc;
}

double now_s() {
    static const auto t0 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

struct Job {
    long long id = 0;
    int kind = 0;                      /* 0 render, 1 ray query */
    int scene = 0;
    lh2g_view view;
    lh2g_render_params params;
    void* hostOut = nullptr;
    const lh2g_ray* hostRays = nullptr;
    long long n = 0;                   /* rays of a query */
    int mode = 0;
    long long paths = 0;
    long long admittedPaths = 0;       /* paths generated so far (a job enters the queues in ranges) */
    int slot = -1;
    long long admitTick = -1;
    int state = 0;                     /* 0 pending, 1 running, 2 finishing, 3 done, 4 failed */
    bool express = false;              /* traced whole in one tick beside the waves (no queue memory) */
    double tSubmit = 0, tAdmit = 0, tDone = 0;
    JobGPU gpu;
};

}  // namespace srv
}  // namespace lh2g

using namespace lh2g::srv;

struct lh2g_server {
    int device = 0;
    cudaStream_t st = nullptr;         /* render ticks */
    cudaStream_t io = nullptr;         /* worker: result copies, ray queries */
    cudaStream_t side = nullptr;       /* second branch of the tick graph (express jobs) */
    cudaEvent_t evFork = nullptr, evJoin = nullptr;
    std::string err;
    std::vector<SceneGPU> scenes;
    int graphScenes = -1;              /* scene count the tick graph was captured with */
    JobGPU* dJobs = nullptr;
    int* dAlive = nullptr;
    int* hAlive = nullptr;             /* pinned snapshot, refreshed by every tick */
    ServerState* dState = nullptr;
    ServerState* hTick = nullptr;      /* pinned staging of the tick parameters, one per tick-event ring entry */
    Queues Q;
    long long capacity = 0;
    long long tickBudget = 0;          /* new paths per tick */
    long long expressMax = 0;          /* jobs of at most this many paths are express jobs (0: none) */
    long long expressBudget = 1ll << 20;   /* express paths per tick */
    double maxWaitS = 0.2;             /* a job waiting longer than this is admitted before smaller ones */
    cudaGraphExec_t tickExec = nullptr;
    cudaGraph_t tickGraph = nullptr;
    /* the device-side tick loop (setting "deviceLoop"): a graph whose WHILE node runs the tick body */
    bool deviceLoop = true;
    long long loopLimit = 256;         /* ticks per launch at most (setting "loopTicks") */
    cudaGraphExec_t loopExec = nullptr;
    cudaGraph_t loopGraph = nullptr;
    int loopScenes = -1;               /* scene count the loop graph was built with */
    LoopState* dLoop = nullptr;
    LoopState* hLoop = nullptr;        /* pinned: [0] staged for a launch, [1] read back after it */
    int* hDoorbell = nullptr;          /* mapped host word: set when a job is submitted, cleared before a launch */
    int* dDoorbell = nullptr;
    long long loopLaunches = 0;
    std::vector<cudaEvent_t> tickEv;   /* ring of tick-completion events */
    long long ticksLaunched = 0, ticksDone = 0;
    int blocksGen = 0, blocksExtend = 0, blocksShade = 0, blocksConnect = 0, blocksTrace0 = 0, blocksTrace1 = 0, blocksExpress = 0, blocksPart = 0;
    /* jobs */
    std::mutex mu;
    std::condition_variable cvWork, cvDone;
    std::deque<Job*> pending;
    std::vector<Job*> partial;         /* admitted jobs with paths still to generate */
    std::map<long long, Job*> jobs;
    Job* slots[MAX_SLOTS] = {};
    long long nextId = 1;
    long long pathsInFlight = 0;
    bool stop = false;                 /* finish the jobs held, then exit */
    bool abortLoop = false;            /* exit now (a drain that does not end) */
    bool loopExited = false;
    std::thread loop, worker;
    std::deque<std::function<void()>> tasks;
    std::mutex tmu;
    std::condition_variable tcv;
    /* statistics */
    long long jobsDone = 0;
    unsigned long long raysDone = 0;
    /* Large jobs (at least largeMin paths; setting "largeJobPaths", 0 = none) skip the shared queues: they run one at a
     * time as plain frames (the plain core's stages, waves then the tail kernel) on their own stream and buffers,
     * beside the ticks. A job that fills the GPU alone gains nothing from sharing queues, and in the queues it
     * lengthens every tick the small jobs need. */
    long long largeMin = 8ll << 20;
    std::deque<Job*> largeQ;
    std::condition_variable lcv;
    std::thread large;
    cudaStream_t lst = nullptr;
    lh2g::WaveBuffers LB{};
    long long lcap = 0, lpix = 0;
    lh2g::Counters* lhost = nullptr;   /* pinned copy of a large job's counters */
    uint32_t largeStatus = 0;          /* traversal status bits of large jobs (reported with the device status) */
};

namespace lh2g {
namespace srv {

int sfail(lh2g_server* s, int code, const std::string& m) {
    if (s) {
        std::lock_guard<std::mutex> g(s->mu);
        s->err = m;
    }
    return code;
}

void post(lh2g_server* s, std::function<void()> f) {
    {
        std::lock_guard<std::mutex> g(s->tmu);
        s->tasks.push_back(std::move(f));
    }
    s->tcv.notify_one();
}

void finish(lh2g_server* s, Job* j, int state) {
    std::lock_guard<std::mutex> g(s->mu);
    j->state = state;
    j->tDone = now_s();
    s->jobsDone++;
    s->cvDone.notify_all();
}

/* the worker: copies finished images out and runs ray queries, in submission order, on its own stream */
void worker_loop(lh2g_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        std::function<void()> f;
        {
            std::unique_lock<std::mutex> g(s->tmu);
            s->tcv.wait(g, [&] { return s->stop || !s->tasks.empty(); });
            if (s->tasks.empty()) return;
            f = std::move(s->tasks.front());
            s->tasks.pop_front();
        }
        f();
    }
}

void run_query(lh2g_server* s, Job* j) {
    const SceneGPU S = s->scenes[j->scene];
    lh2g_ray* dr = nullptr;
    void* dout = nullptr;
    uint32_t* fetch = nullptr;
    const size_t outBytes = (size_t)j->n * (j->mode == 1 ? 4 : 16);
    bool ok = cudaMallocAsync((void**)&dr, sizeof(lh2g_ray) * (size_t)j->n, s->io) == cudaSuccess &&
              cudaMallocAsync(&dout, outBytes, s->io) == cudaSuccess && cudaMallocAsync((void**)&fetch, 16, s->io) == cudaSuccess;
    if (ok) ok = cudaMemcpyAsync(dr, j->hostRays, sizeof(lh2g_ray) * (size_t)j->n, cudaMemcpyHostToDevice, s->io) == cudaSuccess;
    if (ok) ok = cudaMemsetAsync(fetch, 0, 16, s->io) == cudaSuccess;
    if (ok) {
        launch_trace(S, dr, dout, j->n, j->mode, fetch, fetch + 1, j->mode == 1 ? s->blocksTrace1 : s->blocksTrace0, s->io);
        ok = cudaGetLastError() == cudaSuccess;
    }
    if (ok) ok = cudaMemcpyAsync(j->hostOut, dout, outBytes, cudaMemcpyDeviceToHost, s->io) == cudaSuccess;
    if (dr) cudaFreeAsync(dr, s->io);
    if (dout) cudaFreeAsync(dout, s->io);
    if (fetch) cudaFreeAsync(fetch, s->io);
    ok = cudaStreamSynchronize(s->io) == cudaSuccess && ok;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->raysDone += (unsigned long long)j->n;
    }
    finish(s, j, ok ? 3 : 4);
}

/* One large job as a plain frame (the waves of lh2g_render_ex, then the tail kernel and the finalize that leaves the
 * per-pixel sums), on the server's large-job stream; false on a CUDA error. */
bool render_large(lh2g_server* s, Job* j, const SceneGPU& S) {
    const lh2g_render_params& p = j->params;
    const long long P = (long long)p.width * p.height * p.spp, WH = (long long)p.width * p.height;
    WaveBuffers& B = s->LB;
    bool ok = true;
    if (P > s->lcap) {
        for (int k = 0; k < 2; k++) cudaFree(B.O[k]), cudaFree(B.D[k]), cudaFree(B.T[k]);
        cudaFree(B.hits), cudaFree(B.shO), cudaFree(B.shD), cudaFree(B.shE), cudaFree(B.pathAcc), cudaFree(B.order);
        for (int k = 0; k < 2 && ok; k++)
            ok = cudaMalloc((void**)&B.O[k], 16 * (size_t)P) == cudaSuccess && cudaMalloc((void**)&B.D[k], 16 * (size_t)P) == cudaSuccess &&
                 cudaMalloc((void**)&B.T[k], 16 * (size_t)P) == cudaSuccess;
        ok = ok && cudaMalloc((void**)&B.hits, 16 * (size_t)P) == cudaSuccess && cudaMalloc((void**)&B.shO, 16 * (size_t)P) == cudaSuccess &&
             cudaMalloc((void**)&B.shD, 16 * (size_t)P) == cudaSuccess && cudaMalloc((void**)&B.shE, 16 * (size_t)P) == cudaSuccess &&
             cudaMalloc((void**)&B.pathAcc, 16 * (size_t)P) == cudaSuccess && cudaMalloc((void**)&B.order, 4 * (size_t)P) == cudaSuccess;
        s->lcap = ok ? P : 0;
    }
    if (ok && WH > s->lpix) {
        cudaFree(B.accum), cudaFree(B.frame);
        ok = cudaMalloc((void**)&B.accum, 16 * (size_t)WH) == cudaSuccess && cudaMalloc((void**)&B.frame, 16 * (size_t)WH) == cudaSuccess;
        s->lpix = ok ? WH : 0;
    }
    if (ok && !B.counters) ok = cudaMalloc((void**)&B.counters, sizeof(Counters)) == cudaSuccess;
    if (ok && !s->lhost) ok = cudaMallocHost((void**)&s->lhost, sizeof(Counters)) == cudaSuccess;
    if (!ok) return false;
    FrameGPU F = frame_of(&j->view, &p);
    F.stride = s->lcap;
    cudaStream_t st = s->lst;
    ok = cudaMemsetAsync(B.counters, 0, sizeof(Counters), st) == cudaSuccess;
    launch_generate(F, B, st);
    constexpr int TAIL = 5;   /* the plain core's default waveTail */
    const int waves = std::min(F.maxDepth, TAIL - 1);
    for (int d = 1; d <= waves; d++) {
        launch_extend(S, F, B, d, persistent_blocks_wave(0), st);
        launch_shade(S, F, B, d, persistent_blocks_wave(2), st);
        launch_connect(S, F, B, d, persistent_blocks_wave(1), st);
    }
    if (waves < F.maxDepth) launch_tail(S, F, B, waves + 1, persistent_blocks_wave(3), st);
    launch_finalize(F, B, 1.0f / (float)(p.samplesTaken + F.spp), 1, st);
    ok = ok && cudaGetLastError() == cudaSuccess;
    ok = ok && cudaMemcpyAsync(j->hostOut, B.accum, 16 * (size_t)WH, cudaMemcpyDeviceToHost, st) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(s->lhost, B.counters, sizeof(Counters), cudaMemcpyDeviceToHost, st) == cudaSuccess;
    ok = cudaStreamSynchronize(st) == cudaSuccess && ok;
    if (ok) {
        unsigned long long rays = (unsigned long long)P;
        for (int d = 0; d < F.maxDepth; d++) rays += s->lhost->extension[d] + s->lhost->shadow[d];
        std::lock_guard<std::mutex> g(s->mu);
        s->raysDone += rays;
        s->largeStatus |= s->lhost->status;
    }
    return ok;
}

void large_loop(lh2g_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        Job* j = nullptr;
        SceneGPU S;
        {
            std::unique_lock<std::mutex> g(s->mu);
            s->lcv.wait(g, [&] { return s->stop || s->abortLoop || !s->largeQ.empty(); });
            if (s->largeQ.empty()) return;   /* stopping, nothing held */
            j = s->largeQ.front();
            s->largeQ.pop_front();
            S = s->scenes[j->scene];
        }
        const bool ok = render_large(s, j, S);
        finish(s, j, ok ? 3 : 4);
    }
}

/* A path range of a job entering the queues at the next tick. */
struct Range { Job* job; long long start, count; bool first, express; };

/* Admission for the next tick. Ray queries go to the worker. Render jobs are admitted when their paths fit in the
 * capacity beside the live paths of the jobs in flight and a slot is free: the smallest pending job first, unless one has waited longer than
 * maxWaitS (then the oldest); a job that does not fit stops admission, so no job waits forever. The paths of
 * admitted jobs enter the queues in ranges, at most tickBudget new paths per tick, so that one large job does not
 * stretch the ticks that every small job needs. */
void admit(lh2g_server* s, std::vector<Range>& ranges) {
    std::lock_guard<std::mutex> g(s->mu);
    long long budget = s->tickBudget, expBudget = s->expressBudget;
    /* Queue slots the next tick can need for the jobs in flight. A job's live count (its paths not yet ended,
     * including those not yet in the queue) only falls, and the host's copy of it is at most one tick old, so it
     * bounds the job's share of the next queue from above; a job whose first tick has not completed yet counts
     * all its paths. Capacity is thus released as paths end, not when the job's last path ends. */
    long long inUse = 0;
    for (int k = 0; k < MAX_SLOTS; k++) {
        const Job* j = s->slots[k];
        if (!j || j->express) continue;
        inUse += (j->admitTick >= 0 && j->admitTick < s->ticksDone) ? std::min<long long>(std::max(s->hAlive[k], 0), j->paths) : j->paths;
    }
    int nNew = 0, nExp = 0;
    auto take = [&](Job* j, bool first) {
        const long long n = std::min(j->paths - j->admittedPaths, std::max(budget, 1ll));
        ranges.push_back({j, j->admittedPaths, n, first, false});
        j->admittedPaths += n;
        budget -= n;
        nNew++;
    };
    /* ranges of jobs admitted earlier, in admission order */
    for (size_t k = 0; k < s->partial.size() && budget > 0 && nNew < MAX_NEW;) {
        Job* j = s->partial[k];
        take(j, false);
        if (j->admittedPaths == j->paths) s->partial.erase(s->partial.begin() + (long)k);
        else k++;
    }
    const double now = now_s();
    /* large jobs go to their own lane, in arrival order, without queue memory */
    if (s->largeMin > 0) {
        bool moved = false;
        for (size_t k = 0; k < s->pending.size();) {
            Job* j = s->pending[k];
            if (j->kind == 0 && j->paths >= s->largeMin) {
                s->pending.erase(s->pending.begin() + (long)k);
                j->state = 1, j->tAdmit = now;
                s->largeQ.push_back(j);
                moved = true;
            } else {
                k++;
            }
        }
        if (moved) s->lcv.notify_all();
    }
    while (!s->pending.empty()) {
        size_t pick = 0;
        if (now - s->pending.front()->tSubmit <= s->maxWaitS)
            for (size_t k = 1; k < s->pending.size(); k++)
                if (s->pending[k]->paths < s->pending[pick]->paths) pick = k;
        Job* j = s->pending[pick];
        if (j->kind == 1) {
            s->pending.erase(s->pending.begin() + (long)pick);
            j->state = 1, j->tAdmit = now;
            post(s, [s, j] { run_query(s, j); });
            continue;
        }
        if (j->scene >= s->graphScenes) break;                  /* its scene is not in the tick graph yet */
        const bool express = j->paths <= s->expressMax;
        if (express) {
            /* a small job runs whole, beside the waves, in the next tick: no queue memory, its own budget */
            if (j->paths > expBudget || nExp >= MAX_EXPRESS) break;
            int slot = -1;
            for (int k = 0; k < MAX_SLOTS; k++)
                if (!s->slots[k]) { slot = k; break; }
            if (slot < 0) break;
            s->pending.erase(s->pending.begin() + (long)pick);
            j->slot = slot;
            j->express = true;
            s->slots[slot] = j;
            j->state = 1, j->tAdmit = now;
            ranges.push_back({j, 0, j->paths, true, true});
            j->admittedPaths = j->paths;
            expBudget -= j->paths;
            nExp++;
            continue;
        }
        if (budget <= 0 || nNew >= MAX_NEW) break;
        if (inUse + j->paths > s->capacity) break;   /* wait for path memory */
        int slot = -1;
        for (int k = 0; k < MAX_SLOTS; k++)
            if (!s->slots[k]) { slot = k; break; }
        if (slot < 0) break;
        s->pending.erase(s->pending.begin() + (long)pick);
        j->slot = slot;
        s->slots[slot] = j;
        s->pathsInFlight += j->paths;
        inUse += j->paths;
        j->state = 1, j->tAdmit = now;
        take(j, true);
        if (j->admittedPaths < j->paths) s->partial.push_back(j);
    }
}

void tick_loop_body(lh2g_server* s);
int build_tick_graph(lh2g_server* s);
int build_loop_graph(lh2g_server* s);

void tick_loop(lh2g_server* s) {
    tick_loop_body(s);
    cudaStreamSynchronize(s->st);
    std::lock_guard<std::mutex> g(s->mu);
    s->loopExited = true;
    s->cvDone.notify_all();
}

void tick_loop_body(lh2g_server* s) {
    cudaSetDevice(s->device);
    const int ring = (int)s->tickEv.size();
    std::vector<Range> admitted;
    for (;;) {
        {
            /* scenes added since the tick graph was captured: capture it again (the scene table is a kernel
             * parameter) */
            int n;
            {
                std::lock_guard<std::mutex> g(s->mu);
                n = (int)s->scenes.size();
            }
            if (n != s->graphScenes && build_tick_graph(s) != LH2G_OK) {
                std::lock_guard<std::mutex> g(s->mu);
                s->err = "tick graph capture failed";
            }
            bool wantLoop;
            {
                std::lock_guard<std::mutex> g(s->mu);
                wantLoop = s->deviceLoop;
            }
            if (wantLoop && n != s->loopScenes && build_loop_graph(s) != LH2G_OK) {
                cudaGetLastError();
                if (s->loopExec) cudaGraphExecDestroy(s->loopExec), s->loopExec = nullptr;
                std::lock_guard<std::mutex> g(s->mu);
                s->err = "device loop graph build failed: ticks stay host-driven";
                s->deviceLoop = false;
            }
        }
        admitted.clear();
        admit(s, admitted);
        bool active = false;
        {
            std::unique_lock<std::mutex> g(s->mu);
            if (s->abortLoop) return;
            for (int k = 0; k < MAX_SLOTS && !active; k++) active = s->slots[k] != nullptr;
            if (!active && admitted.empty()) {
                if (s->stop) return;
                s->cvWork.wait_for(g, std::chrono::milliseconds(2));
                continue;
            }
        }
        /* new jobs: device records, live counts, per-job memory (stream-ordered), tick parameters */
        uint32_t total = 0, expTotal = 0, nNew = 0, nExp = 0;
        /* staging entry of this tick: its previous user (ticksLaunched - ring) has completed, since at most two
         * ticks are in flight */
        ServerState& tp = s->hTick[s->ticksLaunched % ring];
        for (size_t k = 0; k < admitted.size(); k++) {
            Job* j = admitted[k].job;
            if (admitted[k].first) {
                JobGPU& G = j->gpu;
                G.F = frame_of(&j->view, &j->params);
                G.scene = j->scene;
                G.pathAcc = nullptr, G.out = nullptr;
                if (cudaMallocAsync((void**)&G.pathAcc, sizeof(float4) * (size_t)j->paths, s->st) != cudaSuccess ||
                    cudaMallocAsync((void**)&G.out, sizeof(float4) * (size_t)G.F.W * G.F.H, s->st) != cudaSuccess) {
                    /* no device memory for this job: it fails, the others go on */
                    if (G.pathAcc) cudaFreeAsync(G.pathAcc, s->st);
                    {
                        std::lock_guard<std::mutex> g(s->mu);
                        s->slots[j->slot] = nullptr;
                        if (!j->express) s->pathsInFlight -= j->paths;
                        s->partial.erase(std::remove(s->partial.begin(), s->partial.end(), j), s->partial.end());
                    }
                    finish(s, j, 4);
                    continue;
                }
                cudaMemcpyAsync(s->dJobs + j->slot, &G, sizeof(JobGPU), cudaMemcpyHostToDevice, s->st);
                const int live = (int)j->paths;
                cudaMemcpyAsync(s->dAlive + j->slot, &live, sizeof(int), cudaMemcpyHostToDevice, s->st);
                j->admitTick = s->ticksLaunched;
            }
            if (admitted[k].express) {
                tp.expSlot[nExp] = (uint32_t)j->slot;
                tp.expPrefix[nExp] = expTotal;
                expTotal += (uint32_t)admitted[k].count;
                nExp++;
            } else {
                tp.newSlot[nNew] = (uint32_t)j->slot;
                tp.newStart[nNew] = (uint32_t)admitted[k].start;
                tp.newPrefix[nNew] = total;
                total += (uint32_t)admitted[k].count;
                nNew++;
            }
        }
        tp.newCount = nNew, tp.newPrefix[nNew] = total, tp.newTotal = total;
        tp.expCount = nExp, tp.expPrefix[nExp] = expTotal, tp.expTotal = expTotal;
        cudaMemcpyAsync(&s->dState->newCount, &tp.newCount, offsetof(ServerState, rays) - offsetof(ServerState, newCount), cudaMemcpyHostToDevice,
                        s->st);
        bool loopLaunch;
        {
            std::lock_guard<std::mutex> g(s->mu);
            loopLaunch = s->deviceLoop && s->loopExec && s->loopScenes == s->graphScenes;
        }
        if (loopLaunch) {
            /* the device-side loop: this tick's ranges as staged above, later ticks' ranges of the jobs still
             * entering the queues from the device; the launch ends when the host is needed */
            while (s->ticksLaunched > s->ticksDone) {   /* (host-driven ticks still in flight) */
                cudaEventSynchronize(s->tickEv[s->ticksDone % ring]);
                s->ticksDone++;
            }
            LoopState& L = s->hLoop[0];
            {
                std::lock_guard<std::mutex> g(s->mu);
                L.ticks = 0, L.limit = (uint32_t)std::max(1ll, std::min(s->loopLimit, 1ll << 20));
                L.budget = (uint32_t)std::min(std::max(s->tickBudget, 1ll), (long long)UINT32_MAX);
                L.nPart = 0;
                for (Job* j : s->partial) {
                    L.partSlot[L.nPart] = (uint32_t)j->slot, L.partNext[L.nPart] = (uint32_t)j->admittedPaths;
                    L.partEnd[L.nPart] = (uint32_t)j->paths, L.nPart++;
                }
                for (int k = 0; k < MAX_SLOTS; k++) L.active[k] = s->slots[k] ? 1u : 0u;
                L.doorbell = s->dDoorbell;
                *(volatile int*)s->hDoorbell = 0;   /* jobs submitted from now on end the launch after their tick */
            }
            cudaMemcpyAsync(s->dLoop, &L, sizeof(LoopState), cudaMemcpyHostToDevice, s->st);
            cudaGraphLaunch(s->loopExec, s->st);
            cudaMemcpyAsync(&s->hLoop[1], s->dLoop, sizeof(LoopState), cudaMemcpyDeviceToHost, s->st);
            cudaStreamSynchronize(s->st);
            const LoopState& R = s->hLoop[1];
            s->ticksLaunched += std::max(R.ticks, 1u);
            s->ticksDone = s->ticksLaunched;
            std::lock_guard<std::mutex> g(s->mu);
            s->loopLaunches++;
            for (uint32_t p = 0; p < R.nPart; p++) {
                Job* j = s->slots[R.partSlot[p]];
                if (j) j->admittedPaths = R.partNext[p];
            }
            s->partial.erase(std::remove_if(s->partial.begin(), s->partial.end(), [](const Job* j) { return j->admittedPaths == j->paths; }),
                             s->partial.end());
        } else {
            /* the tick */
            cudaGraphLaunch(s->tickExec, s->st);
            cudaEventRecord(s->tickEv[s->ticksLaunched % ring], s->st);
            s->ticksLaunched++;
            /* at most two ticks in flight: the host prepares the next tick while the GPU runs the current one; the
             * live counts on the host are then at least as new as the older of the two */
            while (s->ticksLaunched - s->ticksDone > 1) {
                cudaEventSynchronize(s->tickEv[s->ticksDone % ring]);
                s->ticksDone++;
            }
        }
        /* jobs with no live path left: finalize, release, copy out */
        std::vector<Job*> done;
        {
            std::lock_guard<std::mutex> g(s->mu);
            for (int k = 0; k < MAX_SLOTS; k++) {
                Job* j = s->slots[k];
                if (j && j->admitTick < s->ticksDone && j->admittedPaths == j->paths && s->hAlive[k] <= 0) done.push_back(j);
            }
        }
        for (Job* j : done) {
            JobGPU& G = j->gpu;
            const int64_t WH = (int64_t)G.F.W * G.F.H;
            k_srv_finalize<<<(unsigned)((WH + 255) / 256), 256, 0, s->st>>>(G);
            cudaFreeAsync(G.pathAcc, s->st);
            cudaEvent_t ev;
            cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
            cudaEventRecord(ev, s->st);
            {
                std::lock_guard<std::mutex> g(s->mu);
                s->slots[j->slot] = nullptr;
                if (!j->express) s->pathsInFlight -= j->paths;
                j->state = 2;
            }
            post(s, [s, j, ev] {
                JobGPU& G2 = j->gpu;
                cudaStreamWaitEvent(s->io, ev, 0);
                const size_t bytes = sizeof(float4) * (size_t)G2.F.W * G2.F.H;
                bool ok = cudaMemcpyAsync(j->hostOut, G2.out, bytes, cudaMemcpyDeviceToHost, s->io) == cudaSuccess;
                cudaFreeAsync(G2.out, s->io);
                ok = cudaStreamSynchronize(s->io) == cudaSuccess && ok;
                cudaEventDestroy(ev);
                finish(s, j, ok ? 3 : 4);
            });
        }
        if (!done.empty()) s->cvWork.notify_all();
    }
}

/* the launches of one tick, on s->st (being captured) */
void capture_tick_body(lh2g_server* s, const SceneTable& T, int n) {
    k_srv_generate<<<s->blocksGen, 256, 0, s->st>>>(s->dJobs, s->dState, s->Q);
    /* express jobs on a second branch, beside the waves; the tick ends when both are done */
    cudaEventRecord(s->evFork, s->st);
    cudaStreamWaitEvent(s->side, s->evFork, 0);
    k_srv_express<<<s->blocksExpress, WAVE_BLOCK, 0, s->side>>>(T, s->dJobs, s->dState, s->dAlive);
    cudaEventRecord(s->evJoin, s->side);
    k_srv_extend<<<s->blocksExtend, 128, 0, s->st>>>(T, s->dJobs, s->dState, s->Q);
    k_srv_partition<<<s->blocksPart, PART_TILE, 0, s->st>>>(s->dState, s->Q);
    int lights = 1;   /* at most 64 per scene (lh2g_set_lights) */
    for (int k = 0; k < n; k++) lights = std::max(lights, T.s[k].nTri + T.s[k].nPoint + T.s[k].nSpot + T.s[k].nDir);
    k_srv_shade<<<s->blocksShade, WAVE_BLOCK, (size_t)lights * WAVE_BLOCK * sizeof(float), s->st>>>(T, s->dJobs, s->dState, s->Q, s->dAlive);
    k_srv_connect<<<s->blocksConnect, 128, 0, s->st>>>(T, s->dJobs, s->dState, s->Q);
    cudaStreamWaitEvent(s->st, s->evJoin, 0);
    k_srv_end<<<1, 1, 0, s->st>>>(s->dState);
    cudaMemcpyAsync(s->hAlive, s->dAlive, sizeof(int) * MAX_SLOTS, cudaMemcpyDeviceToHost, s->st);
}

int scene_table(lh2g_server* s, SceneTable& T) {
    memset(&T, 0, sizeof(T));
    std::lock_guard<std::mutex> g(s->mu);
    const int n = (int)s->scenes.size();
    for (int k = 0; k < n; k++) T.s[k] = s->scenes[k];
    return n;
}

int build_tick_graph(lh2g_server* s) {
    SceneTable T;
    const int n = scene_table(s, T);
    if (s->tickExec) cudaGraphExecDestroy(s->tickExec), s->tickExec = nullptr;
    if (s->tickGraph) cudaGraphDestroy(s->tickGraph), s->tickGraph = nullptr;
    if (cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return LH2G_ERR_CUDA;
    capture_tick_body(s, T, n);
    if (cudaStreamEndCapture(s->st, &s->tickGraph) != cudaSuccess) return LH2G_ERR_CUDA;
    if (cudaGraphInstantiate(&s->tickExec, s->tickGraph, 0) != cudaSuccess) return LH2G_ERR_CUDA;
    s->graphScenes = n;
    return LH2G_OK;
}

/* the device-side loop: a conditional WHILE node (its condition set to 1 at every launch) whose body is the tick
 * followed by k_srv_loop_end, which sets the condition for the next iteration */
int build_loop_graph(lh2g_server* s) {
    SceneTable T;
    const int n = scene_table(s, T);
    if (s->loopExec) cudaGraphExecDestroy(s->loopExec), s->loopExec = nullptr;
    if (s->loopGraph) cudaGraphDestroy(s->loopGraph), s->loopGraph = nullptr;
    if (cudaGraphCreate(&s->loopGraph, 0) != cudaSuccess) return LH2G_ERR_CUDA;
    cudaGraphConditionalHandle handle;
    if (cudaGraphConditionalHandleCreate(&handle, s->loopGraph, 1, cudaGraphCondAssignDefault) != cudaSuccess) return LH2G_ERR_CUDA;
    alignas(cudaGraphNodeParams) unsigned char cpBytes[sizeof(cudaGraphNodeParams)];   /* (no default constructor: a union) */
    memset(cpBytes, 0, sizeof(cpBytes));
    cudaGraphNodeParams& cp = *reinterpret_cast<cudaGraphNodeParams*>(cpBytes);
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, s->loopGraph, nullptr, nullptr, 0, &cp) != cudaSuccess) return LH2G_ERR_CUDA;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if (cudaStreamBeginCaptureToGraph(s->st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return LH2G_ERR_CUDA;
    capture_tick_body(s, T, n);
    k_srv_loop_end<<<1, MAX_SLOTS, 0, s->st>>>(s->dState, s->dLoop, s->dAlive, handle);
    cudaGraph_t captured = nullptr;
    if (cudaStreamEndCapture(s->st, &captured) != cudaSuccess) return LH2G_ERR_CUDA;
    if (cudaGraphInstantiate(&s->loopExec, s->loopGraph, 0) != cudaSuccess) return LH2G_ERR_CUDA;
    s->loopScenes = n;
    return LH2G_OK;
}

template <typename K>
int occupancy_blocks(K kernel, int threads) {
    int dev = 0, sms = 1, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
    return sms * std::max(per, 1);
}

}  // namespace srv
}  // namespace lh2g

extern "C" {

int lh2g_server_create(int device, long long pathCapacity, lh2g_server** out) {
    if (!out || pathCapacity <= 0 || pathCapacity >= (1ll << 31)) return LH2G_ERR_INVALID;
    *out = nullptr;
    lh2g_server* s = new lh2g_server();
    s->device = device;
    s->capacity = pathCapacity;
    s->tickBudget = std::max(1ll << 20, std::min(pathCapacity, 1ll << 22));
    memset(&s->Q, 0, sizeof(s->Q));
    bool ok = cudaSetDevice(device) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&s->io, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&s->evFork, cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&s->evJoin, cudaEventDisableTiming) == cudaSuccess;
    const size_t cap = (size_t)pathCapacity;
    for (int k = 0; k < 2 && ok; k++)
        ok = cudaMalloc((void**)&s->Q.O[k], 16 * cap) == cudaSuccess && cudaMalloc((void**)&s->Q.D[k], 16 * cap) == cudaSuccess &&
             cudaMalloc((void**)&s->Q.T[k], 16 * cap) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&s->Q.hits, 16 * cap) == cudaSuccess && cudaMalloc((void**)&s->Q.shO, 16 * cap) == cudaSuccess &&
         cudaMalloc((void**)&s->Q.shD, 16 * cap) == cudaSuccess && cudaMalloc((void**)&s->Q.shE, 16 * cap) == cudaSuccess &&
         cudaMalloc((void**)&s->Q.order, 4 * cap) == cudaSuccess;
    s->Q.cap = (uint32_t)cap;
    ok = ok && cudaMalloc((void**)&s->dJobs, sizeof(JobGPU) * MAX_SLOTS) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&s->dAlive, sizeof(int) * MAX_SLOTS) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&s->dState, sizeof(ServerState)) == cudaSuccess;
    ok = ok && cudaMallocHost((void**)&s->hAlive, sizeof(int) * MAX_SLOTS) == cudaSuccess;
    ok = ok && cudaMallocHost((void**)&s->hTick, sizeof(ServerState) * 4) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&s->dLoop, sizeof(LoopState)) == cudaSuccess;
    ok = ok && cudaMallocHost((void**)&s->hLoop, sizeof(LoopState) * 2) == cudaSuccess;
    ok = ok && cudaHostAlloc((void**)&s->hDoorbell, sizeof(int), cudaHostAllocMapped) == cudaSuccess;
    ok = ok && cudaHostGetDevicePointer((void**)&s->dDoorbell, s->hDoorbell, 0) == cudaSuccess;
    if (ok) {
        cudaMemset(s->dAlive, 0, sizeof(int) * MAX_SLOTS);
        cudaMemset(s->dState, 0, sizeof(ServerState));
        memset(s->hAlive, 0, sizeof(int) * MAX_SLOTS);
        memset(s->hTick, 0, sizeof(ServerState) * 4);
        memset(s->hLoop, 0, sizeof(LoopState) * 2);
        *s->hDoorbell = 0;
        /* per-job memory comes from the stream-ordered pool: keep what it holds between jobs */
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        s->blocksGen = occupancy_blocks(k_srv_generate, 256);
        s->blocksExtend = occupancy_blocks(k_srv_extend, 128);
        s->blocksShade = occupancy_blocks(k_srv_shade, WAVE_BLOCK);
        s->blocksConnect = occupancy_blocks(k_srv_connect, 128);
        /* a modest share of the SMs (two CTAs each): the express branch runs beside the waves */
        int sms = 1;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        s->blocksExpress = 2 * sms;
        s->blocksPart = 2 * sms;
        s->blocksTrace0 = persistent_blocks_trace(0);
        s->blocksTrace1 = persistent_blocks_trace(1);
        s->tickEv.resize(4);
        for (auto& e : s->tickEv) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
        ok = ok && cudaDeviceSynchronize() == cudaSuccess;
    }
    if (!ok) {
        lh2g_server_destroy(s);
        return LH2G_ERR_CUDA;
    }
    ok = ok && cudaStreamCreateWithFlags(&s->lst, cudaStreamNonBlocking) == cudaSuccess;
    if (!ok) {
        lh2g_server_destroy(s);
        return LH2G_ERR_CUDA;
    }
    s->loop = std::thread(tick_loop, s);
    s->worker = std::thread(worker_loop, s);
    s->large = std::thread(large_loop, s);
    *out = s;
    return LH2G_OK;
}

int lh2g_server_destroy(lh2g_server* s) {
    if (!s) return LH2G_ERR_INVALID;
    {
        std::unique_lock<std::mutex> g(s->mu);
        s->stop = true;
        s->cvWork.notify_all();
        /* let the loop finish the jobs it holds; a drain longer than 30 s ends it */
        if (s->loop.joinable() && !s->cvDone.wait_for(g, std::chrono::seconds(30), [&] { return s->loopExited; })) s->abortLoop = true;
    }
    s->cvWork.notify_all();
    if (s->loop.joinable()) s->loop.join();
    {
        std::lock_guard<std::mutex> g(s->tmu);
    }
    s->tcv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->lcv.notify_all();
    }
    if (s->large.joinable()) s->large.join();
    cudaSetDevice(s->device);
    if (s->st) cudaStreamSynchronize(s->st);
    if (s->io) cudaStreamSynchronize(s->io);
    if (s->side) cudaStreamSynchronize(s->side);
    if (s->tickExec) cudaGraphExecDestroy(s->tickExec);
    if (s->tickGraph) cudaGraphDestroy(s->tickGraph);
    if (s->loopExec) cudaGraphExecDestroy(s->loopExec);
    if (s->loopGraph) cudaGraphDestroy(s->loopGraph);
    cudaFree(s->dLoop);
    if (s->hLoop) cudaFreeHost(s->hLoop);
    if (s->hDoorbell) cudaFreeHost(s->hDoorbell);
    for (auto& e : s->tickEv) if (e) cudaEventDestroy(e);
    for (int k = 0; k < 2; k++) cudaFree(s->Q.O[k]), cudaFree(s->Q.D[k]), cudaFree(s->Q.T[k]);
    cudaFree(s->Q.hits), cudaFree(s->Q.shO), cudaFree(s->Q.shD), cudaFree(s->Q.shE), cudaFree(s->Q.order);
    cudaFree(s->dJobs), cudaFree(s->dAlive), cudaFree(s->dState);
    if (s->lst) cudaStreamSynchronize(s->lst), cudaStreamDestroy(s->lst);
    {
        WaveBuffers& B = s->LB;
        for (int k = 0; k < 2; k++) cudaFree(B.O[k]), cudaFree(B.D[k]), cudaFree(B.T[k]);
        cudaFree(B.hits), cudaFree(B.shO), cudaFree(B.shD), cudaFree(B.shE), cudaFree(B.pathAcc), cudaFree(B.order);
        cudaFree(B.accum), cudaFree(B.frame), cudaFree(B.counters);
        if (s->lhost) cudaFreeHost(s->lhost);
    }
    if (s->hAlive) cudaFreeHost(s->hAlive);
    if (s->hTick) cudaFreeHost(s->hTick);
    for (auto& kv : s->jobs) delete kv.second;
    if (s->st) cudaStreamDestroy(s->st);
    if (s->io) cudaStreamDestroy(s->io);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->evFork) cudaEventDestroy(s->evFork);
    if (s->evJoin) cudaEventDestroy(s->evJoin);
    delete s;
    return LH2G_OK;
}

const char* lh2g_server_last_error(lh2g_server* s) { return s ? s->err.c_str() : "null server"; }

int lh2g_server_setting(lh2g_server* s, const char* name, double value) {
    if (!s || !name || !(value >= 0.0)) return LH2G_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    if (!strcmp(name, "expressMaxPaths")) s->expressMax = (long long)value;
    else if (!strcmp(name, "expressBudget")) s->expressBudget = (long long)value;
    else if (!strcmp(name, "tickBudget")) s->tickBudget = std::max(1ll, (long long)value);
    else if (!strcmp(name, "maxWaitSeconds")) s->maxWaitS = value;
    else if (!strcmp(name, "largeJobPaths")) s->largeMin = (long long)value;
    else if (!strcmp(name, "deviceLoop")) s->deviceLoop = value != 0.0;
    else if (!strcmp(name, "loopTicks")) s->loopLimit = std::max(1ll, (long long)value);
    else {
        s->err = std::string("unknown server setting ") + name;
        return LH2G_ERR_INVALID;
    }
    if (s->expressMax > s->expressBudget) s->expressBudget = s->expressMax;   /* every express job fits a tick */
    return LH2G_OK;
}

int lh2g_server_add_scene(lh2g_server* s, lh2g_context* ctx, int* sceneId) {
    if (!s || !ctx || !sceneId) return LH2G_ERR_INVALID;
    SceneGPU S;
    int dev = 0, blocks[4], tail = 0;
    const int r = context_scene(ctx, &S, &dev, blocks, &tail);
    if (r != LH2G_OK) return sfail(s, r, "add_scene: the context has no finalized scene");
    if (dev != s->device) return sfail(s, LH2G_ERR_INVALID, "add_scene: the context is on another device");
    if (S.nTri + S.nPoint + S.nSpot + S.nDir > 64)
        return sfail(s, LH2G_ERR_INVALID, "add_scene: at most 64 lights (the serving loop selects lights by their potentials)");
    {
        std::lock_guard<std::mutex> g(s->mu);
        if ((int)s->scenes.size() >= MAX_SCENES) { s->err = "add_scene: at most 16 scenes"; return LH2G_ERR_OVERFLOW; }
        *sceneId = (int)s->scenes.size();
        s->scenes.push_back(S);
    }
    /* the tick loop captures its graph again with the new table before it admits a job of this scene */
    s->cvWork.notify_all();
    return LH2G_OK;
}

int lh2g_server_submit_render(lh2g_server* s, int sceneId, const lh2g_view* view, const lh2g_render_params* p, float* hostOut, long long* jobId) {
    if (!s || !view || !p || !hostOut || !jobId) return LH2G_ERR_INVALID;
    if (p->width <= 0 || p->height <= 0 || p->spp <= 0 || p->maxDepth < 1 || p->maxDepth > 64 ||
        (p->flags & (LH2G_RP_FILTER | LH2G_RP_NRC | LH2G_RP_OPTIX7 | LH2G_RP_ADAPTIVE | LH2G_RP_DISNEY | LH2G_RP_LIGHTTREE)) || p->rowCount != 0)
        return sfail(s, LH2G_ERR_INVALID, "submit_render: bad parameters (filter frames are not served)");
    const long long P = (long long)p->width * p->height * p->spp;
    Job* j = new Job();
    j->kind = 0, j->view = *view, j->params = *p, j->hostOut = hostOut, j->paths = P, j->tSubmit = now_s();
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (sceneId < 0 || sceneId >= (int)s->scenes.size()) { delete j; s->err = "submit_render: unknown scene"; return LH2G_ERR_INVALID; }
        if (P > s->capacity && !(s->largeMin > 0 && P >= s->largeMin)) {
            delete j;
            s->err = "submit_render: the job has more paths than the server's capacity";
            return LH2G_ERR_OVERFLOW;
        }
        j->scene = sceneId;
        j->id = s->nextId++;
        s->jobs[j->id] = j;
        s->pending.push_back(j);
        *jobId = j->id;
        *(volatile int*)s->hDoorbell = 1;   /* a running device loop ends after its tick */
    }
    s->cvWork.notify_all();
    return LH2G_OK;
}

int lh2g_server_submit_trace(lh2g_server* s, int sceneId, const lh2g_ray* hostRays, long long n, int mode, void* hostOut, long long* jobId) {
    if (!s || !hostRays || !hostOut || !jobId || n <= 0 || n >= (1ll << 31) || (mode != 0 && mode != 1)) return LH2G_ERR_INVALID;
    Job* j = new Job();
    j->kind = 1, j->hostRays = hostRays, j->n = n, j->mode = mode, j->hostOut = hostOut, j->tSubmit = now_s();
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (sceneId < 0 || sceneId >= (int)s->scenes.size()) { delete j; s->err = "submit_trace: unknown scene"; return LH2G_ERR_INVALID; }
        j->scene = sceneId;
        j->id = s->nextId++;
        s->jobs[j->id] = j;
        s->pending.push_back(j);
        *jobId = j->id;
        *(volatile int*)s->hDoorbell = 1;   /* a running device loop ends after its tick */
    }
    s->cvWork.notify_all();
    return LH2G_OK;
}

int lh2g_server_wait(lh2g_server* s, long long jobId, int timeoutMs, lh2g_job_times* times) {
    if (!s) return LH2G_ERR_INVALID;
    std::unique_lock<std::mutex> g(s->mu);
    auto it = s->jobs.find(jobId);
    if (it == s->jobs.end()) return LH2G_ERR_INVALID;
    Job* j = it->second;
    const bool done = s->cvDone.wait_for(g, std::chrono::milliseconds(timeoutMs < 0 ? 0 : timeoutMs), [&] { return j->state >= 3; });
    if (!done) return LH2G_ERR_STATE;
    if (times) times->submit = j->tSubmit, times->admit = j->tAdmit, times->done = j->tDone;
    return j->state == 3 ? LH2G_OK : LH2G_ERR_CUDA;
}

int lh2g_server_release(lh2g_server* s, long long jobId) {
    if (!s) return LH2G_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->jobs.find(jobId);
    if (it == s->jobs.end() || it->second->state < 3) return LH2G_ERR_STATE;
    delete it->second;
    s->jobs.erase(it);
    return LH2G_OK;
}

int lh2g_server_get_stats(lh2g_server* s, lh2g_server_stats* out) {
    if (!s || !out) return LH2G_ERR_INVALID;
    ServerState st;
    cudaSetDevice(s->device);
    /* a plain read of two counters; the copy may overlap a running tick (values from some tick boundary) */
    if (cudaMemcpy(&st, s->dState, sizeof(ServerState), cudaMemcpyDeviceToHost) != cudaSuccess) return LH2G_ERR_CUDA;
    std::lock_guard<std::mutex> g(s->mu);
    out->ticks = st.ticks;
    out->raysTraced = st.rays + s->raysDone;
    out->jobsDone = s->jobsDone;
    out->pathsInFlight = s->pathsInFlight;
    out->pending = (long long)s->pending.size();
    out->deviceStatus = st.status | s->largeStatus;
    out->loopLaunches = s->loopLaunches;
    return LH2G_OK;
}

}  // extern "C"

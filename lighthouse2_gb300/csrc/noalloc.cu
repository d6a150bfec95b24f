/* noalloc.cu - a frame render that allocates no device memory.
 *
 * Some callers cannot call cudaMalloc at render time: a host that hands the core a fixed memory budget up front
 * and forbids further allocation (a game engine or a plugin host with its own device allocator), or a process
 * that must not grow its device footprint after start-up. lh2g_render_noalloc serves them: it renders one frame
 * of at most LH2G_NOALLOC_MAX_PATHS paths with every scratch buffer of the wavefront stages (path-state queues,
 * hit records, connections, per-path radiance, queue counters, the finalized frame) placed in the file-scope
 * device array below. The scene still comes from the context (uploaded earlier by the setters), and the caller
 * passes the per-pixel accumulator it wants the frame added to.
 *
 * The array (about 6 MB) is part of the library image: every GPU that loads the library holds it until the
 * process exits. All calls share it and it keeps the last call's contents; the queue counters are cleared at the
 * start of every call and every other buffer is written before it is read. Calls whose work overlaps on the GPU
 * (two streams, two threads, two contexts on one device) race on the array.
 *
 * The array's device address belongs to the CUDA context that loaded the module: it is looked up per device
 * and cached together with the unique id of the context current at the time (cuCtxGetId). A call from another
 * context on the device, or after cudaDeviceReset ended the old one, sees a different id and looks the address up
 * again instead of using a stale one.
 */
#include <algorithm>
#include <mutex>

#include <cuda.h>

#include "kernels.cuh"
#include "lh2g.h"

namespace {

constexpr size_t PATH_BYTES = 176;   /* 2 x (O, D, T) + hit + 3 connection float4 + per-path radiance */
constexpr size_t MAX_DEVICES = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[(size_t)LH2G_NOALLOC_MAX_PATHS * PATH_BYTES + sizeof(lh2g::Counters) +
                                                          (size_t)LH2G_NOALLOC_MAX_PATHS * 16 + 1024];

std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[MAX_DEVICES] = {nullptr};
unsigned long long g_scratch_ctx[MAX_DEVICES] = {0};   /* cuCtxGetId of the context the address belongs to */

/* unique id of the current context (0 when it cannot be had), through the runtime's driver entry points so that
 * the library needs no link against the driver library */
unsigned long long current_context_id() {
    typedef CUresult (*GetCurrent)(CUcontext*);
    typedef CUresult (*GetId)(CUcontext, unsigned long long*);
    static GetCurrent getCurrent = nullptr;
    static GetId getId = nullptr;
    static bool looked = false;
    if (!looked) {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess && qa == cudaDriverEntryPointSuccess)
            getCurrent = (GetCurrent)a;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess && qb == cudaDriverEntryPointSuccess)
            getId = (GetId)b;
        looked = true;
    }
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!getCurrent || !getId || getCurrent(&c) != CUDA_SUCCESS || !c || getId(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

}  // namespace

namespace lh2g {
/* defined in capi.cu: the scene and launch configuration of a context */
int context_scene(lh2g_context* ctx, SceneGPU* scene, int* device, int* blocks4, int* tailDepth);
}

extern "C" LH2G_API int lh2g_render_noalloc(lh2g_context* ctx, const lh2g_view* view, const lh2g_render_params* p, float* accumDevice,
                                             void* stream, uint32_t* statusHost) {
    using namespace lh2g;
    if (!ctx || !view || !p || !accumDevice) return LH2G_ERR_INVALID;
    if (p->width <= 0 || p->height <= 0 || p->spp <= 0 || p->maxDepth < 1 || p->maxDepth > 64) return LH2G_ERR_INVALID;
    /* filter, radiance-cache and adaptive frames need the context's own buffers; this path renders the plain estimator */
    if ((p->flags & (LH2G_RP_FILTER | LH2G_RP_NRC | LH2G_RP_OPTIX7 | LH2G_RP_ADAPTIVE | LH2G_RP_DISNEY | LH2G_RP_LIGHTTREE)) || p->rowCount != 0) return LH2G_ERR_INVALID;
    const long long P = (long long)p->width * p->height * p->spp;
    if (P > LH2G_NOALLOC_MAX_PATHS) return LH2G_ERR_OVERFLOW;   /* width * height * spp above the static capacity */
    SceneGPU S;
    int device = 0, blocks[4] = {0, 0, 0, 0}, tailDepth = 0;
    const int r = context_scene(ctx, &S, &device, blocks, &tailDepth);
    if (r != LH2G_OK) return r;
    if (device < 0 || (size_t)device >= MAX_DEVICES) return LH2G_ERR_INVALID;
    if (S.nTri + S.nPoint + S.nSpot + S.nDir > 64) return LH2G_ERR_INVALID;   /* the plain estimator selects lights by potential */
    int current = -1;
    if (cudaGetDevice(&current) != cudaSuccess) return LH2G_ERR_CUDA;
    if (current != device && cudaSetDevice(device) != cudaSuccess) return LH2G_ERR_CUDA;
    unsigned char* base;
    {
        /* once per device, with that device current: the device address of the array (in host code its name
         * only stands for it) */
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        const unsigned long long cid = current_context_id();
        if (!g_scratch_addr[device] || cid == 0 || cid != g_scratch_ctx[device]) {
            void* a = nullptr;
            if (cudaGetSymbolAddress(&a, g_noalloc_scratch) != cudaSuccess || !a) {
                if (current != device) cudaSetDevice(current);
                return LH2G_ERR_CUDA;
            }
            g_scratch_addr[device] = (unsigned char*)a;
            g_scratch_ctx[device] = cid;
        }
        base = g_scratch_addr[device];
    }
    cudaStream_t st = (cudaStream_t)stream;
    WaveBuffers B{};   /* every buffer not set below is null */
    float4* f = (float4*)base;
    const size_t n = (size_t)LH2G_NOALLOC_MAX_PATHS;
    B.O[0] = f, B.D[0] = f + n, B.T[0] = f + 2 * n, B.O[1] = f + 3 * n, B.D[1] = f + 4 * n, B.T[1] = f + 5 * n;
    B.hits = f + 6 * n, B.shO = f + 7 * n, B.shD = f + 8 * n, B.shE = f + 9 * n, B.pathAcc = f + 10 * n;
    B.frame = f + 11 * n;
    B.counters = (Counters*)(f + 12 * n);
    B.accum = (float4*)accumDevice;
    B.capHits = nullptr, B.capSeeds = nullptr;
    B.features = nullptr, B.worldPos = nullptr, B.deltaDepth = nullptr, B.nrcRec = nullptr;
    FrameGPU F{};
    F.rowCount = p->height;   /* the whole frame (bandPix 0) */
    F.W = p->width, F.H = p->height, F.spp = p->spp, F.maxDepth = p->maxDepth, F.rrStart = p->rrStartDepth, F.samplesTaken = p->samplesTaken;
    F.cameraR0 = p->cameraR0, F.frameSeed = p->frameSeed, F.eps = p->geometryEpsilon, F.flags = p->flags;
    F.spreadAngle = view->spreadAngle, F.aperture = view->aperture;
    F.pos = make_float3(view->pos[0], view->pos[1], view->pos[2]);
    F.p1 = make_float3(view->p1[0], view->p1[1], view->p1[2]);
    F.right = make_float3(view->p2[0] - view->p1[0], view->p2[1] - view->p1[1], view->p2[2] - view->p1[2]);
    F.up = make_float3(view->p3[0] - view->p1[0], view->p3[1] - view->p1[1], view->p3[2] - view->p1[2]);
    F.P = P;
    F.stride = (int64_t)n;
    if (cudaMemsetAsync(B.counters, 0, sizeof(Counters), st) != cudaSuccess) {
        if (current != device) cudaSetDevice(current);
        return LH2G_ERR_CUDA;
    }
    launch_generate(F, B, st);
    const int waves = tailDepth > 0 ? std::min(F.maxDepth, tailDepth - 1) : F.maxDepth;
    for (int d = 1; d <= waves; d++) {
        launch_extend(S, F, B, d, blocks[0], st);
        launch_shade(S, F, B, d, blocks[2], st);
        launch_connect(S, F, B, d, blocks[1], st);
    }
    if (waves < F.maxDepth) launch_tail(S, F, B, waves + 1, blocks[3], st);
    launch_finalize(F, B, 1.0f / (float)(p->samplesTaken + F.spp), 0, st);
    /* the status word (LH2G_STATUS_* bits: traversal stack overflow, step limit) to the caller, on the stream */
    cudaError_t e = statusHost ? cudaMemcpyAsync(statusHost, &B.counters->status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) : cudaSuccess;
    const cudaError_t le = cudaGetLastError();
    if (e == cudaSuccess) e = le;
    if (current != device) cudaSetDevice(current);
    return e == cudaSuccess ? LH2G_OK : LH2G_ERR_CUDA;
}

/* capi.cu - host side of the GB300 render core: context, scene upload, device BVH finalisation, frame
 * orchestration and ray queries behind the C ABI of include/lh2g.h.
 *
 * Host-side semantics follow the reference core:
 *   scene setters        lib/RenderCore_PrimeRef/rendercore.cpp:214-478 (meshes appended in index order,
 *                        SetInstance(n, -1) truncates, textures before materials, lights <= 64)
 *   material packing     rendercore.cpp:360-402 (half colours, 8-bit parameters, 16-byte texture maps)
 *   instance inverse     mat4::Inverted, lib/RenderSystem/common_types.h:559-604
 *   Render               rendercore.cpp:535-632 (Restart resets the accumulator, samplesTaken and the camera
 *                        seed 0x12345678; R0 = RandomUInt(camRNGseed); shading R0 = samplesTaken * 7907 +
 *                        pathLength * 91771; output = accumulator / samplesTaken)
 *   Render, "filter" on  lib/RenderCore_Optix7Filter/rendercore.cpp:737-797, 897-935 (Halton subpixel jitter
 *                        when TAA is on, aperture 0, camRNGseed never reset; then SVGF and the history swaps).
 *                        One RandomUInt(camRNGseed) per frame seeds every wave (the reference draws one per wave,
 *                        and its wave count depends on queue sizes read back by the host, which this core never
 *                        reads). The first filtered frame after SetTarget reprojects onto its own view.
 * No stage of a frame waits for the host: queue sizes stay on the device.
 */
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "bvh_build.cuh"
#include "kernels.cuh"
#include "lh2g.h"
#include "light_tree.h"
#include "svgf.cuh"
#include "raster.cuh"

using namespace lh2g;

namespace lh2g {
FrameGPU frame_of(const lh2g_view* view, const lh2g_render_params* p);
}

namespace {

struct MeshDev {
    float4* verts = nullptr;   /* 3 per triangle */
    float4* tris = nullptr;    /* CoreTri4, 13 float4 per triangle */
    float4* rsNorms = nullptr; /* rasterizer: face normal + material per triangle, packed at its first raster frame */
    uint32_t n = 0;
    uint32_t maxMaterial = 0;  /* largest material index of its triangles (checked against the materials at render) */
    float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
};

struct InstHost { int mesh; float T[16]; float inv[16]; };

uint16_t f2h(float f) {   /* round-to-nearest-even float -> half */
    uint32_t x;
    memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u, ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);
    if (ax < 0x38800000u) {
        const uint32_t e = ax >> 23;
        if (e < 102) return (uint16_t)sign;
        const uint32_t m = (ax & 0x7fffffu) | 0x800000u, shift = 126 - e;
        uint32_t h = m >> shift;
        const uint32_t rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1u);
        if (rem > half || (rem == half && (h & 1u))) h++;
        return (uint16_t)(sign | h);
    }
    uint32_t h = (ax >> 13) - (112u << 10);
    const uint32_t rem = ax & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
    return (uint16_t)(sign | h);
}

uint32_t f2u_sat(float x) { if (!(x > 0.0f)) return 0u; if (x >= 4294967296.0f) return 0xffffffffu; return (uint32_t)x; }
uint32_t tochar(float a) { return f2u_sat(a * 255.0f); }
uint32_t touint4(float a, float b, float c, float d) { return tochar(a) + (tochar(b) << 8) + (tochar(c) << 16) + (tochar(d) << 24); }
uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

void pack_material(const lh2g_material& m, const std::vector<uint32_t>& first, const std::vector<uint32_t>& wh, lh2g_gpu_material& g) {
    memset(&g, 0, sizeof(g));
    g.base[0] = (uint32_t)f2h(m.color[0]) | ((uint32_t)f2h(m.color[1]) << 16);
    g.base[1] = (uint32_t)f2h(m.color[2]) | ((uint32_t)f2h(1 - m.absorption[0]) << 16);
    g.base[2] = (uint32_t)f2h(1 - m.absorption[1]) | ((uint32_t)f2h(1 - m.absorption[2]) << 16);
    g.params[0] = touint4(m.metallic, m.subsurface, m.specular, m.roughness);
    g.params[1] = touint4(m.specularTint, m.anisotropic, m.sheen, m.sheenTint);
    g.params[2] = touint4(m.clearcoat, m.clearcoatGloss, m.transmission, 0);
    g.params[3] = fbits(m.eta);
    const lh2g_map_ref* refs[6] = {&m.color_map, &m.detail_color_map, &m.normal_map, &m.detail_normal_map, &m.specular_map, &m.roughness_map};
    for (int i = 0; i < 6; i++) {
        const lh2g_map_ref& r = *refs[i];
        if (r.texture < 0) continue;
        g.maps[i][0] = (wh[2 * r.texture] & 0xffffu) | ((wh[2 * r.texture + 1] & 0xffffu) << 16);
        g.maps[i][1] = (uint32_t)f2h(r.uvscale[0]) | ((uint32_t)f2h(r.uvscale[1]) << 16);
        g.maps[i][2] = (uint32_t)f2h(r.uvoffset[0]) | ((uint32_t)f2h(r.uvoffset[1]) << 16);
        g.maps[i][3] = first[r.texture];
    }
    uint32_t flags = m.eta < 1 ? 1u : 0u;
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

/* mat4::Inverted, cofactor expansion (common_types.h:559-604). */
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

uint32_t xorshift(uint32_t& s) { s ^= s << 13; s ^= s >> 17; s ^= s << 5; return s; }

}  // namespace

constexpr uint32_t NRC_TRAIN_CAP = 65536;   /* training samples per radiance-cache frame */
struct NrcBuffers {
    float4* rec = nullptr;       /* 6 float4 per path (stride = path capacity) */
    float4* queries = nullptr;   /* 4 float4 per query */
    uint32_t* qPath = nullptr;
    float4* pred = nullptr;
    float4* trainQ = nullptr;
    float4* trainT = nullptr;
    uint32_t* counts = nullptr;
    uint32_t* hostCounts = nullptr;
    int64_t cap = 0;
};

struct lh2g_context {
    int device = 0;
    cudaStream_t st = nullptr;
    std::string err;
    std::vector<MeshDev> meshes;
    std::vector<InstHost> inst;
    std::vector<lh2g_material> hostMats;
    uint4* mats = nullptr;
    uint32_t* texels = nullptr;
    std::vector<uint32_t> texFirst, texWH;
    float4 *triL = nullptr, *ptL = nullptr, *spL = nullptr, *dirL = nullptr;
    float4* lightTree = nullptr;       /* 4 float4 per record (light_tree.h) */
    int nTreeNodes = 0;
    int lightTreeOn = 0;               /* setting "lightTree": the OptiX 7 estimator selects lights through the tree */
    int nTri = 0, nPt = 0, nSpot = 0, nDir = 0;
    float4* sky = nullptr;
    float4* skySmall = nullptr;       /* the sky's 64x scaled-down copy (OptiX 7 estimator after a bounce) */
    uint32_t* blueNoise = nullptr;    /* expanded blue-noise tables (lh2g_set_blue_noise) */
    int skyW = 0, skyH = 0;
    float w2s[16];
    /* acceleration structure */
    uint4* pool = nullptr;
    float4* triData = nullptr;
    InstanceGPU* instGPU = nullptr;
    uint32_t* tlasPrims = nullptr;
    uint32_t tlasRoot = 0xffffffffu;
    const float4** instTris = nullptr;
    float4* instInvRows = nullptr;
    bool finalized = false;
    /* target */
    int W = 0, H = 0, spp = 1;
    int64_t cap = 0;
    WaveBuffers B;
    /* settings and accumulation state (RenderCore_PrimeRef/rendercore.cpp:535-550) */
    float eps = 1e-3f, clampValue = 10.0f;
    int maxDepth = 3, rrStart = 1, nee = 1;
    int samplesTaken = 0;
    uint32_t camSeed = 0x12345678u;
    bool firstConverging = true;
    int probeX = -1, probeY = -1;
    lh2g_stats stats;
    Counters* hostCounters = nullptr;   /* pinned copy of the frame's counters */
    int lastDepth = 0;
    int64_t lastP = 0;
    bool statsPending = false;
    uint32_t* traceFetch = nullptr;     /* 64-bit fetch counter + status word */
    lh2g_ray* hostRaysDev = nullptr;
    void* hostOutDev = nullptr;
    long long hostCap = 0;
    cudaEvent_t ev[2];
    bool launchTiming = false;
    std::vector<cudaEvent_t> lev;   /* 2 per launch */
    int timedLaunches = 0;             /* launches timed since the last lh2g_get_launch_times */
    static constexpr int MAX_TIMED_LAUNCHES = 1 << 14;
    int blocksExtend = 0, blocksConnect = 0, blocksShade = 0, blocksTail = 0;
    int fullBlocks[3] = {0, 0, 0};     /* extend, connect, shade grids at full occupancy (setting "waveOccupancy" scales them) */
    /* path length from which the remaining paths run to their end in one persistent kernel (0: wave loop
     * to the end); a scheduling choice only, results are the same */
    int tailDepth = 5;
    /* SVGF (filter core) state: settings of lib/RenderCore_Optix7Filter/rendercore.h:32-35 (this core renders
     * the unfiltered PrimeRef estimator unless "filter" is set) */
    int filterEnabled = 0, taaEnabled = 1;
    float clampDirect = 2.5f, clampIndirect = 15.0f;
    SvgfBuffers sv;
    bool svAlloc = false;
    int64_t pathAccCap = 0;            /* paths that pathAcc holds (2 * cap once a filter frame was rendered) */
    uint32_t filterSeed = 0x12345678u; /* camRNGseed of the filter core */
    int frameCycle = 0;
    float prevj0 = 0, prevj1 = 0;
    lh2g_view prevView;
    bool havePrevView = false;
    cudaEvent_t fev[2] = {nullptr, nullptr};   /* around the filter passes: coreStats.filterTime */
    bool filterPending = false;
    lh2g_filter_params lastFilter;
    NrcBuffers nrcBuf[8];              /* radiance-cache frame buffers per lane, MAX_LANES (lane 0 also for frames on the context stream) */
    cudaEvent_t cacheEv = nullptr;     /* the last queued radiance-cache work: the next frame's cache work waits for it */
    bool cacheEvValid = false;
    lh2g_view lastJittered;
    lh2g_render_params lastParams;
    /* Frame pipelining (setting "pipelineFrames" = frames in flight, default 6, at most MAX_LANES): plain frames rotate over lanes,
     * each with its own stream and path-state buffers (lane 0 uses B's, the others their own), so that the sparse
     * last waves of one frame overlap the first waves of the next. The accumulator and the frame are shared: finalizes run
     * in submission order (finEv). A lane frame waits for everything enqueued on the context stream before it
     * (forkEv); every other operation first orders the context stream after the lanes' frames (join_frames). */
    struct Lane {
        cudaStream_t st = nullptr;
        WaveBuffers B;
        Counters* hostCounters = nullptr;
        cudaEvent_t ev[2] = {nullptr, nullptr};
        cudaEvent_t done = nullptr;
        bool pending = false;
        bool ready = false;
    };
    static constexpr int MAX_LANES = 8;
    static_assert(sizeof(nrcBuf) / sizeof(nrcBuf[0]) == MAX_LANES, "a radiance-cache buffer set per lane");
    Lane lanes[MAX_LANES];
    int pipelineFrames = 6;            /* lanes in use; 0 or 1: one frame at a time */
    int sortConnections = 0;           /* group each wave's connections by light before the any-hit queries */
    int sortRays = 0;                  /* group each bounce wave's extension rays by direction octant before the closest-hit queries */
    int nextLane = 0;
    int lastSlot = -1;                 /* lane of the last frame, -1: the context stream */
    cudaEvent_t forkEv = nullptr, finEv = nullptr;
    bool finValid = false;
    static constexpr int64_t PIPE_MAX_PATHS = 8ll << 20;   /* larger targets render one frame at a time */
    /* estimator of lh2g_render (setting "estimator": 0 PrimeRef, 1 OptiX 7; "adaptive" 1: PrimeAdaptive frames) and
     * the OptiX 7 cores' blue-noise shift seed (rendercore.h: shiftSeed = 0x11331445, never reset) */
    int estimator = 0, adaptive = 0;
    int bsdf = 0;                      /* setting "bsdf" for those two estimators: 0 lambert.h, 1 disney.h (LH2G_RP_DISNEY) */
    uint32_t shiftSeed = 0x11331445u;
    /* PrimeAdaptive frames: the second wave's per-slot radiance and layer, the first wave's features, per-pixel
     * deviation / requested / kept counts and slots, scan scratch, the device state and the second wave's counters */
    struct Adaptive {
        float4* pathAcc2 = nullptr;
        uint32_t* slotLayer = nullptr;
        float4* features = nullptr;
        float* deviation = nullptr;
        uint32_t *want = nullptr, *tmp = nullptr, *rank = nullptr, *kept = nullptr, *first = nullptr, *sums = nullptr;
        AdaptiveState* state = nullptr;
        Counters* counters2 = nullptr;
        AdaptiveState* hostState = nullptr;
        Counters* hostCounters2 = nullptr;
        int64_t cap = 0, pixels = 0;
        float pendingScale = 10.0f;     /* devScale to start the next adaptive frame from (rendercore.h: 10) */
        bool scaleDirty = true;
        bool last = false;              /* the last frame was adaptive: its statistics include the second wave */
    } ad;
    /* SoftRasterizer frames (lh2g_raster_render): pixels, depth keys, the passes' triangle lists and counters, the
     * kept instances and the materials as the rasterizer reads them */
    struct Raster {
        uint32_t* pixels = nullptr;
        unsigned long long* keys = nullptr;
        float* depth = nullptr;
        uint32_t *list = nullptr, *counters = nullptr;
        uint2 *big = nullptr, *owner = nullptr;
        float4* ck = nullptr;
        uint32_t ckCap = 0;
        RasterInst* inst = nullptr;
        RasterMat* mats = nullptr;
        int64_t pixCap = 0, triCap = 0;
        int instCap = 0, matCap = 0;
        int W = 0, H = 0;               /* size of the last frame */
        bool valid = false;
    } rs;
};

namespace {

int fail(lh2g_context* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_check(lh2g_context* c, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return LH2G_OK;
    return fail(c, e == cudaErrorMemoryAllocation ? LH2G_ERR_OOM : LH2G_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                      \
    do {                                                              \
        const int _r = cuda_check(ctx, (call), #call);                \
        if (_r != LH2G_OK) return _r;                                 \
    } while (0)

/* orders the context stream after every lane frame submitted so far (no host wait) */
int join_frames(lh2g_context* ctx) {
    for (auto& L : ctx->lanes)
        if (L.pending) {
            CK(cudaStreamWaitEvent(ctx->st, L.done, 0));
            L.pending = false;
        }
    return LH2G_OK;
}
/* every instanced triangle's material index must name a material: shading reads the material array with it */
bool materials_cover_meshes(const lh2g_context* ctx) {
    for (const InstHost& in : ctx->inst)
        if (in.mesh >= 0 && in.mesh < (int)ctx->meshes.size() && ctx->meshes[in.mesh].n &&
            ctx->meshes[in.mesh].maxMaterial >= ctx->hostMats.size())
            return false;
    return true;
}

#define JOIN()                                  \
    do {                                        \
        const int _j = join_frames(ctx);        \
        if (_j != LH2G_OK) return _j;           \
    } while (0)

template <typename T>
void dfree(T*& p) { if (p) cudaFree((void*)p); p = nullptr; }

template <typename T>
cudaError_t dalloc(T*& p, size_t count) {
    dfree(p);
    return cudaMalloc((void**)&p, std::max<size_t>(1, count) * sizeof(T));
}

void free_filter(lh2g_context* ctx) {
    SvgfBuffers& v = ctx->sv;
    dfree(v.features), dfree(v.worldPos), dfree(v.prevWorldPos), dfree(v.deltaDepth), dfree(v.motion), dfree(v.moments);
    dfree(v.prevMoments), dfree(v.shading), dfree(v.filteredIN), dfree(v.filteredOUT), dfree(v.prevPixels), dfree(v.taaPixels);
    ctx->svAlloc = false;
    ctx->havePrevView = false;
}

void free_lane_buffers(lh2g_context* ctx) {
    for (int l = 1; l < lh2g_context::MAX_LANES; l++) {
        WaveBuffers& B = ctx->lanes[l].B;
        if (!ctx->lanes[l].ready) continue;
        for (int k = 0; k < 2; k++) dfree(B.O[k]), dfree(B.D[k]), dfree(B.T[k]);
        dfree(B.hits), dfree(B.shO), dfree(B.shD), dfree(B.shE), dfree(B.pathAcc), dfree(B.counters);
        dfree(B.sortO), dfree(B.sortD), dfree(B.sortE), dfree(B.connBins), dfree(B.order);
        ctx->lanes[l].ready = false;
    }
}

void free_target(lh2g_context* ctx) {
    free_lane_buffers(ctx);
    WaveBuffers& B = ctx->B;
    for (int k = 0; k < 2; k++) dfree(B.O[k]), dfree(B.D[k]), dfree(B.T[k]);
    dfree(B.hits), dfree(B.shO), dfree(B.shD), dfree(B.shE), dfree(B.pathAcc), dfree(B.accum), dfree(B.frame), dfree(B.counters);
    dfree(B.sortO), dfree(B.sortD), dfree(B.sortE), dfree(B.connBins), dfree(B.order);
    free_filter(ctx);
    for (NrcBuffers& n : ctx->nrcBuf) {
        dfree(n.rec), dfree(n.queries), dfree(n.qPath), dfree(n.pred), dfree(n.trainQ), dfree(n.trainT), dfree(n.counts);
        n.cap = 0;
    }
    {
        auto& a = ctx->ad;
        dfree(a.pathAcc2), dfree(a.slotLayer), dfree(a.features), dfree(a.deviation), dfree(a.want), dfree(a.tmp), dfree(a.rank);
        dfree(a.kept), dfree(a.first), dfree(a.sums), dfree(a.counters2);
        if (a.state) {   /* keep devScale across a new target, as the reference's core does */
            if (!a.scaleDirty && a.hostState) {
                cudaMemcpy(a.hostState, a.state, sizeof(AdaptiveState), cudaMemcpyDeviceToHost);
                a.pendingScale = a.hostState->devScale, a.scaleDirty = true;
            }
            dfree(a.state);
        }
        a.cap = 0, a.pixels = 0;
    }
    ctx->cap = 0, ctx->pathAccCap = 0;
}

/* The filter's buffers, a second (indirect) half for the per-path radiance and the accumulator; all zeroed. */
int ensure_filter(lh2g_context* ctx) {
    if (ctx->svAlloc) return LH2G_OK;
    const size_t WH = (size_t)ctx->W * ctx->H;
    SvgfBuffers& v = ctx->sv;
    WaveBuffers& B = ctx->B;
    cudaError_t e = cudaSuccess;
    CK(cudaStreamSynchronize(ctx->st));
    if (!e) e = dalloc(B.pathAcc, 2 * (size_t)ctx->cap);
    if (!e) e = dalloc(B.accum, 2 * WH);
    float4** f4[] = {&v.worldPos, &v.prevWorldPos, &v.deltaDepth, &v.moments, &v.prevMoments, &v.shading, &v.filteredIN, &v.filteredOUT,
                     &v.prevPixels, &v.taaPixels};
    for (float4** q : f4)
        if (!e) e = dalloc(*q, WH);
    if (!e) e = dalloc(v.features, WH);
    if (!e) e = dalloc(v.motion, WH);
    if (e) { free_target(ctx); return cuda_check(ctx, e, "filter buffer allocation"); }
    ctx->pathAccCap = 2 * ctx->cap;
    CK(cudaMemsetAsync(B.accum, 0, sizeof(float4) * 2 * WH, ctx->st));
    for (float4** q : f4) CK(cudaMemsetAsync(*q, 0, sizeof(float4) * WH, ctx->st));
    CK(cudaMemsetAsync(v.features, 0, sizeof(uint4) * WH, ctx->st));
    CK(cudaMemsetAsync(v.motion, 0, sizeof(float2) * WH, ctx->st));
    ctx->svAlloc = true;
    return LH2G_OK;
}

/* host part of prepareFilter (lib/CUDA/shared_kernel_code/finalize_shared.h:297-313) */
float3 h3(const float* p) { return make_float3(p[0], p[1], p[2]); }
float3 hsub(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
float3 hadd(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
float3 hmul(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
float hdot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
float3 hnormalize(float3 v) { const float inv = 1.0f / sqrtf(hdot(v, v)); return hmul(v, inv); }
SvgfView svgf_view(const lh2g_view& v, int h) {
    const float3 pos = h3(v.pos), p1 = h3(v.p1), p2 = h3(v.p2), p3 = h3(v.p3);
    const float3 centre = make_float3(0.5f * (p2.x + p3.x), 0.5f * (p2.y + p3.y), 0.5f * (p2.z + p3.z));
    const float3 direction = hnormalize(hsub(centre, pos));
    const float3 right = hnormalize(hsub(p2, p1));
    const float3 up = hnormalize(hsub(p3, p1));
    const float screenSize = sqrtf(hdot(hsub(p3, p1), hsub(p3, p1)));
    const float lenReci = (float)h / screenSize;
    SvgfView r;
    r.prevPos = make_float4(pos.x, pos.y, pos.z, -(hdot(pos, direction) - hdot(centre, direction)));
    r.prevE = make_float4(direction.x, direction.y, direction.z, 0);
    const float3 rr = hmul(right, lenReci), uu = hmul(up, lenReci);
    r.prevRight = make_float4(rr.x, rr.y, rr.z, hdot(p1, right) * lenReci);
    r.prevUp = make_float4(uu.x, uu.y, uu.z, hdot(p1, up) * lenReci);
    return r;
}

SceneGPU scene_of(const lh2g_context* c) {
    SceneGPU S;
    memset(&S, 0, sizeof(S));
    S.nodes = c->pool, S.triData = c->triData, S.inst = c->instGPU, S.tlasPrims = c->tlasPrims, S.tlasRoot = c->tlasRoot;
    S.instCount = (int)c->inst.size();
    S.instTris = c->instTris, S.instInvRows = c->instInvRows;
    S.materials = c->mats, S.texels = c->texels;
    S.nMaterials = (int)std::max<size_t>(c->hostMats.size(), 1);
    S.triLights = c->triL, S.pointLights = c->ptL, S.spotLights = c->spL, S.dirLights = c->dirL;
    S.nTri = c->nTri, S.nPoint = c->nPt, S.nSpot = c->nSpot, S.nDir = c->nDir;
    S.lightTree = c->lightTree, S.nTreeNodes = c->nTreeNodes;
    S.skyPixels = c->sky, S.skyW = c->skyW, S.skyH = c->skyH;
    S.skySmall = c->skySmall, S.blueNoise = c->blueNoise;
    for (int r = 0; r < 3; r++) S.worldToSky[r] = make_float4(c->w2s[4 * r], c->w2s[4 * r + 1], c->w2s[4 * r + 2], c->w2s[4 * r + 3]);
    return S;
}

}  // namespace

extern "C" {

int lh2g_create(int device, lh2g_context** out) {
    if (!out) return LH2G_ERR_INVALID;
    *out = nullptr;
    lh2g_context* ctx = new lh2g_context();
    memset(&ctx->B, 0, sizeof(ctx->B));
    memset(&ctx->stats, 0, sizeof(ctx->stats));
    memset(&ctx->sv, 0, sizeof(ctx->sv));
    memset(&ctx->prevView, 0, sizeof(ctx->prevView));
    memset(&ctx->lastFilter, 0, sizeof(ctx->lastFilter));
    memset(&ctx->lastJittered, 0, sizeof(ctx->lastJittered));
    memset(&ctx->lastParams, 0, sizeof(ctx->lastParams));
    for (int i = 0; i < 16; i++) ctx->w2s[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    ctx->device = device;
    int r = cuda_check(ctx, cudaSetDevice(device), "cudaSetDevice");
    if (r == LH2G_OK) r = cuda_check(ctx, cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking), "cudaStreamCreate");
    if (r == LH2G_OK) r = cuda_check(ctx, cudaMallocHost((void**)&ctx->hostCounters, sizeof(Counters)), "cudaMallocHost");
    if (r == LH2G_OK) r = cuda_check(ctx, cudaMalloc((void**)&ctx->traceFetch, 16), "cudaMalloc");
    if (r == LH2G_OK) r = cuda_check(ctx, cudaEventCreate(&ctx->ev[0]), "cudaEventCreate");
    if (r == LH2G_OK) r = cuda_check(ctx, cudaEventCreate(&ctx->ev[1]), "cudaEventCreate");
    if (r == LH2G_OK) r = cuda_check(ctx, cudaEventCreate(&ctx->fev[0]), "cudaEventCreate");
    if (r == LH2G_OK) r = cuda_check(ctx, cudaEventCreate(&ctx->fev[1]), "cudaEventCreate");
    if (r == LH2G_OK) r = cuda_check(ctx, cudaEventCreateWithFlags(&ctx->forkEv, cudaEventDisableTiming), "cudaEventCreate");
    if (r == LH2G_OK) r = cuda_check(ctx, cudaEventCreateWithFlags(&ctx->finEv, cudaEventDisableTiming), "cudaEventCreate");
    if (r != LH2G_OK) {
        fprintf(stderr, "lh2g_create: %s\n", ctx->err.c_str());
        delete ctx;
        return r;
    }
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, device);
    ctx->stats.SMcount = (uint32_t)prop.multiProcessorCount;
    ctx->stats.ccMajor = (uint32_t)prop.major, ctx->stats.ccMinor = (uint32_t)prop.minor;
    ctx->stats.VRAM = (uint32_t)(prop.totalGlobalMem >> 20);
    ctx->stats.probedTriid = -1;
    ctx->blocksExtend = ctx->fullBlocks[0] = persistent_blocks_wave(0);
    ctx->blocksConnect = ctx->fullBlocks[1] = persistent_blocks_wave(1);
    ctx->blocksShade = ctx->fullBlocks[2] = persistent_blocks_wave(2);
    ctx->blocksTail = persistent_blocks_wave(3);
    *out = ctx;
    return LH2G_OK;
}

int lh2g_destroy(lh2g_context* ctx) {
    if (!ctx) return LH2G_ERR_INVALID;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->st);
    for (auto& L : ctx->lanes)
        if (L.st) cudaStreamSynchronize(L.st);
    for (MeshDev& m : ctx->meshes) dfree(m.verts), dfree(m.tris), dfree(m.rsNorms);
    dfree(ctx->mats), dfree(ctx->texels), dfree(ctx->triL), dfree(ctx->ptL), dfree(ctx->spL), dfree(ctx->dirL), dfree(ctx->sky);
    dfree(ctx->lightTree);
    dfree(ctx->skySmall), dfree(ctx->blueNoise);
    dfree(ctx->pool), dfree(ctx->triData), dfree(ctx->instGPU), dfree(ctx->tlasPrims), dfree(ctx->instTris), dfree(ctx->instInvRows);
    dfree(ctx->traceFetch), dfree(ctx->hostRaysDev), dfree(ctx->hostOutDev);
    dfree(ctx->B.capHits), dfree(ctx->B.capSeeds);
    dfree(ctx->rs.pixels), dfree(ctx->rs.keys), dfree(ctx->rs.depth), dfree(ctx->rs.list), dfree(ctx->rs.big), dfree(ctx->rs.counters);
    dfree(ctx->rs.inst), dfree(ctx->rs.mats), dfree(ctx->rs.owner), dfree(ctx->rs.ck);
    free_target(ctx);
    if (ctx->hostCounters) cudaFreeHost(ctx->hostCounters);
    if (ctx->ad.hostState) cudaFreeHost(ctx->ad.hostState);
    if (ctx->ad.hostCounters2) cudaFreeHost(ctx->ad.hostCounters2);
    for (NrcBuffers& n : ctx->nrcBuf)
        if (n.hostCounts) cudaFreeHost(n.hostCounts);
    if (ctx->cacheEv) cudaEventDestroy(ctx->cacheEv);
    cudaEventDestroy(ctx->ev[0]), cudaEventDestroy(ctx->ev[1]);
    if (ctx->fev[0]) cudaEventDestroy(ctx->fev[0]);
    if (ctx->fev[1]) cudaEventDestroy(ctx->fev[1]);
    for (cudaEvent_t e : ctx->lev) cudaEventDestroy(e);
    for (auto& L : ctx->lanes) {
        if (!L.st) continue;
        cudaEventDestroy(L.ev[0]), cudaEventDestroy(L.ev[1]), cudaEventDestroy(L.done);
        if (L.hostCounters) cudaFreeHost(L.hostCounters);
        cudaStreamDestroy(L.st);
    }
    if (ctx->forkEv) cudaEventDestroy(ctx->forkEv);
    if (ctx->finEv) cudaEventDestroy(ctx->finEv);
    cudaStreamDestroy(ctx->st);
    delete ctx;
    return LH2G_OK;
}

const char* lh2g_last_error(lh2g_context* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int lh2g_set_geometry(lh2g_context* ctx, int meshIdx, const float* v4, int vertexCount, int triangleCount, const lh2g_core_tri* tris) {
    if (!ctx) return LH2G_ERR_INVALID;
    if (meshIdx < 0 || meshIdx > (int)ctx->meshes.size() || triangleCount < 0 || vertexCount != 3 * triangleCount || (triangleCount && (!v4 || !tris)))
        return fail(ctx, LH2G_ERR_INVALID, "set_geometry: meshes must arrive in index order with 3 vertices per triangle");
    if (triangleCount >= (1 << 28)) return fail(ctx, LH2G_ERR_INVALID, "set_geometry: at most 2^28 triangles per mesh");
    JOIN();   /* frames in flight read the scene */
    cudaSetDevice(ctx->device);
    if (meshIdx == (int)ctx->meshes.size()) ctx->meshes.emplace_back();
    MeshDev& m = ctx->meshes[meshIdx];
    m.n = (uint32_t)triangleCount;
    CK(dalloc(m.verts, (size_t)3 * triangleCount));
    CK(dalloc(m.tris, (size_t)13 * triangleCount));
    dfree(m.rsNorms);
    CK(cudaMemcpyAsync(m.verts, v4, sizeof(float4) * 3 * (size_t)triangleCount, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(m.tris, tris, sizeof(lh2g_core_tri) * (size_t)triangleCount, cudaMemcpyHostToDevice, ctx->st));
    m.maxMaterial = 0;
    for (int i = 0; i < triangleCount; i++) m.maxMaterial = std::max(m.maxMaterial, tris[i].material);
    for (int k = 0; k < 3; k++) m.bmin[k] = 1e30f, m.bmax[k] = -1e30f;
    for (size_t i = 0; i < (size_t)vertexCount; i++)
        for (int k = 0; k < 3; k++) m.bmin[k] = std::min(m.bmin[k], v4[4 * i + k]), m.bmax[k] = std::max(m.bmax[k], v4[4 * i + k]);
    CK(cudaStreamSynchronize(ctx->st));   /* the caller may free its arrays on return */
    ctx->finalized = false;
    return LH2G_OK;
}

int lh2g_set_instance(lh2g_context* ctx, int instIdx, int meshIdx, const float* T) {
    if (!ctx || instIdx < 0) return LH2G_ERR_INVALID;
    if (meshIdx == -1) {
        if ((int)ctx->inst.size() > instIdx) ctx->inst.resize(instIdx);
        ctx->finalized = false;
        return LH2G_OK;
    }
    if (instIdx > (int)ctx->inst.size() || meshIdx < 0 || !T) return fail(ctx, LH2G_ERR_INVALID, "set_instance: instances must arrive in index order");
    if (instIdx == (int)ctx->inst.size()) ctx->inst.emplace_back();
    InstHost& in = ctx->inst[instIdx];
    in.mesh = meshIdx;
    memcpy(in.T, T, 64);
    invert4x4(T, in.inv);
    ctx->finalized = false;
    return LH2G_OK;
}

int lh2g_finalize_instances(lh2g_context* ctx) {
    if (!ctx) return LH2G_ERR_INVALID;
    cudaSetDevice(ctx->device);
    JOIN();
    for (const InstHost& in : ctx->inst)
        if (in.mesh >= (int)ctx->meshes.size()) return fail(ctx, LH2G_ERR_INVALID, "finalize: instance of a mesh that was never set");
    const auto t0 = std::chrono::high_resolution_clock::now();
    const uint32_t M = (uint32_t)ctx->meshes.size(), I = (uint32_t)ctx->inst.size();
    std::vector<uint32_t> segStart(M + 1, 0);
    for (uint32_t m = 0; m < M; m++) segStart[m + 1] = segStart[m] + ctx->meshes[m].n;
    const uint32_t N = segStart[M];
    float4 *triIn = nullptr, *lo = nullptr, *hi = nullptr;
    uint32_t *segOf = nullptr, *leafPrim = nullptr;
    auto cleanup = [&]() { dfree(triIn), dfree(lo), dfree(hi), dfree(segOf), dfree(leafPrim); };
    if (dalloc(triIn, (size_t)3 * N) || dalloc(lo, std::max(N, I)) || dalloc(hi, std::max(N, I)) || dalloc(segOf, std::max(N, I)) ||
        dalloc(leafPrim, std::max(N, I))) {
        cleanup();
        return fail(ctx, LH2G_ERR_OOM, "finalize: out of device memory for the BVH build");
    }
    for (uint32_t m = 0; m < M; m++)
        launch_tri_prep(ctx->meshes[m].verts, ctx->meshes[m].n, m, triIn + 3 * (size_t)segStart[m], lo + segStart[m], hi + segStart[m],
                        segOf + segStart[m], ctx->st);
    const uint32_t cap = N + M + 2 * (I + 1) + 64;
    if (dalloc(ctx->pool, (size_t)5 * cap) || dalloc(ctx->triData, (size_t)3 * std::max(N, 1u))) {
        cleanup();
        return fail(ctx, LH2G_ERR_OOM, "finalize: out of device memory for the node pool");
    }
    std::vector<uint32_t> meshRoot(M);
    uint32_t used = 0, slots = 0;
    int r = build_bvh8(lo, hi, segOf, N, segStart, ctx->pool, 0, cap, leafPrim, 3, meshRoot.data(), &used, &slots, ctx->st);
    if (r != 0) { cleanup(); return fail(ctx, r == 3 ? LH2G_ERR_OOM : (r == 5 ? LH2G_ERR_OVERFLOW : LH2G_ERR_CUDA), "finalize: BLAS build failed"); }
    launch_gather_tris(triIn, leafPrim, N, ctx->triData, ctx->st);
    /* TLAS over instance world boxes (8 transformed corners of the mesh box, widened) */
    std::vector<float4> ilo(std::max(I, 1u)), ihi(std::max(I, 1u));
    std::vector<uint32_t> iseg(std::max(I, 1u), 0);
    for (uint32_t i = 0; i < I; i++) {
        const InstHost& in = ctx->inst[i];
        const MeshDev& m = ctx->meshes[in.mesh];
        float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
        for (int c = 0; c < 8; c++) {
            const float p[3] = {(c & 1) ? m.bmax[0] : m.bmin[0], (c & 2) ? m.bmax[1] : m.bmin[1], (c & 4) ? m.bmax[2] : m.bmin[2]};
            for (int k = 0; k < 3; k++) {
                const float w = in.T[4 * k] * p[0] + in.T[4 * k + 1] * p[1] + in.T[4 * k + 2] * p[2] + in.T[4 * k + 3];
                mn[k] = std::min(mn[k], w), mx[k] = std::max(mx[k], w);
            }
        }
        for (int k = 0; k < 3; k++) {
            const float pad = (mx[k] - mn[k]) * 1e-5f + (fabsf(mn[k]) + fabsf(mx[k])) * 1e-6f + 1e-30f;
            mn[k] -= pad, mx[k] += pad;
        }
        ilo[i] = make_float4(mn[0], mn[1], mn[2], 0), ihi[i] = make_float4(mx[0], mx[1], mx[2], 0);
    }
    std::vector<InstanceGPU> ig(std::max(I, 1u));
    std::vector<const float4*> itris(std::max(I, 1u), nullptr);
    std::vector<float4> irows(3 * std::max(I, 1u));
    for (uint32_t i = 0; i < I; i++) {
        const InstHost& in = ctx->inst[i];
        memset(&ig[i], 0, sizeof(InstanceGPU));
        memcpy(ig[i].inv, in.inv, 48);
        ig[i].blasRoot = meshRoot[in.mesh];
        ig[i].mesh = (uint32_t)in.mesh;
        itris[i] = ctx->meshes[in.mesh].tris;
        for (int k = 0; k < 3; k++) irows[3 * i + k] = make_float4(in.inv[4 * k], in.inv[4 * k + 1], in.inv[4 * k + 2], in.inv[4 * k + 3]);
    }
    if (dalloc(ctx->instGPU, std::max(I, 1u)) || dalloc(ctx->instTris, std::max(I, 1u)) || dalloc(ctx->instInvRows, 3 * (size_t)std::max(I, 1u)) ||
        dalloc(ctx->tlasPrims, std::max(I, 1u))) {
        cleanup();
        return fail(ctx, LH2G_ERR_OOM, "finalize: out of device memory for instances");
    }
    CK(cudaMemcpyAsync(ctx->instGPU, ig.data(), sizeof(InstanceGPU) * ig.size(), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync((void*)ctx->instTris, itris.data(), sizeof(void*) * itris.size(), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->instInvRows, irows.data(), sizeof(float4) * irows.size(), cudaMemcpyHostToDevice, ctx->st));
    ctx->tlasRoot = 0xffffffffu;
    if (I > 0) {
        CK(cudaMemcpyAsync(lo, ilo.data(), sizeof(float4) * I, cudaMemcpyHostToDevice, ctx->st));
        CK(cudaMemcpyAsync(hi, ihi.data(), sizeof(float4) * I, cudaMemcpyHostToDevice, ctx->st));
        CK(cudaMemcpyAsync(segOf, iseg.data(), sizeof(uint32_t) * I, cudaMemcpyHostToDevice, ctx->st));
        std::vector<uint32_t> tseg = {0, I};
        uint32_t troot = 0, tused = 0, tslots = 0;
        r = build_bvh8(lo, hi, segOf, I, tseg, ctx->pool, used, cap, ctx->tlasPrims, 1, &troot, &tused, &tslots, ctx->st);
        if (r != 0) { cleanup(); return fail(ctx, LH2G_ERR_CUDA, "finalize: TLAS build failed"); }
        ctx->tlasRoot = troot;
    }
    CK(cudaStreamSynchronize(ctx->st));
    cleanup();
    ctx->finalized = true;
    ctx->stats.bvhBuildTime = std::chrono::duration<float, std::milli>(std::chrono::high_resolution_clock::now() - t0).count();
    return LH2G_OK;
}

int lh2g_pack_materials(const lh2g_material* mats, int count, const lh2g_texture* tex, int ntex, lh2g_gpu_material* out) {
    if (count < 0 || ntex < 0 || (count && (!mats || !out))) return LH2G_ERR_INVALID;
    std::vector<uint32_t> first, wh;
    uint32_t off = 0;
    for (int i = 0; i < ntex; i++) first.push_back(off), wh.push_back(tex[i].width), wh.push_back(tex[i].height), off += tex[i].pixelCount;
    for (int i = 0; i < count; i++) {
        const lh2g_map_ref* refs[6] = {&mats[i].color_map, &mats[i].detail_color_map, &mats[i].normal_map, &mats[i].detail_normal_map, &mats[i].specular_map, &mats[i].roughness_map};
        for (const lh2g_map_ref* r : refs) if (r->texture >= ntex) return LH2G_ERR_INVALID;
        pack_material(mats[i], first, wh, out[i]);
    }
    return LH2G_OK;
}

int lh2g_set_textures(lh2g_context* ctx, const lh2g_texture* tex, int count) {
    if (!ctx || count < 0 || (count && !tex)) return LH2G_ERR_INVALID;
    cudaSetDevice(ctx->device);
    JOIN();
    ctx->texFirst.clear(), ctx->texWH.clear();
    size_t total = 0, slack = 64;
    for (int i = 0; i < count; i++) {
        slack = std::max(slack, (size_t)tex[i].width * tex[i].height + 64);   /* MIP reads past a short chain stay in bounds */
        if (tex[i].storage != 0) return fail(ctx, LH2G_ERR_INVALID, "set_textures: only ARGB32 storage is supported");
        ctx->texFirst.push_back((uint32_t)total), ctx->texWH.push_back(tex[i].width), ctx->texWH.push_back(tex[i].height);
        total += tex[i].pixelCount;
    }
    CK(dalloc(ctx->texels, total + slack));
    CK(cudaMemsetAsync(ctx->texels, 0, sizeof(uint32_t) * (total + slack), ctx->st));
    for (int i = 0; i < count; i++)
        CK(cudaMemcpyAsync(ctx->texels + ctx->texFirst[i], tex[i].texels, sizeof(uint32_t) * tex[i].pixelCount, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return LH2G_OK;
}

int lh2g_set_materials(lh2g_context* ctx, const lh2g_material* mats, int count) {
    if (!ctx || count < 0 || (count && !mats)) return LH2G_ERR_INVALID;
    cudaSetDevice(ctx->device);
    JOIN();
    std::vector<lh2g_gpu_material> packed(std::max(count, 1));
    for (int i = 0; i < count; i++) {
        const lh2g_map_ref* refs[6] = {&mats[i].color_map, &mats[i].detail_color_map, &mats[i].normal_map, &mats[i].detail_normal_map, &mats[i].specular_map, &mats[i].roughness_map};
        for (const lh2g_map_ref* r : refs)
            if (r->texture >= (int)ctx->texFirst.size()) return fail(ctx, LH2G_ERR_INVALID, "set_materials: texture index out of range (set textures first)");
        pack_material(mats[i], ctx->texFirst, ctx->texWH, packed[i]);
    }
    ctx->hostMats.assign(mats, mats + count);
    CK(dalloc(ctx->mats, (size_t)8 * packed.size()));
    CK(cudaMemcpyAsync(ctx->mats, packed.data(), sizeof(lh2g_gpu_material) * packed.size(), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return LH2G_OK;
}

int lh2g_set_lights(lh2g_context* ctx, const lh2g_light_tri* tri, int ntri, const lh2g_point_light* pt, int npt, const lh2g_spot_light* spot, int nspot,
                    const lh2g_dir_light* dir, int ndir) {
    if (!ctx || ntri < 0 || npt < 0 || nspot < 0 || ndir < 0) return LH2G_ERR_INVALID;
    if ((long long)ntri + npt + nspot > LH2G_MAX_TREE_LIGHTS || ndir > 64)
        return fail(ctx, LH2G_ERR_INVALID, "set_lights: at most LH2G_MAX_TREE_LIGHTS area, point and spot lights and 64 directional lights");
    cudaSetDevice(ctx->device);
    JOIN();
    const std::vector<LightTreeNode> tree = build_light_tree(tri, ntri, pt, npt, spot, nspot);
    CK(dalloc(ctx->lightTree, (size_t)4 * std::max<size_t>(tree.size(), 1)));
    if (!tree.empty()) CK(cudaMemcpyAsync(ctx->lightTree, tree.data(), sizeof(LightTreeNode) * tree.size(), cudaMemcpyHostToDevice, ctx->st));
    ctx->nTreeNodes = (int)tree.size();
    CK(dalloc(ctx->triL, (size_t)6 * std::max(ntri, 1)));
    CK(dalloc(ctx->ptL, (size_t)2 * std::max(npt, 1)));
    CK(dalloc(ctx->spL, (size_t)3 * std::max(nspot, 1)));
    CK(dalloc(ctx->dirL, (size_t)2 * std::max(ndir, 1)));
    if (ntri) CK(cudaMemcpyAsync(ctx->triL, tri, sizeof(lh2g_light_tri) * ntri, cudaMemcpyHostToDevice, ctx->st));
    if (npt) CK(cudaMemcpyAsync(ctx->ptL, pt, sizeof(lh2g_point_light) * npt, cudaMemcpyHostToDevice, ctx->st));
    if (nspot) CK(cudaMemcpyAsync(ctx->spL, spot, sizeof(lh2g_spot_light) * nspot, cudaMemcpyHostToDevice, ctx->st));
    if (ndir) CK(cudaMemcpyAsync(ctx->dirL, dir, sizeof(lh2g_dir_light) * ndir, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->nTri = ntri, ctx->nPt = npt, ctx->nSpot = nspot, ctx->nDir = ndir;
    return LH2G_OK;
}

int lh2g_build_light_tree(const lh2g_light_tri* tri, int ntri, const lh2g_point_light* pt, int npt, const lh2g_spot_light* spot, int nspot,
                          void* nodes, int capacity) {
    if (ntri < 0 || npt < 0 || nspot < 0 || (long long)ntri + npt + nspot > LH2G_MAX_TREE_LIGHTS || capacity < 0) return -LH2G_ERR_INVALID;
    if ((ntri && !tri) || (npt && !pt) || (nspot && !spot)) return -LH2G_ERR_INVALID;
    const std::vector<LightTreeNode> tree = build_light_tree(tri, ntri, pt, npt, spot, nspot);
    if ((size_t)capacity < tree.size() || (!nodes && !tree.empty())) return -LH2G_ERR_OVERFLOW;
    if (!tree.empty()) memcpy(nodes, tree.data(), sizeof(LightTreeNode) * tree.size());
    return (int)tree.size();
}

int lh2g_set_sky(lh2g_context* ctx, const float* rgb, int w, int h, const float* m16) {
    if (!ctx || w < 0 || h < 0 || ((size_t)w * h && !rgb)) return LH2G_ERR_INVALID;
    cudaSetDevice(ctx->device);
    JOIN();
    std::vector<float4> px((size_t)std::max(1, w * h));
    for (size_t i = 0; i < (size_t)w * h; i++) px[i] = make_float4(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2], 0.0f);
    CK(dalloc(ctx->sky, px.size()));
    CK(cudaMemcpyAsync(ctx->sky, px.data(), sizeof(float4) * px.size(), cudaMemcpyHostToDevice, ctx->st));
    /* the average of every 64 x 64 tile, summed row by row (RenderCore::SetSkyData, rendercore_optix7/rendercore.cpp:726-737) */
    const int sw = w >> 6, sh = h >> 6;
    std::vector<float4> small((size_t)std::max(1, sw * sh), make_float4(0, 0, 0, 0));
    for (int y = 0; y < sh; y++)
        for (int x = 0; x < sw; x++) {
            float tx = 0, ty = 0, tz = 0;
            for (int v = 0; v < 64; v++)
                for (int u = 0; u < 64; u++) {
                    const float4& q = px[(size_t)(x * 64 + u) + (size_t)(y * 64 + v) * w];
                    tx += q.x, ty += q.y, tz += q.z;
                }
            const float k = 1.0f / (64 * 64);
            small[(size_t)x + (size_t)y * sw] = make_float4(tx * k, ty * k, tz * k, 0.0f);
        }
    CK(dalloc(ctx->skySmall, small.size()));
    CK(cudaMemcpyAsync(ctx->skySmall, small.data(), sizeof(float4) * small.size(), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->skyW = w, ctx->skyH = h;
    for (int i = 0; i < 16; i++) ctx->w2s[i] = m16 ? m16[i] : ((i % 5 == 0) ? 1.0f : 0.0f);
    return LH2G_OK;
}

int lh2g_set_blue_noise(lh2g_context* ctx, const uint8_t* sobol, const uint8_t* scrambling, const uint8_t* ranking) {
    if (!ctx) return LH2G_ERR_INVALID;
    cudaSetDevice(ctx->device);
    JOIN();
    CK(cudaStreamSynchronize(ctx->st));
    if (!sobol || !scrambling || !ranking) {
        dfree(ctx->blueNoise);
        return LH2G_OK;
    }
    /* one uint per entry as rendercore_optix7/rendercore.cpp:247-256 expands them, then 64 zeros: the ranking
     * reads of deep path lengths at the last tile pixel reach past the tables (the reference reads past its buffer) */
    std::vector<uint32_t> bn(65536 * 5 + 64, 0u);
    for (int i = 0; i < 65536; i++) bn[i] = sobol[i];
    for (int i = 0; i < 128 * 128 * 8; i++) bn[i + 65536] = scrambling[i], bn[i + 3 * 65536] = ranking[i];
    CK(dalloc(ctx->blueNoise, bn.size()));
    CK(cudaMemcpy(ctx->blueNoise, bn.data(), sizeof(uint32_t) * bn.size(), cudaMemcpyHostToDevice));
    return LH2G_OK;
}

int lh2g_setting(lh2g_context* ctx, const char* name, float value) {
    if (!ctx || !name) return LH2G_ERR_INVALID;
    if (!strcmp(name, "epsilon")) ctx->eps = value;
    else if (!strcmp(name, "clampValue")) ctx->clampValue = value;
    else if (!strcmp(name, "maxDepth")) {
        if (value < 1 || value > 64) return fail(ctx, LH2G_ERR_INVALID, "setting maxDepth: 1..64");
        ctx->maxDepth = (int)value;
    } else if (!strcmp(name, "rrStartDepth")) ctx->rrStart = (int)value;
    else if (!strcmp(name, "nee")) ctx->nee = value != 0.0f;
    else if (!strcmp(name, "estimator")) {
        if (value != 0.0f && value != 1.0f) return fail(ctx, LH2G_ERR_INVALID, "setting estimator: 0 (PrimeRef) or 1 (OptiX 7)");
        ctx->estimator = (int)value;
    } else if (!strcmp(name, "adaptive")) ctx->adaptive = value != 0.0f;
    else if (!strcmp(name, "bsdf")) {
        if (value != 0.0f && value != 1.0f) return fail(ctx, LH2G_ERR_INVALID, "setting bsdf: 0 (lambert.h) or 1 (disney.h)");
        ctx->bsdf = (int)value;
    } else if (!strcmp(name, "lightTree")) {
        if (value != 0.0f && value != 1.0f) return fail(ctx, LH2G_ERR_INVALID, "setting lightTree: 0 (potentials) or 1 (the light tree)");
        ctx->lightTreeOn = (int)value;
    }
    else if (!strcmp(name, "waveTail")) {
        if (value < 0 || value > 65) return fail(ctx, LH2G_ERR_INVALID, "setting waveTail: 0 (off) or 1..65");
        ctx->tailDepth = (int)value;
    }
    /* the filter core's settings (lib/RenderCore_Optix7Filter/rendercore.cpp:674-677) */
    else if (!strcmp(name, "clampDirect")) ctx->clampDirect = value;
    else if (!strcmp(name, "clampIndirect")) ctx->clampIndirect = value;
    else if (!strcmp(name, "filter")) ctx->filterEnabled = value == 0 ? 0 : 1;
    else if (!strcmp(name, "TAA")) ctx->taaEnabled = value == 0 ? 0 : 1;
    else if (!strcmp(name, "sortConnections")) {
        if (value != 0.0f && value != 1.0f && value != 2.0f) return fail(ctx, LH2G_ERR_INVALID, "setting sortConnections: 0, 1 (by light) or 2 (by light within chunks)");
        ctx->sortConnections = (int)value;
    }
    else if (!strcmp(name, "sortRays")) {
        if (value != 0.0f && value != 1.0f && value != 2.0f) return fail(ctx, LH2G_ERR_INVALID, "setting sortRays: 0, 1 (by octant) or 2 (by octant within chunks)");
        ctx->sortRays = (int)value;
    }
    else if (!strcmp(name, "waveOccupancy")) {
        /* fraction of a full GPU the persistent wave kernels of one frame take (frames in flight share the rest) */
        if (!(value > 0.0f && value <= 1.0f)) return fail(ctx, LH2G_ERR_INVALID, "setting waveOccupancy: (0, 1]");
        JOIN();
        int* blocks[3] = {&ctx->blocksExtend, &ctx->blocksConnect, &ctx->blocksShade};
        for (int k = 0; k < 3; k++) *blocks[k] = std::max(1, (int)((float)ctx->fullBlocks[k] * value + 0.5f));
    } else if (!strcmp(name, "pipelineFrames")) {
        if (value < 0 || value > lh2g_context::MAX_LANES) return fail(ctx, LH2G_ERR_INVALID, "setting pipelineFrames: 0..8 frames in flight");
        JOIN();
        ctx->pipelineFrames = (int)value;
        ctx->nextLane = 0;
    }
    /* other names are accepted and ignored, as the reference cores ignore settings they do not know
     * (rendercore.cpp:484-502) */
    return LH2G_OK;
}

int lh2g_set_target(lh2g_context* ctx, int w, int h, int spp) {
    if (!ctx || w <= 0 || h <= 0 || spp <= 0 || w > 16384 || h > 16384) return fail(ctx, LH2G_ERR_INVALID, "set_target: bad size");
    const int64_t P = (int64_t)w * h * spp;
    if (P >= (1ll << 31)) return fail(ctx, LH2G_ERR_INVALID, "set_target: more than 2^31 paths");
    cudaSetDevice(ctx->device);
    JOIN();
    CK(cudaStreamSynchronize(ctx->st));
    if (P > ctx->cap || (int64_t)w * h != (int64_t)ctx->W * ctx->H) {
        free_target(ctx);
        WaveBuffers& B = ctx->B;
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < 2 && e == cudaSuccess; k++) {
            if ((e = dalloc(B.O[k], P))) break;
            if ((e = dalloc(B.D[k], P))) break;
            e = dalloc(B.T[k], P);
        }
        if (!e) e = dalloc(B.hits, P);
        if (!e) e = dalloc(B.shO, P);
        if (!e) e = dalloc(B.shD, P);
        if (!e) e = dalloc(B.shE, P);
        if (!e) e = dalloc(B.pathAcc, P);
        if (!e) e = dalloc(B.accum, (size_t)w * h);
        if (!e) e = dalloc(B.frame, (size_t)w * h);
        if (!e) e = dalloc(B.counters, 1);
        if (!e) e = dalloc(B.sortO, P);
        if (!e) e = dalloc(B.sortD, P);
        if (!e) e = dalloc(B.sortE, P);
        if (!e) e = dalloc(B.connBins, 128);
        if (!e) e = cudaMemset(B.connBins, 0, 128 * sizeof(uint32_t));
        if (!e) e = dalloc(B.order, P);
        if (e) { free_target(ctx); return cuda_check(ctx, e, "set_target allocation"); }
        ctx->cap = P, ctx->pathAccCap = P;
        CK(cudaMemsetAsync(B.accum, 0, sizeof(float4) * (size_t)w * h, ctx->st));
        CK(cudaMemsetAsync(B.frame, 0, sizeof(float4) * (size_t)w * h, ctx->st));
    }
    ctx->havePrevView = false;
    ctx->W = w, ctx->H = h, ctx->spp = spp;
    ctx->samplesTaken = 0;
    ctx->firstConverging = true;
    return LH2G_OK;
}

int lh2g_set_probe(lh2g_context* ctx, int x, int y) {
    if (!ctx) return LH2G_ERR_INVALID;
    ctx->probeX = x, ctx->probeY = y;
    return LH2G_OK;
}

}  // extern "C"

namespace {
/* Work a frame adds around its finalize (radiance-cache frames), enqueued on the frame's stream: before runs between
 * the last wave and the finalize, after follows the finalize. async: the hooks never wait for the device, so the
 * frame may run on a lane. */
struct FrameHooks {
    std::function<int(const FrameGPU&, const WaveBuffers&, cudaStream_t, int lane)> before, after;
    bool async = false;
};

int ensure_nrc(lh2g_context* ctx, int lane) {
    NrcBuffers& n = ctx->nrcBuf[lane];
    if (n.cap >= ctx->cap) return LH2G_OK;
    JOIN();
    CK(cudaStreamSynchronize(ctx->st));
    dfree(n.rec), dfree(n.queries), dfree(n.qPath), dfree(n.pred), dfree(n.trainQ), dfree(n.trainT), dfree(n.counts);
    const size_t cap = (size_t)ctx->cap;
    cudaError_t e = dalloc(n.rec, 6 * cap);
    if (!e) e = dalloc(n.queries, 4 * cap);
    if (!e) e = dalloc(n.qPath, cap);
    if (!e) e = dalloc(n.pred, cap);
    if (!e) e = dalloc(n.trainQ, 4 * (size_t)NRC_TRAIN_CAP);
    if (!e) e = dalloc(n.trainT, (size_t)NRC_TRAIN_CAP);
    if (!e) e = dalloc(n.counts, 4);
    if (!e && !n.hostCounts) e = cudaMallocHost((void**)&n.hostCounts, 16);
    if (e) return cuda_check(ctx, e, "radiance-cache buffers");
    n.cap = ctx->cap;
    return LH2G_OK;
}

/* the stream, events and pinned counters of lane l; lanes above 0 also get their own path-state buffers */
int ensure_lane(lh2g_context* ctx, int l) {
    auto& L = ctx->lanes[l];
    if (!L.st) {
        CK(cudaStreamCreateWithFlags(&L.st, cudaStreamNonBlocking));
        CK(cudaEventCreate(&L.ev[0]));
        CK(cudaEventCreate(&L.ev[1]));
        CK(cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming));
        CK(cudaMallocHost((void**)&L.hostCounters, sizeof(Counters)));
    }
    if (l > 0 && !L.ready) {
        memset(&L.B, 0, sizeof(L.B));
        const size_t P = (size_t)ctx->cap;
        WaveBuffers& B = L.B;
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < 2 && e == cudaSuccess; k++) {
            if ((e = dalloc(B.O[k], P))) break;
            if ((e = dalloc(B.D[k], P))) break;
            e = dalloc(B.T[k], P);
        }
        if (!e) e = dalloc(B.hits, P);
        if (!e) e = dalloc(B.shO, P);
        if (!e) e = dalloc(B.shD, P);
        if (!e) e = dalloc(B.shE, P);
        if (!e) e = dalloc(B.pathAcc, P);
        if (!e) e = dalloc(B.counters, 1);
        if (!e) e = dalloc(B.sortO, P);
        if (!e) e = dalloc(B.sortD, P);
        if (!e) e = dalloc(B.sortE, P);
        if (!e) e = dalloc(B.connBins, 128);
        if (!e) e = cudaMemset(B.connBins, 0, 128 * sizeof(uint32_t));
        if (!e) e = dalloc(B.order, P);
        if (e) { free_lane_buffers(ctx); return cuda_check(ctx, e, "frame lane buffers"); }
        L.ready = true;
    }
    return LH2G_OK;
}

int render_frame(lh2g_context* ctx, const lh2g_view* view, const lh2g_render_params* p, int accumulate, lh2g_hit* capHits, uint32_t* capSeeds,
                 uint32_t* countersOut, const FrameHooks* hook, float* hostFrame = nullptr) {
    if (!ctx || !view || !p) return LH2G_ERR_INVALID;
    if (!ctx->finalized) return fail(ctx, LH2G_ERR_STATE, "render: scene not finalized (call lh2g_finalize_instances)");
    if (!ctx->cap) return fail(ctx, LH2G_ERR_STATE, "render: no target (call lh2g_set_target)");
    const bool band = p->rowCount > 0;
    if (p->width != ctx->W || (band ? p->rowCount : p->height) != ctx->H || p->spp != ctx->spp || p->maxDepth < 1 || p->maxDepth > 64)
        return fail(ctx, LH2G_ERR_INVALID, "render: parameters do not match the target");
    if (band && (p->rowBegin < 0 || p->rowBegin + p->rowCount > p->height || (int64_t)p->width * p->height * p->spp >= (1ll << 32) ||
                 (p->flags & (LH2G_RP_FILTER | LH2G_RP_NRC | LH2G_RP_OPTIX7 | LH2G_RP_ADAPTIVE))))
        return fail(ctx, LH2G_ERR_INVALID, "render: a band must lie in the frame and render the PrimeRef estimator");
    if (!ctx->mats) return fail(ctx, LH2G_ERR_STATE, "render: no materials");
    if (!materials_cover_meshes(ctx)) return fail(ctx, LH2G_ERR_INVALID, "render: a triangle's material index exceeds the material count");
    cudaSetDevice(ctx->device);
    const bool filt = (p->flags & LH2G_RP_FILTER) != 0, nrcFrame = (p->flags & LH2G_RP_NRC) != 0;
    if (filt && nrcFrame) return fail(ctx, LH2G_ERR_INVALID, "render: filter and radiance-cache frames do not combine");
    if (p->flags & LH2G_RP_ADAPTIVE) return fail(ctx, LH2G_ERR_INVALID, "render: adaptive frames go through lh2g_render_adaptive");
    if ((p->flags & LH2G_RP_DISNEY) && !(p->flags & LH2G_RP_OPTIX7))
        return fail(ctx, LH2G_ERR_INVALID, "render: the Disney BSDF belongs to the OptiX 7 estimator and adaptive frames");
    if ((p->flags & LH2G_RP_LIGHTTREE) && !(p->flags & LH2G_RP_OPTIX7))
        return fail(ctx, LH2G_ERR_INVALID, "render: the light tree belongs to the OptiX 7 estimator");
    if (!(p->flags & LH2G_RP_LIGHTTREE) && ctx->nTri + ctx->nPt + ctx->nSpot + ctx->nDir > 64)
        return fail(ctx, LH2G_ERR_INVALID, "render: more than 64 lights need the OptiX 7 estimator's light tree (LH2G_RP_LIGHTTREE)");
    if ((p->flags & LH2G_RP_OPTIX7) && (filt || nrcFrame || (p->flags & LH2G_RP_DEPTH_W)))
        return fail(ctx, LH2G_ERR_INVALID, "render: the OptiX 7 estimator combines with none of filter, radiance-cache or depth frames");
    if ((p->flags & LH2G_RP_OPTIX7) && ctx->cap >= (1ll << MIS_SLOT_BITS))
        return fail(ctx, LH2G_ERR_INVALID, "render: the OptiX 7 estimator takes at most 2^26 paths per frame");
    /* plain frames without host read-backs go to the next lane; everything else runs on the context stream after
     * the lanes' frames */
    const bool pipe = ctx->pipelineFrames > 1 && !filt && !capHits && !capSeeds && !countersOut && (!hook || hook->async) &&
                      ctx->cap <= lh2g_context::PIPE_MAX_PATHS;
    if (!pipe) JOIN();
    if (filt) {
        const int r = ensure_filter(ctx);
        if (r != LH2G_OK) return r;
    }
    const int nrcLane = pipe ? ctx->nextLane : 0;
    if (nrcFrame) {
        const int r = ensure_nrc(ctx, nrcLane);
        if (r != LH2G_OK) return r;
    }
    cudaStream_t st = ctx->st;
    Counters* hostCounters = ctx->hostCounters;
    cudaEvent_t* fev = ctx->ev;
    WaveBuffers B = ctx->B;
    int slot = -1;
    if (pipe) {
        slot = ctx->nextLane;
        const int r = ensure_lane(ctx, slot);
        if (r != LH2G_OK) return r;
        auto& L = ctx->lanes[slot];
        st = L.st, hostCounters = L.hostCounters, fev = L.ev;
        if (slot > 0) {
            for (int k = 0; k < 2; k++) B.O[k] = L.B.O[k], B.D[k] = L.B.D[k], B.T[k] = L.B.T[k];
            B.hits = L.B.hits, B.shO = L.B.shO, B.shD = L.B.shD, B.shE = L.B.shE, B.pathAcc = L.B.pathAcc, B.counters = L.B.counters;
            B.sortO = L.B.sortO, B.sortD = L.B.sortD, B.sortE = L.B.sortE, B.connBins = L.B.connBins, B.order = L.B.order;
        }
        CK(cudaEventRecord(ctx->forkEv, ctx->st));
        CK(cudaStreamWaitEvent(st, ctx->forkEv, 0));
        ctx->nextLane = (ctx->nextLane + 1) % ctx->pipelineFrames;
    }
    FrameGPU F = frame_of(view, p);
    F.stride = ctx->cap;
    B.capHits = nullptr, B.capSeeds = nullptr;
    B.features = filt ? ctx->sv.features : nullptr;
    B.worldPos = filt ? ctx->sv.worldPos : nullptr;
    B.deltaDepth = filt ? ctx->sv.deltaDepth : nullptr;
    B.nrcRec = nrcFrame ? ctx->nrcBuf[nrcLane].rec : nullptr;
    const size_t capN = (size_t)F.maxDepth * F.P;
    if (capHits || capSeeds) {
        CK(dalloc(ctx->B.capHits, capN));
        CK(dalloc(ctx->B.capSeeds, capN));
        std::vector<lh2g_hit> init(capN, lh2g_hit{0u, -1, -2, 0.0f});
        CK(cudaMemcpyAsync(ctx->B.capHits, init.data(), sizeof(lh2g_hit) * capN, cudaMemcpyHostToDevice, ctx->st));
        CK(cudaMemsetAsync(ctx->B.capSeeds, 0, sizeof(uint32_t) * capN, ctx->st));
        B.capHits = ctx->B.capHits, B.capSeeds = ctx->B.capSeeds;
    }
    const SceneGPU S = scene_of(ctx);
    /* a frame that does not accumulate overwrites the accumulator in its finalize (filter frames clear both halves
     * here, on the context stream) */
    if (!accumulate && filt) CK(cudaMemsetAsync(B.accum, 0, sizeof(float4) * (size_t)F.W * F.H * 2, st));
    CK(cudaMemsetAsync(B.counters, 0, sizeof(Counters), st));
    const int waves = ctx->tailDepth > 0 ? std::min(F.maxDepth, ctx->tailDepth - 1) : F.maxDepth;
    const bool tail = waves < F.maxDepth;
    const int launches = 2 + 3 * waves + (tail ? 1 : 0);
    const bool timing = ctx->launchTiming;
    if (timing && ctx->timedLaunches + launches > lh2g_context::MAX_TIMED_LAUNCHES) ctx->timedLaunches = 0;   /* never read: start over */
    if (timing)
        while ((int)ctx->lev.size() < 2 * (ctx->timedLaunches + launches)) {
            cudaEvent_t e;
            CK(cudaEventCreate(&e));
            ctx->lev.push_back(e);
        }
    int li = 2 * ctx->timedLaunches;
    auto mark = [&]() { if (timing) cudaEventRecord(ctx->lev[li++], st); };
    CK(cudaEventRecord(fev[0], st));
    mark();
    if (p->flags & LH2G_RP_OPTIX7) launch_generate_mis(S, F, B, st);
    else launch_generate(F, B, st);
    mark();
    for (int d = 1; d <= waves; d++) {
        WaveBuffers Bq = B;   /* with "sortRays": the queue of a bounce wave regrouped by direction octant */
        if (ctx->sortRays && d >= 2) {
            const int q = (d - 1) & 1;
            Bq.O[q] = B.sortO, Bq.D[q] = B.sortD, Bq.T[q] = B.sortE;
            mark();
            if (ctx->sortRays == 2) launch_sort_rays_local(B, d, st);
            else launch_sort_rays(B, d, st);
            launch_extend(S, F, Bq, d, ctx->blocksExtend, st), mark();
        } else {
            mark(), launch_extend(S, F, Bq, d, ctx->blocksExtend, st), mark();
        }
        mark(), launch_shade(S, F, Bq, d, ctx->blocksShade, st), mark();
        if (ctx->sortConnections) {   /* one timed slot: the regrouping and the any-hit queries */
            WaveBuffers Bs = B;
            Bs.shO = B.sortO, Bs.shD = B.sortD, Bs.shE = B.sortE;
            mark();
            if (ctx->sortConnections == 2) launch_sort_connections_local(B, d, st);
            else launch_sort_connections(B, d, st);
            launch_connect(S, F, Bs, d, ctx->blocksConnect, st), mark();
        } else {
            mark(), launch_connect(S, F, B, d, ctx->blocksConnect, st), mark();
        }
    }
    if (tail) mark(), launch_tail(S, F, B, waves + 1, ctx->blocksTail, st), mark();
    if (hook && hook->before) {
        const int r = hook->before(F, B, st, nrcLane);
        if (r != LH2G_OK) return r;
    }
    const int after = p->samplesTaken + F.spp;
    if (pipe && ctx->finValid) CK(cudaStreamWaitEvent(st, ctx->finEv, 0));   /* the previous frame's finalize first */
    mark(), launch_finalize(F, B, 1.0f / (float)after, !accumulate && !filt, st), mark();
    /* the frame to the caller's host buffer, before the next frame's finalize overwrites it */
    if (hostFrame) CK(cudaMemcpyAsync(hostFrame, B.frame, sizeof(float4) * (size_t)F.W * F.rowCount, cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(ctx->finEv, st));
    ctx->finValid = true;
    if (hook && hook->after) {
        const int r = hook->after(F, B, st, nrcLane);
        if (r != LH2G_OK) return r;
    }
    if (timing) ctx->timedLaunches += launches;
    CK(cudaGetLastError());
    CK(cudaEventRecord(fev[1], st));
    CK(cudaMemcpyAsync(hostCounters, B.counters, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    ctx->statsPending = true, ctx->lastDepth = F.maxDepth, ctx->lastP = F.P, ctx->lastSlot = slot;
    if (pipe) {
        CK(cudaEventRecord(ctx->lanes[slot].done, st));
        ctx->lanes[slot].pending = true;
    }
    if (capHits || capSeeds || countersOut) {
        CK(cudaStreamSynchronize(st));
        if (capHits) CK(cudaMemcpy(capHits, ctx->B.capHits, sizeof(lh2g_hit) * capN, cudaMemcpyDeviceToHost));
        if (capSeeds) CK(cudaMemcpy(capSeeds, ctx->B.capSeeds, sizeof(uint32_t) * capN, cudaMemcpyDeviceToHost));
        if (countersOut)
            for (int d = 0; d < F.maxDepth; d++) countersOut[2 * d] = hostCounters->extension[d], countersOut[2 * d + 1] = hostCounters->shadow[d];
        if (hostCounters->status) return fail(ctx, LH2G_ERR_OVERFLOW, "render: traversal stack overflow, step limit or path-state copy timeout");
    }
    return LH2G_OK;
}

/* buffers of PrimeAdaptive frames for the current target */
int ensure_adaptive(lh2g_context* ctx) {
    auto& a = ctx->ad;
    const int64_t WH = (int64_t)ctx->W * ctx->H;
    if (!a.hostState) {
        CK(cudaMallocHost((void**)&a.hostState, sizeof(AdaptiveState)));
        CK(cudaMallocHost((void**)&a.hostCounters2, sizeof(Counters)));
    }
    if (a.cap < ctx->cap || a.pixels < WH) {
        dfree(a.pathAcc2), dfree(a.slotLayer), dfree(a.features), dfree(a.deviation), dfree(a.want), dfree(a.tmp), dfree(a.rank);
        dfree(a.kept), dfree(a.first), dfree(a.sums), dfree(a.counters2);
        const size_t P = (size_t)ctx->cap, n = (size_t)WH;
        cudaError_t e = dalloc(a.pathAcc2, P);
        if (!e) e = dalloc(a.slotLayer, P);
        if (!e) e = dalloc(a.features, P);
        if (!e) e = dalloc(a.deviation, n);
        if (!e) e = dalloc(a.want, n);
        if (!e) e = dalloc(a.tmp, n);
        if (!e) e = dalloc(a.rank, n);
        if (!e) e = dalloc(a.kept, n);
        if (!e) e = dalloc(a.first, n);
        if (!e) e = dalloc(a.sums, n / 4096 + 2);
        if (!e) e = dalloc(a.counters2, 1);
        if (!e && !a.state) e = dalloc(a.state, 1);
        if (e) return cuda_check(ctx, e, "adaptive frame buffers");
        a.cap = ctx->cap, a.pixels = WH;
    }
    if (a.scaleDirty) {
        AdaptiveState init;
        memset(&init, 0, sizeof(init));
        init.devScale = a.pendingScale;
        CK(cudaMemcpyAsync(a.state, &init, sizeof(init), cudaMemcpyHostToDevice, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        a.scaleDirty = false;
    }
    return LH2G_OK;
}

/* One PrimeAdaptive frame (lib/RenderCore_PrimeAdaptive/rendercore.cpp:600-713 and FinalizeRender :749-755) on the
 * context stream: the first wave over the target's sample layers, the variance estimate, the second wave of
 * adaptively placed samples, finalizeASRender. */
int render_adaptive(lh2g_context* ctx, const lh2g_view* view, const lh2g_render_params* p, int accumulate, lh2g_hit* capHits, uint32_t* capSeeds,
                    uint32_t* countersOut, lh2g_adaptive_stats* statsOut) {
    if (!ctx || !view || !p) return LH2G_ERR_INVALID;
    if (!ctx->finalized) return fail(ctx, LH2G_ERR_STATE, "render: scene not finalized (call lh2g_finalize_instances)");
    if (!ctx->cap) return fail(ctx, LH2G_ERR_STATE, "render: no target (call lh2g_set_target)");
    if (p->width != ctx->W || p->height != ctx->H || p->spp != ctx->spp || p->maxDepth < 1 || p->maxDepth > 32)
        return fail(ctx, LH2G_ERR_INVALID, "render_adaptive: parameters do not match the target (or maxDepth beyond 32)");
    if ((p->flags & ~(LH2G_RP_NEE | LH2G_RP_DISNEY)) || p->rowCount != 0)
        return fail(ctx, LH2G_ERR_INVALID, "render_adaptive: only LH2G_RP_NEE and LH2G_RP_DISNEY combine with adaptive frames (whole frames)");
    if (ctx->cap >= (1ll << MIS_SLOT_BITS)) return fail(ctx, LH2G_ERR_INVALID, "render_adaptive: at most 2^26 paths per frame");
    if (ctx->nTri + ctx->nPt + ctx->nSpot + ctx->nDir > 64)
        return fail(ctx, LH2G_ERR_INVALID, "render_adaptive: at most 64 lights (the light tree is the OptiX 7 estimator's)");
    if (!ctx->mats) return fail(ctx, LH2G_ERR_STATE, "render: no materials");
    if (!materials_cover_meshes(ctx)) return fail(ctx, LH2G_ERR_INVALID, "render: a triangle's material index exceeds the material count");
    cudaSetDevice(ctx->device);
    JOIN();
    {
        const int r = ensure_adaptive(ctx);
        if (r != LH2G_OK) return r;
    }
    auto& a = ctx->ad;
    cudaStream_t st = ctx->st;
    const SceneGPU S = scene_of(ctx);
    FrameGPU F = frame_of(view, p);
    F.stride = ctx->cap;
    F.flags |= LH2G_RP_ADAPTIVE;
    F.pass = (uint32_t)p->samplesTaken;
    F.r0Base = (uint32_t)p->samplesTaken * 7907u, F.r0Depth = 91771u;
    WaveBuffers B = ctx->B;
    B.capHits = nullptr, B.capSeeds = nullptr;
    B.features = nullptr, B.worldPos = nullptr, B.deltaDepth = nullptr, B.nrcRec = nullptr;
    B.misFeatures = a.features, B.slotLayer = nullptr, B.firstCount = nullptr;
    const size_t capN = (size_t)F.maxDepth * F.P;
    if (capHits || capSeeds) {
        CK(dalloc(ctx->B.capHits, capN));
        CK(dalloc(ctx->B.capSeeds, capN));
        std::vector<lh2g_hit> init(capN, lh2g_hit{0u, -1, -2, 0.0f});
        CK(cudaMemcpyAsync(ctx->B.capHits, init.data(), sizeof(lh2g_hit) * capN, cudaMemcpyHostToDevice, st));
        CK(cudaMemsetAsync(ctx->B.capSeeds, 0, sizeof(uint32_t) * capN, st));
        B.capHits = ctx->B.capHits, B.capSeeds = ctx->B.capSeeds;
    }
    const int waves = ctx->tailDepth > 0 ? std::min(F.maxDepth, ctx->tailDepth - 1) : F.maxDepth;
    auto run_waves = [&](const FrameGPU& Fw, const WaveBuffers& Bw) {
        for (int d = 1; d <= waves; d++) {
            launch_extend(S, Fw, Bw, d, ctx->blocksExtend, st);
            launch_shade(S, Fw, Bw, d, ctx->blocksShade, st);
            launch_connect(S, Fw, Bw, d, ctx->blocksConnect, st);
        }
        if (waves < Fw.maxDepth) launch_tail(S, Fw, Bw, waves + 1, ctx->blocksTail, st);
    };
    CK(cudaEventRecord(ctx->ev[0], st));
    /* first wave */
    CK(cudaMemsetAsync(B.counters, 0, sizeof(Counters), st));
    launch_generate_mis(S, F, B, st);
    run_waves(F, B);
    /* variance estimate, budget, kept samples and their slots */
    CK(cudaMemsetAsync(a.state->hist, 0, sizeof(a.state->hist), st));
    launch_adaptive_estimate(F, B, a.deviation, a.want, a.state, st);
    launch_adaptive_keep(F, a.want, a.tmp, a.rank, a.kept, a.first, a.sums, a.state, st);
    /* second wave: pass samplesTaken + spp, shading seeds samplesTaken * 59071 + depth * 31771 (rendercore.cpp:689-691) */
    FrameGPU F2 = F;
    F2.pass = (uint32_t)(p->samplesTaken + p->spp);
    F2.r0Base = (uint32_t)p->samplesTaken * 59071u, F2.r0Depth = 31771u;
    WaveBuffers B2 = B;
    B2.pathAcc = a.pathAcc2, B2.slotLayer = a.slotLayer, B2.misFeatures = nullptr, B2.firstCount = &a.state->pathCount;
    B2.counters = a.counters2, B2.capHits = nullptr, B2.capSeeds = nullptr;
    CK(cudaMemsetAsync(B2.counters, 0, sizeof(Counters), st));
    launch_adaptive_generate(S, F2, B2, a.kept, a.first, a.slotLayer, p->frameSeed, st);
    run_waves(F2, B2);
    /* finalizeASRender after samplesTaken += spp */
    const int frames = (p->samplesTaken + p->spp) / p->spp;
    launch_adaptive_finalize(F, B.pathAcc, a.pathAcc2, a.kept, a.first, B.accum, B.frame, 1.0f / (float)frames, accumulate ? 0 : 1, st);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev[1], st));
    CK(cudaMemcpyAsync(ctx->hostCounters, B.counters, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(a.hostCounters2, a.counters2, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(a.hostState, a.state, sizeof(AdaptiveState), cudaMemcpyDeviceToHost, st));
    ctx->statsPending = true, ctx->lastDepth = F.maxDepth, ctx->lastP = F.P, ctx->lastSlot = -1;
    a.last = true;
    if (capHits || capSeeds || countersOut || statsOut) {
        CK(cudaStreamSynchronize(st));
        if (capHits) CK(cudaMemcpy(capHits, ctx->B.capHits, sizeof(lh2g_hit) * capN, cudaMemcpyDeviceToHost));
        if (capSeeds) CK(cudaMemcpy(capSeeds, ctx->B.capSeeds, sizeof(uint32_t) * capN, cudaMemcpyDeviceToHost));
        if (countersOut)
            for (int d = 0; d < F.maxDepth; d++) {
                countersOut[2 * d] = ctx->hostCounters->extension[d], countersOut[2 * d + 1] = ctx->hostCounters->shadow[d];
                countersOut[2 * (F.maxDepth + d)] = a.hostCounters2->extension[d];
                countersOut[2 * (F.maxDepth + d) + 1] = a.hostCounters2->shadow[d];
            }
        if (statsOut) {
            statsOut->devScale = a.hostState->devScale;
            statsOut->adaptivePaths = a.hostState->pathCount;
            statsOut->requested = a.hostState->requested;
        }
        if (ctx->hostCounters->status | a.hostCounters2->status) return fail(ctx, LH2G_ERR_OVERFLOW, "render: traversal stack overflow, step limit or path-state copy timeout");
    }
    return LH2G_OK;
}

}  // namespace

extern "C" {

int lh2g_render_ex(lh2g_context* ctx, const lh2g_view* view, const lh2g_render_params* p, int accumulate, lh2g_hit* capHits, uint32_t* capSeeds,
                   uint32_t* countersOut) {
    if (ctx) ctx->ad.last = false;
    return render_frame(ctx, view, p, accumulate, capHits, capSeeds, countersOut, nullptr);
}

int lh2g_render_adaptive(lh2g_context* ctx, const lh2g_view* view, const lh2g_render_params* p, int accumulate, lh2g_hit* capHits,
                         uint32_t* capSeeds, uint32_t* counters, lh2g_adaptive_stats* stats) {
    return render_adaptive(ctx, view, p, accumulate, capHits, capSeeds, counters, stats);
}

int lh2g_set_adaptive_scale(lh2g_context* ctx, float devScale) {
    if (!ctx || !(devScale > 0.0f)) return LH2G_ERR_INVALID;
    ctx->ad.pendingScale = devScale, ctx->ad.scaleDirty = true;
    return LH2G_OK;
}

int lh2g_render_to_host(lh2g_context* ctx, const lh2g_view* view, const lh2g_render_params* p, int accumulate, float* hostFrame) {
    if (!hostFrame) return LH2G_ERR_INVALID;
    if (p && (p->flags & LH2G_RP_FILTER)) return fail(ctx, LH2G_ERR_INVALID, "render_to_host: filter frames are presented by lh2g_filter");
    return render_frame(ctx, view, p, accumulate, nullptr, nullptr, nullptr, nullptr, hostFrame);
}

int lh2g_render_nrc(lh2g_context* ctx, lh2g_nrc* cache, const lh2g_view* view, const lh2g_render_params* params, int accumulate, int train,
                    lh2g_nrc_frame_stats* stats) {
    if (!ctx || !cache || !view || !params) return LH2G_ERR_INVALID;
    if (params->flags & LH2G_RP_FILTER) return fail(ctx, LH2G_ERR_INVALID, "render_nrc: filter frames do not combine with the cache");
    lh2g_render_params p = *params;
    p.flags |= LH2G_RP_NRC;
    if (!ctx->cacheEv) CK(cudaEventCreateWithFlags(&ctx->cacheEv, cudaEventDisableTiming));
    FrameHooks hooks;
    hooks.async = stats == nullptr;   /* nothing waits for the device: the frame may overlap others */
    /* after the waves: gather the queries and training samples, infer, add throughput x prediction. The cache
     * work waits for the previous frame's (its update), all counts stay on the device. */
    hooks.before = [&](const FrameGPU& F, const WaveBuffers& B, cudaStream_t st, int lane) -> int {
        NrcBuffers& n = ctx->nrcBuf[lane];
        CK(cudaMemsetAsync(n.counts, 0, 16, st));
        launch_nrc_collect(F, B, n.queries, n.qPath, n.trainQ, n.trainT, n.counts, NRC_TRAIN_CAP, st);
        if (ctx->cacheEvValid) CK(cudaStreamWaitEvent(st, ctx->cacheEv, 0));
        const int r = lh2g_nrc_infer_counted(cache, (const float*)n.queries, n.counts, F.P, (float*)n.pred, st);
        if (r != LH2G_OK) return fail(ctx, r, std::string("radiance-cache inference: ") + lh2g_nrc_last_error(cache));
        launch_nrc_apply(F, B, n.pred, n.qPath, n.counts, st);
        if (!train) {
            CK(cudaEventRecord(ctx->cacheEv, st));
            ctx->cacheEvValid = true;
        }
        return LH2G_OK;
    };
    /* after the finalize: one training step on the frame's samples */
    if (train)
        hooks.after = [&](const FrameGPU&, const WaveBuffers&, cudaStream_t st, int lane) -> int {
            NrcBuffers& n = ctx->nrcBuf[lane];
            const int r = lh2g_nrc_train_counted(cache, (const float*)n.trainQ, (const float*)n.trainT, n.counts + 1, NRC_TRAIN_CAP, st);
            if (r != LH2G_OK) return fail(ctx, r, std::string("radiance-cache training: ") + lh2g_nrc_last_error(cache));
            CK(cudaEventRecord(ctx->cacheEv, st));
            ctx->cacheEvValid = true;
            return LH2G_OK;
        };
    int r = render_frame(ctx, view, &p, accumulate, nullptr, nullptr, nullptr, &hooks);
    if (r != LH2G_OK) return r;
    if (stats) {   /* the frame ran on the context stream with lane 0's buffers */
        NrcBuffers& n = ctx->nrcBuf[0];
        CK(cudaMemcpyAsync(n.hostCounts, n.counts, 8, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        stats->queries = n.hostCounts[0];
        stats->trainSamples = std::min<uint32_t>(n.hostCounts[1], NRC_TRAIN_CAP);
        stats->loss = 0.0f;
        if (train && stats->trainSamples > 0) {
            r = lh2g_nrc_last_loss(cache, &stats->loss);
            if (r != LH2G_OK) return fail(ctx, r, std::string("radiance-cache training: ") + lh2g_nrc_last_error(cache));
        }
    }
    return LH2G_OK;
}

namespace {

/* RenderCore::Render + FinalizeRender of the filter core (lib/RenderCore_Optix7Filter/rendercore.cpp:737-797,
 * 897-935) */
int render_filtered(lh2g_context* ctx, const lh2g_view* view, int converge) {
    if (converge == 1 || ctx->firstConverging) {
        ctx->samplesTaken = 0;
        ctx->firstConverging = true;   /* camRNGseed is not reset: every frame gets new noise */
    }
    if (converge == 0) ctx->firstConverging = false;
    static const float haltonx[4] = {0.3f, 0.7f, 0.2f, 0.8f}, haltony[4] = {0.2f, 0.8f, 0.7f, 0.3f};
    const float j0 = ctx->taaEnabled ? haltonx[ctx->frameCycle] : 0.0f;
    const float j1 = ctx->taaEnabled ? haltony[ctx->frameCycle] : 0.0f;
    ctx->frameCycle = (ctx->frameCycle + 1) & 3;
    lh2g_view jv = *view;
    for (int k = 0; k < 3; k++) {
        const float right = view->p2[k] - view->p1[k], up = view->p3[k] - view->p1[k];
        const float jitter = (j0 / (float)ctx->W) * right + (j1 / (float)ctx->H) * up;
        jv.p1[k] += jitter, jv.p2[k] += jitter, jv.p3[k] += jitter;
    }
    jv.aperture = 0;
    lh2g_render_params p;
    memset(&p, 0, sizeof(p));
    p.width = ctx->W, p.height = ctx->H, p.spp = ctx->spp, p.maxDepth = ctx->maxDepth, p.rrStartDepth = ctx->rrStart;
    p.samplesTaken = ctx->samplesTaken;
    p.frameSeed = xorshift(ctx->filterSeed);
    p.geometryEpsilon = ctx->eps, p.clampValue = ctx->clampValue;
    p.flags = LH2G_RP_FILTER | (ctx->nee ? LH2G_RP_NEE : 0) | LH2G_RP_DEPTH_W;
    int r = lh2g_render_ex(ctx, &jv, &p, ctx->samplesTaken > 0 ? 1 : 0, nullptr, nullptr, nullptr);
    if (r != LH2G_OK) return r;
    ctx->samplesTaken += ctx->spp;
    lh2g_filter_params fp;
    memset(&fp, 0, sizeof(fp));
    fp.prevView = ctx->havePrevView ? ctx->prevView : *view;
    fp.j0 = j0, fp.j1 = j1, fp.prevj0 = ctx->prevj0, fp.prevj1 = ctx->prevj1;
    fp.clampDirect = ctx->clampDirect, fp.clampIndirect = ctx->clampIndirect;
    fp.samplesTaken = ctx->samplesTaken;
    fp.camIsStationary = ctx->samplesTaken == ctx->spp ? 0 : 1;
    fp.taa = ctx->taaEnabled;
    r = lh2g_filter(ctx, &fp);
    if (r != LH2G_OK) return r;
    ctx->prevj0 = j0, ctx->prevj1 = j1;
    ctx->prevView = *view, ctx->havePrevView = true;
    ctx->lastFilter = fp, ctx->lastJittered = jv, ctx->lastParams = p;
    return LH2G_OK;
}

}  // namespace

int lh2g_filter(lh2g_context* ctx, const lh2g_filter_params* fp) {
    if (!ctx || !fp) return LH2G_ERR_INVALID;
    if (!ctx->svAlloc) return fail(ctx, LH2G_ERR_STATE, "filter: no filter-core frame rendered on this target");
    if (fp->samplesTaken <= 0) return fail(ctx, LH2G_ERR_INVALID, "filter: samplesTaken must be positive");
    cudaSetDevice(ctx->device);
    JOIN();
    SvgfBuffers b = ctx->sv;
    b.accum = ctx->B.accum, b.target = ctx->B.frame;
    SvgfArgs a;
    a.W = ctx->W, a.H = ctx->H;
    a.scale = 1.0f / (float)fp->samplesTaken;
    a.j0 = fp->j0, a.j1 = fp->j1, a.prevj0 = fp->prevj0, a.prevj1 = fp->prevj1;
    a.clampDirect = fp->clampDirect, a.clampIndirect = fp->clampIndirect;
    a.camIsStationary = fp->camIsStationary;
    a.view = svgf_view(fp->prevView, ctx->H);
    CK(cudaEventRecord(ctx->fev[0], ctx->st));
    launch_svgf(b, a, fp->taa != 0, ctx->st);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->fev[1], ctx->st));
    ctx->filterPending = true;
    SvgfBuffers& v = ctx->sv;
    if (fp->taa) std::swap(v.taaPixels, v.prevPixels);
    else std::swap(v.shading, v.prevPixels);
    std::swap(v.filteredIN, v.filteredOUT);
    std::swap(v.prevWorldPos, v.worldPos);
    std::swap(v.moments, v.prevMoments);
    return LH2G_OK;
}

int lh2g_read_filter_buffer(lh2g_context* ctx, int slot, void* host) {
    if (!ctx || !host || slot < 0 || slot >= LH2G_FB_COUNT) return LH2G_ERR_INVALID;
    if (!ctx->svAlloc) return fail(ctx, LH2G_ERR_STATE, "read_filter_buffer: no filter buffers");
    JOIN();
    const size_t WH = (size_t)ctx->W * ctx->H;
    const SvgfBuffers& v = ctx->sv;
    const void* src = nullptr;
    size_t bytes = sizeof(float4) * WH;
    switch (slot) {
        case LH2G_FB_FEATURES: src = v.features; break;
        case LH2G_FB_WORLDPOS: src = v.worldPos; break;
        case LH2G_FB_PREV_WORLDPOS: src = v.prevWorldPos; break;
        case LH2G_FB_DELTADEPTH: src = v.deltaDepth; break;
        case LH2G_FB_MOTION: src = v.motion, bytes = sizeof(float2) * WH; break;
        case LH2G_FB_MOMENTS: src = v.moments; break;
        case LH2G_FB_PREV_MOMENTS: src = v.prevMoments; break;
        case LH2G_FB_SHADING: src = v.shading; break;
        case LH2G_FB_FILTERED_IN: src = v.filteredIN; break;
        case LH2G_FB_FILTERED_OUT: src = v.filteredOUT; break;
        case LH2G_FB_PREV_PIXELS: src = v.prevPixels; break;
        default: src = ctx->B.accum, bytes = 2 * sizeof(float4) * WH; break;
    }
    CK(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return LH2G_OK;
}

int lh2g_get_last_filter_frame(lh2g_context* ctx, lh2g_filter_params* filter, lh2g_view* jitteredView, lh2g_render_params* params) {
    if (!ctx) return LH2G_ERR_INVALID;
    if (filter) *filter = ctx->lastFilter;
    if (jitteredView) *jitteredView = ctx->lastJittered;
    if (params) *params = ctx->lastParams;
    return LH2G_OK;
}

int lh2g_render(lh2g_context* ctx, const lh2g_view* view, int converge) {
    if (!ctx || !view) return LH2G_ERR_INVALID;
    if (ctx->filterEnabled) {
        if (!ctx->cap) return fail(ctx, LH2G_ERR_STATE, "render: no target (call lh2g_set_target)");
        return render_filtered(ctx, view, converge);
    }
    if (converge == 1 || ctx->firstConverging) {
        ctx->samplesTaken = 0;
        ctx->firstConverging = true;
        ctx->camSeed = 0x12345678u;
    }
    if (converge == 0) ctx->firstConverging = false;
    lh2g_render_params p;
    memset(&p, 0, sizeof(p));
    p.width = ctx->W, p.height = ctx->H, p.spp = ctx->spp, p.maxDepth = ctx->maxDepth, p.rrStartDepth = ctx->rrStart;
    p.samplesTaken = ctx->samplesTaken;
    p.geometryEpsilon = ctx->eps, p.clampValue = ctx->clampValue;
    int r;
    if (ctx->adaptive) {
        /* RenderCore_PrimeAdaptive/rendercore.cpp:606-609: one shift draw, then two camera draws per frame */
        p.shift = xorshift(ctx->shiftSeed);
        p.cameraR0 = xorshift(ctx->camSeed);
        p.frameSeed = xorshift(ctx->camSeed);
        p.maxDepth = std::min(ctx->maxDepth, 32);
        p.flags = (ctx->nee ? LH2G_RP_NEE : 0) | (ctx->bsdf ? LH2G_RP_DISNEY : 0);
        r = lh2g_render_adaptive(ctx, view, &p, ctx->samplesTaken > 0 ? 1 : 0, nullptr, nullptr, nullptr, nullptr);
    } else if (ctx->estimator == 1) {
        /* rendercore_optix7/rendercore.cpp:855,900: one shift draw per frame, one camera draw per wave (here every
         * wave of maxDepth is drawn for, also where the reference's loop ends early) */
        p.shift = xorshift(ctx->shiftSeed);
        p.cameraR0 = xorshift(ctx->camSeed);
        for (int d = 1; d < p.maxDepth; d++) xorshift(ctx->camSeed);
        p.flags = (ctx->nee ? LH2G_RP_NEE : 0) | LH2G_RP_OPTIX7 | (ctx->bsdf ? LH2G_RP_DISNEY : 0) | (ctx->lightTreeOn ? LH2G_RP_LIGHTTREE : 0);
        r = lh2g_render_ex(ctx, view, &p, ctx->samplesTaken > 0 ? 1 : 0, nullptr, nullptr, nullptr);
    } else {
        p.cameraR0 = xorshift(ctx->camSeed);
        p.flags = (ctx->nee ? LH2G_RP_NEE : 0) | LH2G_RP_DEPTH_W;
        r = lh2g_render_ex(ctx, view, &p, ctx->samplesTaken > 0 ? 1 : 0, nullptr, nullptr, nullptr);
    }
    if (r == LH2G_OK) ctx->samplesTaken += ctx->spp;
    return r;
}

int lh2g_wait(lh2g_context* ctx) {
    if (!ctx) return LH2G_ERR_INVALID;
    JOIN();
    CK(cudaStreamSynchronize(ctx->st));
    return LH2G_OK;
}

int lh2g_get_stats(lh2g_context* ctx, lh2g_stats* out) {
    if (!ctx || !out) return LH2G_ERR_INVALID;
    JOIN();
    if (ctx->statsPending) {
        CK(cudaStreamSynchronize(ctx->st));
        const bool lane = ctx->lastSlot >= 0;
        const Counters& C = lane ? *ctx->lanes[ctx->lastSlot].hostCounters : *ctx->hostCounters;
        uint32_t ext = (uint32_t)ctx->lastP, sh = 0;
        for (int d = 0; d < ctx->lastDepth; d++) ext += C.extension[d], sh += C.shadow[d];
        uint32_t primary = (uint32_t)ctx->lastP;
        if (ctx->ad.last) {   /* an adaptive frame: its second wave's rays too */
            const Counters& C2 = *ctx->ad.hostCounters2;
            const uint32_t n2 = ctx->ad.hostState->pathCount;
            ext += n2, primary += n2;
            for (int d = 0; d < ctx->lastDepth; d++) ext += C2.extension[d], sh += C2.shadow[d];
        }
        ctx->stats.totalExtensionRays = ext, ctx->stats.totalShadowRays = sh, ctx->stats.totalRays = ext + sh;
        ctx->stats.primaryRayCount = primary;
        ctx->stats.bounce1RayCount = ctx->lastDepth > 1 ? C.extension[0] : 0;
        uint32_t deep = 0;
        for (int d = 1; d < ctx->lastDepth - 1; d++) deep += C.extension[d];
        ctx->stats.deepRayCount = deep;
        float ms = 0;
        cudaEvent_t* fev = lane ? ctx->lanes[ctx->lastSlot].ev : ctx->ev;
        cudaEventElapsedTime(&ms, fev[0], fev[1]);
        ctx->stats.renderTime = ms;
        ctx->stats.deviceStatus = C.status;
        ctx->statsPending = false;
    }
    if (ctx->filterPending) {   /* RenderCore_Optix7Filter/rendercore.cpp:868 */
        CK(cudaEventSynchronize(ctx->fev[1]));
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->fev[0], ctx->fev[1]);
        ctx->stats.filterTime = ms;
        ctx->filterPending = false;
    }
    *out = ctx->stats;
    return LH2G_OK;
}

int lh2g_get_framebuffer(lh2g_context* ctx, void** dev) {
    if (!ctx || !dev) return LH2G_ERR_INVALID;
    if (!ctx->cap) return fail(ctx, LH2G_ERR_STATE, "no target");
    JOIN();
    *dev = ctx->B.frame;
    return LH2G_OK;
}

int lh2g_read_framebuffer(lh2g_context* ctx, float* host) {
    if (!ctx || !host) return LH2G_ERR_INVALID;
    if (!ctx->cap) return fail(ctx, LH2G_ERR_STATE, "no target");
    JOIN();
    CK(cudaMemcpyAsync(host, ctx->B.frame, sizeof(float4) * (size_t)ctx->W * ctx->H, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return LH2G_OK;
}

int lh2g_read_accumulator(lh2g_context* ctx, float* host) {
    if (!ctx || !host) return LH2G_ERR_INVALID;
    if (!ctx->cap) return fail(ctx, LH2G_ERR_STATE, "no target");
    /* the direct half only when filter frames split it (LH2G_FB_ACCUM reads both) */
    JOIN();
    CK(cudaMemcpyAsync(host, ctx->B.accum, sizeof(float4) * (size_t)ctx->W * ctx->H, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return LH2G_OK;
}

int lh2g_get_traversal_stats(lh2g_context* ctx, unsigned long long* out4) {
    if (!ctx || !out4) return LH2G_ERR_INVALID;
    JOIN();
    CK(cudaStreamSynchronize(ctx->st));
    const Counters* C = ctx->lastSlot >= 0 ? ctx->lanes[ctx->lastSlot].hostCounters : ctx->hostCounters;
    for (int k = 0; k < 4; k++) out4[k] = C->travStats[k];
    return LH2G_OK;
}

int lh2g_get_stream(lh2g_context* ctx, void** stream) {
    if (!ctx || !stream) return LH2G_ERR_INVALID;
    JOIN();
    *stream = (void*)ctx->st;
    return LH2G_OK;
}

int lh2g_enable_launch_timing(lh2g_context* ctx, int enable) {
    if (!ctx) return LH2G_ERR_INVALID;
    ctx->launchTiming = enable != 0;
    ctx->timedLaunches = 0;
    return LH2G_OK;
}

int lh2g_get_launch_times(lh2g_context* ctx, float* ms, int capacity, int* count) {
    if (!ctx || !count || (capacity > 0 && !ms)) return LH2G_ERR_INVALID;
    JOIN();
    CK(cudaStreamSynchronize(ctx->st));
    *count = ctx->timedLaunches;
    for (int k = 0; k < ctx->timedLaunches && k < capacity; k++) {
        float t = 0;
        CK(cudaEventElapsedTime(&t, ctx->lev[2 * k], ctx->lev[2 * k + 1]));
        ms[k] = t;
    }
    ctx->timedLaunches = 0;
    return LH2G_OK;
}

int lh2g_trace(lh2g_context* ctx, const lh2g_ray* rays, void* out, long long n, int mode, void* stream) {
    if (!ctx || n < 0 || (n && (!rays || !out)) || (mode != 0 && mode != 1)) return LH2G_ERR_INVALID;
    if (!ctx->finalized) return fail(ctx, LH2G_ERR_STATE, "trace: scene not finalized");
    if (n == 0) return LH2G_OK;
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->st;
    const long long chunk = 1ll << 31;   /* the work counter is 32-bit */
    const int blocks = persistent_blocks_trace(mode);
    CK(cudaMemsetAsync(ctx->traceFetch + 2, 0, 4, st));
    for (long long b = 0; b < n; b += chunk) {
        const long long m = std::min(chunk, n - b);
        CK(cudaMemsetAsync(ctx->traceFetch, 0, 4, st));
        void* o = (char*)out + (size_t)b * (mode == 0 ? sizeof(lh2g_hit) : sizeof(uint32_t));
        launch_trace(scene_of(ctx), rays + b, o, m, mode, ctx->traceFetch, ctx->traceFetch + 2, blocks, st);
    }
    CK(cudaGetLastError());
    return LH2G_OK;
}

int lh2g_trace_host(lh2g_context* ctx, const lh2g_ray* rays, void* out, long long n, int mode) {
    if (!ctx || n < 0 || (n && (!rays || !out)) || (mode != 0 && mode != 1)) return LH2G_ERR_INVALID;
    if (n == 0) return LH2G_OK;
    cudaSetDevice(ctx->device);
    if (n > ctx->hostCap) {
        CK(dalloc(ctx->hostRaysDev, (size_t)n));
        CK(cudaMalloc(&ctx->hostOutDev, sizeof(lh2g_hit) * (size_t)n));
        ctx->hostCap = n;
    }
    const size_t outBytes = (mode == 0 ? sizeof(lh2g_hit) : sizeof(uint32_t)) * (size_t)n;
    CK(cudaMemcpyAsync(ctx->hostRaysDev, rays, sizeof(lh2g_ray) * (size_t)n, cudaMemcpyHostToDevice, ctx->st));
    const int r = lh2g_trace(ctx, ctx->hostRaysDev, ctx->hostOutDev, n, mode, nullptr);
    if (r != LH2G_OK) return r;
    CK(cudaMemcpyAsync(out, ctx->hostOutDev, outBytes, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    uint32_t status = 0;
    CK(cudaMemcpy(&status, ctx->traceFetch + 2, 4, cudaMemcpyDeviceToHost));
    if (status) return fail(ctx, LH2G_ERR_OVERFLOW, "trace: traversal stack overflow or step limit");
    return LH2G_OK;
}

}  // extern "C"

namespace lh2g {
/* The device frame parameters of a view and estimator parameters (shared by render_ex and the serving loop). */
FrameGPU frame_of(const lh2g_view* view, const lh2g_render_params* p) {
    FrameGPU F;
    memset(&F, 0, sizeof(F));
    F.W = p->width, F.H = p->height, F.spp = p->spp, F.maxDepth = p->maxDepth, F.rrStart = p->rrStartDepth, F.samplesTaken = p->samplesTaken;
    F.cameraR0 = p->cameraR0, F.frameSeed = p->frameSeed, F.eps = p->geometryEpsilon, F.flags = p->flags;
    F.spreadAngle = view->spreadAngle, F.aperture = view->aperture;
    F.pos = make_float3(view->pos[0], view->pos[1], view->pos[2]);
    F.p1 = make_float3(view->p1[0], view->p1[1], view->p1[2]);
    F.right = make_float3(view->p2[0] - view->p1[0], view->p2[1] - view->p1[1], view->p2[2] - view->p1[2]);
    F.up = make_float3(view->p3[0] - view->p1[0], view->p3[1] - view->p1[1], view->p3[2] - view->p1[2]);
    F.P = (int64_t)F.W * F.H * F.spp;
    F.stride = F.P;
    F.distortion = view->distortion, F.shift = p->shift, F.pass = (uint32_t)p->samplesTaken, F.clampValue = p->clampValue;
    F.rowBegin = 0, F.rowCount = F.H, F.bandPix = 0;
    if (p->rowCount > 0) {   /* a band of rows: its paths, with their seeds of the whole frame */
        F.rowBegin = p->rowBegin, F.rowCount = p->rowCount;
        F.bandPix = (uint32_t)F.W * (uint32_t)p->rowCount;
        F.P = (int64_t)F.bandPix * F.spp;
        F.stride = F.P;
    }
    return F;
}

/* Scene and persistent-grid sizes of a finalized context (for the allocation-free render in noalloc.cu). */
int context_scene(lh2g_context* ctx, SceneGPU* scene, int* device, int* blocks4, int* tailDepth) {
    if (!ctx || !scene || !device || !blocks4 || !tailDepth) return LH2G_ERR_INVALID;
    if (!ctx->finalized) return fail(ctx, LH2G_ERR_STATE, "render: scene not finalized (call lh2g_finalize_instances)");
    if (!ctx->mats) return fail(ctx, LH2G_ERR_STATE, "render: no materials");
    if (!materials_cover_meshes(ctx)) return fail(ctx, LH2G_ERR_INVALID, "render: a triangle's material index exceeds the material count");
    *scene = scene_of(ctx);
    *device = ctx->device;
    blocks4[0] = ctx->blocksExtend, blocks4[1] = ctx->blocksConnect, blocks4[2] = ctx->blocksShade, blocks4[3] = ctx->blocksTail;
    *tailDepth = ctx->tailDepth;
    return LH2G_OK;
}
}  // namespace lh2g

/* ======================================================================================================
 * SoftRasterizer core (lib/RenderCore_SoftRasterizer): the frame's host half. The camera transform
 * (rendercore.cpp:215-222), its inverse (rasterizer.cpp:239), the per-mesh transforms (SGNode::Render,
 * rasterizer.cpp:185-190), the frustum planes (Rasterizer::Reinit, :205-214) and the mesh culling (:69-75) are a
 * few hundred flops per frame and run here, in the reference's operation order (host code is built without FMA
 * contraction); the triangles run on the device (raster.cu).
 * ==================================================================================================== */
namespace {

struct RsM { float m[16]; };
struct RsV { float x, y, z; };
RsV rs_sub(RsV a, RsV b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
float rs_dot(RsV a, RsV b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
RsV rs_cross(RsV a, RsV b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
RsV rs_normalize(RsV v) { const float inv = 1.0f / sqrtf(rs_dot(v, v)); return {v.x * inv, v.y * inv, v.z * inv}; }
/* operator*(mat4, mat4), lib/platform/system.cpp:57-68 */
RsM rs_mul(const float* a, const float* b) {
    RsM r;
    for (int i = 0; i < 16; i += 4)
        for (int j = 0; j < 4; j++) r.m[i + j] = a[i] * b[j] + a[i + 1] * b[j + 4] + a[i + 2] * b[j + 8] + a[i + 3] * b[j + 12];
    return r;
}
int rs_f2i(float x) {   /* truncation, saturating, NaN -> 0 (as the device's conversion) */
    if (x != x) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int)0x80000000u;
    return (int)x;
}

}  // namespace

int lh2g_raster_render(lh2g_context* ctx, const lh2g_view* view, uint32_t* pixelsHost, float* depthHost, lh2g_raster_stats* stats) {
    if (!ctx || !view) return LH2G_ERR_INVALID;
    const int W = ctx->W, H = ctx->H;
    if (W < 3 || H < 3 || W > 8192 || H > 8192) return fail(ctx, LH2G_ERR_INVALID, "raster_render: the target must be 3..8192 pixels on each side");
    if (!materials_cover_meshes(ctx)) return fail(ctx, LH2G_ERR_INVALID, "raster_render: a triangle names a missing material");
    cudaSetDevice(ctx->device);
    JOIN();
    auto& R0 = ctx->rs;
    /* frustum planes (rasterizer.cpp:205-214) */
    float4 fr[5];
    {
        const float w = (float)W, h = (float)H;
        const float C = -1.0f, x1 = 0.5f, x2 = W - 1.5f, y1 = 0.5f, y2 = H - 1.5f;
        const RsV p0 = {0.0f, 0.0f, 0.0f};
        const RsV p1 = {((x1 - w * 0.5f) * C) / w, ((y1 - h * 0.5f) * C) / w, 1.0f};
        const RsV p2 = {((x2 - w * 0.5f) * C) / w, ((y1 - h * 0.5f) * C) / w, 1.0f};
        const RsV p3 = {((x2 - w * 0.5f) * C) / w, ((y2 - h * 0.5f) * C) / w, 1.0f};
        const RsV p4 = {((x1 - w * 0.5f) * C) / w, ((y2 - h * 0.5f) * C) / w, 1.0f};
        const RsV a = rs_normalize(rs_cross(rs_sub(p1, p0), rs_sub(p4, p1))), b = rs_normalize(rs_cross(rs_sub(p2, p0), rs_sub(p1, p2)));
        const RsV c = rs_normalize(rs_cross(rs_sub(p3, p0), rs_sub(p2, p3))), d = rs_normalize(rs_cross(rs_sub(p4, p0), rs_sub(p3, p4)));
        fr[0] = make_float4(0.0f, 0.0f, -1.0f, 0.2f);
        fr[1] = make_float4(a.x, a.y, a.z, 0.0f), fr[2] = make_float4(b.x, b.y, b.z, 0.0f);
        fr[3] = make_float4(c.x, c.y, c.z, 0.0f), fr[4] = make_float4(d.x, d.y, d.z, 0.0f);
    }
    /* camera transform, inverted, times the scene root's identity (rendercore.cpp:215-222, rasterizer.cpp:187,239) */
    RsM root;
    {
        const RsV pos = {view->pos[0], view->pos[1], view->pos[2]}, p1 = {view->p1[0], view->p1[1], view->p1[2]};
        const RsV p2 = {view->p2[0], view->p2[1], view->p2[2]}, p3 = {view->p3[0], view->p3[1], view->p3[2]};
        const RsV X = rs_normalize(rs_sub(p2, p1)), Y = rs_normalize(rs_sub(p1, p3));
        const RsV mid = {0.5f * (p2.x + p3.x), 0.5f * (p2.y + p3.y), 0.5f * (p2.z + p3.z)};
        const RsV Z = rs_normalize(rs_sub(pos, mid));
        float Rm[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        Rm[0] = X.x, Rm[4] = X.y, Rm[8] = X.z;
        Rm[1] = Y.x, Rm[5] = Y.y, Rm[9] = Y.z;
        Rm[2] = Z.x, Rm[6] = Z.y, Rm[10] = Z.z;
        const float Tr[16] = {1, 0, 0, pos.x, 0, 1, 0, pos.y, 0, 0, 1, pos.z, 0, 0, 0, 1};
        const RsM cam = rs_mul(Tr, Rm);
        float inv[16];
        invert4x4(cam.m, inv);
        const float I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        root = rs_mul(inv, I);
    }
    /* instances sharing a mesh share its scene-graph node and with it the transform set last (rendercore.cpp:118-131) */
    std::vector<const float*> meshT(ctx->meshes.size(), nullptr);
    for (const InstHost& in : ctx->inst) meshT[in.mesh] = in.T;
    std::vector<RasterInst> kept;
    std::vector<int> keptMesh;
    uint32_t total = 0;
    for (const InstHost& in : ctx->inst) {
        const MeshDev& m = ctx->meshes[in.mesh];
        if (!m.n) continue;
        const RsM M = rs_mul(root.m, meshT[in.mesh]);
        /* cull the mesh's bounding box (rasterizer.cpp:69-75): out when every corner is outside one plane */
        bool culled = false;
        for (int p = 0; p < 5 && !culled; p++) {
            int i = 0;
            for (; i < 8; i++) {
                const float bx = (i & 1) ? m.bmax[0] : m.bmin[0], by = ((i >> 1) & 1) ? m.bmax[1] : m.bmin[1], bz = (i >> 2) ? m.bmax[2] : m.bmin[2];
                const RsV c = {M.m[0] * bx + M.m[1] * by + M.m[2] * bz + M.m[3] * 1.0f, M.m[4] * bx + M.m[5] * by + M.m[6] * bz + M.m[7] * 1.0f,
                               M.m[8] * bx + M.m[9] * by + M.m[10] * bz + M.m[11] * 1.0f};
                if ((rs_dot({fr[p].x, fr[p].y, fr[p].z}, c) - fr[p].w) > 0) break;
            }
            culled = i == 8;
        }
        if (culled) continue;
        if ((uint64_t)total + m.n >= (1ull << 32)) return fail(ctx, LH2G_ERR_INVALID, "raster_render: more than 2^32 triangles in view");
        RasterInst r;
        memcpy(r.M, M.m, sizeof(r.M));
        r.verts = m.verts, r.tris = m.tris, r.norms = nullptr, r.first = total, r.count = m.n;
        keptMesh.push_back(in.mesh);
        kept.push_back(r);
        total += m.n;
    }
    /* materials (rendercore.cpp:166-185) */
    std::vector<RasterMat> mats(std::max<size_t>(1, ctx->hostMats.size()));
    for (size_t i = 0; i < ctx->hostMats.size(); i++) {
        const lh2g_material& hm = ctx->hostMats[i];
        const int t = hm.color_map.texture;
        RasterMat rm;
        rm.diffuse = ((uint32_t)rs_f2i(hm.color[2] * 255.0f) << 16) + ((uint32_t)rs_f2i(hm.color[1] * 255.0f) << 8) + (uint32_t)rs_f2i(hm.color[0] * 255.0f);
        if (t >= 0 && t < (int)ctx->texFirst.size()) rm.texFirst = ctx->texFirst[t], rm.width = ctx->texWH[2 * t], rm.height = ctx->texWH[2 * t + 1];
        else rm.texFirst = 0, rm.width = 0, rm.height = 0;
        mats[i] = rm;
    }
    /* buffers */
    const int64_t WH = (int64_t)W * H;
    if (WH > R0.pixCap) {
        CK(dalloc(R0.pixels, WH));
        CK(dalloc(R0.keys, WH));
        dfree(R0.depth);
        R0.pixCap = WH;
    }
    if ((int64_t)total > R0.triCap) {
        CK(dalloc(R0.list, total));
        CK(dalloc(R0.big, total));
        R0.triCap = total;
    }
    /* chunks of the block path: up to 2^20 (88 MB); triangles that find the arrays full are filled one per thread */
    const uint32_t ckCap = std::min<uint32_t>(1u << 20, std::max<uint32_t>(1u << 14, total));
    if (ckCap > R0.ckCap) {
        CK(dalloc(R0.owner, ckCap));
        CK(dalloc(R0.ck, (size_t)ckCap * 5));
        R0.ckCap = ckCap;
    }
    if (!R0.counters) CK(dalloc(R0.counters, 8));
    if ((int)kept.size() > R0.instCap) {
        CK(dalloc(R0.inst, kept.size()));
        R0.instCap = (int)kept.size();
    }
    if ((int)mats.size() > R0.matCap) {
        CK(dalloc(R0.mats, mats.size()));
        R0.matCap = (int)mats.size();
    }
    cudaStream_t st = ctx->st;
    /* the first pass's compact per-triangle records, once per mesh geometry */
    for (size_t k = 0; k < kept.size(); k++) {
        MeshDev& m = ctx->meshes[keptMesh[k]];
        if (!m.rsNorms) {
            CK(dalloc(m.rsNorms, m.n));
            launch_raster_pack(m.tris, m.n, m.rsNorms, st);
            CK(cudaGetLastError());
        }
        kept[k].norms = m.rsNorms;
    }
    if (!kept.empty()) CK(cudaMemcpyAsync(R0.inst, kept.data(), sizeof(RasterInst) * kept.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(R0.mats, mats.data(), sizeof(RasterMat) * mats.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(R0.pixels, 0, sizeof(uint32_t) * WH, st));
    CK(cudaMemsetAsync(R0.keys, 0xff, sizeof(unsigned long long) * WH, st));
    CK(cudaMemsetAsync(R0.counters, 0, 8 * sizeof(uint32_t), st));
    RasterFrame F;
    F.W = W, F.H = H, F.nearPlane = fr[0], F.leftPlane = fr[1];
    F.inst = R0.inst, F.nInst = (int)kept.size(), F.total = total;
    F.mats = R0.mats, F.nMats = (uint32_t)ctx->hostMats.size(), F.texels = ctx->texels;
    F.pixels = R0.pixels, F.keys = R0.keys, F.list = R0.list, F.big = R0.big, F.counters = R0.counters;
    F.owner = R0.owner, F.ck = R0.ck, F.ckCap = R0.ckCap;
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    launch_raster(F, sms, st);
    CK(cudaGetLastError());
    if (depthHost) {
        if (!R0.depth) CK(dalloc(R0.depth, R0.pixCap));
        launch_raster_depth(F, R0.depth, st);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(depthHost, R0.depth, sizeof(float) * WH, cudaMemcpyDeviceToHost, st));
    }
    if (pixelsHost) CK(cudaMemcpyAsync(pixelsHost, R0.pixels, sizeof(uint32_t) * WH, cudaMemcpyDeviceToHost, st));
    R0.W = W, R0.H = H, R0.valid = true;
    if (stats) {
        uint32_t c[4];
        CK(cudaMemcpyAsync(c, R0.counters, sizeof(c), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        stats->instancesDrawn = (uint32_t)kept.size(), stats->triangles = total;
        stats->smallTriangles = c[0], stats->bigTriangles = c[1], stats->fragments = c[2], stats->status = c[3];
    } else if (pixelsHost || depthHost) {
        CK(cudaStreamSynchronize(st));
    }
    return LH2G_OK;
}

uint32_t* lh2g_raster_pixels_device(lh2g_context* ctx) { return ctx && ctx->rs.valid ? ctx->rs.pixels : nullptr; }

int lh2g_raster_read(lh2g_context* ctx, uint32_t* pixelsHost) {
    if (!ctx || !pixelsHost) return LH2G_ERR_INVALID;
    if (!ctx->rs.valid) return fail(ctx, LH2G_ERR_INVALID, "raster_read: no raster frame yet");
    cudaSetDevice(ctx->device);
    CK(cudaMemcpyAsync(pixelsHost, ctx->rs.pixels, sizeof(uint32_t) * (size_t)ctx->rs.W * ctx->rs.H, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return LH2G_OK;
}

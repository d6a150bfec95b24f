/* kernels.cuh - the wavefront stages and ray-query kernels of the GB300 render core. */
#pragma once
#include "core_types.cuh"
#include "lh2g_types.h"

namespace lh2g {

/* Path-state buffers of one render target (capacity = W * H * spp paths). */
struct WaveBuffers {
    float4* O[2];          /* ping-pong queues: O4 (w = path index), D4 (w = flags), T4 (w = tmin) */
    float4* D[2];
    float4* T[2];
    float4* hits;          /* OptiX-style hit record per queue slot */
    float4* shO;           /* connections: origin (w = path index), direction (w = tmax), contribution */
    float4* shD;
    float4* shE;
    float4* pathAcc;       /* per-path radiance (w = primary distance); LH2G_RP_FILTER frames add an indirect half at + P */
    float4* accum;         /* per-pixel accumulator across frames */
    float4* frame;         /* finalized output: accum / samplesTaken */
    Counters* counters;
    float4* nrcRec;        /* LH2G_RP_NRC: per path 6 float4 with stride P: query (4), throughput + state, radiance so far */
    uint4* features;       /* LH2G_RP_FILTER: SVGF features, world position and depth derivatives of sample 0 (W*H) */
    float4* worldPos;
    float4* deltaDepth;
    lh2g_hit* capHits;     /* optional per-(depth, path) capture */
    uint32_t* capSeeds;
    float4* sortO;         /* connections grouped by light (setting "sortConnections"): a second O, D, E set */
    float4* sortD;
    float4* sortE;
    uint32_t* connBins;    /* 64 per-light counts, then their running offsets */
    uint32_t* order = nullptr;   /* shading order of the extension queue: the slots whose ray hit something first,
                                  * those that missed after them (null: queue order) */
    /* the OptiX 7 / PrimeAdaptive estimators */
    const uint32_t* slotLayer = nullptr;   /* adaptive second wave: the sample layer (pathIdx) each slot shades as */
    float4* misFeatures = nullptr;         /* adaptive first wave: albedo + packed normal per sample (variance estimate) */
    const uint32_t* firstCount = nullptr;  /* paths in the first queue when a device count gives it (else F.P) */
};

void launch_generate(const FrameGPU& F, const WaveBuffers& B, cudaStream_t st);
/* primary rays of the OptiX 7 estimator (LH2G_RP_OPTIX7) or of a PrimeAdaptive frame's first wave (LH2G_RP_ADAPTIVE);
 * the other stages choose their estimator by the same flags */
void launch_generate_mis(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, cudaStream_t st);
void launch_extend(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, int depth, int persistentBlocks, cudaStream_t st);
/* with B.order: the partition of the queue into hits and misses (k_partition), then the shading */
void launch_shade(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, int depth, int blocks, cudaStream_t st);
void launch_connect(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, int depth, int persistentBlocks, cudaStream_t st);
/* path lengths startDepth..maxDepth of the frame's remaining paths, one persistent launch */
void launch_tail(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, int startDepth, int persistentBlocks, cudaStream_t st);
/* the extension queue of wave `depth` (>= 2) regrouped by direction octant into sortO/D/E (O, D, T) */
void launch_sort_rays(const WaveBuffers& B, int depth, cudaStream_t st);
/* extension rays grouped by direction octant within chunks of consecutive queue entries, into sortO/D/E */
void launch_sort_rays_local(const WaveBuffers& B, int depth, cudaStream_t st);
/* the connections of wave `depth` regrouped by light into sortO/D/E (counting sort over 64 bins) */
void launch_sort_connections(const WaveBuffers& B, int depth, cudaStream_t st);
/* connections grouped by light within chunks of consecutive queue entries, into sortO/D/E */
void launch_sort_connections_local(const WaveBuffers& B, int depth, cudaStream_t st);
/* per-pixel sums of the frame's paths into the accumulator (from zero when overwrite != 0), then the frame */
void launch_finalize(const FrameGPU& F, const WaveBuffers& B, float scale, int overwrite, cudaStream_t st);
/* radiance-cache frames: gather queries / training samples (counts[0], counts[1]), then add the predictions */
void launch_nrc_collect(const FrameGPU& F, const WaveBuffers& B, float4* queries, uint32_t* qPath, float4* trainQ, float4* trainT, uint32_t* counts,
                        uint32_t trainCap, cudaStream_t st);
void launch_nrc_apply(const FrameGPU& F, const WaveBuffers& B, const float4* pred, const uint32_t* qPath, const uint32_t* counts, cudaStream_t st);
void launch_trace(const SceneGPU& S, const lh2g_ray* rays, void* out, long long n, int mode, uint32_t* fetch, uint32_t* status,
                  int persistentBlocks, cudaStream_t st);

/* scene preparation */
void launch_tri_prep(const float4* verts, uint32_t n, uint32_t seg, float4* triData, float4* lo, float4* hi, uint32_t* segOf, cudaStream_t st);
void launch_gather_tris(const float4* triIn, const uint32_t* leafPrim, uint32_t n, float4* triOut, cudaStream_t st);

/* PrimeAdaptive frames (adaptive.cu): device state between the two waves. devScale carries over to the next frame;
 * hist must be zero before launch_adaptive_estimate. */
struct AdaptiveState {
    float devScale;
    uint32_t requested;   /* samples the pixels asked for */
    uint32_t pathCount;   /* second-wave paths: requested, capped at W*H*spp */
    uint32_t sStar, room; /* the cap keeps requests with S < sStar, and S = sStar for the first `room` pixels asking for it */
    uint32_t hist[25];    /* pixels per requested sample count 0..24 */
};
void launch_adaptive_estimate(const FrameGPU& F, const WaveBuffers& B, float* deviation, uint32_t* want, AdaptiveState* state, cudaStream_t st);
/* per pixel its kept sample count and first second-wave slot (tmp, rank, kept, first: W*H; sums: W*H / 4096 + 1) */
void launch_adaptive_keep(const FrameGPU& F, const uint32_t* want, uint32_t* tmp, uint32_t* rank, uint32_t* kept, uint32_t* first, uint32_t* sums,
                          const AdaptiveState* state, cudaStream_t st);
void launch_adaptive_generate(const SceneGPU& S, const FrameGPU& F, const WaveBuffers& B, const uint32_t* kept, const uint32_t* first,
                              uint32_t* slotLayer, uint32_t R1, cudaStream_t st);
void launch_adaptive_finalize(const FrameGPU& F, const float4* layers, const float4* extra, const uint32_t* kept, const uint32_t* first, float4* accum,
                              float4* frame, float scale, int overwrite, cudaStream_t st);

int persistent_blocks_trace(int mode);
int persistent_blocks_wave(int which);   /* 0 extend, 1 connect, 2 shade, 3 tail */

}  // namespace lh2g

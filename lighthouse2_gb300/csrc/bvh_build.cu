/* bvh_build.cu - device BVH build for the GB300 render core.
 *
 * Replaces the closed acceleration-structure builds of the reference (optixAccelBuild,
 * lib/rendercore_optix7/core_mesh.cpp:67-129 and rendercore.cpp:767-797; rtpModelUpdate,
 * lib/RenderCore_PrimeRef/core_mesh.cpp:63-64). All meshes (segments) are built in one batch:
 *
 *   1. primitive boxes, widened by 2^-20 of the coordinate magnitude (absorbs the rounding of dequantised
 *      planes and of v0 + e1 in the traversal);
 *   2. 64-bit keys (segment << 32 | 30-bit Morton code of the box centre in the segment's bounds);
 *   3. stable LSD radix sort, 8-bit digits, only over the key bits in use;
 *   4. binary tree over Morton-sorted ranges, level by level, one warp per node: the range is cut into
 *      min(32, n) equal chunks and the split with the lowest surface-area cost among the chunk boundaries is
 *      taken (binned SAH over the Morton order; ranges of at most leafMax primitives become leaves);
 *   5. top-down greedy collapse into 8-wide nodes (repeatedly open the interior child of largest area) with
 *      child boxes quantised outward to 8 bits per plane relative to the parent box;
 *   6. leaf primitives stored contiguously per wide node (leafPrim gives the original primitive index).
 */
#include <climits>
#include "bvh_build.cuh"

#include <algorithm>
#include <cfloat>
#include <vector>

namespace lh2g {

namespace {

constexpr int SORT_TILE = 2048;  /* 256 threads x 8 rounds */

__global__ void k_radix_hist(const uint64_t* __restrict__ keys, uint32_t n, int shift, uint32_t* __restrict__ hist, uint32_t tiles) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * SORT_TILE;
    for (int r = 0; r < SORT_TILE / 256; r++) {
        const uint32_t i = base + r * 256 + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * tiles + blockIdx.x] = cnt[threadIdx.x];
}

/* exclusive scan of len counts with a single block of 1024 threads */
__global__ void k_scan_single(uint32_t* __restrict__ data, uint32_t len) {
    __shared__ uint32_t part[1024];
    const uint32_t per = (len + 1023) / 1024;
    const uint32_t b = threadIdx.x * per, e = min(len, b + per);
    uint32_t s = 0;
    for (uint32_t i = b; i < e; i++) s += data[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const uint32_t v = threadIdx.x >= (uint32_t)off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
    for (uint32_t i = b; i < e; i++) { const uint32_t v = data[i]; data[i] = run; run += v; }
}

__global__ void k_radix_scatter(const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
                                uint32_t* __restrict__ vout, uint32_t n, int shift, const uint32_t* __restrict__ hist, uint32_t tiles) {
    __shared__ uint32_t digitBase[256];
    __shared__ uint32_t warpCnt[8][257];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    digitBase[tid] = hist[tid * tiles + blockIdx.x];
    for (int w = 0; w < 8; w++) warpCnt[w][tid] = 0;
    __syncthreads();
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    const uint32_t base = blockIdx.x * SORT_TILE;
    for (int r = 0; r < SORT_TILE / 256; r++) {
        const uint32_t i = base + r * 256 + tid;
        const bool valid = i < n;
        const uint64_t key = valid ? kin[i] : 0ull;
        const uint32_t val = valid ? vin[i] : 0u;
        const uint32_t d = valid ? (uint32_t)((key >> shift) & 255u) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & lanemask_lt);
        if (valid && (__ffs(peers) - 1) == lane) warpCnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = digitBase[tid];
            for (int w = 0; w < 8; w++) { const uint32_t c = warpCnt[w][tid]; warpCnt[w][tid] = run; run += c; }
            digitBase[tid] = run;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = warpCnt[warp][d] + rank;
            kout[pos] = key, vout[pos] = val;
        }
        __syncthreads();
        for (int w = 0; w < 8; w++) warpCnt[w][tid] = 0;
        __syncthreads();
    }
}

__device__ __forceinline__ uint32_t expand_bits10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ int f2ord(float f) { const int i = __float_as_int(f); return i >= 0 ? i : i ^ 0x7fffffff; }
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

/* Segment boxes by atomics on order-preserving integers. Segments are runs of consecutive primitives, so a warp
 * almost always lies in one segment: it then reduces its 32 boxes with shuffles and one lane does the 6 atomics
 * (per-primitive atomics on a few dozen addresses serialise). Min and max do not depend on the order. */
__global__ void k_seg_bounds(const float4* __restrict__ lo, const float4* __restrict__ hi, const uint32_t* __restrict__ seg, uint32_t n,
                             int* __restrict__ segBox /* 6 ints per segment: min xyz, max xyz (ordered ints) */) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;   /* blockDim is a multiple of 32: whole warps */
    const bool ok = i < n;
    const uint32_t s = ok ? seg[i] : 0xffffffffu;
    int v[6] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};
    if (ok) {
        const float4 a = lo[i], b = hi[i];
        v[0] = f2ord(a.x), v[1] = f2ord(a.y), v[2] = f2ord(a.z), v[3] = f2ord(b.x), v[4] = f2ord(b.y), v[5] = f2ord(b.z);
    }
    const uint32_t s0 = __shfl_sync(0xffffffffu, s, 0);
    if (__all_sync(0xffffffffu, s == s0 || s == 0xffffffffu)) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
            for (int k = 0; k < 3; k++) v[k] = min(v[k], __shfl_xor_sync(0xffffffffu, v[k], off));
#pragma unroll
            for (int k = 3; k < 6; k++) v[k] = max(v[k], __shfl_xor_sync(0xffffffffu, v[k], off));
        }
        if ((threadIdx.x & 31u) != 0u || s0 == 0xffffffffu) return;
    } else if (!ok) {
        return;
    }
    atomicMin(&segBox[6 * s + 0], v[0]), atomicMin(&segBox[6 * s + 1], v[1]), atomicMin(&segBox[6 * s + 2], v[2]);
    atomicMax(&segBox[6 * s + 3], v[3]), atomicMax(&segBox[6 * s + 4], v[4]), atomicMax(&segBox[6 * s + 5], v[5]);
}

__global__ void k_morton(const float4* __restrict__ lo, const float4* __restrict__ hi, const uint32_t* __restrict__ seg, uint32_t n,
                         const int* __restrict__ segBox, uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t s = seg[i];
    const float4 a = lo[i], b = hi[i];
    const float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
    uint32_t q[3];
    for (int k = 0; k < 3; k++) {
        const float mn = ord2f(segBox[6 * s + k]), mx = ord2f(segBox[6 * s + 3 + k]);
        const float ext = mx - mn;
        float f = ext > 0.0f ? (c[k] - mn) / ext : 0.5f;
        f = fminf(fmaxf(f, 0.0f), 1.0f);
        q[k] = min(1023u, (uint32_t)(f * 1024.0f));
    }
    const uint32_t m = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
    keys[i] = ((uint64_t)s << 32) | m;
    vals[i] = i;
}

__global__ void k_gather_boxes(const float4* __restrict__ lo, const float4* __restrict__ hi, const uint32_t* __restrict__ order, uint32_t n,
                               float4* __restrict__ slo, float4* __restrict__ shi) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t p = order[i];
    slo[i] = lo[p], shi[i] = hi[p];
}

__device__ __forceinline__ float half_area(float lx, float ly, float lz, float hx, float hy, float hz) {
    const float dx = fmaxf(hx - lx, 0.0f), dy = fmaxf(hy - ly, 0.0f), dz = fmaxf(hz - lz, 0.0f);
    return dx * dy + dy * dz + dz * dx;
}

/* One warp per node of the current level. */
__global__ void k_build_level(const float4* __restrict__ pLo, const float4* __restrict__ pHi, float4* __restrict__ nLo, float4* __restrict__ nHi,
                              int* __restrict__ nLeft, const uint32_t* __restrict__ cur, uint32_t curCount, uint32_t* __restrict__ next,
                              uint32_t* __restrict__ nextCount, uint32_t* __restrict__ nodeCount, int leafMax) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= curCount) return;
    const uint32_t node = cur[warp];
    const uint32_t b = __float_as_uint(nLo[node].w), e = __float_as_uint(nHi[node].w), n = e - b;
    const uint32_t K = min(32u, n);
    float lx = FLT_MAX, ly = FLT_MAX, lz = FLT_MAX, hx = -FLT_MAX, hy = -FLT_MAX, hz = -FLT_MAX;
    uint32_t ce = b;
    if ((uint32_t)lane < K) {
        const uint32_t cb = b + (uint32_t)(((uint64_t)lane * n) / K);
        ce = b + (uint32_t)(((uint64_t)(lane + 1) * n) / K);
        for (uint32_t i = cb; i < ce; i++) {
            const float4 a = __ldg(pLo + i), c = __ldg(pHi + i);
            lx = fminf(lx, a.x), ly = fminf(ly, a.y), lz = fminf(lz, a.z);
            hx = fmaxf(hx, c.x), hy = fmaxf(hy, c.y), hz = fmaxf(hz, c.z);
        }
    }
    float plx = lx, ply = ly, plz = lz, phx = hx, phy = hy, phz = hz;   /* inclusive prefix */
    float slx = lx, sly = ly, slz = lz, shx = hx, shy = hy, shz = hz;   /* inclusive suffix */
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const float a0 = __shfl_up_sync(~0u, plx, off), a1 = __shfl_up_sync(~0u, ply, off), a2 = __shfl_up_sync(~0u, plz, off);
        const float a3 = __shfl_up_sync(~0u, phx, off), a4 = __shfl_up_sync(~0u, phy, off), a5 = __shfl_up_sync(~0u, phz, off);
        if (lane >= off) plx = fminf(plx, a0), ply = fminf(ply, a1), plz = fminf(plz, a2), phx = fmaxf(phx, a3), phy = fmaxf(phy, a4), phz = fmaxf(phz, a5);
        const float b0 = __shfl_down_sync(~0u, slx, off), b1 = __shfl_down_sync(~0u, sly, off), b2 = __shfl_down_sync(~0u, slz, off);
        const float b3 = __shfl_down_sync(~0u, shx, off), b4 = __shfl_down_sync(~0u, shy, off), b5 = __shfl_down_sync(~0u, shz, off);
        if (lane + off < 32) slx = fminf(slx, b0), sly = fminf(sly, b1), slz = fminf(slz, b2), shx = fmaxf(shx, b3), shy = fmaxf(shy, b4), shz = fmaxf(shz, b5);
    }
    const float bx0 = __shfl_sync(~0u, plx, 31), by0 = __shfl_sync(~0u, ply, 31), bz0 = __shfl_sync(~0u, plz, 31);
    const float bx1 = __shfl_sync(~0u, phx, 31), by1 = __shfl_sync(~0u, phy, 31), bz1 = __shfl_sync(~0u, phz, 31);
    if (lane == 0) {
        nLo[node] = make_float4(bx0, by0, bz0, __uint_as_float(b));
        nHi[node] = make_float4(bx1, by1, bz1, __uint_as_float(e));
    }
    if (n <= (uint32_t)leafMax) {
        if (lane == 0) nLeft[node] = -1;
        return;
    }
    const float nlx = __shfl_down_sync(~0u, slx, 1), nly = __shfl_down_sync(~0u, sly, 1), nlz = __shfl_down_sync(~0u, slz, 1);
    const float nhx = __shfl_down_sync(~0u, shx, 1), nhy = __shfl_down_sync(~0u, shy, 1), nhz = __shfl_down_sync(~0u, shz, 1);
    /* candidate splits are the boundaries after chunks 0..K-2; other lanes get +inf, non-finite costs of valid
     * candidates are clamped to FLT_MAX so that the argmin always lands on a valid boundary */
    float cost = __int_as_float(0x7f800000);
    if ((uint32_t)lane + 1 < K) {
        const float nl = (float)(ce - b), nr = (float)(e - ce);
        cost = half_area(plx, ply, plz, phx, phy, phz) * nl + half_area(nlx, nly, nlz, nhx, nhy, nhz) * nr;
        if (!(cost <= FLT_MAX)) cost = FLT_MAX;
    }
    int bj = lane;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float oc = __shfl_xor_sync(~0u, cost, off);
        const int oj = __shfl_xor_sync(~0u, bj, off);
        if (oc < cost || (oc == cost && oj < bj)) cost = oc, bj = oj;
    }
    if (lane == 0) {
        bj = min(bj, (int)K - 2);
        const uint32_t split = b + (uint32_t)(((uint64_t)(bj + 1) * n) / K);
        const uint32_t idx = atomicAdd(nodeCount, 2u);
        nLeft[node] = (int)idx;
        nLo[idx] = make_float4(0, 0, 0, __uint_as_float(b));
        nHi[idx] = make_float4(0, 0, 0, __uint_as_float(split));
        nLo[idx + 1] = make_float4(0, 0, 0, __uint_as_float(split));
        nHi[idx + 1] = make_float4(0, 0, 0, __uint_as_float(e));
        const uint32_t q = atomicAdd(nextCount, 2u);
        next[q] = idx, next[q + 1] = idx + 1;
    }
}

__device__ __forceinline__ uint32_t quant_exp(float ext) {
    /* biased exponent e with 2^(e-127) * 255 >= ext */
    if (!(ext > 0.0f)) return 1u;
    int ex;
    frexp((double)ext / 255.0, &ex);
    ex = max(-126, min(127, ex));
    return (uint32_t)(ex + 127);
}

/* One thread per wide node of the current level. */
__global__ void k_collapse(const float4* __restrict__ nLo, const float4* __restrict__ nHi, const int* __restrict__ nLeft,
                           const uint32_t* __restrict__ sortedPrim, const uint32_t* __restrict__ work, const uint32_t* __restrict__ workWide,
                           uint32_t count, uint4* __restrict__ pool, uint32_t* __restrict__ leafPrim, uint32_t* __restrict__ wideCount,
                           uint32_t* __restrict__ slotCount, uint32_t* __restrict__ nextWork, uint32_t* __restrict__ nextWide,
                           uint32_t* __restrict__ nextCount, uint32_t poolCapacity, uint32_t* __restrict__ error) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint32_t X = work[i], W = workWide[i];
    int ch[8];
    int nc;
    if (nLeft[X] < 0) ch[0] = (int)X, nc = 1;
    else ch[0] = nLeft[X], ch[1] = nLeft[X] + 1, nc = 2;
    while (nc < 8) {
        int best = -1;
        float bestA = -1.0f;
        for (int k = 0; k < nc; k++) {
            const int c = ch[k];
            if (nLeft[c] < 0) continue;
            const float4 a = nLo[c], b = nHi[c];
            const float ar = half_area(a.x, a.y, a.z, b.x, b.y, b.z);
            if (ar > bestA) bestA = ar, best = k;
        }
        if (best < 0) break;
        const int c = ch[best];
        ch[best] = nLeft[c];
        ch[nc++] = nLeft[c] + 1;
    }
    uint32_t nInt = 0, nTri = 0;
    for (int k = 0; k < nc; k++) {
        if (nLeft[ch[k]] >= 0) nInt++;
        else nTri += __float_as_uint(nHi[ch[k]].w) - __float_as_uint(nLo[ch[k]].w);
    }
    const uint32_t childBase = nInt ? atomicAdd(wideCount, nInt) : 0u;
    if (childBase + nInt > poolCapacity || W >= poolCapacity) { atomicOr(error, 1u); return; }
    const uint32_t primBase = nTri ? atomicAdd(slotCount, nTri) : 0u;
    const uint32_t nextPos = nInt ? atomicAdd(nextCount, nInt) : 0u;
    const float4 plo = nLo[X], phi = nHi[X];
    const uint32_t ex = quant_exp(phi.x - plo.x), ey = quant_exp(phi.y - plo.y), ez = quant_exp(phi.z - plo.z);
    const double sx = ldexp(1.0, (int)ex - 127), sy = ldexp(1.0, (int)ey - 127), sz = ldexp(1.0, (int)ez - 127);
    uint32_t meta[2] = {0, 0}, qlx[2] = {0, 0}, qly[2] = {0, 0}, qlz[2] = {0, 0}, qhx[2] = {0, 0}, qhy[2] = {0, 0}, qhz[2] = {0, 0};
    uint32_t imask = 0, intIdx = 0, off = 0;
    for (int k = 0; k < nc; k++) {
        const int c = ch[k];
        const float4 a = nLo[c], b = nHi[c];
        auto qlo = [](double v, double p, double s) { return (uint32_t)max(0.0, min(255.0, floor((v - p) / s))); };
        auto qhi = [](double v, double p, double s) { return (uint32_t)max(0.0, min(255.0, ceil((v - p) / s))); };
        const int w = k >> 2, sh = (k & 3) * 8;
        qlx[w] |= qlo(a.x, plo.x, sx) << sh, qly[w] |= qlo(a.y, plo.y, sy) << sh, qlz[w] |= qlo(a.z, plo.z, sz) << sh;
        qhx[w] |= qhi(b.x, plo.x, sx) << sh, qhy[w] |= qhi(b.y, plo.y, sy) << sh, qhz[w] |= qhi(b.z, plo.z, sz) << sh;
        uint32_t m;
        if (nLeft[c] >= 0) {
            m = 0x80u | intIdx;
            imask |= 1u << k;
            nextWork[nextPos + intIdx] = (uint32_t)c;
            nextWide[nextPos + intIdx] = childBase + intIdx;
            intIdx++;
        } else {
            const uint32_t pb = __float_as_uint(a.w), pe = __float_as_uint(b.w);
            m = ((pe - pb) << 5) | off;
            for (uint32_t j = pb; j < pe; j++) leafPrim[primBase + off + (j - pb)] = sortedPrim[j];
            off += pe - pb;
        }
        meta[w] |= m << sh;
    }
    uint4* np = pool + (size_t)W * 5;
    np[0] = make_uint4(__float_as_uint(plo.x), __float_as_uint(plo.y), __float_as_uint(plo.z), ex | (ey << 8) | (ez << 16) | (imask << 24));
    np[1] = make_uint4(childBase, primBase, meta[0], meta[1]);
    np[2] = make_uint4(qlx[0], qlx[1], qly[0], qly[1]);
    np[3] = make_uint4(qlz[0], qlz[1], qhx[0], qhx[1]);
    np[4] = make_uint4(qhy[0], qhy[1], qhz[0], qhz[1]);
}

template <typename T>
T* alloc(size_t n, std::vector<void*>& owned) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T)) != cudaSuccess) return nullptr;
    owned.push_back(p);
    return (T*)p;
}

}  // namespace

/* Builds BVH8s for nseg segments of primitives (prims of a segment contiguous, segment s = [segStart[s], segStart[s+1])).
 * Wide nodes are written to pool starting at node index poolBase; the root of segment s is poolBase + s (segments
 * with no primitive get no root, rootOut[s] = 0xffffffff). leafPrimOut receives, per leaf slot (slotBase + k), the
 * original primitive index. Returns 0 on success; *nodesUsed / *slotsUsed receive the counts written. */
int build_bvh8(const float4* primLo, const float4* primHi, const uint32_t* primSeg, uint32_t n, const std::vector<uint32_t>& segStart,
               uint4* pool, uint32_t poolBase, uint32_t poolCapacity, uint32_t* leafPrimOut, int leafMax, uint32_t* rootOut,
               uint32_t* nodesUsed, uint32_t* slotsUsed, cudaStream_t st) {
    const uint32_t nseg = (uint32_t)segStart.size() - 1;
    std::vector<void*> owned;
    auto cleanup = [&]() { for (void* p : owned) cudaFree(p); };
    *nodesUsed = nseg, *slotsUsed = 0;
    for (uint32_t s = 0; s < nseg; s++) rootOut[s] = segStart[s + 1] > segStart[s] ? poolBase + s : 0xffffffffu;
    if (n == 0) return 0;
    uint64_t* keys[2] = {alloc<uint64_t>(n, owned), alloc<uint64_t>(n, owned)};
    uint32_t* vals[2] = {alloc<uint32_t>(n, owned), alloc<uint32_t>(n, owned)};
    const uint32_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    uint32_t* hist = alloc<uint32_t>((size_t)256 * tiles, owned);
    int* segBox = alloc<int>((size_t)6 * nseg, owned);
    float4* sLo = alloc<float4>(n, owned);
    float4* sHi = alloc<float4>(n, owned);
    float4* nLo = alloc<float4>(2 * (size_t)n, owned);
    float4* nHi = alloc<float4>(2 * (size_t)n, owned);
    int* nLeft = alloc<int>(2 * (size_t)n, owned);
    uint32_t* lists[2] = {alloc<uint32_t>(2 * (size_t)n, owned), alloc<uint32_t>(2 * (size_t)n, owned)};
    uint32_t* wl[4] = {alloc<uint32_t>(n + nseg, owned), alloc<uint32_t>(n + nseg, owned), alloc<uint32_t>(n + nseg, owned),
                       alloc<uint32_t>(n + nseg, owned)};
    uint32_t* counters = alloc<uint32_t>(8, owned);
    for (void* p : owned) if (!p) { cleanup(); return 3; }
    std::vector<int> initBox(6 * nseg);
    for (uint32_t s = 0; s < nseg; s++)
        for (int k = 0; k < 3; k++) initBox[6 * s + k] = 0x7f7fffff, initBox[6 * s + 3 + k] = (int)(0xff7fffffu ^ 0x7fffffffu);
    cudaMemcpyAsync(segBox, initBox.data(), sizeof(int) * 6 * nseg, cudaMemcpyHostToDevice, st);
    const int B = 256;
    const uint32_t G = (n + B - 1) / B;
    k_seg_bounds<<<G, B, 0, st>>>(primLo, primHi, primSeg, n, segBox);
    k_morton<<<G, B, 0, st>>>(primLo, primHi, primSeg, n, segBox, keys[0], vals[0]);
    int segBits = 0;
    while ((1u << segBits) < nseg) segBits++;
    std::vector<int> shifts = {0, 8, 16, 24};   /* Morton codes use 30 of the low 32 bits */
    for (int sb = 0; sb < segBits; sb += 8) shifts.push_back(32 + sb);
    int cur = 0;
    for (int shift : shifts) {
        k_radix_hist<<<tiles, 256, 0, st>>>(keys[cur], n, shift, hist, tiles);
        k_scan_single<<<1, 1024, 0, st>>>(hist, 256 * tiles);
        k_radix_scatter<<<tiles, 256, 0, st>>>(keys[cur], vals[cur], keys[1 - cur], vals[1 - cur], n, shift, hist, tiles);
        cur = 1 - cur;
    }
    const uint32_t* sorted = vals[cur];
    k_gather_boxes<<<G, B, 0, st>>>(primLo, primHi, sorted, n, sLo, sHi);
    /* level-by-level binary build */
    std::vector<uint32_t> roots;
    std::vector<float4> initLo, initHi;
    for (uint32_t s = 0; s < nseg; s++) {
        if (segStart[s + 1] == segStart[s]) continue;
        const uint32_t idx = (uint32_t)roots.size();
        roots.push_back(idx);
        float4 a, b;
        a.x = a.y = a.z = 0, b.x = b.y = b.z = 0;
        uint32_t bb = segStart[s], ee = segStart[s + 1];
        memcpy(&a.w, &bb, 4), memcpy(&b.w, &ee, 4);
        initLo.push_back(a), initHi.push_back(b);
    }
    const uint32_t nroots = (uint32_t)roots.size();
    cudaMemcpyAsync(nLo, initLo.data(), sizeof(float4) * nroots, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(nHi, initHi.data(), sizeof(float4) * nroots, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(lists[0], roots.data(), sizeof(uint32_t) * nroots, cudaMemcpyHostToDevice, st);
    uint32_t hc[8] = {nroots, 0, 0, 0, 0, 0, 0, 0};   /* [0] node count, [1] next count */
    cudaMemcpyAsync(counters, hc, sizeof(hc), cudaMemcpyHostToDevice, st);
    uint32_t curCount = nroots;
    int li = 0, levels = 0;
    while (curCount > 0) {
        if (++levels > 256) { cleanup(); return 5; }   /* a range halves at least every ~32 levels: never reached */
        cudaMemsetAsync(counters + 1, 0, 4, st);
        const uint32_t threads = curCount * 32;
        k_build_level<<<(threads + 127) / 128, 128, 0, st>>>(sLo, sHi, nLo, nHi, nLeft, lists[li], curCount, lists[1 - li], counters + 1, counters, leafMax);
        cudaMemcpyAsync(&curCount, counters + 1, 4, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) { cleanup(); return 2; }
        li = 1 - li;
    }
    /* collapse, level by level; wide roots are poolBase + segment index */
    std::vector<uint32_t> work, wide;
    {
        uint32_t r = 0;
        for (uint32_t s = 0; s < nseg; s++) if (segStart[s + 1] > segStart[s]) work.push_back(r++), wide.push_back(poolBase + s);
    }
    cudaMemcpyAsync(wl[0], work.data(), 4 * work.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(wl[1], wide.data(), 4 * wide.size(), cudaMemcpyHostToDevice, st);
    uint32_t h2[4] = {poolBase + nseg, 0, 0, 0};   /* wide count, slot count, next count, error */
    cudaMemcpyAsync(counters + 4, h2, sizeof(h2), cudaMemcpyHostToDevice, st);
    curCount = (uint32_t)work.size();
    int wi = 0;
    levels = 0;
    while (curCount > 0) {
        if (++levels > 256) { cleanup(); return 5; }
        cudaMemsetAsync(counters + 6, 0, 4, st);
        k_collapse<<<(curCount + 127) / 128, 128, 0, st>>>(nLo, nHi, nLeft, sorted, wl[2 * wi], wl[2 * wi + 1], curCount, pool, leafPrimOut,
                                                            counters + 4, counters + 5, wl[2 * (1 - wi)], wl[2 * (1 - wi) + 1], counters + 6,
                                                            poolCapacity, counters + 7);
        cudaMemcpyAsync(&curCount, counters + 6, 4, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) { cleanup(); return 2; }
        wi = 1 - wi;
    }
    uint32_t used[4];
    cudaMemcpyAsync(used, counters + 4, 16, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) { cleanup(); return 2; }
    *nodesUsed = used[0] - poolBase, *slotsUsed = used[1];
    cleanup();
    return (used[3] == 0 && used[0] <= poolCapacity) ? 0 : 5;
}

}  // namespace lh2g

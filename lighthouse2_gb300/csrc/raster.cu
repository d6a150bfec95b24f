/* raster.cu - the SoftRasterizer core's kernels (see raster.cuh for the scheme).
 *
 * Arithmetic follows lib/RenderCore_SoftRasterizer/rasterizer.cpp:66-171 operation for operation (compiled with
 * --fmad=false and IEEE division, like the rest of the core), with the conversions the C++ source leaves to the
 * platform fixed as: float -> int truncating and saturating (cvt.rzi.s32.f32), float -> unsigned through a 64-bit
 * truncation keeping the low 32 bits (0 beyond the 64-bit range and for NaN), as x86-64 compilers emit the cast.
 * Two guards the reference lacks: a span whose left end lies at x <= -1 is dropped (the reference would write
 * into the previous row; after clipping against the left plane only a rounding error of more than a pixel could
 * produce one), and a fragment whose 1/z is NaN is dropped (the reference's z-test lets it through and every later
 * fragment after it; 1/z is finite for every finite vertex in front of the near plane). */
#include <climits>

#include "device_math.cuh"
#include "raster.cuh"

namespace lh2g {
namespace {

constexpr int RS_MAXV = 5;           /* a triangle clipped by two planes has at most 5 vertices */
constexpr float RS_SMALL_WORK = 64.0f;    /* rows x columns above which a triangle takes the block path */

LH2G_DEV int rs_f2i(float x) { return __float2int_rz(x); }
LH2G_DEV uint32_t rs_f2u(float x) {
    if (!(x > -9223372036854775808.0f && x < 9223372036854775808.0f)) return 0u;
    return (uint32_t)(unsigned long long)__float2ll_rz(x);
}
/* ScaleColor (rasterizer.cpp:20-25) */
LH2G_DEV uint32_t rs_scale_color(uint32_t c, uint32_t scale) {
    const uint32_t rb = (((c & 0xff00ffu) * scale) >> 8) & 0xff00ffu;
    const uint32_t g = (((c & 0xff00u) * scale) >> 8) & 0xff00u;
    return rb + g;
}
LH2G_DEV unsigned long long rs_key(float z, uint32_t order) { return ((unsigned long long)(~__float_as_uint(z)) << 32) | order; }

struct Poly {
    float x[RS_MAXV], y[RS_MAXV], z[RS_MAXV], u[RS_MAXV], v[RS_MAXV];
    int n;
};

/* one Sutherland-Hodgman stage (rasterizer.cpp:93-105): keeps the part of the polygon where dot(P.xyz, p) - P.w >= 0 */
template <bool UV>
LH2G_DEV void clip(const Poly& in, Poly& out, const float4 P) {
    out.n = 0;
    auto emit = [&](float x, float y, float z, float u, float v) {
#pragma unroll
        for (int k = 0; k < RS_MAXV; k++)
            if (k == out.n) {
                out.x[k] = x, out.y[k] = y, out.z[k] = z;
                if (UV) out.u[k] = u, out.v[k] = v;
            }
        out.n++;
    };
#pragma unroll
    for (int a = 0; a < RS_MAXV - 1; a++) {   /* inputs have at most 4 vertices */
        if (a < in.n) {
            const int bn = a + 1 < RS_MAXV ? a + 1 : 0;
            const bool wrap = a + 1 >= in.n;
            const float Ax = in.x[a], Ay = in.y[a], Az = in.z[a];
            const float Bx = wrap ? in.x[0] : in.x[bn], By = wrap ? in.y[0] : in.y[bn], Bz = wrap ? in.z[0] : in.z[bn];
            float Au = 0.0f, Av = 0.0f, Bu = 0.0f, Bv = 0.0f;
            if (UV) Au = in.u[a], Av = in.v[a], Bu = wrap ? in.u[0] : in.u[bn], Bv = wrap ? in.v[0] : in.v[bn];
            const float t1 = P.x * Ax + P.y * Ay + P.z * Az - P.w, t2 = P.x * Bx + P.y * By + P.z * Bz - P.w;
            if (t1 < 0.0f && t2 >= 0.0f) {
                const float f = t1 / (t1 - t2);
                emit(Ax + f * (Bx - Ax), Ay + f * (By - Ay), Az + f * (Bz - Az), Au + (Bu - Au) * f, Av + (Bv - Av) * f);
                emit(Bx, By, Bz, Bu, Bv);
            } else if (t1 >= 0.0f && t2 >= 0.0f) {
                emit(Bx, By, Bz, Bu, Bv);
            } else if (t1 >= 0.0f && t2 < 0.0f) {
                const float f = t1 / (t1 - t2);
                emit(Ax + f * (Bx - Ax), Ay + f * (By - Ay), Az + f * (Bz - Az), Au + (Bu - Au) * f, Av + (Bv - Av) * f);
            }
        }
    }
}

/* a triangle after culling, clipping and projection: its edges' running values at their first row */
struct Setup {
    int n, miny, maxy;
    int iy0[RS_MAXV], iy1[RS_MAXV];   /* iy0 > iy1: the edge fills no row */
    float x[RS_MAXV], dx[RS_MAXV], z[RS_MAXV], dz[RS_MAXV], u[RS_MAXV], du[RS_MAXV], v[RS_MAXV], dv[RS_MAXV];
    float xmin, xmax;
    uint32_t shade, mat;
};

/* the kept instances' first draw-order indices in shared memory (the first RS_SHARED_INST of them), for the
 * binary search of a triangle's instance; kernels that call setup() fill it first (load_instance_table) */
constexpr int RS_SHARED_INST = 1024;
__shared__ uint32_t instFirst[RS_SHARED_INST];

LH2G_DEV void load_instance_table(const RasterFrame& R) {
    for (int i = threadIdx.x; i < R.nInst && i < RS_SHARED_INST; i += blockDim.x) instFirst[i] = R.inst[i].first;
    __syncthreads();
}
LH2G_DEV uint32_t first_of(const RasterFrame& R, int i) { return i < RS_SHARED_INST ? instFirst[i] : R.inst[i].first; }

LH2G_DEV int find_instance(const RasterFrame& R, uint32_t g) {
    int lo = 0, hi = R.nInst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first_of(R, mid) <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

/* rasterizer.cpp:78-137 for triangle g of the draw order; false when nothing of it reaches a row */
template <bool UV>
LH2G_DEV bool setup(const RasterFrame& R, const uint32_t g, Setup& E) {
    const RasterInst& I = R.inst[find_instance(R, g)];
    const uint32_t t = g - I.first;
    float M[12];
#pragma unroll
    for (int k = 0; k < 12; k++) M[k] = I.M[k];
    const float4* vp = I.verts + 3 * (size_t)t;
    const float4* tp = I.tris + 13 * (size_t)t;
    const float4 p0 = __ldg(vp), p1 = __ldg(vp + 1), p2 = __ldg(vp + 2);
    const float4 nm = __ldg(I.norms + t);
    const float Nx = nm.x, Ny = nm.y, Nz = nm.z;
    /* make_float4(pos, 1) * T and make_float4(N, 0) * T (system.cpp:90-103: the matrix times the column) */
    auto tx = [&](int r, float x, float y, float z, float w) { return M[4 * r] * x + M[4 * r + 1] * y + M[4 * r + 2] * z + M[4 * r + 3] * w; };
    Poly A;
    A.n = 3;
    const float4 ps[3] = {p0, p1, p2};
#pragma unroll
    for (int k = 0; k < 3; k++) A.x[k] = tx(0, ps[k].x, ps[k].y, ps[k].z, 1.0f), A.y[k] = tx(1, ps[k].x, ps[k].y, ps[k].z, 1.0f),
                                A.z[k] = tx(2, ps[k].x, ps[k].y, ps[k].z, 1.0f);
    const float ntx = tx(0, Nx, Ny, Nz, 0.0f), nty = tx(1, Nx, Ny, Nz, 0.0f), ntz = tx(2, Nx, Ny, Nz, 0.0f);
    if (A.x[0] * ntx + A.y[0] * nty + A.z[0] * ntz > 0.0f) return false;
    if (UV) {
        const float4 t0 = __ldg(tp), t1 = __ldg(tp + 1);
        A.u[0] = t0.x, A.u[1] = t0.y, A.u[2] = t0.z, A.v[0] = t1.x, A.v[1] = t1.y, A.v[2] = t1.z;
        E.mat = __float_as_uint(nm.w);
        E.shade = rs_f2u((Nz + 1.0f) * 64.0f + 127.9f);
    }
    Poly B, P;
    clip<UV>(A, B, R.nearPlane);
    clip<UV>(B, P, R.leftPlane);
    if (P.n == 0) return false;
    const float Wf = (float)R.W, hw = (float)(R.W / 2), hh = (float)(R.H / 2), Hf = (float)R.H;
    E.n = P.n;
    E.xmin = 1e30f, E.xmax = -1e30f;
#pragma unroll
    for (int k = 0; k < RS_MAXV; k++)
        if (k < P.n) {
            P.x[k] = ((P.x[k] * Wf) / -P.z[k]) + hw;
            P.y[k] = ((P.y[k] * Wf) / P.z[k]) + hh;
            E.xmin = fminf(E.xmin, P.x[k]), E.xmax = fmaxf(E.xmax, P.x[k]);
        }
    E.miny = R.H - 1, E.maxy = 0;
#pragma unroll
    for (int j = 0; j < RS_MAXV; j++) {
        E.iy0[j] = INT_MAX, E.iy1[j] = INT_MIN;
        if (j >= P.n) continue;
        const int bn = j + 1 < RS_MAXV ? j + 1 : 0;
        const bool wrap = j + 1 >= P.n;
        float xa = P.x[j], ya = P.y[j], za = P.z[j], ua = 0.0f, va = 0.0f;
        float xb = wrap ? P.x[0] : P.x[bn], yb = wrap ? P.y[0] : P.y[bn], zb = wrap ? P.z[0] : P.z[bn], ub = 0.0f, vb = 0.0f;
        if (UV) ua = P.u[j], va = P.v[j], ub = wrap ? P.u[0] : P.u[bn], vb = wrap ? P.v[0] : P.v[bn];
        if (ya > yb) {
            float s;
            s = xa, xa = xb, xb = s;
            s = ya, ya = yb, yb = s;
            s = za, za = zb, zb = s;
            s = ua, ua = ub, ub = s;
            s = va, va = vb, vb = s;
        }
        const float y0 = ya, y1 = yb, rydiff = 1.0f / (y1 - y0);
        if (y0 == y1 || y0 >= Hf || y1 < 1.0f) continue;
        const int iy0 = max(1, rs_f2i(y0) + 1), iy1 = min(R.H - 2, rs_f2i(y1));
        float x0 = xa;
        const float dx = (xb - x0) * rydiff;
        float z0 = 1.0f / za;
        const float z1 = 1.0f / zb, dz = (z1 - z0) * rydiff;
        const float f = (float)iy0 - y0;
        x0 += dx * f;
        if (UV) {
            float u0 = ua * z0;
            const float du = (ub * z1 - u0) * rydiff;
            float v0 = va * z0;
            const float dv = (vb * z1 - v0) * rydiff;
            u0 += du * f, v0 += dv * f;
            E.u[j] = u0, E.du[j] = du, E.v[j] = v0, E.dv[j] = dv;
        }
        z0 += dz * f;
        E.x[j] = x0, E.dx[j] = dx, E.z[j] = z0, E.dz[j] = dz;
        E.iy0[j] = iy0, E.iy1[j] = iy1;
        E.miny = min(E.miny, iy0), E.maxy = max(E.maxy, iy1);
    }
    return E.miny <= E.maxy;
}

/* work estimate of a set-up triangle: rows x columns of its clamped extent */
LH2G_DEV float work_of(const RasterFrame& R, const Setup& E) {
    const float x0 = fmaxf(E.xmin, 1.0f), x1 = fminf(E.xmax, (float)(R.W - 2));
    return (float)(E.maxy - E.miny + 1) * fmaxf(x1 - x0 + 1.0f, 1.0f);
}

/* the texel colour of pass 2 (rasterizer.cpp:162-166) */
struct Shader {
    const uint32_t* src;
    uint32_t diffuse, umask, vmask, shade;
    float tw, th;
    bool pow2;   /* both sizes powers of two: the modulo is a mask */
    __device__ __forceinline__ void init(const RasterFrame& R, const Setup& E) {
        const RasterMat m = R.mats[E.mat];
        diffuse = m.diffuse, shade = E.shade;
        if (m.width) src = R.texels + m.texFirst, umask = m.width, vmask = m.height, tw = (float)m.width, th = (float)m.height;
        else src = nullptr, umask = vmask = 1u, tw = th = 1.0f;
        pow2 = !(umask & (umask - 1u)) && !(vmask & (vmask - 1u));
    }
    /* the texel index of a fragment */
    __device__ __forceinline__ uint32_t texel(float u0, float v0, float z0) const {
        const float z = 1.0f / z0;
        const uint32_t uu = rs_f2u(u0 * z * tw), vv = rs_f2u(v0 * z * th);
        const uint32_t u = pow2 ? uu & (umask - 1u) : uu % umask, v = pow2 ? vv & (vmask - 1u) : vv % vmask;
        return u + v * umask;
    }
    __device__ __forceinline__ uint32_t fetch(uint32_t idx) const { return src ? __ldg(src + idx) : diffuse; }
};

constexpr int RS_BATCH = 8;   /* pass 2 handles a span's pixels in groups: their key and texel loads are independent */

/* one row's span (rasterizer.cpp:140-168): pass 1 offers depth keys, pass 2 writes the colour where its key won */
template <int PASS>
LH2G_DEV uint32_t span(const RasterFrame& R, const int y, const float xl, const float xr, const float ul, const float ur, const float vl,
                       const float vr, const float zl, const float zr, const uint32_t g, const Shader& sh) {
    const float rxdiff = 1.0f / (xr - xl);
    float u0 = ul, v0 = vl, z0 = zl;
    const float du = (ur - u0) * rxdiff, dv = (vr - v0) * rxdiff, dz = (zr - z0) * rxdiff;
    const int ix0 = rs_f2i(xl) + 1, ix1 = min(R.W - 2, rs_f2i(xr));
    if (ix0 < 1) return 0;
    const float f = (float)ix0 - xl;
    if (PASS == 2) u0 += f * du, v0 += f * dv;
    z0 += f * dz;
    uint32_t offered = 0;
    unsigned long long* keys = R.keys + (size_t)y * R.W;
    if (PASS == 1) {
        /* the minimum is all pass 1 needs: a reduction without a returned value does not wait for memory */
        for (int x = ix0; x <= ix1; x++) {
            if (z0 < 0.0f) atomicMin(keys + x, rs_key(z0, g)), offered++;
            z0 += dz;
        }
        return offered;
    }
    uint32_t* out = R.pixels + (size_t)y * R.W;
    for (int xb = ix0; xb <= ix1; xb += RS_BATCH) {
        unsigned long long k[RS_BATCH];
#pragma unroll
        for (int i = 0; i < RS_BATCH; i++) k[i] = xb + i <= ix1 ? __ldg(keys + xb + i) : 0ull;
        uint32_t idx[RS_BATCH];
        bool win[RS_BATCH];
#pragma unroll
        for (int i = 0; i < RS_BATCH; i++) {
            win[i] = false;
            if (xb + i <= ix1) {
                win[i] = z0 < 0.0f && k[i] == rs_key(z0, g);
                idx[i] = win[i] ? sh.texel(u0, v0, z0) : 0u;
                u0 += du, v0 += dv, z0 += dz;
            }
        }
        uint32_t c[RS_BATCH];
#pragma unroll
        for (int i = 0; i < RS_BATCH; i++) c[i] = win[i] ? sh.fetch(idx[i]) : 0u;
#pragma unroll
        for (int i = 0; i < RS_BATCH; i++)
            if (win[i]) out[xb + i] = rs_scale_color(c[i], sh.shade);
    }
    return 0;
}

/* a whole small triangle in one thread: rows in order, each edge advanced on the rows it covers */
template <int PASS>
LH2G_DEV uint32_t rasterize(const RasterFrame& R, Setup& E, const uint32_t g, const Shader& sh) {
    uint32_t offered = 0;
    const float xinit = (float)(R.W - 1);
    for (int y = E.miny; y <= E.maxy; y++) {
        float xl = xinit, xr = 0.0f, ul = 0.0f, ur = 0.0f, vl = 0.0f, vr = 0.0f, zl = 0.0f, zr = 0.0f;
#pragma unroll
        for (int j = 0; j < RS_MAXV; j++) {
            if (y < E.iy0[j] || y > E.iy1[j]) continue;
            const float x = E.x[j];
            if (x < xl) {
                xl = x, zl = E.z[j];
                if (PASS == 2) ul = E.u[j], vl = E.v[j];
            }
            if (x > xr) {
                xr = x, zr = E.z[j];
                if (PASS == 2) ur = E.u[j], vr = E.v[j];
            }
            E.x[j] += E.dx[j], E.z[j] += E.dz[j];
            if (PASS == 2) E.u[j] += E.du[j], E.v[j] += E.dv[j];
        }
        offered += span<PASS>(R, y, xl, xr, ul, ur, vl, vr, zl, zr, g, sh);
    }
    return offered;
}

/* warp-aggregated append of g to a list */
LH2G_DEV void append(uint32_t* list, uint32_t* count, bool take, uint32_t g) {
    const uint32_t m = __ballot_sync(0xffffffffu, take);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (take) list[base + __popc(m & ((1u << lane) - 1u))] = g;
}

constexpr uint32_t RS_NO_OWNER = 0xffffffffu;

/* pass 1: every triangle of the kept instances. A triangle past the one-thread size takes its chunks from the
 * chunk arrays; when they are full it is filled here, in one thread (slower, same result). */
__global__ void __launch_bounds__(128) k_rs_cover(const RasterFrame R) {
    load_instance_table(R);
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    Setup E;
    bool small = false, big = false;
    uint32_t offered = 0, base = 0;
    if (g < R.total && setup<false>(R, g, E)) {
        if (work_of(R, E) > RS_SMALL_WORK) {
            const uint32_t n = (uint32_t)(E.maxy - E.miny) / RS_CHUNK + 1u;
            base = atomicAdd(R.counters + 4, n);
            if (base < R.ckCap && n <= R.ckCap - base) {
                big = true;
                for (uint32_t k = 0; k < n; k++) R.owner[base + k] = make_uint2(g, k);
            } else {
                for (uint32_t k = base; k < R.ckCap && k < base + n; k++) R.owner[k] = make_uint2(RS_NO_OWNER, 0u);
            }
        }
        if (!big) {
            Shader none{};
            offered = rasterize<1>(R, E, g, none);
            small = offered > 0;
        }
    }
    append(R.list, R.counters + 0, small, g);
    {   /* the block-path list, entries (draw order, first chunk) */
        const uint32_t m = __ballot_sync(0xffffffffu, big);
        if (m) {
            const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
            uint32_t b0 = 0;
            if (lane == leader) b0 = atomicAdd(R.counters + 1, (uint32_t)__popc(m));
            b0 = __shfl_sync(0xffffffffu, b0, leader);
            if (big) R.big[b0 + __popc(m & ((1u << lane) - 1u))] = make_uint2(g, base);
        }
    }
    unsigned long long o = offered;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) o += __shfl_down_sync(0xffffffffu, o, s);
    if ((threadIdx.x & 31) == 0 && o) atomicAdd(R.counters + 2, (uint32_t)o);
}

/* pass 2: the small triangles that offered fragments */
__global__ void __launch_bounds__(128) k_rs_color(const RasterFrame R) {
    load_instance_table(R);
    const uint32_t n = R.counters[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t g = R.list[i];
        Setup E;
        if (!setup<true>(R, g, E)) continue;
        if (E.mat >= R.nMats) { atomicOr(R.counters + 3, 1u); continue; }
        Shader sh;
        sh.init(R, E);
        rasterize<2>(R, E, g, sh);
    }
}

/* one row's span by a whole warp (the block path): every lane runs the span's running sums (u0 += du, v0 += dv,
 * z0 += dz, the reference's exact sequence) and lane i keeps the values of pixel i of each group of 32; then each lane
 * handles its pixel. The serial part is a few adds per pixel; the key, texel and store work spreads over the lanes. */
constexpr int RS_SEG = 512;   /* columns of a row one warp fills in the block path */

template <int PASS>
LH2G_DEV uint32_t warp_span(const RasterFrame& R, const int y, const float xl, const float xr, const float ul, const float ur, const float vl,
                            const float vr, const float zl, const float zr, const uint32_t g, const Shader& sh, const int lane, const int seg) {
    const float rxdiff = 1.0f / (xr - xl);
    float u0 = ul, v0 = vl, z0 = zl;
    const float du = (ur - u0) * rxdiff, dv = (vr - v0) * rxdiff, dz = (zr - z0) * rxdiff;
    const int ix0 = rs_f2i(xl) + 1, ix1 = min(R.W - 2, rs_f2i(xr));
    if (ix0 < 1) return 0;
    const float f = (float)ix0 - xl;
    if (PASS == 2) u0 += f * du, v0 += f * dv;
    z0 += f * dz;
    /* this warp's columns: segment seg of the row; the running sums first advance to its first pixel */
    const int xs = max(ix0, 1 + seg * RS_SEG), xe = min(ix1, seg * RS_SEG + RS_SEG);
    if (xs > xe) return 0;
    for (int x = ix0; x < xs; x++) {
        z0 += dz;
        if (PASS == 2) u0 += du, v0 += dv;
    }
    uint32_t offered = 0;
    unsigned long long* keys = R.keys + (size_t)y * R.W;
    uint32_t* out = R.pixels + (size_t)y * R.W;
    for (int xb = xs; xb <= xe; xb += 32) {
        const int cnt = min(32, xe - xb + 1);
        float mu = 0.0f, mv = 0.0f, mz = 0.0f;
        if (cnt == 32) {
#pragma unroll
            for (int i = 0; i < 32; i++) {
                if (lane == i) {
                    mz = z0;
                    if (PASS == 2) mu = u0, mv = v0;
                }
                z0 += dz;
                if (PASS == 2) u0 += du, v0 += dv;
            }
        } else {
            for (int i = 0; i < cnt; i++) {
                if (lane == i) {
                    mz = z0;
                    if (PASS == 2) mu = u0, mv = v0;
                }
                z0 += dz;
                if (PASS == 2) u0 += du, v0 += dv;
            }
        }
        if (lane < cnt && mz < 0.0f) {
            const int x = xb + lane;
            const unsigned long long key = rs_key(mz, g);
            if (PASS == 1) {
                atomicMin(keys + x, key);
                offered++;
            } else if (__ldg(keys + x) == key) {
                out[x] = rs_scale_color(sh.fetch(sh.texel(mu, mv, mz)), sh.shade);
            }
        }
    }
    return offered;
}

/* a warp per block-path triangle: lanes 0..n-1 walk one edge each over its rows and keep its running values at the
 * first row of every chunk the edge continues into (the chunk then starts from them instead of from the edge's
 * first row) */
__global__ void __launch_bounds__(256) k_rs_edges(const RasterFrame R) {
    load_instance_table(R);
    const uint32_t n = R.counters[1];
    const int lane = threadIdx.x & 31;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += (gridDim.x * blockDim.x) >> 5) {
        const uint2 e = R.big[i];
        Setup E;
        if (!setup<true>(R, e.x, E)) continue;
#pragma unroll
        for (int j = 0; j < RS_MAXV; j++) {
            if (lane != j || E.iy0[j] > E.iy1[j]) continue;
            float x = E.x[j], z = E.z[j], u = E.u[j], v = E.v[j];
            const float dx = E.dx[j], dz = E.dz[j], du = E.du[j], dv = E.dv[j];
            const int iy0 = E.iy0[j], iy1 = E.iy1[j];
            /* rows iy0 .. the next chunk start, one step each; then whole chunks of RS_CHUNK steps, storing at each
             * chunk start (the same additions in the same order as row by row) */
            int y = iy0;
            const int first = E.miny + ((iy0 - E.miny) / RS_CHUNK + 1) * RS_CHUNK;
            for (; y < first && y <= iy1; y++) x += dx, z += dz, u += du, v += dv;
            for (; y <= iy1; y += RS_CHUNK) {
                R.ck[(size_t)(e.y + (uint32_t)(y - E.miny) / RS_CHUNK) * RS_MAXV + j] = make_float4(x, z, u, v);
#pragma unroll
                for (int k = 0; k < RS_CHUNK; k++) x += dx, z += dz, u += du, v += dv;
            }
        }
    }
}

/* Triangles past the one-thread size: one block per (triangle, chunk of RS_CHUNK rows, segment of RS_SEG columns).
 * Threads 0..n-1 walk one edge each from its first row to the chunk's end and leave the chunk's values in shared
 * memory; then warp w fills the segment of row w of the chunk (warp_span). */
constexpr int RS_BIG_WARPS = RS_CHUNK;
template <int PASS>
__global__ void __launch_bounds__(32 * RS_BIG_WARPS) k_rs_big(const RasterFrame R, const int segsPerRow) {
    __shared__ float4 rows[RS_MAXV][RS_CHUNK];   /* x, z, u, v of each edge on each row of the chunk */
    __shared__ Setup shared;                     /* the triangle's set-up, by warp 0 */
    __shared__ int valid;
    const uint32_t items = min(R.counters[4], R.ckCap) * (uint32_t)segsPerRow;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t offered = 0;
    load_instance_table(R);
    for (uint32_t item = blockIdx.x; item < items; item += gridDim.x) {
        const uint32_t c = item / (uint32_t)segsPerRow;
        const int seg = (int)(item % (uint32_t)segsPerRow);
        const uint2 own = R.owner[c];
        if (own.x == RS_NO_OWNER) continue;
        const uint32_t g = own.x;
        const int chunk = (int)own.y;
        if (warp == 0) {
            Setup E0;
            const bool ok = setup<PASS == 2>(R, g, E0);
            if (lane == 0) shared = E0, valid = ok;
        }
        __syncthreads();
        const Setup E = shared;
        const bool ok = valid != 0;
        __syncthreads();   /* every thread has its copy before warp 0 writes the next item's */
        if (!ok) continue;
        const int c0 = E.miny + chunk * RS_CHUNK;
        if (c0 > E.maxy) continue;
        const int c1 = min(c0 + RS_CHUNK - 1, E.maxy);
        if (PASS == 2 && E.mat >= R.nMats) {
            if (t == 0 && chunk == 0) atomicOr(R.counters + 3, 1u);
            continue;
        }
#pragma unroll
        for (int j = 0; j < RS_MAXV; j++) {
            if (t != j || E.iy0[j] > c1 || E.iy1[j] < c0) continue;
            /* from the edge's first row, or from its values at the chunk's first row (k_rs_edges) */
            const int start = max(c0, E.iy0[j]);
            float x, z, u = 0.0f, v = 0.0f;
            if (start == E.iy0[j]) {
                x = E.x[j], z = E.z[j];
                if (PASS == 2) u = E.u[j], v = E.v[j];
            } else {
                const float4 k4 = R.ck[(size_t)c * RS_MAXV + j];
                x = k4.x, z = k4.y;
                if (PASS == 2) u = k4.z, v = k4.w;
            }
            const int last = min(E.iy1[j], c1);
            for (int y = start; y <= last; y++) {
                rows[j][y - c0] = make_float4(x, z, u, v);
                x += E.dx[j], z += E.dz[j];
                if (PASS == 2) u += E.du[j], v += E.dv[j];
            }
        }
        __syncthreads();
        Shader sh{};
        if (PASS == 2) sh.init(R, E);
        for (int r = warp; r <= c1 - c0; r += RS_BIG_WARPS) {
            const int y = c0 + r;
            float xl = (float)(R.W - 1), xr = 0.0f, ul = 0.0f, ur = 0.0f, vl = 0.0f, vr = 0.0f, zl = 0.0f, zr = 0.0f;
#pragma unroll
            for (int j = 0; j < RS_MAXV; j++) {
                if (y < E.iy0[j] || y > E.iy1[j]) continue;
                const float4 e = rows[j][r];
                if (e.x < xl) xl = e.x, zl = e.y, ul = e.z, vl = e.w;
                if (e.x > xr) xr = e.x, zr = e.y, ur = e.z, vr = e.w;
            }
            offered += warp_span<PASS>(R, y, xl, xr, ul, ur, vl, vr, zl, zr, g, sh, lane, seg);
        }
        __syncthreads();
    }
    if (PASS == 1) {
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) offered += __shfl_down_sync(0xffffffffu, offered, s);
        if (lane == 0 && offered) atomicAdd(R.counters + 2, offered);
    }
}

__global__ void k_rs_pack(const float4* __restrict__ tris, const uint32_t n, float4* __restrict__ norms) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const float4* r = tris + 13 * (size_t)t;
    norms[t] = make_float4(r[2].w, r[3].w, r[4].w, r[1].w);
}

__global__ void k_rs_depth(const RasterFrame R, float* zbuffer) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)R.W * R.H) return;
    const unsigned long long k = R.keys[i];
    zbuffer[i] = k == ~0ull ? 0.0f : __uint_as_float(~(uint32_t)(k >> 32));
}

}  // namespace

void launch_raster(const RasterFrame& R, int smCount, cudaStream_t st) {
    const int segsPerRow = (R.W - 2 + RS_SEG - 1) / RS_SEG;
    if (R.total) k_rs_cover<<<(R.total + 127) / 128, 128, 0, st>>>(R);
    k_rs_edges<<<smCount * 2, 256, 0, st>>>(R);
    k_rs_big<1><<<smCount * 8, 32 * RS_BIG_WARPS, 0, st>>>(R, segsPerRow);
    k_rs_color<<<smCount * 12, 128, 0, st>>>(R);
    k_rs_big<2><<<smCount * 8, 32 * RS_BIG_WARPS, 0, st>>>(R, segsPerRow);
}

void launch_raster_pack(const float4* tris, uint32_t n, float4* norms, cudaStream_t st) {
    if (n) k_rs_pack<<<(n + 255) / 256, 256, 0, st>>>(tris, n, norms);
}

void launch_raster_depth(const RasterFrame& R, float* zbuffer, cudaStream_t st) {
    const size_t n = (size_t)R.W * R.H;
    k_rs_depth<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(R, zbuffer);
}

}  // namespace lh2g

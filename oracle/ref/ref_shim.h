/* ref_shim.h - host-compilation shim for the reference's own device headers (TEST INFRASTRUCTURE ONLY).
 *
 * Lets g++ compile, by path from the reference tree, the PrimeRef path-tracer kernels
 * (lib/RenderCore_PrimeRef/kernels/{camera,pathtracer,connections}.h) together with the shared device code
 * (lib/CUDA/shared_kernel_code/{tools,sampling,material,lights}_shared.h) and lib/sharedBSDFs/lambert.h.
 * It supplies what nvcc would: the device-only intrinsics, the kernel globals of
 * lib/RenderCore_PrimeRef/kernels/.cuda.cu:22-43, and the parts of lib/RenderCore_PrimeRef/core_settings.h that
 * device code reads (that header pulls in OptiX Prime and OpenGL on the host).
 * The CUDA transcendental intrinsics the kernels call (__sincosf, __expf, sincosf, expf, log2f) are routed to the
 * oracle's own implementations, the same functions the GPU core uses, so the comparison isolates the
 * restatement of the algorithm from libm differences. */
#pragma once
#include <cstdint>
#include <cstring>
#include <cmath>
#include <cuda_runtime.h>   /* vector types only: no CUDA runtime call is made */
#include <immintrin.h>      /* the host aabb of common_types.h is SSE-based; this harness only builds on x86 */

extern "C" {
void lh2o_sincos(float x, float* s, float* c);
float lh2o_expf(float x);
float lh2o_log2f(float x);
float lh2o_half2float(uint16_t h);
}

typedef unsigned int uint;
typedef unsigned char uchar;
#define CUDABUILD
#define LH2_DEVFUNC static inline
#undef __global__
#define __global__
#define NEXTMULTIPLEOF(a, b) (((a) + ((b)-1)) & (0x7fffffff - ((b)-1)))
#define __launch_bounds__(a, b)
#define REFERENCE_OF(x) x&

/* CUDA's float and unsigned overloads of min/max (device code calls them on floats; on the host only the
 * int versions of helper_math.h would be found and would truncate). */
inline float max(float a, float b) { return fmaxf(a, b); }
inline float min(float a, float b) { return fminf(a, b); }
inline unsigned int max(unsigned int a, unsigned int b) { return a > b ? a : b; }
inline unsigned int min(unsigned int a, unsigned int b) { return a < b ? a : b; }
inline float __uint_as_float(uint u) { float f; memcpy(&f, &u, 4); return f; }
inline uint __float_as_uint(float f) { uint u; memcpy(&u, &f, 4); return u; }
inline float __int_as_float(int u) { float f; memcpy(&f, &u, 4); return f; }
inline int __float_as_int(float f) { int u; memcpy(&u, &f, 4); return u; }
inline unsigned short __ushort_as_half(unsigned int x) { return (unsigned short)x; }
inline ushort2 __halves2half2(unsigned short a, unsigned short b) { ushort2 r; r.x = a, r.y = b; return r; }
inline float2 __half22float2(ushort2 h) { float2 r; r.x = lh2o_half2float(h.x), r.y = lh2o_half2float(h.y); return r; }
inline void __sincosf(float a, float* s, float* c) { lh2o_sincos(a, s, c); }
inline float __expf(float x) { return lh2o_expf(x); }
#define sincosf(a, s, c) lh2o_sincos(a, s, c)
#define expf(x) lh2o_expf(x)
#define log2f(x) lh2o_log2f(x)
/* float -> unsigned conversion with the GPU's semantics (cvt.rzi.u32.f32: truncation, saturation at the range
 * ends, NaN -> 0). The Makefile rewrites the float casts "(uint)(...)" of tools_shared.h to it. */
inline uint REF_F2U(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xffffffffu;
    return (uint)x;
}
/* single-threaded host execution: atomics are plain read-modify-writes */
inline uint atomicAdd(uint* p, uint v) { const uint o = *p; *p = o + v; return o; }
struct ref_dim3 { uint x, y, z; };
extern ref_dim3 threadIdx, blockIdx, blockDim;

/* lh2g_types.h - wire formats of the GB300 wavefront render core.
 *
 * Plain C structs shared by the C-ABI (lh2g.h), the CUDA kernels and the CPU oracle.
 * Every struct here is laid out byte-for-byte like the Lighthouse 2 type it stands for, so that
 * arrays built by the Lighthouse 2 RenderSystem can be handed over without conversion:
 *
 *   lh2g_core_tri      <-> CoreTri            lib/RenderSystem/common_classes.h:57-97   (208 B)
 *   lh2g_light_tri     <-> CoreLightTri       lib/RenderSystem/common_classes.h:365-385 (96 B)
 *   lh2g_point_light   <-> CorePointLight     lib/RenderSystem/common_classes.h:392-404 (32 B)
 *   lh2g_spot_light    <-> CoreSpotLight      lib/RenderSystem/common_classes.h:411-426 (48 B)
 *   lh2g_dir_light     <-> CoreDirectionalLight lib/RenderSystem/common_classes.h:433-445 (32 B)
 *   lh2g_view          <-> ViewPyramid        lib/RenderSystem/common_classes.h:452-475 (68 B)
 *   lh2g_texture       <-> CoreTexDesc (host) lib/RenderSystem/common_classes.h:336-359 (40 B)
 *   lh2g_ray           <-> Ray (OptiX Prime ORIGIN_TMIN_DIRECTION_TMAX)
 *                                             lib/RenderCore_PrimeRef/core_settings.h:151 (32 B)
 *   lh2g_hit           <-> hit float4 {u|v<<16, inst, prim, t}
 *                                             lib/rendercore_optix7/optix/.optix.cu:180-183 (16 B)
 *   lh2g_gpu_material  <-> CUDAMaterial       lib/rendercore_optix7/core_settings.h:136-185 (128 B)
 */
#ifndef LH2G_TYPES_H
#define LH2G_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One triangle with all shading attributes (CoreTri). Vertex positions are in object space. */
typedef struct lh2g_core_tri {
    float u0, u1, u2; int32_t ltriIdx;      /* texture u per vertex; light index for emissive tris */
    float v0, v1, v2; uint32_t material;    /* texture v per vertex; material index */
    float vN0[3]; float Nx;                 /* vertex normal 0; face normal x */
    float vN1[3]; float Ny;
    float vN2[3]; float Nz;
    float T[3]; float area;                 /* tangent; area */
    float B[3]; float invArea;              /* bitangent */
    float alpha[3]; float LOD;              /* consistent-normal alphas; texture LOD bias */
    float vertex0[3]; float dummy0;
    float vertex1[3]; float dummy1;
    float vertex2[3]; float dummy2;
    float u1_0, u1_1, u1_2; float dummy3;   /* second uv layer */
    float v1_0, v1_1, v1_2; float dummy4;
} lh2g_core_tri;

typedef struct lh2g_light_tri {
    float centre[3]; float energy;
    float N[3]; float area;
    float radiance[3]; int32_t dummy2;
    float vertex0[3]; int32_t triIdx;
    float vertex1[3]; int32_t instIdx;
    float vertex2[3]; int32_t dummy1;
} lh2g_light_tri;

typedef struct lh2g_point_light {
    float position[3]; float energy;
    float radiance[3]; int32_t dummy;
} lh2g_point_light;

typedef struct lh2g_spot_light {
    float position[3]; float cosInner;
    float radiance[3]; float cosOuter;
    float direction[3]; int32_t dummy;
} lh2g_spot_light;

typedef struct lh2g_dir_light {
    float direction[3]; float energy;
    float radiance[3]; int32_t dummy;
} lh2g_dir_light;

/* Camera: eye position and three corners of the screen plane (p1 top-left, p2 top-right, p3 bottom-left). */
typedef struct lh2g_view {
    float pos[3], p1[3], p2[3], p3[3];
    float aperture, spreadAngle, imagePlane, focalDistance, distortion;
} lh2g_view;

/* Texture descriptor (host layout of CoreTexDesc). texels points at pixelCount ARGB32 words holding every
 * MIP level back to back; firstPixel is filled in by the core. */
typedef struct lh2g_texture {
    const uint32_t* texels;
    uint32_t width, height, flags, pixelCount, firstPixel, MIPlevels;
    int32_t storage;                        /* 0 = ARGB32 (the only storage this core reads) */
} lh2g_texture;

/* Ray query formats. */
typedef struct lh2g_ray { float ox, oy, oz, tmin, dx, dy, dz, tmax; } lh2g_ray;
typedef struct lh2g_hit { uint32_t bary; int32_t inst; int32_t prim; float t; } lh2g_hit;

/* Host-side material description: the value fields of CoreMaterial (common_classes.h:219-328) that the
 * Lambert shading path reads, plus the texture slots it samples. Textures are indices into the array given
 * to lh2g_set_textures (-1 = none). */
typedef struct lh2g_map_ref { int32_t texture; float uvscale[2]; float uvoffset[2]; } lh2g_map_ref;
typedef struct lh2g_material {
    float color[3];                         /* base colour; any channel > 1 marks an emitter */
    float absorption[3];                    /* transmittance = 1 - absorption */
    float metallic, subsurface, specular, roughness;
    float specularTint, anisotropic, sheen, sheenTint;
    float clearcoat, clearcoatGloss, transmission, eta;
    uint32_t flags;                         /* 1 = smooth normals, 2 = alpha tested */
    lh2g_map_ref color_map, detail_color_map, normal_map, detail_normal_map, specular_map, roughness_map;
} lh2g_material;

/* Packed device material (128 bytes): half diffuse rgb + half transmittance rgb + flags, 16 8-bit
 * parameters (eta as float bits in the last word), six 16-byte texture maps
 * {short w, h; half uscale, vscale, uoffs, voffs; uint addr}. */
typedef struct lh2g_gpu_material { uint32_t base[4]; uint32_t params[4]; uint32_t maps[6][4]; } lh2g_gpu_material;

/* Material flag bits (core_settings.h:160-171 of the OptiX7 core). */
#define LH2G_MAT_ISDIELECTRIC     (1u << 0)
#define LH2G_MAT_DIFFUSEMAPISHDR  (1u << 1)
#define LH2G_MAT_HASDIFFUSEMAP    (1u << 2)
#define LH2G_MAT_HASNORMALMAP     (1u << 3)
#define LH2G_MAT_HASSPECULARITYMAP (1u << 4)
#define LH2G_MAT_HASROUGHNESSMAP  (1u << 5)
#define LH2G_MAT_HAS2NDNORMALMAP  (1u << 7)
#define LH2G_MAT_HAS2NDDIFFUSEMAP (1u << 9)
#define LH2G_MAT_HASSMOOTHNORMALS (1u << 11)
#define LH2G_MAT_HASALPHA         (1u << 12)

/* Per-frame estimator parameters. The defaults reproduce the PrimeRef reference path tracer
 * (lib/RenderCore_PrimeRef/kernels/pathtracer.h:45-168): uniform xorshift numbers, NEE without MIS,
 * Russian roulette from the first bounce. */
typedef struct lh2g_render_params {
    int32_t width, height, spp;
    int32_t maxDepth;                       /* MAXPATHLENGTH: paths stop after this many segments */
    int32_t rrStartDepth;                   /* Russian roulette applies from this path length on (1 = always) */
    int32_t samplesTaken;                   /* samples already accumulated (the 'pass' of the reference) */
    uint32_t cameraR0;                      /* R0 of the primary-ray kernel (RandomUInt(camRNGseed)) */
    float geometryEpsilon;                  /* ray offset / tmin, 'epsilon' setting (rendersystem.h:67) */
    float clampValue;                       /* 'clampValue' setting (kept for the settings interface) */
    int32_t flags;                          /* LH2G_RP_* */
    uint32_t frameSeed;                     /* LH2G_RP_FILTER: shading R0 = frameSeed + pathLength * 91771;
                                             * adaptive frames: R0 of the second wave's primary rays */
    uint32_t shift;                         /* LH2G_RP_OPTIX7 / adaptive frames: blue-noise tile shift (shiftSeed) */
    /* A band of the frame (rowCount > 0): only pixel rows [rowBegin, rowBegin + rowCount) of the width x height
     * frame are rendered, each path with the seeds it has in the whole frame, so the bands of one frame rendered
     * apart (one per GPU) and put together equal the frame bit for bit. The target is the band (width x rowCount x
     * spp); the accumulator holds the band's rows. PrimeRef estimator only. rowCount 0: the whole frame. */
    int32_t rowBegin, rowCount;
} lh2g_render_params;

#define LH2G_RP_NEE        1                /* next-event estimation (connections buffer present) */
#define LH2G_RP_DEPTH_W    2                /* add the primary hit distance to accumulator.w (DOF data) */
/* Filter-core frame (lib/RenderCore_Optix7Filter): primary rays through the pixel corner of the (jittered)
 * view without lens sampling (optix/.optix.cu:66-100), SVGF features of sample 0 written while shading
 * (kernels/pathtracer.h:44-57,95-232), radiance split into a direct half (accumulator[0, W*H)) and an
 * indirect half (accumulator[W*H, 2*W*H)) at the first diffuse bounce, and a per-frame shading seed
 * (rendercore.cpp:834: RandomUInt(camRNGseed) + pathLength * 91771). */
#define LH2G_RP_FILTER     4
/* Radiance-cache frame (lh2g_render_nrc): a path that reaches its second vertex through a diffuse bounce records
 * a cache query there; 15 of 16 such paths end and receive throughput x cache, the others trace on and train it. */
#define LH2G_RP_NRC        8
/* The OptiX 7 core's estimator (lib/rendercore_optix7/kernels/pathtracer.h:54-238 with the ray generation of
 * optix/.optix.cu:85-129): primary rays seeded WangHash(pathIdx * 16789 + pass * 1791) through RayTarget, blue-noise
 * samples (blueNoiseSampler4, tools_shared.h:324-337) for sample indices below 64 when tables are set
 * (lh2g_set_blue_noise), MIS weights on emissive hits and on light connections (lights_shared.h:111-190), path
 * regularisation after the first diffuse bounce, paths capped at their second diffuse vertex, intensity clamp
 * ('clampValue'), NaN suppression, the small sky after a bounce, connections traced with tmin = epsilon and counted
 * in accumulator.w. cameraR0 is the frame's first draw of RandomUInt(camRNGseed): wave d shades with the d-th draw
 * + d * 91771 (rendercore.cpp:900). Radiance per path: the terminal sky or emitter term, then the connections. */
#define LH2G_RP_OPTIX7     16
/* Set by lh2g_render_adaptive (not by callers): the PrimeAdaptive core's shading (the OptiX 7 estimator with
 * per-sample accumulators, a sample count in w and albedo/normal features for the variance estimate). */
#define LH2G_RP_ADAPTIVE   32
/* With LH2G_RP_OPTIX7 or LH2G_RP_ADAPTIVE: the Disney principled BSDF (lib/sharedBSDFs/disney.h with ggxmdf.h and
 * frosted.h, the default branch of those cores' kernels/bsdf.h) instead of lambert.h; light connections then take
 * the BSDF value without lambert.h's ROUGHNESS factor (BSDF_HAS_PURE_SPECULARS is lambert.h's), and the sampler
 * uses the third random number that lambert.h draws and ignores. */
#define LH2G_RP_DISNEY     64
/* With LH2G_RP_OPTIX7: stochastic-lightcuts light selection through the binary light tree that lh2g_set_lights builds
 * (lights_shared.h:120-156 CalculateChildNodeWeights, :198-217 LightPickProbLTree, :322-395 RandomPointOnLightLTree;
 * the calls the OptiX 7 shading kernel has commented out beside its potential-based ones, pathtracer.h:145,187, with
 * LIGHTTREE defined). Each tree level draws six numbers from the path's shading seed. Directional lights are not in
 * the tree. Scenes of more than 64 lights render only with it. */
#define LH2G_RP_LIGHTTREE  128

/* Bits of the device status word (lh2g_core_stats.deviceStatus, lh2g_render_noalloc's statusHost, the serving
 * loop's stats): the frame they come with is incomplete. */
#define LH2G_STATUS_STACK_OVERFLOW 1u    /* a traversal stack was full: entries were dropped */
#define LH2G_STATUS_TRAVERSAL_LIMIT 2u   /* a traversal exceeded its step limit (a malformed tree) */
#define LH2G_STATUS_QUEUE_OVERFLOW 4u    /* serving loop: new paths would not have fit the queue (skipped) */
#define LH2G_STATUS_COPY_TIMEOUT 8u      /* a staged copy of path state did not complete within its bound (batch skipped) */

/* One SVGF pass over the accumulator of a LH2G_RP_FILTER frame (lib/RenderCore_Optix7Filter/rendercore.cpp:
 * 897-935 with the kernels of lib/CUDA/shared_kernel_code/finalize_shared.h:169-600). */
typedef struct lh2g_filter_params {
    lh2g_view prevView;                     /* unjittered view of the previous frame (reprojection) */
    float j0, j1;                           /* subpixel jitter of this frame, in pixels */
    float prevj0, prevj1;                   /* jitter of the previous filtered frame */
    float clampDirect, clampIndirect;       /* demodulated-light clamps ('clampDirect' 2.5, 'clampIndirect' 15) */
    int32_t samplesTaken;                   /* samples in the accumulator, this frame included (scale = 1 / this) */
    int32_t camIsStationary;                /* 1 while converging: specular pixels keep their own position */
    int32_t taa;                            /* 1: TAA + unsharpen (TAApassKernel, unsharpenTAAKernel); 0: finalizeNoTAA */
} lh2g_filter_params;

/* Filter buffer slots (lh2g_read_filter_buffer), named by their role at the time of the call: after
 * lh2g_filter the history buffers have been swapped, so PREV_* hold this frame's data. */
#define LH2G_FB_FEATURES       0            /* uint4: albedo 10:11:11, normal 10:10:10 + specular bits, depth, w = history | spec << 4 | mat << 6 */
#define LH2G_FB_WORLDPOS       1            /* float4: first diffuse vertex, w = packed normal */
#define LH2G_FB_PREV_WORLDPOS  2
#define LH2G_FB_DELTADEPTH     3            /* float4: z, w = depth derivatives in x and y */
#define LH2G_FB_MOTION         4            /* float2: position in the previous frame (+0.5) */
#define LH2G_FB_MOMENTS        5            /* float4: luminance moments direct (x, y) and indirect (z, w) */
#define LH2G_FB_PREV_MOMENTS   6
#define LH2G_FB_SHADING        7            /* float4: 5:11 packed direct + indirect light; after filtering the gamma image */
#define LH2G_FB_FILTERED_IN    8            /* float4: packed light, history of the temporal blend */
#define LH2G_FB_FILTERED_OUT   9
#define LH2G_FB_PREV_PIXELS    10           /* float4: the previous frame's image (TAA history) */
#define LH2G_FB_ACCUM          11           /* float4 x 2*W*H: direct and indirect accumulators */
#define LH2G_FB_COUNT          12

/* Per-path, per-depth capture used by the parity tests: the hit record each path saw at each depth and
 * its RNG state after shading. Entries of paths that were no longer alive carry prim = -2. */
typedef struct lh2g_capture { lh2g_hit* hits; uint32_t* seeds; } lh2g_capture;

#ifdef __cplusplus
}
#endif
#endif /* LH2G_TYPES_H */

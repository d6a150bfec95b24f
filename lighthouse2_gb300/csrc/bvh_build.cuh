/* bvh_build.cuh - device BVH8 builder (see bvh_build.cu). */
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

namespace lh2g {
int build_bvh8(const float4* primLo, const float4* primHi, const uint32_t* primSeg, uint32_t n, const std::vector<uint32_t>& segStart,
               uint4* pool, uint32_t poolBase, uint32_t poolCapacity, uint32_t* leafPrimOut, int leafMax, uint32_t* rootOut,
               uint32_t* nodesUsed, uint32_t* slotsUsed, cudaStream_t st);
}

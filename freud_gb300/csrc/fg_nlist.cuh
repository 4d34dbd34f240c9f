// Launch interface of the NeighborList construction helpers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fg_common.cuh"

namespace fg {
void launch_from_arrays(const uint32_t* qi, const uint32_t* pi, const float* vec, uint64_t nb, uint2* ij, float* dist,
                        cudaStream_t s);
void launch_all_pairs(const DevBox& b, const float* pts, uint32_t np, const float* qpts, uint32_t nq, int exclude_ii,
                      uint64_t nb, uint2* ij, float* dist, float* vec, cudaStream_t s);
void launch_keep_r(const float* dist, uint64_t nb, float r_max, float r_min, uint32_t* keep, cudaStream_t s);
void launch_keep_u8(const uint8_t* in, uint64_t nb, uint32_t* keep, cudaStream_t s);
void launch_compact(const uint32_t* keep, const uint64_t* pos, uint64_t nb, const uint2* ij, const float* dist,
                    const float* w, const float* vec, uint2* ij2, float* dist2, float* w2, float* vec2, cudaStream_t s);
void launch_first_index(const uint2* ij, uint64_t nb, uint32_t i, uint64_t* out, cudaStream_t s);
} // namespace fg

// noalloc_kernels.h -- the pheromone step on caller-owned device buffers
// with a fixed file-scope scratch (faco_noalloc.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace faco {

// Largest instance the fixed scratch holds: 65,535 nodes (the engine's node
// limit; 16-bit node ids), i.e. 256 KiB of packed neighbours + an 8 KiB
// permutation bitmap per device.
constexpr std::uint32_t kNoAllocMaxNodes = 65535;

// Problems found on the device (bits of the error word read back).
constexpr std::uint32_t kNoAllocParentRange = 1;   // a parent entry >= n
constexpr std::uint32_t kNoAllocParentRepeat = 2;  // the parent repeats a node
constexpr std::uint32_t kNoAllocPrimaryRange = 4;  // a candidate id >= n

// Enqueues the step on `stream` and waits for it; *error_bits receives the
// device-side checks (0: trails and products were updated; otherwise neither
// was touched).  The caller checks n <= kNoAllocMaxNodes and k >= 1.
cudaError_t pheromone_step_noalloc(std::uint32_t n, std::uint32_t k, const std::uint32_t* primary,
                                   const std::uint32_t* parent, float retention, float minimum, float maximum,
                                   float increment, const float* eta, float* trails, float* products,
                                   cudaStream_t stream, std::uint32_t* error_bits);

}  // namespace faco

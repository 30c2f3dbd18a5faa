// prior_mlp.cuh -- the learned edge prior: an 8 -> 64 -> 64 -> 1 MLP scored
// per candidate edge (8 features), BF16 operands with FP32 accumulation on
// the tcgen05 tensor cores (prior_mlp_tc.cuh), forward and backward.
//
// The reference has no learned prior (its only prior is an external LKH
// candidate export, python/gp_faco/candidate_prior.py:20-36); this is the
// engine's own component.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

namespace faco {

constexpr int kMlpIn = 8;       // feature slots per edge
constexpr int kMlpFeatures = 8;
constexpr int kMlpHidden = 64;

// FP32 master parameters (4,673 used values) and their BF16 operand copies.
struct MlpParams {
    float w1[kMlpHidden * kMlpIn];      // [out][in]
    float b1[kMlpHidden];
    float w2[kMlpHidden * kMlpHidden];  // [out][in]
    float b2[kMlpHidden];
    float w3[kMlpHidden];
    float b3;
    float pad[3];
};

struct MlpOperands {
    __nv_bfloat16 w1[kMlpHidden * kMlpIn];          // [out][in]
    __nv_bfloat16 w2[kMlpHidden * kMlpHidden];      // [out][in]
};

constexpr int kMlpParamCount = sizeof(MlpParams) / sizeof(float);

__device__ __forceinline__ std::uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const std::uint32_t*>(&v);
}

}  // namespace faco

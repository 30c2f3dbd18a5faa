// prior_kernels.h -- kernels of the learned edge prior.
#pragma once

#include <cstdint>

#include "faco_common.cuh"
#include "prior_mlp.cuh"
#include "prior_mlp_tc.cuh"

namespace faco {

// tcgen05 kernels (prior_mlp_tc.cuh), 128 threads: the forward pass with
// tc::kLaunchSmemBytes of dynamic shared memory (at most tc::kCtasPerSm CTAs
// per SM), the gradient with tc::kGradSmemBytes (tc::kGradCtasPerSm).
__global__ void mlp_forward_kernel(const MlpParams* P, const MlpOperands* O, const __nv_bfloat16* x, std::uint32_t E,
                                   float* prob, unsigned* error);
__global__ void mlp_grad_kernel(const MlpParams* P, const MlpOperands* O, const __nv_bfloat16* x, const float* y,
                                std::uint32_t E, float inv_count, MlpParams* partials, float* loss_partials,
                                unsigned* error);
__global__ void mlp_grad_reduce_kernel(const MlpParams* partials, const float* loss_partials, std::uint32_t blocks,
                                       MlpParams* grad, float* loss);
__global__ void adam_kernel(MlpParams* P, const MlpParams* grad, MlpParams* m, MlpParams* v, float lr, float beta1,
                            float beta2, float eps, float bias1, float bias2);
__global__ void refresh_operands_kernel(const MlpParams* P, MlpOperands* O);
__global__ void edge_features_kernel(const InstanceView* instances, const ColonyView* colonies,
                                     const ColonyState* states, std::uint32_t first, const std::uint64_t* row_offset,
                                     __nv_bfloat16* x_out, float* y_out);
__global__ void global_neighbours_kernel(const ColonyView* colonies, std::uint32_t* gnbr_all,
                                         const std::uint32_t* node_offset);
__global__ void prior_apply_kernel(const InstanceView* instances, const ColonyView* colonies,
                                   const ColonyState* states, const std::uint8_t* enabled, const MlpParams* P,
                                   const MlpOperands* O, float floor, int gamma, const std::uint32_t* gnbr_all,
                                   const std::uint32_t* node_offset, unsigned* error);

}  // namespace faco

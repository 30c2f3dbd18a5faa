// faco_kernels.h -- kernel declarations shared by faco_kernels.cu and the
// host engine.
#pragma once

#include <cstdint>

#include "faco_ant.cuh"
#include "faco_control.cuh"

namespace faco {

// Ants (warps) per block of the ant kernel, and the resident blocks per SM the
// register budget is sized for (6 x 4 warps x 85 registers fills the file;
// the variants use 72-80 registers without spills, where 8 blocks per SM
// forced 64 registers and spills, and ran slower on every workload).
constexpr std::uint32_t kMaxWarpsPerBlock = 4;
constexpr std::uint32_t kAntBlocksPerSM = 6;

struct ColonyParams {
    std::uint32_t ants;
    std::uint32_t mne_target;
    double retention;
    float retention_f;
    double p_root;                   // p_best^(1/k), computed once on the host
    double epoch_source_probability;
    std::uint32_t controlled;        // GP controllers choose MNE, start region and restarts
    std::uint32_t total_iterations;  // T of the evaluation (iteration-fraction feature)
    float log2k;                     // log2(k) by the engine's own log2
    std::uint32_t ref_control;       // 1: the 12-feature controller (feature spec 2)
    std::uint32_t zero_fingerprints; // diagnostic: every tour fingerprint 0 (forced collisions)
    unsigned long long ls_limit;     // LS evaluation budget per ant (LS-work feedback)
    DecisionCapture capture;         // decisions to record (count 0: none)
    const std::uint32_t* prior_rows; // per colony: 1 = the prior re-ranks departures only (device; may be null)
    std::uint32_t trail_blocks;      // > 1: colony_trails_kernel updates the trails with this many blocks per
                                     // colony, after the colony update (uncontrolled evaluations only)
};

// Candidate rows of registration on the GPU (faco_knn.cu): per node its
// `needed` nearest nodes in (EUC_2D length, id) order, ids and lengths
// [n][needed]; needed <= kKnnMaxNeeded and < n, shared memory 8 n bytes.
constexpr std::uint32_t kKnnMaxNeeded = 256;
std::uint32_t knn_smem_bytes(std::uint32_t n);
cudaError_t launch_knn(const int2* xy, std::uint32_t n, std::uint32_t needed, node_t* near_ids,
                       std::int32_t* near_dist, cudaStream_t stream);

// Host-side launchers (the kernels are defined in faco_kernels.cu).
cudaError_t prepare_ant_kernel(int mode, std::uint32_t smem_bytes);
cudaError_t launch_ant_kernel(int mode, const AntLaunch& L, std::uint32_t blocks, std::uint32_t warps,
                              std::uint32_t smem_bytes, cudaStream_t stream);

__global__ void colony_init_kernel(const InstanceView* instances, const ColonyView* colonies, ColonyState* states,
                                   ColonyParams P, std::uint32_t colony_count);
__global__ void prior_rows_kernel(const InstanceView* instances, const ColonyView* colonies,
                                  const std::uint32_t* modes);
__global__ void fingerprint_kernel(const ColonyView* colonies, const std::uint32_t* list, std::uint32_t ants,
                                   std::uint32_t colony_count, std::uint32_t zero);
__global__ void colony_update_kernel(const InstanceView* instances, const ColonyView* colonies,
                                     ColonyState* states, ColonyParams P, TraceRow* trace,
                                     const std::uint32_t* list, std::uint32_t colony_count,
                                     std::uint32_t trace_cap);
__global__ void colony_trails_kernel(const InstanceView* instances, const ColonyView* colonies,
                                     const ColonyState* states, ColonyParams P, const std::uint32_t* list);
__global__ void pheromone_step_kernel(std::uint32_t n, std::uint32_t k, const node_t* primary,
                                      const std::uint32_t* parent_nbr, float ret, float tmin, float tmax, float inc,
                                      const float* eta, float* trails, float* products);
__global__ void score_controllers_kernel(const Program* trees, const std::uint32_t* kinds, std::uint32_t replicas,
                                         const float* features, const std::uint32_t* masks, float* scores,
                                         std::int32_t* actions, std::uint32_t colonies);
__global__ void score_kernel(const Program* programs, std::uint32_t replicas, const float* features,
                             const std::uint32_t* masks, float* scores, std::int32_t* actions,
                             std::uint32_t colonies);

}  // namespace faco

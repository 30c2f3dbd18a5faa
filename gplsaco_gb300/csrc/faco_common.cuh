// faco_common.cuh -- device types and primitives shared by the FACO kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace faco {

using node_t = std::uint16_t;   // node ids on the device (n <= 65535)
constexpr std::uint32_t kMaxNodes = 65535;
constexpr std::uint32_t kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

// Device error word bits (the host turns a non-zero word into FACO_EDEVICE).
enum DeviceError : unsigned {
    kErrNone = 0,
    kErrQueueOverflow = 1u << 0,
    kErrBadChoice = 1u << 1,
    kErrLoopCap = 1u << 2,
    kErrShape = 1u << 3,
    kErrTensorWait = 1u << 4,   // a tcgen05 MMA completion wait ran out
};

// TSPLIB EUC_2D: round(sqrt(dx^2+dy^2)) with halves up.  sqrt(s) is never a
// half-integer for integer s, so the result is the unique m with
// m*m - m < s <= m*m + m (m > 0) -- found from an FP32 estimate and at most
// a few exact int64 corrections.  Equal to floor(sqrt((double)s) + 0.5)
// for lengths below 2^25, which covers every instance registration admits
// (coordinate spans below 2^24 per axis).
// The estimate comes from 32-bit dx, dy in FP32 (GB300 runs 64-bit
// integer/float conversions on its narrow FP64 pipe, so none are used).
// The estimate only has to be close: m is the exact result iff
// m^2 - m < s <= m^2 + m, which one 64-bit product decides; the correction
// loops run only when that test fails (an estimate off by one or more).
__device__ __forceinline__ float sqrt_estimate(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ int euc2d(int2 p, int2 q) {
    const int dx = p.x - q.x, dy = p.y - q.y;  // |dx|, |dy| < 2^27
    const float fx = (float)dx, fy = (float)dy;
    int m = __float2int_rn(sqrt_estimate(fx * fx + fy * fy));
    const long long s = (long long)dx * dx + (long long)dy * dy;
    const long long t = s - (long long)m * m;
    if (t > m || t <= -m) {
        while (s > (long long)m * m + m) ++m;
        while (m > 0 && s <= (long long)m * m - m) --m;
    }
    return m;
}

// Philox4x32 with 10 rounds (Salmon, Moraes, Dror, Shaw, SC'11).
struct uint4v { std::uint32_t x, y, z, w; };
__device__ __forceinline__ uint4v philox4x32(std::uint32_t c0, std::uint32_t c1, std::uint32_t c2,
                                             std::uint32_t c3, std::uint32_t k0, std::uint32_t k1) {
#pragma unroll
    for (int round = 0; round < 10; ++round) {
        const std::uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        const std::uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
        c0 = hi1 ^ c1 ^ k0; c1 = lo1; c2 = hi0 ^ c3 ^ k1; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    return {c0, c1, c2, c3};
}

// The same generator with its rounds in a loop: fewer instructions in the
// code, for call sites where code size matters more than the loop overhead.
__device__ __forceinline__ uint4v philox4x32_rolled(std::uint32_t c0, std::uint32_t c1, std::uint32_t c2,
                                                    std::uint32_t c3, std::uint32_t k0, std::uint32_t k1) {
#pragma unroll 1
    for (int round = 0; round < 10; ++round) {
        const std::uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        const std::uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
        c0 = hi1 ^ c1 ^ k0; c1 = lo1; c2 = hi0 ^ c3 ^ k1; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    return {c0, c1, c2, c3};
}

__device__ __forceinline__ double u53(std::uint32_t hi, std::uint32_t lo) {
    return (double)(((((unsigned long long)hi) << 32) | lo) >> 11) * 0x1.0p-53;
}

// Counter layout: (step, ant, batch, tag).  tag 0 construction uniform,
// 1 start node, 2 colony source draw (ant = 0xffffffff).
__device__ __forceinline__ double step_uniform(unsigned long long key, std::uint32_t batch, std::uint32_t ant,
                                               std::uint32_t step) {
    const uint4v r = philox4x32(step, ant, batch, 0, (std::uint32_t)key, (std::uint32_t)(key >> 32));
    return u53(r.x, r.y);
}
__device__ __forceinline__ std::uint32_t start_node(unsigned long long key, std::uint32_t batch,
                                                    std::uint32_t ant, std::uint32_t n) {
    const uint4v r = philox4x32(0, ant, batch, 1, (std::uint32_t)key, (std::uint32_t)(key >> 32));
    return (std::uint32_t)(((unsigned long long)r.x * n) >> 32);
}
__device__ __forceinline__ double source_uniform(unsigned long long key, std::uint32_t batch) {
    const uint4v r = philox4x32(0, 0xffffffffu, batch, 2, (std::uint32_t)key, (std::uint32_t)(key >> 32));
    return u53(r.x, r.y);
}

// One registered instance resident on the device.
struct InstanceView {
    std::uint32_t n;
    std::uint32_t k, b, w;         // primary / backup / LS widths (clipped to n)
    const int2* xy;                // [n]
    const node_t* primary;         // [n][k]
    const node_t* backup;          // [n][b]
    const node_t* ls;              // [n][w], distance ordered
    const int* ls_dist;            // [n][w]
    const float* eta;              // [n][k]
    const node_t* initial;         // [n]
    long long initial_cost;
    const node_t* region_list;     // nodes grouped by quadrant of the bounding box
    std::uint32_t region_offsets[5];
    float mean_nn;                 // mean nearest-neighbour distance (prior features)
    // 12-feature controller (feature spec 2)
    const node_t* samples;         // min(n, 64) sample nodes drawn from the instance key
    std::uint32_t sample_count;
    const double* local_scale;     // [n] mean of the min(8, n-1) nearest lengths
    double scale_epsilon;          // 1e-12 * max(coordinate span, 1)
    const float* alpha;            // [n][k] alpha-nearness of the primary entries (prior features)
};

// GP program (postfix IR; device mirror of faco_program).
struct Program {
    std::uint16_t ir_version, numeric_spec_id, feature_spec_id, length, constants_count;
    std::uint8_t opcode[63];
    std::uint8_t operand[63];
    float constants[63];
};

// Start node from a start region (quadrant) when one is set and non-empty,
// else uniform over all nodes; the same Philox draw either way.
__device__ __forceinline__ std::uint32_t region_start(unsigned long long key, std::uint32_t batch,
                                                      std::uint32_t ant, const InstanceView* in,
                                                      std::uint32_t region) {
    const uint4v r = philox4x32(0, ant, batch, 1, (std::uint32_t)key, (std::uint32_t)(key >> 32));
    if (region < 4) {
        const std::uint32_t lo = in->region_offsets[region], size = in->region_offsets[region + 1] - lo;
        if (size) return in->region_list[lo + (std::uint32_t)(((unsigned long long)r.x * size) >> 32)];
    }
    return (std::uint32_t)(((unsigned long long)r.x * in->n) >> 32);
}

// Per-colony mutable state (one per work item of an evaluation).
struct ColonyState {
    long long epoch_cost, global_cost, parent_cost;
    long long iteration_best_cost;
    float tau_min, tau_max, default_trail;
    std::uint32_t iteration;       // completed batches
    std::uint32_t iteration_best;
    std::uint32_t source_is_epoch;
    std::uint32_t mne_target;
    std::int32_t action;
    unsigned long long construction_steps, ls_evaluations, reversed_elements;
    // controller state (GP-controlled evaluations)
    std::uint32_t region;          // start region of the next iteration (4 = all nodes, 5 = the controller's start list)
    std::uint32_t restarts, last_improvement, last_restart;
};

struct RefControl;

// Per-colony constant view.
struct ColonyView {
    std::uint32_t instance;        // index into the instance table
    std::uint32_t n;
    unsigned long long key;        // Philox key
    float* trails;                 // [n][k]
    float* products;               // [n][k]
    float* eta;                    // [n][k] heuristic of this colony (instance eta, or reweighted by the prior)
    node_t* parent;                // [n_pad] (16-byte aligned)
    std::uint32_t* parent_nbr;     // [n]: parent successor | predecessor << 16
    node_t* epoch;                 // [n]
    node_t* global;                // [n]
    node_t* ant_tours;             // [ants][n_pad] (16-byte aligned rows)
    std::uint32_t n_pad;           // row stride of ant_tours (n rounded up to 8)
    long long* ant_costs;          // [ants] final (after LS)
    long long* ant_ccosts;         // [ants] after construction
    unsigned* ant_counts;          // [ants][3]: construction steps, LS evaluations, moved elements
    const Program* program;        // GP controller of this colony: 3 tree slots (null: plain FACO)
    std::uint32_t action_mask;     // legal actions
    std::uint32_t controller_kind; // 0 joint_single (slot 0), 1 conditional_three (slots 0-2 = roles)
    // 12-feature controller (feature spec 2; null otherwise)
    RefControl* control;
    node_t* archive;               // [2 sides][4 slots][tour, positions][n_pad]
    unsigned long long* ant_ids;   // [ants][2] fingerprints of the batch's tours
    std::uint32_t* ant_p0;         // [ants] position of node 0 in each tour
};

struct TraceRow {
    long long iteration_best_cost, global_cost, parent_cost;
    std::uint32_t iteration_best, source_is_epoch;
    float tau_min, tau_max;
    std::uint32_t mne_target;
    std::int32_t action;
    unsigned long long construction_steps, ls_evaluations;
};

}  // namespace faco

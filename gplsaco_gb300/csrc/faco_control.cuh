// faco_control.cuh -- the reference's 12-feature colony controller (feature
// spec 2) on the device: tour fingerprints, the reference-tour archive,
// controller feedback, start regions and the 12 x 32 action features
// (cpp/include/gp_faco/control_ops.hpp:15-214, cpp/src/control_cpu.cpp:25-118,
// cuda/control_state.cuh:45-364).
//
// The control hash (SplitMix64's output function) and its salts are kept
// equal to the reference's, so sample nodes, start regions and fingerprints
// -- and with them the archive order of equal-cost tours -- are the same
// for the same keys.  Lengths are exact EUC_2D integers.
#pragma once

#include "faco_common.cuh"

namespace faco {

constexpr std::uint32_t kArchive = 4, kRegionNodes = 16, kSamples = 64;
constexpr double kArchiveBand = 0.02;
constexpr std::uint32_t kCtlMaxAnts = 1024;   // ants per colony the archive selection tracks

__host__ __device__ __forceinline__ unsigned long long ctl_mix(unsigned long long v) {
    v += 0x9e3779b97f4a7c15ULL;
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31);
}

// Uniform integer in [0, bound) by rejection below (2^64 - bound) mod bound.
struct CtlRandom {
    unsigned long long key, counter;
    __host__ __device__ std::uint32_t bounded(std::uint32_t bound) {
        const unsigned long long threshold = (0ull - (unsigned long long)bound) % bound;
        unsigned long long word;
        do { word = ctl_mix(key + counter++); } while (word < threshold);
        return (std::uint32_t)(word % bound);
    }
};

// The rank-th node outside existing[0..count), count <= 64.
template <class T>
__host__ __device__ std::uint32_t remaining_node(std::uint32_t rank, const T* existing, std::uint32_t count) {
    std::uint32_t sorted[kSamples];
    for (std::uint32_t i = 0; i < count; ++i) {
        std::uint32_t j = i;
        while (j && sorted[j - 1] > (std::uint32_t)existing[i]) { sorted[j] = sorted[j - 1]; --j; }
        sorted[j] = existing[i];
    }
    std::uint32_t node = rank;
    for (std::uint32_t i = 0; i < count; ++i) if (sorted[i] <= node) ++node;
    return node;
}

// min(n, 64) distinct nodes of an instance, drawn from its key.
template <class T>
__host__ __device__ void sample_nodes(std::uint32_t n, unsigned long long instance_key, T* out) {
    const std::uint32_t count = n < kSamples ? n : kSamples;
    CtlRandom r{ctl_mix(instance_key ^ 0x6a09e667f3bcc909ULL), 0};
    for (std::uint32_t i = 0; i < count; ++i) out[i] = (T)remaining_node(r.bounded(n - i), out, i);
}

template <class T>
__host__ __device__ __forceinline__ bool has_node(const T* nodes, std::uint32_t count, std::uint32_t v) {
    for (std::uint32_t i = 0; i < count; ++i) if ((std::uint32_t)nodes[i] == v) return true;
    return false;
}

// Start region (mode, region) of one batch around a reference tour, built by
// one warp (every lane draws the same random sequence): regions 0-1 are 16
// consecutive tour nodes from a random position, region 2 a breadth-first
// walk over the primary candidate rows from a random node (a row's new nodes
// taken in row order), region 3 (and any shortfall of 2) distinct uniform
// nodes -- the rank-th node outside the set is the least fixed point of
// x = rank + |{e in set : e <= x}|.  nodes[16] in shared memory; k <= 32.
__device__ inline void warp_build_region(const node_t* tour, std::uint32_t n, const node_t* primary,
                                         std::uint32_t k, unsigned long long key, std::uint32_t batch,
                                         std::uint32_t mode, std::uint32_t region, node_t* nodes,
                                         std::uint32_t lane) {
    const std::uint32_t count = n < kRegionNodes ? n : kRegionNodes;
    CtlRandom r{ctl_mix(key ^ 0xbb67ae8584caa73bULL ^ ctl_mix((unsigned long long)batch ^ 0x3c6ef372fe94f82bULL) ^
                        ctl_mix((unsigned long long)(mode * 4 + region + 1) ^ 0xa54ff53a5f1d36f1ULL)),
                0};
    if (region < 2) {
        const std::uint32_t start = r.bounded(n);
        if (lane < kRegionNodes) nodes[lane] = lane < count ? tour[(start + lane) % n] : (node_t)0;
        __syncwarp();
        return;
    }
    if (lane < kRegionNodes) nodes[lane] = 0;
    __syncwarp();
    std::uint32_t used = 0;
    if (region == 2) {
        const std::uint32_t first = r.bounded(n);
        if (lane == 0) nodes[0] = (node_t)first;
        used = 1;
        __syncwarp();
        for (std::uint32_t head = 0; head < used && used < count; ++head) {
            const std::uint32_t v = lane < k ? primary[(size_t)nodes[head] * k + lane] : n;
            const bool fresh = v < n && !has_node(nodes, used, v);
            const unsigned ok = __ballot_sync(0xffffffffu, fresh);
            const std::uint32_t take = min((std::uint32_t)__popc(ok), count - used);
            const std::uint32_t rank = __popc(ok & ((1u << lane) - 1u));
            __syncwarp();
            if (fresh && rank < take) nodes[used + rank] = (node_t)v;
            used += take;
            __syncwarp();
        }
    }
    while (used < count) {
        const std::uint32_t rank = r.bounded(n - used);
        const std::uint32_t e = lane < used ? (std::uint32_t)nodes[lane] : 0xffffffffu;
        std::uint32_t x = rank;
        for (;;) {
            const std::uint32_t next = rank + __popc(__ballot_sync(0xffffffffu, e <= x));
            if (next == x) break;
            x = next;
        }
        if (lane == 0) nodes[used] = (node_t)x;
        ++used;
        __syncwarp();
    }
}

// A start node from a start list with the construction's own Philox draw
// (the draw region_start takes).
__device__ __forceinline__ std::uint32_t list_start(unsigned long long key, std::uint32_t batch, std::uint32_t ant,
                                                    const node_t* list, std::uint32_t count) {
    const uint4v r = philox4x32(0, ant, batch, 1, (std::uint32_t)key, (std::uint32_t)(key >> 32));
    return list[((unsigned long long)r.x * count) >> 32];
}

struct Fingerprint {
    unsigned long long first, second;
};
__host__ __device__ __forceinline__ bool fp_equal(Fingerprint a, Fingerprint b) {
    return a.first == b.first && a.second == b.second;
}
__host__ __device__ __forceinline__ bool fp_less(Fingerprint a, Fingerprint b) {
    return a.first < b.first || (a.first == b.first && a.second < b.second);
}
__host__ __device__ __forceinline__ Fingerprint fingerprint_edge(std::uint32_t a, std::uint32_t b) {
    const unsigned long long lo = a < b ? a : b, hi = a < b ? b : a, edge = (lo << 32) | hi;
    return {ctl_mix(edge ^ 0xb5ad4eceda1ce2a9ULL), ctl_mix(edge ^ 0xd6e8feb86659fd93ULL)};
}

// Per-colony controller state (ControllerState + FeedbackState,
// control_ops.hpp:160-173), plus the start list of the next batch.
struct RefControl {
    long long archive_cost[kArchive];
    Fingerprint archive_id[kArchive];
    Fingerprint active_id, epoch_id;
    long long tracked_global, tracked_epoch;
    unsigned long long stagnant_batches, epoch_batches, restarts;
    float return_rate, ls_work;
    std::uint32_t archive_size, side;   // archive entries; which half of the double buffer holds them
    std::uint32_t alternative, legal_mask;
    std::uint32_t start_count, reserved;
    std::uint32_t archive_p0[kArchive];   // position of node 0 in each archive tour
    node_t start_nodes[kRegionNodes];
};

// Decision captures (decision_iterations, batch_engine.cu:620-632): for the
// decision before batch b the slot i with points[i] == b + 1.
struct DecisionCapture {
    const std::uint32_t* points;
    std::uint32_t count;
    float* features;           // [count][colonies][12][32]
    float* scores;             // [count][colonies][32]
    std::uint32_t* masks;      // [count][colonies]
    std::int32_t* actions;     // [count][colonies]
};

}  // namespace faco

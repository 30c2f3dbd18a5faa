// faco_ant.cuh -- one warp runs one ant: focused construction from the
// colony's parent tour, then checklist local search.
//
// Semantics follow the reference's fused kernel construct_and_search
// (cuda/faco_device.cuh:100-501) and its CPU restatement
// (cpp/src/faco_cpu.cpp:82-294): relocation steps until the MNE target,
// candidate-row roulette with backup and global fallbacks, then FIFO
// checklist 2-opt with best-gain moves and the reference's tie, cap and
// reversal rules.  The GB300 design differs throughout:
//   - every per-ant scalar is warp-uniform and lives in registers of all 32
//     lanes (no shared State struct, no lane-0 serial sections beyond the
//     single store of a queue slot or flag word);
//   - the tour and its inverse live in shared memory as 16-bit nodes, the
//     visited/pending flags as bitsets; coordinates are staged once per
//     block for all its ants (one colony per block); the checklist ring
//     lives in the ant's own output-tour slot in global memory (L1-cached),
//     which nothing reads before the ant writes its final tour there;
//   - distances are exact EUC_2D integers computed on the fly, so gains and
//     tour lengths are exact int64 and ties are decided by index only;
//   - the roulette decides from an FP32 warp scan whenever a proven error
//     margin allows and otherwise recomputes the reference's ordered FP64
//     prefix sums, so the choice is always the FP64 one (GB300 runs FP64 at
//     a small fraction of its FP32 rate);
//   - relocation shifts run as register-staged warp chunks, reversals as
//     disjoint swap pairs, the best move by __reduce_max/min_sync, and the
//     LS rows of the next pending node are fetched while the current one is
//     evaluated.
#pragma once

#include <climits>

#include "faco_common.cuh"

namespace faco {

enum AntMode : int {
    kModeEngine = 0,    // Philox choices, colony parent (production path)
    kModeVisits = 1,    // explicit visit orders (diagnostic)
    kModeUniforms = 2,  // injected uniforms + given products (diagnostic)
    kModePrepare = 3,   // no construction; LS over the whole tour (registration)
    kModeEngineGlobal = 4,  // kModeEngine with tour/inverse in global memory and
                            // coordinates read from global (large instances)
    kModeEngineFollow = 5,        // kModeEngine with batched parent-following steps (follow_batch)
    kModeEngineGlobalFollow = 6,  // kModeEngineGlobal with batched parent-following steps
    // kModeEngineFollow compiled for panels beyond one wave of the GPU: the
    // same arithmetic, the batch's roulette loops unrolled by two (72
    // registers against 79: one more block per SM) where mode 5 favours one
    // ant's latency.  The global-workspace variant has no such build: the
    // same unrolling leaves it at 80 registers.
    kModeEngineFollowDense = 7,
};

__host__ __device__ constexpr bool engine_mode(int mode) {
    return mode == kModeEngine || mode == kModeEngineGlobal || mode == kModeEngineFollow ||
           mode == kModeEngineGlobalFollow || mode == kModeEngineFollowDense;
}
__host__ __device__ constexpr bool global_mode(int mode) {
    return mode == kModeEngineGlobal || mode == kModeEngineGlobalFollow;
}
__host__ __device__ constexpr bool dense_mode(int mode) { return mode == kModeEngineFollowDense; }
__host__ __device__ constexpr bool follow_mode(int mode) {
    return mode == kModeEngineFollow || mode == kModeEngineGlobalFollow || mode == kModeEngineFollowDense;
}
// The batched variant of an engine mode (`dense`: the build for panels
// beyond one wave, where there is one).
__host__ __device__ constexpr int with_follow(int mode, bool dense = false) {
    return mode == kModeEngineGlobal ? kModeEngineGlobalFollow
           : mode == kModeEngine     ? (dense ? kModeEngineFollowDense : kModeEngineFollow)
                                     : mode;
}

struct AntLaunch {
    // instance (all ants of a block share one instance)
    const InstanceView* instances;
    // engine mode
    const ColonyView* colonies;
    ColonyState* states;
    const uint2* work;            // per block: (colony, first ant)
    node_t* workspace;            // kModeEngineGlobal: tour + inverse per ant, laid out
                                  // like the colonies' ant_tours with rows of 2 x n_pad
    const node_t* ant_tours_base; // start of the buffer the colonies' ant_tours point into
    std::uint32_t ants;           // ants per colony
    std::uint32_t warps;          // warps per block
    std::uint32_t n_max;          // smem layout size
    unsigned long long ls_limit;
    std::uint32_t ls_mode;
    // diagnostic modes: tasks on instance 0
    std::uint32_t tasks;
    const node_t* task_tours;        // [tasks][n]
    const std::uint32_t* task_nbr;   // [tasks][n] parent successor | predecessor << 16
    const long long* task_costs;     // [tasks]
    const node_t* task_visits;       // [tasks][n]
    const double* task_uniforms;     // [tasks][n]
    const std::uint32_t* task_starts;
    const std::uint32_t* task_targets;
    const float* task_products;      // [n][k]
    // diagnostic outputs (may be null)
    node_t* out_construction;     // [tasks][n]
    node_t* out_tours;            // [tasks][n]; required: also each task's checklist ring during the run
    node_t* out_pos;              // [tasks][n]
    node_t* out_selected;         // [tasks][n]
    std::uint32_t* out_checklist; // [tasks][checklist_cap]
    std::uint32_t checklist_cap;
    long long* out_costs;         // [tasks][2]
    unsigned long long* out_counters;  // [tasks][10]
    unsigned* error;
};

__host__ __device__ inline std::uint32_t pad8(std::uint32_t n) { return (n + 7u) & ~7u; }

// Per-warp shared-memory workspace: tour and inverse (16-bit), visited and
// pending bitsets.
__host__ __device__ inline std::uint32_t ant_smem_bytes(std::uint32_t n) {
    return (4u * pad8(n) + 8u * ((n + 31u) / 32u) + 15u) & ~15u;
}
__host__ __device__ inline std::uint32_t block_smem_bytes(std::uint32_t n, std::uint32_t warps) {
    return ((8u * n + 15u) & ~15u) + warps * ant_smem_bytes(n);
}
// Global-workspace variant: only the two bitsets per ant stay in shared memory.
__host__ __device__ inline std::uint32_t ant_bitset_bytes(std::uint32_t n) {
    return (8u * ((n + 31u) / 32u) + 15u) & ~15u;
}
__host__ __device__ inline std::uint32_t block_smem_bytes_global(std::uint32_t n, std::uint32_t warps) {
    return warps * ant_bitset_bytes(n);
}

struct AntSmem {
    node_t* tour;                 // shared
    node_t* pos;                  // shared
    node_t* ring;                 // global: the ant's checklist ring (n entries)
    std::uint32_t* visited;       // shared
    std::uint32_t* queued;        // shared
    __device__ static AntSmem at(unsigned char* base, std::uint32_t n_max, node_t* ring) {
        const std::uint32_t np = pad8(n_max), words = (n_max + 31u) / 32u;
        return {reinterpret_cast<node_t*>(base), reinterpret_cast<node_t*>(base + 2 * np), ring,
                reinterpret_cast<std::uint32_t*>(base + 4 * np),
                reinterpret_cast<std::uint32_t*>(base + 4 * np) + words};
    }
    // tour/inverse at `global` (2 x n_pad nodes), bitsets at `bits` (shared)
    __device__ static AntSmem split(node_t* global, std::uint32_t n_pad, unsigned char* bits,
                                    std::uint32_t n_max, node_t* ring) {
        const std::uint32_t words = (n_max + 31u) / 32u;
        return {global, global + n_pad, ring, reinterpret_cast<std::uint32_t*>(bits),
                reinterpret_cast<std::uint32_t*>(bits) + words};
    }
};

__device__ __forceinline__ bool test_bit(const std::uint32_t* bits, std::uint32_t v) {
    return (bits[v >> 5] >> (v & 31u)) & 1u;
}

struct Checklist {
    std::uint32_t head, tail, pending, pushed;  // ring indices and counters (warp-uniform)
};

// Appends v unless it is pending (reference append_if_absent,
// cuda/faco_device.cuh:81-92).  Warp-uniform decision, lane 0 stores.
__device__ __forceinline__ bool push_absent(const AntSmem& s, Checklist& q, std::uint32_t n, std::uint32_t v,
                                            std::uint32_t lane, std::uint32_t* log, std::uint32_t log_cap) {
    const bool absent = !test_bit(s.queued, v);
    __syncwarp();   // every lane has read the flag before lane 0 sets it
    if (absent) {
        if (lane == 0) {
            s.queued[v >> 5] |= 1u << (v & 31u);
            s.ring[q.tail] = (node_t)v;
            if (log && q.pushed < log_cap) log[q.pushed] = v;
        }
        q.tail = q.tail + 1 == n ? 0 : q.tail + 1;
        ++q.pending;
        ++q.pushed;
    }
    __syncwarp();
    return absent;
}

__device__ __forceinline__ std::uint32_t pop(const AntSmem& s, Checklist& q, std::uint32_t n,
                                             std::uint32_t lane) {
    const std::uint32_t a = s.ring[q.head];
    q.head = q.head + 1 == n ? 0 : q.head + 1;
    --q.pending;
    __syncwarp();
    if (lane == 0) s.queued[a >> 5] &= ~(1u << (a & 31u));
    return a;
}

struct AntResult {
    long long construction_cost, final_cost;
    std::uint32_t mne, steps, nonidentity;
    unsigned long long processed, checks, evaluations, accepted, reactivations;
    unsigned long long moved;  // tour elements rewritten by relocations and reversals
    std::uint32_t limit_reached, checklist;
};

// Moves `node` right after `target` (CpuTour::relocate): shifts the closed
// interval between their positions by one, register-staged per 64-element
// chunk (two elements per lane) so that every read of a chunk precedes its
// writes; chunks run away from the vacated end.
__device__ __forceinline__ void relocate_shift(const AntSmem& s, std::uint32_t lane, std::uint32_t tpos,
                                               std::uint32_t npos, std::uint32_t node) {
    if (tpos < npos) {
        // new[tpos+1] = node, new[i] = old[i-1] for i in (tpos+1, npos]
        const int lo = (int)tpos + 1;
        for (int base = (int)npos; base >= lo; base -= 64) {
            const int i0 = base - (int)lane, i1 = i0 - 32;
            std::uint32_t v0 = 0, v1 = 0;
            const bool a0 = i0 >= lo, a1 = i1 >= lo;
            if (a0) v0 = i0 == lo ? node : s.tour[i0 - 1];
            if (a1) v1 = i1 == lo ? node : s.tour[i1 - 1];
            __syncwarp();
            if (a0) { s.tour[i0] = (node_t)v0; s.pos[v0] = (node_t)i0; }
            if (a1) { s.tour[i1] = (node_t)v1; s.pos[v1] = (node_t)i1; }
            __syncwarp();
        }
    } else {
        // new[i] = old[i+1] for i in [npos, tpos), new[tpos] = node
        for (std::uint32_t base = npos; base <= tpos; base += 64) {
            const std::uint32_t i0 = base + lane, i1 = i0 + 32;
            std::uint32_t v0 = 0, v1 = 0;
            const bool a0 = i0 <= tpos, a1 = i1 <= tpos;
            if (a0) v0 = i0 == tpos ? node : s.tour[i0 + 1];
            if (a1) v1 = i1 == tpos ? node : s.tour[i1 + 1];
            __syncwarp();
            if (a0) { s.tour[i0] = (node_t)v0; s.pos[v0] = (node_t)i0; }
            if (a1) { s.tour[i1] = (node_t)v1; s.pos[v1] = (node_t)i1; }
            __syncwarp();
        }
    }
}

// Reverses tour[lo..hi] (inclusive, lo <= hi, no wrap) with the inverse.
__device__ __forceinline__ void reverse_range(const AntSmem& s, std::uint32_t lane, std::uint32_t lo,
                                              std::uint32_t hi) {
    const std::uint32_t count = hi - lo + 1;
    for (std::uint32_t o = lane; o < count / 2; o += 32) {
        const std::uint32_t l = lo + o, r = hi - o;
        const node_t a = s.tour[l], b = s.tour[r];
        s.tour[l] = b; s.tour[r] = a;
        s.pos[b] = (node_t)l; s.pos[a] = (node_t)r;
    }
    __syncwarp();
}

// A run of relocations deferred during construction.  Once trails converge
// an ant mostly follows parent edges: after it takes a node x from its place
// to after the current node, its next nodes are x's old tour neighbours,
// taken one at a time from the same place -- each relocation shifting the
// whole span between the two places again.  A run starts at a relocation:
// it keeps the tour as it is before the node moves (`ph`, the node y_1 at
// p, the current node at t) and the number m of nodes taken since
// (y_j = ph[p + dir (j-1)], j = 1..m), and reads the relocated tour through
// a position map; apply() rewrites the span once, by the single shift when
// m == 1, else with two or three reversals.  The tour it reads equals the one the
// relocations one by one would have left (CpuTour::relocate,
// cpp/src/faco_cpu.cpp:82-112):
//   p < t: the taken nodes sit at [t-m+1, t] in order, the span between
//          them and their source moved left by m;
//   p > t: the taken nodes sit at [t+1, t+m] in order, the span moved
//          right by m.
// An ant defers its relocations on instances of more than kDeferAllFrom
// nodes, and on the others after kDeferFromStep construction steps (early,
// short walks rarely continue a run: there a deferred single relocation
// costs more than an immediate one; measured at N=1000 and N=5000-10000).
constexpr std::uint32_t kDeferFromStep = 24;
constexpr std::uint32_t kDeferAllFrom = 2048;

struct RelocationRun {
    std::uint32_t m = 0;   // 0: no run
    std::uint32_t p = 0, t = 0;
    int dir = 1;           // +1: sources taken rightwards; -1: leftwards (either while m == 1)

    // node at position i of the relocated tour
    __device__ __forceinline__ std::uint32_t read(const AntSmem& s, std::uint32_t i) const {
        if (p < t) {
            const std::uint32_t first = t - m + 1;
            if (i >= first && i <= t) return s.tour[dir > 0 ? p + (i - first) : p - (i - first)];
            const std::uint32_t lo = dir > 0 ? p : p - m + 1;
            if (i >= lo && i < first) return s.tour[i + m];
        } else {
            const std::uint32_t last = t + m;
            if (i > t && i <= last) return s.tour[dir > 0 ? p + (i - t - 1) : p - (i - t - 1)];
            const std::uint32_t hi = dir > 0 ? p + m - 1 : p;
            if (i > last && i <= hi) return s.tour[i - m];
        }
        return s.tour[i];
    }
    // position of the current node (the last one taken)
    __device__ __forceinline__ std::uint32_t current_pos() const { return p < t ? t : t + m; }
    // Direction in which a node at position q of ph continues the run (the
    // next source, p + dir m), or 0: not next to the sources, past a tour
    // end, or out of the span between the sources and the taken nodes.
    __device__ __forceinline__ int continues(std::uint32_t q) const {
        if (q + m == p && (p < t || q > t) && (m == 1 || dir < 0)) return -1;
        if (q == p + m && (p > t || q < t) && (m == 1 || dir > 0)) return 1;
        return 0;
    }
    // position of that node in the relocated tour
    __device__ __forceinline__ std::uint32_t source_pos(int d) const {
        return (p < t) == (d < 0) ? (d < 0 ? p - m : p + m) : p;
    }
    // Rewrites the span so that the tour holds the relocated order; the run
    // ends.  `last` is the node taken last (the ant's current node).
    __device__ void apply(const AntSmem& s, std::uint32_t lane, std::uint32_t last) {
        if (m == 1) {
            relocate_shift(s, lane, t, p, last);   // reads before its first write, after a warp barrier
            m = 0;
            return;
        }
        __syncwarp();
        if (p < t) {
            // [sources | span] -> [span | taken in order]
            const std::uint32_t lo = dir > 0 ? p : p - m + 1, span = t - lo + 1 - m;
            reverse_range(s, lane, lo, t);
            if (span > 1) reverse_range(s, lane, lo, lo + span - 1);
            if (dir > 0) reverse_range(s, lane, t - m + 1, t);
        } else {
            // [span | sources] -> [taken in order | span]
            const std::uint32_t hi = dir > 0 ? p + m - 1 : p, span = hi - t - m;
            reverse_range(s, lane, t + 1, hi);
            if (dir > 0) reverse_range(s, lane, t + 1, t + m);
            if (span > 1) reverse_range(s, lane, t + m + 1, hi);
        }
        m = 0;
    }
};

// Construction steps that follow the parent tour, evaluated 16 or 32 at a
// time, one lane per step.  Once trails converge an ant mostly takes a
// parent-tour neighbour of its current node (no new edge): either the node
// after it in its tour (an identity step) or, after a jump, the old tour
// neighbours of the node it jumped to, pulled one by one from their place
// (a relocation run).  Both paths are known before the draws are: lane i
// assumes the walk followed that path for i steps and decides step i's
// roulette on its own -- candidates of its node, available unless visited
// or earlier on the path, its own uniform -- with a serial FP32 sum and a
// proven margin (sequential FP32 prefixes of at most 32 non-negative terms
// are within 31 roundings of the exact ones, the threshold within 33, so
// 2^-17 of the total separates the FP64 decision with room to spare);
// undecided lanes end the batch.  The leading lanes whose choice is their
// hypothesised node are then applied as one: visited bits, counters, the
// run extended by their number (or, for identity steps, nothing else), and
// the exact six-edge deltas of every step summed.  The tour, costs and
// counters equal those of the steps one by one; the first lane that is not
// taken is left to the caller's serial step.  All 32 steps are decided at
// once, so a long walk along the parent tour costs a few steps' latency:
// the variant for panels that leave the GPU under-filled, where an
// iteration lasts as long as its longest walk.
//
// Hypotheses: with a run of m >= 2 nodes, its direction (32 lanes); with a
// run of one node, both directions (lanes 0-15 rightwards, 16-31
// leftwards); with no run, lanes 0-15 the parent successor of the current
// node and 16-31 its parent predecessor -- an identity walk along the tour
// when that node follows the current one, else the start of a run.
// Returns the number of steps taken (0: nothing changed); `full` is set when
// every lane of the chosen hypothesis was taken (the walk may go on).
__device__ __forceinline__ bool on_segment(int lo, int hi, int q) { return q >= lo && q <= hi; }

// The roulette of one lane's step in follow_batch: the candidates of `row`
// still open to the walk (unvisited, and for a relocation run not on the
// run's segment), their FP32 weights summed serially in candidate order,
// and the first prefix at or above uf * total; -1 when that prefix lies
// within the decision margin (the one-step path decides) or no candidate is
// open.  The dense variants unroll both loops by two; the others leave them
// to the compiler.  The loops are written out twice because any rewrite of
// the shared body (a lambda, a helper per candidate) changed the compiler's
// code for the latency-tuned variants.  Both run the same sums in the same
// order.
template <bool kDense>
__device__ __forceinline__ int follow_roulette(const AntSmem& s, const node_t* row, const float* prow,
                                               std::uint32_t n, std::uint32_t k, std::uint32_t rel, std::uint32_t t0,
                                               bool identity, int lo, int hi, float uf) {
    unsigned avail = 0;
    float tot = 0.0f;
    if constexpr (kDense) {
#pragma unroll 2
        for (std::uint32_t j = 0; j < k; ++j) {
            const std::uint32_t x = __ldg(row + j);
            const float w = __ldg(prow + j);
            bool a = x < n && !test_bit(s.visited, x);
            if (a && rel) {
                const std::uint32_t px = s.pos[x];
                const std::uint32_t dx = px >= t0 ? px - t0 : px + n - t0;   // tour positions after the start
                a = identity ? !(dx >= 1 && dx <= rel) : !on_segment(lo, hi, (int)px);
            }
            if (a) {
                avail |= 1u << j;
                tot += w;
            }
        }
    } else {
        for (std::uint32_t j = 0; j < k; ++j) {
            const std::uint32_t x = __ldg(row + j);
            const float w = __ldg(prow + j);
            bool a = x < n && !test_bit(s.visited, x);
            if (a && rel) {
                const std::uint32_t px = s.pos[x];
                const std::uint32_t dx = px >= t0 ? px - t0 : px + n - t0;   // tour positions after the start
                a = identity ? !(dx >= 1 && dx <= rel) : !on_segment(lo, hi, (int)px);
            }
            if (a) {
                avail |= 1u << j;
                tot += w;
            }
        }
    }
    int choice = -1;
    if (avail && tot >= 0x1p-100f) {
        const float thr = uf * tot, delta = tot * 0x1p-17f;
        float prefix = 0.0f;
        if constexpr (kDense) {
#pragma unroll 2
            for (std::uint32_t j = 0; j < k; ++j) {
                if (!((avail >> j) & 1u)) continue;
                prefix += __ldg(prow + j);
                const float diff = prefix - thr;
                if (diff >= -delta) {
                    if (diff > delta) choice = (int)j;
                    break;
                }
            }
        } else {
            for (std::uint32_t j = 0; j < k; ++j) {
                if (!((avail >> j) & 1u)) continue;
                prefix += __ldg(prow + j);
                const float diff = prefix - thr;
                if (diff >= -delta) {
                    if (diff > delta) choice = (int)j;
                    break;
                }
            }
        }
    }
    return choice;
}

template <bool kDense>
__device__ inline std::uint32_t follow_batch(const AntSmem& s, const int2* xy, const InstanceView& in,
                                             const float* products, const std::uint32_t* parent_nbr, std::uint32_t n,
                                             std::uint32_t lane, unsigned long long key, std::uint32_t batch,
                                             std::uint32_t ant, std::uint32_t& current, AntResult& r,
                                             long long& cost, RelocationRun& run, std::uint32_t& draw_base,
                                             std::uint32_t& draw_hi, std::uint32_t& draw_lo, bool& full) {
    const std::uint32_t k = in.k;
    const std::uint32_t m0 = run.m;
    const bool split = m0 <= 1;
    const std::uint32_t half = split ? lane >> 4 : 0u, rel = split ? lane & 15u : lane;
    // the draws of the next 32 steps, lane i holding step base + i (the
    // caller's layout, which it reuses afterwards)
    const std::uint32_t base = r.steps + 1;
    if (base != draw_base) {
        const uint4v rb = philox4x32_rolled(base + lane, ant, batch, 0, (std::uint32_t)key, (std::uint32_t)(key >> 32));
        draw_base = base;
        draw_hi = rb.x;
        draw_lo = rb.y;
    }
    const std::uint32_t rhi = __shfl_sync(kFull, draw_hi, rel);
    const float uf = __uint2float_rn(rhi) * 0x1p-32f;

    // this lane's hypothesis: the node it stands on (cur) and the node it
    // must draw (sel), with the run geometry of its step
    bool identity = false;
    int p = 0, t = 0, D = 1;
    std::uint32_t t0 = 0;
    if (m0 >= 1) {
        p = (int)run.p;
        t = (int)run.t;
        D = m0 >= 2 ? run.dir : (half ? -1 : 1);
    } else {
        const std::uint32_t pn = __ldg(parent_nbr + current);
        const std::uint32_t y = half ? pn >> 16 : pn & 0xffffu;
        t0 = s.pos[current];
        const std::uint32_t ty = s.pos[y];
        if (ty == (t0 + 1 == n ? 0u : t0 + 1)) {
            identity = true;
        } else {
            p = (int)ty;
            t = (int)t0;
            D = half ? -1 : 1;
        }
    }
    const std::uint32_t mr = m0 + rel;   // run nodes taken before this lane's step
    bool ok = rel + 1 < n - r.steps;     // the loop's step budget: steps + rel + 1 < n
    std::uint32_t cur = current, sel = n;
    int lo = 0, hi = -1;                 // path positions taken by the earlier lanes
    if (identity) {
        if (rel) cur = s.tour[(t0 + rel) % n];
        sel = s.tour[(t0 + rel + 1) % n];
    } else {
        const int q = p + D * (int)mr;
        ok = ok && q >= 0 && q < (int)n && (mr == 0 || (D < 0 ? (p < t || q > t) : (p > t || q < t)));
        if (ok) {
            sel = s.tour[q];
            if (rel) cur = s.tour[q - D];
        }
        if (rel) {
            const int a = p + D * (int)m0, b = q - D;
            lo = a < b ? a : b;
            hi = a < b ? b : a;
        }
    }
    if (ok) {
        const std::uint32_t pn = __ldg(parent_nbr + cur);
        ok = (sel == (pn & 0xffffu) || sel == (pn >> 16)) && !test_bit(s.visited, sel);
    }
    // the run as it stands before this lane's step (m = mr): a step onto the
    // node after the current one is an identity step, not a relocation
    RelocationRun v;
    v.m = mr;
    v.p = (std::uint32_t)p;
    v.t = (std::uint32_t)t;
    v.dir = D;
    if (ok && !identity) {
        const std::uint32_t tpos = v.current_pos();
        ok = v.read(s, tpos + 1 == n ? 0 : tpos + 1) != sel;
    }
    // the roulette of this lane's step: serial FP32 sums in candidate order
    if (ok) {
        const node_t* row = in.primary + (size_t)cur * k;
        const float* prow = products + (size_t)cur * k;
        const int choice = follow_roulette<kDense>(s, row, prow, n, k, rel, t0, identity, lo, hi, uf);
        ok = choice >= 0 && __ldg(row + choice) == sel;
    }
    // the leading run of taken steps
    const unsigned okm = __ballot_sync(kFull, ok);
    std::uint32_t f, first_lane;
    if (split) {
        const unsigned m_lo = okm & 0xffffu, m_hi = okm >> 16;
        const std::uint32_t f_lo = __ffs(~m_lo) - 1, f_hi = __ffs(~m_hi) - 1;   // trailing ones, <= 16
        first_lane = f_lo ? 0u : 16u;
        f = f_lo ? f_lo : f_hi;
    } else {
        first_lane = 0;
        f = okm == kFull ? 32u : (std::uint32_t)(__ffs(~okm) - 1);
    }
    full = f == (split ? 16u : 32u);
    if (f == 0) return 0;
    const bool taken = lane >= first_lane && lane < first_lane + f;
    // identity lanes of the chosen half all agree on `identity`
    const bool ident = __shfl_sync(kFull, identity ? 1 : 0, first_lane) != 0;
    long long d = 0;
    std::uint32_t moved = 0;
    if (taken && !ident) {
        // six-edge delta of CpuTour::relocate for this lane's step, its
        // positions and tour neighbours read through the run with m = mr
        const std::uint32_t tpos = v.current_pos(), npos = v.source_pos(D);
        std::uint32_t target_after = n, previous = n, after = n;
#pragma unroll 1
        for (int t = 0; t < 3; ++t) {   // one copy of the run's read in the code
            const std::uint32_t at = t == 0 ? (tpos + 1 == n ? 0 : tpos + 1)
                                   : t == 1 ? (npos == 0 ? n - 1 : npos - 1) : (npos + 1 == n ? 0 : npos + 1);
            const std::uint32_t x = v.read(s, at);
            if (t == 0) target_after = x;
            else if (t == 1) previous = x;
            else after = x;
        }
        // added (previous,after) (cur,sel) (sel,target_after), removed
        // (previous,sel) (sel,after) (cur,target_after): one loop, so that
        // the batch's code holds one copy of the distance
#pragma unroll 1
        for (int t = 0; t < 6; ++t) {
            const std::uint32_t ea = t == 0 || t == 3 ? previous : t == 2 || t == 4 ? sel : cur;
            const std::uint32_t eb = t == 0 || t == 4 ? after : t == 1 || t == 3 ? sel : target_after;
            const int dd = euc2d(xy[ea], xy[eb]);
            d += t < 3 ? dd : -dd;
        }
        moved = tpos < npos ? npos - tpos : tpos - npos + 1;
    }
    if (taken) atomicOr(&s.visited[sel >> 5], 1u << (sel & 31u));
#pragma unroll
    for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(kFull, d, o);
    moved = __reduce_add_sync(kFull, moved);
    current = __shfl_sync(kFull, sel, first_lane + f - 1);
    cost += d;
    r.steps += f;
    if (!ident) {
        const int Dt = __shfl_sync(kFull, D, first_lane);
        const std::uint32_t pt = (std::uint32_t)__shfl_sync(kFull, p, first_lane);
        const std::uint32_t tt = (std::uint32_t)__shfl_sync(kFull, t, first_lane);
        r.nonidentity += f;
        r.moved += moved;
        run.p = pt;
        run.t = tt;
        run.dir = Dt;
        run.m = m0 + f;
    }
    __syncwarp();
    return f;
}

// flip_without_cost (cpp/src/faco_cpu.cpp:114-135) as disjoint swap pairs.
// Returns the number of elements in the reversed segment.
__device__ __forceinline__ std::uint32_t flip(const AntSmem& s, std::uint32_t n, std::uint32_t lane,
                                              std::uint32_t start, std::uint32_t end) {
    std::uint32_t first = s.pos[start], last = s.pos[end];
    if (first > last) { const std::uint32_t t = first; first = last; last = t; }
    const std::uint32_t length = last - first;
    const bool straight = length <= n - length || first == 0;
    const std::uint32_t count = straight ? length : n - length, begin = straight ? first : last;
    __syncwarp();
    for (std::uint32_t o = lane; o < count / 2; o += 32) {
        std::uint32_t l = begin + o, r = begin + count - 1 - o;
        if (l >= n) l -= n;
        if (r >= n) r -= n;
        const node_t a = s.tour[l], b = s.tour[r];
        s.tour[l] = b; s.tour[r] = a;
        s.pos[b] = (node_t)l; s.pos[a] = (node_t)r;
    }
    __syncwarp();
    return count;
}

// LS row of one node: candidate id and its cached distance, one per lane.
struct LsRow {
    std::uint32_t node, b;
    int ab;
};
__device__ __forceinline__ LsRow load_row(const InstanceView& in, std::uint32_t a, std::uint32_t lane) {
    LsRow r{a, in.n, 0};
    if (lane < in.w) {
        r.b = __ldg(in.ls + (size_t)a * in.w + lane);
        r.ab = __ldg(in.ls_dist + (size_t)a * in.w + lane);
    }
    return r;
}

// Pops the next pending node and returns its LS row, taking the prefetched
// row when it belongs to that node; then prefetches the row of the node now
// at the head (it cannot change before it is popped).
__device__ __forceinline__ LsRow pop_with_row(const AntSmem& s, Checklist& q, std::uint32_t n,
                                              std::uint32_t lane, const InstanceView& in, LsRow& next) {
    const std::uint32_t a = pop(s, q, n, lane);
    LsRow row = next.node == a ? next : load_row(in, a, lane);
    row.node = a;
    next.node = n;
    if (q.pending > 0) next = load_row(in, s.ring[q.head], lane);
    return row;
}

// Checklist 2-opt, best gain per popped node, reference tie/cap rules
// (cpp/src/faco_cpu.cpp:148-217; cuda/faco_device.cuh:295-478).
// kCompact (the batched-step variants, bound by instruction fetch): the four
// pushes of a move through one copy of push_absent.
template <bool kCompact = false>
__device__ __forceinline__ void checklist_two_opt(const AntSmem& s, const int2* xy, const InstanceView& in,
                                                  std::uint32_t n, std::uint32_t lane, Checklist& q,
                                                  unsigned long long cap, AntResult& r, long long& gain_sum,
                                                  std::uint32_t* log, std::uint32_t log_cap) {
    const std::uint32_t w = in.w;
    LsRow next{n, n, 0};
    while (q.pending > 0 && r.accepted < n) {
        if (r.evaluations >= cap) { r.limit_reached = 1; break; }
        const LsRow row = pop_with_row(s, q, n, lane, in, next);
        const std::uint32_t a = row.node, b = row.b;
        const int ab = row.ab;
        const std::uint32_t pa = s.pos[a];
        const std::uint32_t an = s.tour[pa + 1 == n ? 0 : pa + 1];
        const std::uint32_t ap = s.tour[pa == 0 ? n - 1 : pa - 1];
        ++r.processed;
        const int2 pa_xy = xy[a];
        const int cur0 = euc2d(pa_xy, xy[an]), cur1 = euc2d(xy[ap], pa_xy);
        // prefix of candidates that pass the distance test, per kind
        const bool bad0 = lane < w && (b >= n || !(cur0 > ab));
        const bool bad1 = lane < w && (b >= n || !(cur1 > ab));
        const unsigned f0m = __ballot_sync(kFull, bad0), f1m = __ballot_sync(kFull, bad1);
        const std::uint32_t f0 = f0m ? __ffs(f0m) - 1 : w, f1 = f1m ? __ffs(f1m) - 1 : w;
        unsigned long long remaining = cap - r.evaluations;
        const std::uint32_t used0 = remaining < f0 ? (std::uint32_t)remaining : f0;
        r.evaluations += used0;
        r.checks += used0 + (used0 < w ? 1 : 0);
        if (used0 < f0) { r.limit_reached = 1; break; }
        remaining = cap - r.evaluations;
        const std::uint32_t used1 = remaining < f1 ? (std::uint32_t)remaining : f1;
        r.evaluations += used1;
        r.checks += used1 + (used1 < w ? 1 : 0);
        if (used1 < f1) { r.limit_reached = 1; break; }
        // gains
        int g0 = INT_MIN, g1 = INT_MIN;
        std::uint32_t nb0 = 0, nb1 = 0;
        if (lane < used0 || lane < used1) {
            const std::uint32_t pb = s.pos[b];
            const int2 bxy = xy[b];
            if (lane < used0) {
                nb0 = s.tour[pb + 1 == n ? 0 : pb + 1];
                g0 = (nb0 == a || b == an) ? 0 : cur0 + euc2d(bxy, xy[nb0]) - ab - euc2d(xy[an], xy[nb0]);
            }
            if (lane < used1) {
                nb1 = s.tour[pb == 0 ? n - 1 : pb - 1];
                g1 = (nb1 == a || b == ap) ? 0 : cur1 + euc2d(bxy, xy[nb1]) - ab - euc2d(xy[ap], xy[nb1]);
            }
        }
        const int best = __reduce_max_sync(kFull, g0 > g1 ? g0 : g1);
        if (best > 0) {
            const std::uint32_t mine = g0 == best ? lane : g1 == best ? w + lane : 0xffu;
            const std::uint32_t index = __reduce_min_sync(kFull, mine);
            const std::uint32_t kind = index >= w, j = kind ? index - w : index;
            const std::uint32_t bj = __shfl_sync(kFull, b, j);
            const std::uint32_t nbj = __shfl_sync(kFull, kind ? nb1 : nb0, j);
            std::uint32_t m0, m1, m2, m3;
            if (kind == 0) { m0 = an; m1 = nbj; m2 = a; m3 = bj; }
            else { m0 = a; m1 = bj; m2 = ap; m3 = nbj; }
            r.moved += flip(s, n, lane, m0, m1);
            if constexpr (kCompact) {
#pragma unroll 1
                for (int t = 0; t < 4; ++t)
                    r.reactivations += push_absent(s, q, n, t == 0 ? m0 : t == 1 ? m1 : t == 2 ? m2 : m3, lane, log,
                                                   log_cap);
            } else {
                r.reactivations += push_absent(s, q, n, m0, lane, log, log_cap);
                r.reactivations += push_absent(s, q, n, m1, lane, log, log_cap);
                r.reactivations += push_absent(s, q, n, m2, lane, log, log_cap);
                r.reactivations += push_absent(s, q, n, m3, lane, log, log_cap);
            }
            ++r.accepted;
            gain_sum -= best;
        }
        __syncwarp();
    }
}

// Checklist local search with first-improvement 2-opt then Or-opt (segments
// of 1-3 nodes starting at the popped node).  The reference has no Or-opt;
// the move order, pruning and counting rules are this engine's own (stated in
// full beside the CPU restatement).  Every lane evaluates one candidate; the
// first improving move in scan order is found with one ballot.
__device__ __forceinline__ void checklist_ls_first(const AntSmem& s, const int2* xy, const InstanceView& in,
                                                   std::uint32_t n, std::uint32_t lane, Checklist& q,
                                                   unsigned long long cap, AntResult& r, long long& gain_sum,
                                                   std::uint32_t* log, std::uint32_t log_cap) {
    const std::uint32_t w = in.w;
    LsRow next{n, n, 0};
    while (q.pending > 0 && r.accepted < n) {
        if (r.evaluations >= cap) { r.limit_reached = 1; break; }
        const LsRow row = pop_with_row(s, q, n, lane, in, next);
        const std::uint32_t a = row.node, c = row.b;
        const int ac = row.ab;
        const std::uint32_t pa = s.pos[a];
        const std::uint32_t an = s.tour[pa + 1 == n ? 0 : pa + 1];
        const std::uint32_t ap = s.tour[pa == 0 ? n - 1 : pa - 1];
        ++r.processed;
        const int2 a_xy = xy[a];
        const int cur0 = euc2d(a_xy, xy[an]), cur1 = euc2d(xy[ap], a_xy);
        const bool valid = lane < w && c < n;
        std::uint32_t pc = 0, c_next = 0, c_prev = 0;
        int2 c_xy = make_int2(0, 0);
        if (valid) {
            pc = s.pos[c];
            c_next = s.tour[pc + 1 == n ? 0 : pc + 1];
            c_prev = s.tour[pc == 0 ? n - 1 : pc - 1];
            c_xy = xy[c];
        }
        bool interrupted = false, found = false;
        // ---- 2-opt, first improvement in (kind, j) order
        for (std::uint32_t kind = 0; kind < 2 && !found && !interrupted; ++kind) {
            const int cur = kind == 0 ? cur0 : cur1;
            const std::uint32_t closing_end = kind == 0 ? an : ap;
            const unsigned badm = __ballot_sync(kFull, lane < w && (!valid || !(cur > ac)));
            const std::uint32_t f = badm ? __ffs(badm) - 1 : w;
            const unsigned long long remaining = cap - r.evaluations;
            const std::uint32_t used = remaining < f ? (std::uint32_t)remaining : f;
            int g = INT_MIN;
            const std::uint32_t nb = kind == 0 ? c_next : c_prev;
            if (lane < used)
                g = (nb == a || c == closing_end) ? 0 : cur + euc2d(c_xy, xy[nb]) - ac - euc2d(xy[closing_end], xy[nb]);
            const unsigned improving = __ballot_sync(kFull, lane < used && g > 0);
            if (improving) {
                const std::uint32_t j = __ffs(improving) - 1;
                r.evaluations += j + 1;
                r.checks += j + 1;
                const int gain = __shfl_sync(kFull, g, j);
                const std::uint32_t bj = __shfl_sync(kFull, c, j), nbj = __shfl_sync(kFull, nb, j);
                std::uint32_t m0, m1, m2, m3;
                if (kind == 0) { m0 = an; m1 = nbj; m2 = a; m3 = bj; }
                else { m0 = a; m1 = bj; m2 = ap; m3 = nbj; }
                r.moved += flip(s, n, lane, m0, m1);
                r.reactivations += push_absent(s, q, n, m0, lane, log, log_cap);
                r.reactivations += push_absent(s, q, n, m1, lane, log, log_cap);
                r.reactivations += push_absent(s, q, n, m2, lane, log, log_cap);
                r.reactivations += push_absent(s, q, n, m3, lane, log, log_cap);
                ++r.accepted;
                gain_sum -= gain;
                found = true;
            } else {
                r.evaluations += used;
                r.checks += used + (used < w ? 1 : 0);
                if (used < f) interrupted = true;
            }
        }
        if (interrupted) { r.limit_reached = 1; break; }
        if (found) {
            __syncwarp();
            continue;
        }
        // ---- Or-opt: segment a.. of L nodes, first improvement in (L, j, variant) order
        std::uint32_t seg0 = a, seg1 = n, seg2 = n;
        const int d_pa = cur1;
        for (std::uint32_t L = 1; L <= 3 && !found && !interrupted; ++L) {
            if (n < L + 3) break;
            if (L == 2) seg1 = an;
            if (L == 3) { const std::uint32_t p1 = s.pos[seg1]; seg2 = s.tour[p1 + 1 == n ? 0 : p1 + 1]; }
            const std::uint32_t e = L == 1 ? seg0 : L == 2 ? seg1 : seg2;
            const std::uint32_t pe = s.pos[e];
            const std::uint32_t qn = s.tour[pe + 1 == n ? 0 : pe + 1];
            const int2 e_xy = xy[e];
            const int G = d_pa + euc2d(e_xy, xy[qn]) - euc2d(xy[ap], xy[qn]);
            const unsigned badm = __ballot_sync(kFull, lane < w && (!valid || !(G > ac)));
            const std::uint32_t f = badm ? __ffs(badm) - 1 : w;
            const unsigned long long remaining = cap - r.evaluations;
            const std::uint32_t used = remaining < f ? (std::uint32_t)remaining : f;
            int g1 = INT_MIN, g2 = INT_MIN;
            if (lane < used) {
                const bool inside = c == seg0 || c == seg1 || c == seg2;
                if (!inside) {
                    if (!(c_next == seg0 || c_next == seg1 || c_next == seg2))
                        g1 = G + euc2d(c_xy, xy[c_next]) - ac - euc2d(e_xy, xy[c_next]);
                    if (!(c_prev == seg0 || c_prev == seg1 || c_prev == seg2))
                        g2 = G + euc2d(xy[c_prev], c_xy) - euc2d(xy[c_prev], e_xy) - ac;
                }
            }
            const unsigned improving = __ballot_sync(kFull, lane < used && (g1 > 0 || g2 > 0));
            if (improving) {
                const std::uint32_t j = __ffs(improving) - 1;
                r.evaluations += j + 1;
                r.checks += j + 1;
                const int g1j = __shfl_sync(kFull, g1, j), g2j = __shfl_sync(kFull, g2, j);
                const std::uint32_t cj = __shfl_sync(kFull, c, j);
                const std::uint32_t c2 = __shfl_sync(kFull, c_next, j), c0 = __shfl_sync(kFull, c_prev, j);
                const bool first_variant = g1j > 0;
                // (i) c, a .. e, c2: relocate a after c, then each next node after the last moved
                // (ii) c0, e .. a, c: relocate e after c0, then each previous node
                std::uint32_t target = first_variant ? cj : c0;
                for (std::uint32_t t = 0; t < L; ++t) {
                    const std::uint32_t idx = first_variant ? t : L - 1 - t;
                    const std::uint32_t node = idx == 0 ? seg0 : idx == 1 ? seg1 : seg2;
                    const std::uint32_t tp = s.pos[target], np = s.pos[node];
                    relocate_shift(s, lane, tp, np, node);
                    r.moved += tp < np ? np - tp : tp - np + 1;
                    target = node;
                }
                r.reactivations += push_absent(s, q, n, ap, lane, log, log_cap);
                r.reactivations += push_absent(s, q, n, a, lane, log, log_cap);
                r.reactivations += push_absent(s, q, n, e, lane, log, log_cap);
                r.reactivations += push_absent(s, q, n, qn, lane, log, log_cap);
                r.reactivations += push_absent(s, q, n, first_variant ? cj : c0, lane, log, log_cap);
                r.reactivations += push_absent(s, q, n, first_variant ? c2 : cj, lane, log, log_cap);
                ++r.accepted;
                gain_sum -= first_variant ? g1j : g2j;
                found = true;
            } else {
                r.evaluations += used;
                r.checks += used + (used < w ? 1 : 0);
                if (used < f) interrupted = true;
            }
        }
        if (interrupted) { r.limit_reached = 1; break; }
        __syncwarp();
    }
}

}  // namespace faco

// faco_kernels.cu -- the FACO iteration kernels for sm_103a.
//
//   ant_kernel<mode>        construction + local search, one warp per ant
//   colony_init_kernel      reset_colony + initialize_products
//                           (cuda/colony_state.cuh:72-110)
//   colony_update_kernel    reduce_and_select + update_pheromone fused, one
//                           block per colony (cuda/colony_state.cuh:148-229),
//                           with the controllers' per-batch work
//   fingerprint_kernel      tour fingerprints for the 12-feature controller,
//                           one warp per ant (cuda/control_state.cuh:45-64)
//   pheromone_step_kernel   the trail update alone (parity hook)
//   score_kernel            GP controller scoring, warp per colony
//                           (cuda/gp_score.cuh:64-102)
#include <mutex>
#include <climits>

#include "faco_ant.cuh"
#include "faco_kernels.h"

namespace faco {

// ---------------------------------------------------------------------------
// Ant kernel
// ---------------------------------------------------------------------------
// Copies a parent tour into the warp's shared tour/inverse.  Engine parents
// are 16-byte aligned with padded rows, so lanes move 8 nodes per load.
__device__ __forceinline__ void load_parent(const AntSmem& s, const node_t* parent, std::uint32_t n,
                                            std::uint32_t lane, bool aligned) {
    if (aligned) {
        const uint4* src = reinterpret_cast<const uint4*>(parent);
        uint4* dst = reinterpret_cast<uint4*>(s.tour);
        for (std::uint32_t c = lane; c * 8 < n; c += 32) {
            const uint4 v = __ldg(src + c);
            dst[c] = v;
            const std::uint32_t words[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const std::uint32_t i = c * 8 + t;
                if (i < n) s.pos[(words[t >> 1] >> (16 * (t & 1))) & 0xffffu] = (node_t)i;
            }
        }
    } else {
        for (std::uint32_t i = lane; i < n; i += 32) {
            const std::uint32_t v = parent[i];
            s.tour[i] = (node_t)v;
            s.pos[v] = (node_t)i;
        }
    }
}

template <int MODE>
__global__ void __launch_bounds__(kMaxWarpsPerBlock * 32, kAntBlocksPerSM) ant_kernel(const AntLaunch L) {
    constexpr bool kEngine = engine_mode(MODE), kGlobalWs = global_mode(MODE), kFollow = follow_mode(MODE),
                   kDense = dense_mode(MODE);
    extern __shared__ __align__(16) unsigned char smem[];
    const std::uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    std::uint32_t colony = 0, ant = 0, task = 0;
    bool active;
    if (kEngine) {
        const uint2 job = L.work[blockIdx.x];
        colony = job.x;
        ant = job.y + warp;
        active = ant < L.ants;
    } else {
        task = blockIdx.x * L.warps + warp;
        ant = task;
        active = task < L.tasks;
    }
    const InstanceView* in_ptr = L.instances + (kEngine ? L.colonies[colony].instance : 0);
    const InstanceView in = *in_ptr;
    const std::uint32_t n = in.n;
    const int2* xy;
    if (kGlobalWs) {
        xy = in.xy;
    } else {
        int2* staged = reinterpret_cast<int2*>(smem);
        for (std::uint32_t i = threadIdx.x; i < n; i += blockDim.x) staged[i] = in.xy[i];
        __syncthreads();
        xy = staged;
    }
    if (!active) return;

    node_t* ring = kEngine ? L.colonies[colony].ant_tours + (size_t)ant * L.colonies[colony].n_pad
                           : L.out_tours + (size_t)task * n;
    AntSmem s;
    if (kGlobalWs) {
        const std::uint32_t n_pad = L.colonies[colony].n_pad;
        node_t* ws = L.workspace + 2 * ((size_t)(L.colonies[colony].ant_tours - L.ant_tours_base) +
                                        (size_t)ant * n_pad);
        s = AntSmem::split(ws, n_pad, smem + warp * ant_bitset_bytes(L.n_max), L.n_max, ring);
    } else {
        s = AntSmem::at(smem + ((8u * L.n_max + 15u) & ~15u) + warp * ant_smem_bytes(L.n_max), L.n_max, ring);
    }
    const node_t* parent;
    const std::uint32_t* parent_nbr;
    long long cost;
    std::uint32_t target, batch = 0, region = 4;
    unsigned long long key = 0;
    ColonyView cv{};
    if (kEngine) {
        cv = L.colonies[colony];
        const ColonyState& st = L.states[colony];
        parent = cv.parent;
        parent_nbr = cv.parent_nbr;
        cost = st.parent_cost;
        target = st.mne_target;
        batch = st.iteration;
        region = st.region;
        key = cv.key;
    } else {
        parent = L.task_tours + (size_t)task * n;
        parent_nbr = L.task_nbr + (size_t)task * n;
        cost = L.task_costs[task];
        target = MODE == kModePrepare ? 0 : L.task_targets[task];
    }
    load_parent(s, parent, n, lane, kEngine);
    const std::uint32_t words = (n + 31) / 32;
    for (std::uint32_t i = lane; i < words; i += 32) {
        s.visited[i] = 0;
        s.queued[i] = MODE == kModePrepare ? ~0u : 0u;
    }
    __syncwarp();

    std::uint32_t* log = L.out_checklist ? L.out_checklist + (size_t)task * L.checklist_cap : nullptr;
    const std::uint32_t log_cap = L.checklist_cap;
    Checklist q{0, 0, 0, 0};
    AntResult r{};

    if (MODE == kModePrepare) {
        // registration: every node pending, in tour order (prepared_problem.cpp:160-162)
        for (std::uint32_t i = lane; i < n; i += 32) {
            s.ring[i] = s.tour[i];
            if (log && i < log_cap) log[i] = s.tour[i];
        }
        q.tail = 0;
        q.pending = n;
        q.pushed = n;
        __syncwarp();
    } else {
        // ---------------- focused construction ----------------
        std::uint32_t current;
        if (kEngine) current = region == 5 ? list_start(key, batch, ant, cv.control->start_nodes,
                                                        cv.control->start_count)
                                           : region_start(key, batch, ant, in_ptr, region);
        else if (MODE == kModeVisits) current = L.task_visits[(size_t)task * n];
        else current = L.task_starts[task];
        if (L.out_selected && lane == 0) L.out_selected[(size_t)task * n] = (node_t)current;
        if (lane == 0) s.visited[current >> 5] |= 1u << (current & 31u);
        __syncwarp();
        const float* products = kEngine ? cv.products : L.task_products;
        const std::uint32_t k = in.k, b = in.b;
        const unsigned long long loop_cap = 2ull * n + 2;
        unsigned long long guard = 0;
        // the construction draws of 32 consecutive steps at a time, lane i
        // holding step draw_base + i (the same counters as one draw per step)
        std::uint32_t draw_base = 0x80000000u, draw_hi = 0, draw_lo = 0;   // steps < 2^16: first step refreshes
        // the candidate row of the likely next node, loaded one step ahead:
        // once trails converge an ant mostly walks the parent tour, so the
        // next node is the parent neighbour of `current` not yet visited
        std::uint32_t next_node = n, next_pnbr = 0, next_cand = n;
        float next_p = 0.0f;
        RelocationRun run;
        // steps along the parent tour are taken in batches (follow_batch)
        // until a batch stops short of its lanes; the step it stopped at is
        // taken alone, then batches resume
        bool follow = true;
        while (r.mne < target && r.steps + 1 < n) {
            if (++guard > loop_cap) { if (lane == 0) atomicOr(L.error, kErrLoopCap); break; }
            if (kFollow && follow) {
                bool full = false;
                const std::uint32_t f = follow_batch<kDense>(s, xy, in, products, parent_nbr, n, lane, key, batch,
                                                             ant, current, r, cost, run, draw_base, draw_hi, draw_lo,
                                                             full);
                follow = full;
                if (f) continue;
            }
            follow = true;
            const std::uint32_t step = r.steps + 1;
            if (kEngine && step - draw_base >= 32u) {
                draw_base = step;
                const uint4v rb = philox4x32(step + lane, ant, batch, 0, (std::uint32_t)key, (std::uint32_t)(key >> 32));
                draw_hi = rb.x;
                draw_lo = rb.y;
            }
            // loads that depend only on `current`, issued first
            std::uint32_t pnbr, cand = n;
            float p = 0.0f;
            if (kEngine && current == next_node) {
                pnbr = next_pnbr;
                cand = next_cand;
                p = next_p;
            } else {
                pnbr = __ldg(parent_nbr + current);
                if (MODE != kModeVisits && lane < k) {
                    cand = __ldg(in.primary + (size_t)current * k + lane);
                    p = __ldg(products + (size_t)current * k + lane);
                }
            }
            if (kEngine) {
                const std::uint32_t ps = pnbr & 0xffffu;
                next_node = test_bit(s.visited, ps) ? pnbr >> 16 : ps;
                next_pnbr = __ldg(parent_nbr + next_node);
                next_cand = n;
                next_p = 0.0f;
                if (lane < k) {
                    next_cand = __ldg(in.primary + (size_t)next_node * k + lane);
                    next_p = __ldg(products + (size_t)next_node * k + lane);
                }
            }
            std::uint32_t selected = n;
            if (MODE == kModeVisits) {
                selected = L.task_visits[(size_t)task * n + step];
            } else {
                std::uint32_t rhi = 0, rlo = 0;
                double u_given = 0.0;
                float uf;
                if (kEngine) {
                    rhi = __shfl_sync(kFull, draw_hi, step - draw_base);
                    rlo = __shfl_sync(kFull, draw_lo, step - draw_base);
                    uf = __uint2float_rn(rhi) * 0x1p-32f;
                } else {
                    u_given = L.task_uniforms[(size_t)task * n + step];
                    uf = (float)u_given;
                }
                const bool avail = cand < n && !test_bit(s.visited, cand);
                const unsigned mask = __ballot_sync(kFull, avail);
                if (mask) {
                    // FP32 inclusive scan of the available weights.  Each prefix is
                    // within 5 roundings (< 3.1e-7 relative) of the exact prefix, the
                    // threshold u*total within 4.3e-7; a choice is taken only when the
                    // first candidate not certainly below the threshold is certainly
                    // above it by delta = total * 2^-19 (> 1.9e-6), which the FP64
                    // ordered sums of the reference then decide identically.
                    const float pv = avail ? p : 0.0f;
                    float scan = pv;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const float t = __shfl_up_sync(kFull, scan, o);
                        if ((int)lane >= o) scan += t;
                    }
                    const float tot = __shfl_sync(kFull, scan, 31);
                    int j = -1;
                    if (tot >= 0x1p-100f) {
                        const float thr = uf * tot, delta = tot * 0x1p-19f, diff = scan - thr;
                        const unsigned yes = __ballot_sync(kFull, avail && diff > delta);
                        const unsigned maybe = __ballot_sync(kFull, avail && diff >= -delta);
                        if (maybe != 0u && (maybe & (0u - maybe)) == (yes & (0u - yes))) j = __ffs(yes) - 1;
                    }
                    if (j < 0) {
                        // exact path: ordered FP64 prefix sums (faco_cpu.cpp:254-279)
                        const double u = kEngine ? u53(rhi, rlo) : u_given;
                        double total = 0.0, mine = 0.0;
                        for (unsigned m = mask; m; m &= m - 1) {
                            const int jj = __ffs(m) - 1;
                            total += (double)__shfl_sync(kFull, p, jj);
                            if ((int)lane == jj) mine = total;
                        }
                        if (total > 0.0) {
                            const double threshold = u * total;
                            const unsigned hit = __ballot_sync(kFull, avail && threshold < mine);
                            j = hit ? __ffs(hit) - 1 : 31 - __clz(mask);
                        } else {
                            const std::uint32_t count = __popc(mask);
                            std::uint32_t t = (std::uint32_t)(u * count);
                            if (t >= count) t = count - 1;
                            unsigned m = mask;
                            for (; t; --t) m &= m - 1;
                            j = __ffs(m) - 1;
                        }
                    }
                    selected = __shfl_sync(kFull, cand, j);
                } else {
                    for (std::uint32_t base_j = 0; base_j < b && selected == n; base_j += 32) {
                        const std::uint32_t jj = base_j + lane;
                        std::uint32_t v = n;
                        bool ok = false;
                        if (jj < b) {
                            v = __ldg(in.backup + (size_t)current * b + jj);
                            ok = v < n && !test_bit(s.visited, v);
                        }
                        const unsigned m = __ballot_sync(kFull, ok);
                        if (m) selected = __shfl_sync(kFull, v, __ffs(m) - 1);
                    }
                    if (selected == n) {
                        // global nearest unvisited, lowest id on ties
                        unsigned long long bestkey = ~0ull;
                        const int2 cxy = xy[current];
                        for (std::uint32_t v = lane; v < n; v += 32) {
                            if (test_bit(s.visited, v)) continue;
                            const unsigned long long kv =
                                ((unsigned long long)(unsigned)euc2d(cxy, xy[v]) << 32) | v;
                            bestkey = kv < bestkey ? kv : bestkey;
                        }
                        for (int o = 16; o; o >>= 1) {
                            const unsigned long long other = __shfl_xor_sync(kFull, bestkey, o);
                            bestkey = other < bestkey ? other : bestkey;
                        }
                        if (bestkey != ~0ull) selected = (std::uint32_t)(bestkey & 0xffffffffu);
                    }
                }
            }
            if (selected >= n || test_bit(s.visited, selected)) {
                // no legal choice (only an invalid explicit visit order can get here)
                if (lane == 0) atomicOr(L.error, kErrBadChoice);
                break;
            }
            if (L.out_selected && lane == 0) L.out_selected[(size_t)task * n + step] = (node_t)selected;
            // positions and tour neighbours, read through the deferred run
            // when `selected` continues it, else from the rewritten tour
            std::uint32_t npos = s.pos[selected], tpos = n, previous = n, after = n, target_after = n;
            int run_dir = 0;
            bool start_run = false;
            if (run.m) {
                // the inverse is that of the tour before the run (unchanged during it)
                run_dir = run.continues(npos);
                if (run_dir) {
                    npos = run.source_pos(run_dir);
                    tpos = run.current_pos();
                    target_after = run.read(s, tpos + 1 == n ? 0 : tpos + 1);
                    if (target_after == selected) run_dir = 0;
                }
                if (run_dir) {
                    if constexpr (kFollow) {
                        // the batched-step variants are bound by instruction
                        // fetch: one copy of the run's read in their code
#pragma unroll 1
                        for (int t = 0; t < 2; ++t) {
                            const std::uint32_t x = run.read(s, t == 0 ? (npos == 0 ? n - 1 : npos - 1)
                                                                       : (npos + 1 == n ? 0 : npos + 1));
                            if (t == 0) previous = x;
                            else after = x;
                        }
                    } else {
                        previous = run.read(s, npos == 0 ? n - 1 : npos - 1);
                        after = run.read(s, npos + 1 == n ? 0 : npos + 1);
                    }
                } else {
                    run.apply(s, lane, current);
                    npos = s.pos[selected];
                }
            }
            if (!run_dir) {
                tpos = s.pos[current];
                previous = s.tour[npos == 0 ? n - 1 : npos - 1];
                after = s.tour[npos + 1 == n ? 0 : npos + 1];
                target_after = s.tour[tpos + 1 == n ? 0 : tpos + 1];
                // relocations are deferred on large instances, and on the
                // others once the walk is long (converged trails)
                start_run = n > kDeferAllFrom || r.steps >= kDeferFromStep;
            }
            ++r.steps;
            __syncwarp();
            if (lane == 0) s.visited[selected >> 5] |= 1u << (selected & 31u);
            if (target_after != selected) {
                ++r.nonidentity;
                // six-edge delta of CpuTour::relocate, one term per lane
                int term = 0;
                if (lane < 6) {
                    // removed: (previous,selected) (selected,after) (current,target_after)
                    // added:   (previous,after) (current,selected) (selected,target_after)
                    const std::uint32_t e0 = lane == 0 || lane == 3 ? previous : lane == 2 || lane == 4 ? current
                                                                                                        : selected;
                    const std::uint32_t e1 = lane == 0 || lane == 4 ? selected : lane == 1 || lane == 3 ? after
                                                                                                        : target_after;
                    const int d = euc2d(xy[e0], xy[e1]);
                    term = lane < 3 ? -d : d;
                }
                cost += __reduce_add_sync(kFull, term);
                if (run_dir) {
                    // the run takes one more node
                    run.dir = run_dir;
                    ++run.m;
                } else if (start_run) {
                    // a deferred run, of this relocation alone so far
                    run.p = npos;
                    run.t = tpos;
                    run.m = 1;
                    run.dir = 1;
                } else {
                    relocate_shift(s, lane, tpos, npos, selected);
                }
                r.moved += tpos < npos ? npos - tpos : tpos - npos + 1;
            }
            const bool new_edge = (pnbr & 0xffffu) != selected && (pnbr >> 16) != selected;
            if (new_edge) {
                ++r.mne;
                if constexpr (kFollow) {
#pragma unroll 1
                    for (int t = 0; t < 3; ++t)
                        push_absent(s, q, n, t == 0 ? current : t == 1 ? selected : previous, lane, log, log_cap);
                } else {
                    push_absent(s, q, n, current, lane, log, log_cap);
                    push_absent(s, q, n, selected, lane, log, log_cap);
                    push_absent(s, q, n, previous, lane, log, log_cap);
                }
            }
            current = selected;
            __syncwarp();
        }
        if (run.m) run.apply(s, lane, current);
        r.construction_cost = cost;
        if (L.out_construction)
            for (std::uint32_t i = lane; i < n; i += 32) L.out_construction[(size_t)task * n + i] = s.tour[i];
        __syncwarp();
    }
    // ---------------- local search ----------------
    long long gain_sum = 0;
    if (L.ls_mode == 1) checklist_ls_first(s, xy, in, n, lane, q, L.ls_limit, r, gain_sum, log, log_cap);
    else checklist_two_opt<kFollow>(s, xy, in, n, lane, q, L.ls_limit, r, gain_sum, log, log_cap);
    r.final_cost = cost + gain_sum;
    r.checklist = q.pushed;
    if (log && q.pushed > log_cap && lane == 0) atomicOr(L.error, kErrQueueOverflow);
    __syncwarp();

    if (kEngine) {
        uint4* out = reinterpret_cast<uint4*>(cv.ant_tours + (size_t)ant * cv.n_pad);
        const uint4* src = reinterpret_cast<const uint4*>(s.tour);
        for (std::uint32_t c = lane; c * 8 < n; c += 32) out[c] = src[c];
        if (lane == 0) {
            cv.ant_costs[ant] = r.final_cost;
            cv.ant_ccosts[ant] = r.construction_cost;
            cv.ant_counts[3 * ant] = r.steps;
            cv.ant_counts[3 * ant + 1] = (unsigned)r.evaluations;
            cv.ant_counts[3 * ant + 2] = (unsigned)r.moved;
        }
    } else {
        if (L.out_tours)
            for (std::uint32_t i = lane; i < n; i += 32) L.out_tours[(size_t)task * n + i] = s.tour[i];
        if (L.out_pos)
            for (std::uint32_t i = lane; i < n; i += 32) L.out_pos[(size_t)task * n + i] = s.pos[i];
        if (lane == 0) {
            if (L.out_costs) {
                L.out_costs[2 * (size_t)task] = r.construction_cost;
                L.out_costs[2 * (size_t)task + 1] = r.final_cost;
            }
            if (L.out_counters) {
                unsigned long long* c = L.out_counters + 10 * (size_t)task;
                c[0] = r.mne; c[1] = r.steps; c[2] = r.nonidentity; c[3] = r.processed; c[4] = r.checks;
                c[5] = r.evaluations; c[6] = r.accepted; c[7] = r.reactivations; c[8] = r.limit_reached;
                c[9] = r.checklist;
            }
        }
    }
}

namespace {
// The dynamic shared-memory limit is a per-kernel, per-device attribute that
// every engine on the device shares, and instantiated graphs launch against
// it: it is only ever raised, so that one engine's smaller classes never
// invalidate another engine's larger ones.
template <int MODE>
cudaError_t prepare_mode(std::uint32_t smem) {
    static std::mutex lock;
    static std::uint32_t raised[64] = {};
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess) return err;
    std::lock_guard<std::mutex> guard(lock);
    std::uint32_t& current = raised[device & 63];
    if (smem <= current) return cudaSuccess;
    err = cudaFuncSetAttribute(ant_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err == cudaSuccess) current = smem;
    return err;
}
}  // namespace

cudaError_t prepare_ant_kernel(int mode, std::uint32_t smem) {
    switch (mode) {
        case kModeEngine: return prepare_mode<kModeEngine>(smem);
        case kModeVisits: return prepare_mode<kModeVisits>(smem);
        case kModeUniforms: return prepare_mode<kModeUniforms>(smem);
        case kModePrepare: return prepare_mode<kModePrepare>(smem);
        case kModeEngineGlobal: return prepare_mode<kModeEngineGlobal>(smem);
        case kModeEngineFollow: return prepare_mode<kModeEngineFollow>(smem);
        case kModeEngineGlobalFollow: return prepare_mode<kModeEngineGlobalFollow>(smem);
        case kModeEngineFollowDense: return prepare_mode<kModeEngineFollowDense>(smem);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_ant_kernel(int mode, const AntLaunch& L, std::uint32_t blocks, std::uint32_t warps,
                              std::uint32_t smem, cudaStream_t stream) {
    const dim3 grid(blocks), block(warps * 32);
    switch (mode) {
        case kModeEngine: ant_kernel<kModeEngine><<<grid, block, smem, stream>>>(L); break;
        case kModeVisits: ant_kernel<kModeVisits><<<grid, block, smem, stream>>>(L); break;
        case kModeUniforms: ant_kernel<kModeUniforms><<<grid, block, smem, stream>>>(L); break;
        case kModePrepare: ant_kernel<kModePrepare><<<grid, block, smem, stream>>>(L); break;
        case kModeEngineGlobal: ant_kernel<kModeEngineGlobal><<<grid, block, smem, stream>>>(L); break;
        case kModeEngineFollow: ant_kernel<kModeEngineFollow><<<grid, block, smem, stream>>>(L); break;
        case kModeEngineGlobalFollow: ant_kernel<kModeEngineGlobalFollow><<<grid, block, smem, stream>>>(L); break;
        case kModeEngineFollowDense: ant_kernel<kModeEngineFollowDense><<<grid, block, smem, stream>>>(L); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Colony kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ void trail_limits(long long cost, double retention, double p_root, std::uint32_t k,
                                             float& tmin, float& tmax) {
    const double mx = 1.0 / ((double)cost * (1.0 - retention));
    double mn = mx * (1.0 - p_root) / (((double)k - 1.0) * p_root);
    mn = mn < mx ? mn : mx;
    tmax = (float)mx;
    tmin = (float)mn;
}

// MMAS evaporate/deposit on FP32 trails (cuda/colony_state.cuh:210-229):
// tau <- max(tau_min, tau * retention); a directed candidate entry (from, to)
// on the parent tour also gains min(tau_max, tau + 1/parent_cost); products
// are refreshed as tau * eta.  The parent-edge test reads the packed parent
// neighbours of `from`.  Threads stride over entries, four at a time when the
// row width allows 16-byte accesses.
__device__ __forceinline__ float trail_value(float tau, std::uint32_t to, std::uint32_t nb, float ret, float tmin,
                                             float tmax, float inc) {
    float v = fmaxf(tmin, tau * ret);
    if (to == (nb & 0xffffu) || to == (nb >> 16)) v = fminf(tmax, v + inc);
    return v;
}

__device__ __forceinline__ void trail_update(std::uint32_t n, std::uint32_t k, const node_t* primary,
                                             const std::uint32_t* nbr, float ret, float tmin, float tmax, float inc,
                                             const float* eta, float* trails, float* products, std::uint32_t first,
                                             std::uint32_t stride) {
    const std::uint32_t cells = n * k;
    if ((k & 3u) == 0) {
        for (std::uint32_t q = first; q * 4 < cells; q += stride) {
            const std::uint32_t idx = q * 4, nb = nbr[idx / k];
            const float4 t = *reinterpret_cast<const float4*>(trails + idx);
            const float4 e = *reinterpret_cast<const float4*>(eta + idx);
            const uint2 pr = *reinterpret_cast<const uint2*>(primary + idx);
            float4 v;
            v.x = trail_value(t.x, pr.x & 0xffffu, nb, ret, tmin, tmax, inc);
            v.y = trail_value(t.y, pr.x >> 16, nb, ret, tmin, tmax, inc);
            v.z = trail_value(t.z, pr.y & 0xffffu, nb, ret, tmin, tmax, inc);
            v.w = trail_value(t.w, pr.y >> 16, nb, ret, tmin, tmax, inc);
            *reinterpret_cast<float4*>(trails + idx) = v;
            *reinterpret_cast<float4*>(products + idx) = make_float4(v.x * e.x, v.y * e.y, v.z * e.z, v.w * e.w);
        }
    } else {
        for (std::uint32_t idx = first; idx < cells; idx += stride) {
            const float v = trail_value(trails[idx], primary[idx], nbr[idx / k], ret, tmin, tmax, inc);
            trails[idx] = v;
            products[idx] = v * eta[idx];
        }
    }
}

// Products of a colony whose prior re-ranks departures only: per node row,
// the parent-tour entries keep the instance heuristic (products = trail *
// eta), and the other entries take the prior's heuristic scaled so that
// their total weight equals the plain total, sum(trail * eta) over the
// non-parent entries.  An ant then leaves the parent tour as often as a
// plain ant does, and the prior only decides where it goes.  Rows over
// [first, n) with the given stride; trails are already updated.
__device__ __forceinline__ void departure_rows(const InstanceView& in, const ColonyView& cv, std::uint32_t first,
                                               std::uint32_t stride, std::uint32_t end) {
    const std::uint32_t k = in.k;
    for (std::uint32_t i = first; i < end; i += stride) {
        const std::uint32_t nb = cv.parent_nbr[i], succ = nb & 0xffffu, pred = nb >> 16;
        const std::size_t row = (std::size_t)i * k;
        float plain = 0.0f, prior = 0.0f;
        for (std::uint32_t j = 0; j < k; ++j) {
            const std::uint32_t node = in.primary[row + j];
            if (node == succ || node == pred) continue;
            const float t = cv.trails[row + j];
            plain += t * in.eta[row + j];
            prior += t * cv.eta[row + j];
        }
        const float scale = prior > 0.0f ? plain / prior : 1.0f;
        for (std::uint32_t j = 0; j < k; ++j) {
            const std::uint32_t node = in.primary[row + j];
            const float t = cv.trails[row + j];
            cv.products[row + j] = node == succ || node == pred ? t * in.eta[row + j] : t * cv.eta[row + j] * scale;
        }
    }
}

// ---------------------------------------------------------------------------
// GP controller pieces (the engine's feature spec 3; the same arithmetic is
// restated on the CPU beside the oracle colony run).
// ---------------------------------------------------------------------------
// log2 from the exponent and the atanh series of the mantissa,
// m in [sqrt(2)/2, sqrt(2)): log2 m = (2/ln 2) (t + t^3/3 + t^5/5 + t^7/7),
// t = (m-1)/(m+1).  Single-rounding FP32 operations only, so that the CPU
// computes identical bits.
__device__ __forceinline__ float own_log2(float x) {
    const std::uint32_t bits = __float_as_uint(x);
    int e = (int)((bits >> 23) & 255u) - 127;
    float m = __uint_as_float((bits & 0x7FFFFFu) | 0x3F800000u);
    if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e += 1; }
    const float t = (m - 1.0f) / (m + 1.0f), t2 = t * t;
    const float s = t * (1.0f + t2 * (0x1.555556p-2f + t2 * (0x1.99999ap-3f + t2 * 0x1.24924ap-3f)));
    return (float)e + s * 0x1.715476p+1f;
}

// Normalised Shannon entropy of one trail row, in units of 2^-20.
__device__ __forceinline__ std::uint32_t row_entropy_q(const float* tau, std::uint32_t k, float log2k) {
    float sum = 0.0f;
    for (std::uint32_t j = 0; j < k; ++j) sum = sum + tau[j];
    if (!(sum > 0.0f)) return 0;
    float h = 0.0f;
    for (std::uint32_t j = 0; j < k; ++j) {
        const float p = tau[j] / sum;
        if (p > 0.0f) h = h - p * own_log2(p);
    }
    float hn = h / log2k;
    hn = hn < 0.0f ? 0.0f : hn > 1.0f ? 1.0f : hn;
    return (std::uint32_t)(hn * 1048576.0f + 0.5f);
}

__device__ __forceinline__ float apply_operation(int op, float l, float r, float t) {
    float v = 0.0f;
    switch (op) {
        case 2: v = l + r; break;
        case 3: v = l - r; break;
        case 4: v = l * r; break;
        case 5: v = fminf(l, r); break;
        case 6: v = fmaxf(l, r); break;
        case 7: v = fabsf(l); break;
        case 8: { const float q = 1.0f + r * r; v = l * (1.0f / sqrtf(q)); break; }
        case 9: v = fabsf(r) < 1e-6f ? 1.0f : l / r; break;
        case 10: v = l > 0.0f ? r : t; break;
        default: break;
    }
    return fminf(8.0f, fmaxf(-8.0f, v));
}

// Postfix interpreter (cuda/gp_score.cuh:64-102); feature(i) supplies terminal i.
template <class Feature>
__device__ __forceinline__ float eval_program(const Program& p, Feature feature) {
    float stack[16];
    int top = 0;
    for (int i = 0; i < p.length; ++i) {
        const int op = p.opcode[i];
        if (op == 0) stack[top++] = feature(p.operand[i]);
        else if (op == 1) stack[top++] = p.constants[p.operand[i]];
        else {
            const int arity = op == 7 ? 1 : op == 10 ? 3 : 2;
            const float t = arity == 3 ? stack[--top] : 0.0f;
            const float r = arity >= 2 ? stack[--top] : 0.0f;
            const float l = stack[--top];
            stack[top++] = apply_operation(op, l, r, t);
        }
    }
    return stack[0];
}

// First maximum within 1e-6 among legal lanes (score_cpu rule); 32 if none.
__device__ __forceinline__ std::uint32_t choose_action(float value, bool legal, std::uint32_t lane) {
    float maximum = legal ? value : -INFINITY;
    for (int o = 16; o; o >>= 1) maximum = fmaxf(maximum, __shfl_xor_sync(kFull, maximum, o));
    return __reduce_min_sync(kFull, legal && maximum - value <= 1e-6f ? lane : 32u);
}

// conditional_three controllers (python/gp_faco/controller.py:60-84,
// cuda/gp_score.cuh role loop): role 0 picks the restart half (2 options,
// stride 16), role 1 the start region (4, stride 4), role 2 the MNE level
// (4, stride 1), each from the prefix the earlier roles fixed.  Lane i <
// width scores the role's tree on the features of action prefix + i*stride
// (feature_of(index, action)); a lane is legal when any action of its
// stride-wide window is; the first maximum within 1e-6 wins.  Role scores
// go to slots 0-1, 2-5 and 6-9 of `role_scores` (may be null).
template <class FeatureOf>
__device__ __forceinline__ std::uint32_t choose_conditional(const Program* trees, FeatureOf feature_of,
                                                            std::uint32_t mask, std::uint32_t lane,
                                                            float* role_scores) {
    std::uint32_t prefix = 0;
#pragma unroll 1
    for (int role = 0; role < 3; ++role) {
        const std::uint32_t width = role == 0 ? 2u : 4u, stride = role == 0 ? 16u : role == 1 ? 4u : 1u;
        const std::uint32_t action = prefix + (lane < width ? lane : 0u) * stride;
        const bool legal = lane < width && ((mask >> action) & ((1u << stride) - 1u)) != 0u;
        const float value = eval_program(trees[role], [&](int i) { return feature_of(i, action); });
        if (role_scores && lane < width) role_scores[(role == 0 ? 0 : role == 1 ? 2 : 6) + lane] = value;
        const std::uint32_t pick = choose_action(value, legal, lane);
        prefix += stride * (pick < 32u ? pick : 0u);
    }
    return prefix;
}

__device__ __forceinline__ float clamp01(double v) { return (float)(v < 0.0 ? 0.0 : v > 1.0 ? 1.0 : v); }

// ---------------------------------------------------------------------------
// The reference's 12-feature controller (feature spec 2): per batch, after
// the trail update, the ants' fingerprints, the archive of distinct
// near-best tours and the feedback (update_control, control_state.cuh:
// 124-245), then the decision for the next batch -- alternative reference,
// 8 start regions, 12 x 32 features, scoring, and the action (MNE target,
// start list, restart from the alternative; build_control_features and
// apply_control_action, :247-364).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double unit_clip(double v) { return v < 0.0 ? 0.0 : v > 1.0 ? 1.0 : v; }

// A tour in device memory: its order, its positions (may be null) and the
// position of node 0.
struct TourRef {
    const node_t* tour;
    const node_t* pos;
    std::uint32_t p0;
};

__device__ __forceinline__ node_t* archive_tour(const ColonyView& cv, std::uint32_t side, std::uint32_t slot) {
    return cv.archive + (size_t)((side * kArchive + slot) * 2u) * cv.n_pad;
}

// canonical_compare (control_ops.hpp:61-74) by one warp: both tours read
// from node 0 towards its smaller neighbour; -1, 0 or 1.  Each lane loads 16
// elements of both tours before the first vote, so the loads overlap.
__device__ __forceinline__ std::uint32_t canonical_index(std::uint32_t p0, bool forward, std::uint32_t i,
                                                         std::uint32_t n) {
    std::uint32_t x = forward ? p0 + i : p0 + n - i;   // < 2n
    return x >= n ? x - n : x;
}
__device__ int warp_canonical_compare(TourRef a, TourRef b, std::uint32_t n, std::uint32_t lane) {
    constexpr std::uint32_t kUnroll = 16;
    const bool fa = a.tour[a.p0 + 1 == n ? 0 : a.p0 + 1] < a.tour[a.p0 == 0 ? n - 1 : a.p0 - 1];
    const bool fb = b.tour[b.p0 + 1 == n ? 0 : b.p0 + 1] < b.tour[b.p0 == 0 ? n - 1 : b.p0 - 1];
    for (std::uint32_t base = 1; base < n; base += 32 * kUnroll) {
        std::uint32_t va[kUnroll], vb[kUnroll];
#pragma unroll
        for (std::uint32_t u = 0; u < kUnroll; ++u) {
            const std::uint32_t i = base + u * 32 + lane;
            va[u] = i < n ? a.tour[canonical_index(a.p0, fa, i, n)] : 0u;
            vb[u] = i < n ? b.tour[canonical_index(b.p0, fb, i, n)] : 0u;
        }
#pragma unroll
        for (std::uint32_t u = 0; u < kUnroll; ++u) {
            const unsigned m = __ballot_sync(kFull, va[u] != vb[u]);
            if (m) return __shfl_sync(kFull, va[u] < vb[u] ? -1 : 1, __ffs(m) - 1);
        }
    }
    return 0;
}

// XOR of the n edge fingerprints (fingerprint_ants, control_state.cuh:45-64)
// and the position of node 0, by one warp.
__device__ Fingerprint warp_fingerprint(const node_t* tour, std::uint32_t n, std::uint32_t lane, std::uint32_t& p0) {
    unsigned long long f1 = 0, f2 = 0;
    std::uint32_t z = 0xffffffffu;
    for (std::uint32_t base = 0; base < n; base += 128) {
        std::uint32_t a[4], b[4];
#pragma unroll
        for (std::uint32_t u = 0; u < 4; ++u) {
            const std::uint32_t i = base + u * 32 + lane;
            a[u] = i < n ? tour[i] : 0u;
            b[u] = i < n ? tour[i + 1 == n ? 0 : i + 1] : 0u;
        }
#pragma unroll
        for (std::uint32_t u = 0; u < 4; ++u) {
            const std::uint32_t i = base + u * 32 + lane;
            if (i >= n) continue;
            const Fingerprint e = fingerprint_edge(a[u], b[u]);
            f1 ^= e.first;
            f2 ^= e.second;
            if (a[u] == 0) z = i;
        }
    }
    for (int o = 16; o; o >>= 1) {
        f1 ^= __shfl_xor_sync(kFull, f1, o);
        f2 ^= __shfl_xor_sync(kFull, f2, o);
        z = min(z, __shfl_xor_sync(kFull, z, o));
    }
    p0 = z;
    return {f1, f2};
}

// Candidates of the archive selection: 0-3 the archive slots, 4 + a ant a.
// Archive fields come from the shared copy of the controller state; the
// ants' costs, fingerprints and node-0 positions from shared memory when the
// colony has at most kStageAnts ants, else from global memory.
constexpr std::uint32_t kStageAnts = 128;
struct CandidateView {
    const ColonyView& cv;
    const RefControl& ctl;
    const long long* costs;
    const Fingerprint* ids;
    const std::uint32_t* p0s;
    __device__ long long cost(std::uint32_t c) const { return c < kArchive ? ctl.archive_cost[c] : costs[c - kArchive]; }
    __device__ Fingerprint id(std::uint32_t c) const { return c < kArchive ? ctl.archive_id[c] : ids[c - kArchive]; }
    __device__ TourRef ref(std::uint32_t c) const {
        if (c < kArchive) {
            const node_t* t = archive_tour(cv, ctl.side, c);
            return {t, t + cv.n_pad, ctl.archive_p0[c]};
        }
        return {cv.ant_tours + (size_t)(c - kArchive) * cv.n_pad, nullptr, p0s[c - kArchive]};
    }
};

constexpr std::uint32_t kCtlWords = (kArchive + kCtlMaxAnts + 31) / 32;

// The archive band as an integer: an integer cost c exceeds the double
// global_cost * (1 + band) exactly when c exceeds its floor.
__device__ __forceinline__ long long band_limit(long long global_cost) {
    return (long long)floor((double)global_cost * (1 + kArchiveBand));
}

// Archive selection by warp 0 (update_control's slot loop): the global best
// first, then up to 3 distinct tours of the old archive and the batch within
// 2 % of the global cost, each the least by (cost, fingerprint, canonical
// order, candidate index).
__device__ std::uint32_t ref_archive_select(const CandidateView& v, const ColonyState& st, std::uint32_t A,
                                            bool improved, std::uint32_t n, std::uint32_t lane,
                                            std::uint32_t* excluded, std::uint32_t* chosen) {
    const std::uint32_t total = kArchive + A;
    for (std::uint32_t w = lane; w < (total + 31) / 32; w += 32) excluded[w] = 0;
    __syncwarp();
    const long long limit = band_limit(st.global_cost);
    auto is_excluded = [&](std::uint32_t c) { return (excluded[c >> 5] >> (c & 31u)) & 1u; };
    auto eligible = [&](std::uint32_t c) {
        if (c < kArchive && c >= v.ctl.archive_size) return false;
        return v.cost(c) <= limit && !is_excluded(c);
    };
    std::uint32_t count = 0;
    auto add = [&](std::uint32_t w) {
        if (lane == 0) {
            chosen[count] = w;
            excluded[w >> 5] |= 1u << (w & 31u);
        }
        ++count;
        __syncwarp();
        const Fingerprint idw = v.id(w);
        const TourRef rw = v.ref(w);
        for (std::uint32_t base = 0; base < total; base += 32) {
            const std::uint32_t c = base + lane;
            unsigned m = __ballot_sync(kFull, c < total && !is_excluded(c) && fp_equal(v.id(c), idw));
            while (m) {
                const std::uint32_t j = base + __ffs(m) - 1;
                m &= m - 1;
                if (warp_canonical_compare(v.ref(j), rw, n, lane) == 0 && lane == 0)
                    excluded[j >> 5] |= 1u << (j & 31u);
                __syncwarp();
            }
        }
        __syncwarp();
    };
    add(improved ? kArchive + st.iteration_best : 0u);
    for (std::uint32_t slot = 1; slot < kArchive; ++slot) {
        std::uint32_t best = 0xffffffffu;
        long long bc = 0;
        Fingerprint bi{0, 0};
        for (std::uint32_t c = lane; c < total; c += 32) {
            if (!eligible(c)) continue;
            const long long cc = v.cost(c);
            const Fingerprint ci = v.id(c);
            if (best == 0xffffffffu || cc < bc || (cc == bc && fp_less(ci, bi))) { best = c; bc = cc; bi = ci; }
        }
        for (int o = 16; o; o >>= 1) {
            const std::uint32_t ob = __shfl_xor_sync(kFull, best, o);
            const long long oc = __shfl_xor_sync(kFull, bc, o);
            const Fingerprint oi{__shfl_xor_sync(kFull, bi.first, o), __shfl_xor_sync(kFull, bi.second, o)};
            const bool take = ob != 0xffffffffu &&
                              (best == 0xffffffffu || oc < bc ||
                               (oc == bc && (fp_less(oi, bi) || (fp_equal(oi, bi) && ob < best))));
            if (take) { best = ob; bc = oc; bi = oi; }
        }
        if (best == 0xffffffffu) break;
        // equal cost and fingerprint with another tour: canonical order decides
        for (std::uint32_t base = 0; base < total; base += 32) {
            const std::uint32_t c = base + lane;
            unsigned m = __ballot_sync(kFull, c < total && c != best && eligible(c) && v.cost(c) == bc &&
                                                  fp_equal(v.id(c), bi));
            while (m) {
                const std::uint32_t j = base + __ffs(m) - 1;
                m &= m - 1;
                if (warp_canonical_compare(v.ref(j), v.ref(best), n, lane) < 0) best = j;
            }
        }
        add(best);
    }
    return count;
}

// The same selection when every pair of candidates with equal fingerprints
// holds the same tour (rep[c]: the first valid candidate with c's cost and
// fingerprint): a group of identical tours acts as its first member, and the
// least by (cost, fingerprint, index) needs no tour comparison.
__device__ std::uint32_t ref_archive_select_groups(const CandidateView& v, const ColonyState& st, std::uint32_t A,
                                                   bool improved, std::uint32_t lane, const std::uint16_t* rep,
                                                   std::uint32_t* excluded, std::uint32_t* chosen) {
    const std::uint32_t total = kArchive + A;
    for (std::uint32_t w = lane; w < (total + 31) / 32; w += 32) excluded[w] = 0;
    __syncwarp();
    const long long limit = band_limit(st.global_cost);
    const std::uint32_t first = improved ? kArchive + st.iteration_best : 0u;
    if (lane == 0) {
        chosen[0] = first;
        excluded[rep[first] >> 5] |= 1u << (rep[first] & 31u);
    }
    __syncwarp();
    std::uint32_t count = 1;
    for (std::uint32_t slot = 1; slot < kArchive; ++slot) {
        std::uint32_t best = 0xffffffffu;
        long long bc = 0;
        Fingerprint bi{0, 0};
        for (std::uint32_t c = lane; c < total; c += 32) {
            if (rep[c] != c || ((excluded[c >> 5] >> (c & 31u)) & 1u)) continue;
            const long long cc = v.cost(c);
            if (cc > limit) continue;
            const Fingerprint ci = v.id(c);
            if (best == 0xffffffffu || cc < bc || (cc == bc && fp_less(ci, bi))) { best = c; bc = cc; bi = ci; }
        }
        for (int o = 16; o; o >>= 1) {
            const std::uint32_t ob = __shfl_xor_sync(kFull, best, o);
            const long long oc = __shfl_xor_sync(kFull, bc, o);
            const Fingerprint oi{__shfl_xor_sync(kFull, bi.first, o), __shfl_xor_sync(kFull, bi.second, o)};
            const bool take = ob != 0xffffffffu &&
                              (best == 0xffffffffu || oc < bc ||
                               (oc == bc && (fp_less(oi, bi) || (fp_equal(oi, bi) && ob < best))));
            if (take) { best = ob; bc = oc; bi = oi; }
        }
        if (best == 0xffffffffu) break;
        if (lane == 0) {
            chosen[count] = best;
            excluded[best >> 5] |= 1u << (best & 31u);
        }
        ++count;
        __syncwarp();
    }
    return count;
}

struct RefShared {
    RefControl ctl;                       // the colony's controller state while the kernel runs
    float feat[12][32];
    float scores[32];
    node_t regions[8][kRegionNodes];
    long long ant_cost[kStageAnts];
    Fingerprint ant_id[kStageAnts];
    std::uint32_t ant_p0[kStageAnts];
    std::uint16_t rep[kArchive + kCtlMaxAnts];
    std::uint32_t collision;
    std::uint32_t excluded[kCtlWords];
    std::uint32_t chosen[kArchive], next_p0[kArchive];
    long long chosen_cost[kArchive];
    Fingerprint chosen_id[kArchive];
    std::uint32_t count, alternative, mask, action, largest;
    float gap[2], difference, elapsed, stagnation;
};

__device__ __forceinline__ CandidateView candidates(const ColonyView& cv, const RefShared& sh, std::uint32_t A) {
    const bool staged = A <= kStageAnts;
    return {cv, sh.ctl, staged ? sh.ant_cost : cv.ant_costs,
            staged ? sh.ant_id : reinterpret_cast<const Fingerprint*>(cv.ant_ids), staged ? sh.ant_p0 : cv.ant_p0};
}

// update_control for one colony (after reduce/select and the trail update);
// sh.ctl holds the controller state.
__device__ void ref_update(const ColonyView& cv, const InstanceView& in, const ColonyState& st,
                           const ColonyParams& P, RefShared& sh) {
    RefControl& ctl = sh.ctl;
    const std::uint32_t n = in.n, A = P.ants;
    const std::uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    const bool staged = A <= kStageAnts;
    // the ants' fingerprints come from fingerprint_kernel
    if (staged)
        for (std::uint32_t a = threadIdx.x; a < A; a += blockDim.x) {
            sh.ant_cost[a] = cv.ant_costs[a];
            sh.ant_id[a] = {cv.ant_ids[2 * a], cv.ant_ids[2 * a + 1]};
            sh.ant_p0[a] = cv.ant_p0[a];
        }
    if (threadIdx.x == 0) sh.collision = 0;
    __syncthreads();
    const bool improved = st.global_cost < ctl.tracked_global;
    const CandidateView v = candidates(cv, sh, A);
    const std::uint32_t total = kArchive + A;
    // groups of equal (cost, fingerprint); a fingerprint shared across costs,
    // or by two different tours, sends the selection to the general path
    for (std::uint32_t c = threadIdx.x; c < total; c += blockDim.x) {
        std::uint16_t r = 0xffffu;
        if (c >= kArchive || c < ctl.archive_size) {
            r = (std::uint16_t)c;
            const Fingerprint fc = v.id(c);
            const long long cc = v.cost(c);
            for (std::uint32_t q = 0; q < c; ++q) {
                if (q < kArchive && q >= ctl.archive_size) continue;
                if (!fp_equal(v.id(q), fc)) continue;
                if (v.cost(q) == cc) { r = (std::uint16_t)q; break; }
                sh.collision = 1;
            }
        }
        sh.rep[c] = r;
    }
    __syncthreads();
    for (std::uint32_t c = warp; c < total; c += warps) {
        const std::uint32_t r = sh.rep[c];
        if (r != 0xffffu && r != c && warp_canonical_compare(v.ref(c), v.ref(r), n, lane) != 0 && lane == 0)
            sh.collision = 1;
    }
    __syncthreads();
    if (warp == 0) {
        const std::uint32_t count =
            sh.collision ? ref_archive_select(v, st, A, improved, n, lane, sh.excluded, sh.chosen)
                         : ref_archive_select_groups(v, st, A, improved, lane, sh.rep, sh.excluded, sh.chosen);
        if (lane == 0) {
            sh.count = count;
            for (std::uint32_t i = 0; i < count; ++i) {
                sh.chosen_cost[i] = v.cost(sh.chosen[i]);
                sh.chosen_id[i] = v.id(sh.chosen[i]);
            }
        }
    } else if (warp == 1) {
        // feedback (update_feedback, control_ops.hpp:177-188), beside the
        // selection: the LS work fractions summed in ant order
        std::uint32_t returned = 0;
        double work = 0;
        for (std::uint32_t base = 0; base < A; base += 32) {
            const std::uint32_t a = base + lane;
            bool back = false;
            double wa = 0.0;
            if (a < A) {
                back = fp_equal(v.id(kArchive + a), ctl.active_id);
                if (P.ls_limit) wa = (double)cv.ant_counts[3 * a + 1] / (double)P.ls_limit;
            }
            returned += __popc(__ballot_sync(kFull, back));
            for (std::uint32_t j = 0; j < 32 && base + j < A; ++j) work += __shfl_sync(kFull, wa, j);
        }
        if (lane == 0) {
            const float rf = (float)unit_clip((double)returned / (double)A), wf = (float)unit_clip(work / (double)A);
            ctl.return_rate += (rf - ctl.return_rate) * 0.0625f;
            ctl.ls_work += (wf - ctl.ls_work) * 0.0625f;
            if (improved) ctl.stagnant_batches = 0;
            else if (ctl.stagnant_batches != ~0ull) ++ctl.stagnant_batches;
            if (ctl.epoch_batches != ~0ull) ++ctl.epoch_batches;
            const Fingerprint best = v.id(kArchive + st.iteration_best);
            if (st.epoch_cost < ctl.tracked_epoch) ctl.epoch_id = best;
            ctl.active_id = st.source_is_epoch ? ctl.epoch_id : best;
            ctl.tracked_global = st.global_cost;
            ctl.tracked_epoch = st.epoch_cost;
        }
    }
    __syncthreads();
    // chosen tours into the other half of the archive buffer
    const std::uint32_t next = ctl.side ^ 1u, count = sh.count;
    for (std::uint32_t i = threadIdx.x; i < count * n; i += blockDim.x) {
        const std::uint32_t slot = i / n, p = i % n;
        const node_t node = v.ref(sh.chosen[slot]).tour[p];
        node_t* dst = archive_tour(cv, next, slot);
        dst[p] = node;
        dst[cv.n_pad + node] = (node_t)p;
        if (node == 0) sh.next_p0[slot] = p;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (std::uint32_t i = 0; i < kArchive; ++i) {
            ctl.archive_cost[i] = i < count ? sh.chosen_cost[i] : 0;
            ctl.archive_id[i] = i < count ? sh.chosen_id[i] : Fingerprint{0, 0};
            ctl.archive_p0[i] = i < count ? sh.next_p0[i] : 0u;
        }
        ctl.archive_size = count;
        ctl.side = next;
    }
    __syncthreads();
}

// The decision before batch `batch` (build_control_features, score and
// apply_control_action).  Called by the whole block; st and sh.ctl shared.
__device__ void ref_decide(const ColonyView& cv, const InstanceView& in, ColonyState& st, const ColonyParams& P,
                           std::uint32_t colony, std::uint32_t colony_count, std::uint32_t batch,
                           std::uint32_t parent_p0, RefShared& sh) {
    RefControl& ctl = sh.ctl;
    const std::uint32_t n = in.n, k = in.k;
    const std::uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    const std::uint32_t side = ctl.side, size = ctl.archive_size;
    if (warp == 0) {
        // alternative reference: the archive tour other than the active one
        // that differs most from it on the sampled nodes (control_cpu.cpp:46-63);
        // each lane takes samples lane and lane + 32 of every archive tour
        const TourRef parent{cv.parent, nullptr, parent_p0};
        std::uint32_t x[2], ps[2], pp[2], missing[kArchive] = {0, 0, 0, 0};
        bool have[2];
        for (std::uint32_t h = 0; h < 2; ++h) {
            have[h] = lane + 32 * h < in.sample_count;
            x[h] = have[h] ? in.samples[lane + 32 * h] : 0u;
        }
        std::uint32_t pos[kArchive][2];
        for (std::uint32_t h = 0; h < 2; ++h) {
            const std::uint32_t nb = have[h] ? cv.parent_nbr[x[h]] : 0u;
            ps[h] = nb & 0xffffu;
            pp[h] = nb >> 16;
#pragma unroll
            for (std::uint32_t i = 0; i < kArchive; ++i)
                pos[i][h] = have[h] && i < size ? archive_tour(cv, side, i)[cv.n_pad + x[h]] : 0u;
        }
#pragma unroll
        for (std::uint32_t i = 0; i < kArchive; ++i) {
            if (i >= size) continue;
            const node_t* t = archive_tour(cv, side, i);
            for (std::uint32_t h = 0; h < 2; ++h) {
                if (!have[h]) continue;
                const std::uint32_t px = pos[i][h];
                const std::uint32_t cs = t[px + 1 == n ? 0 : px + 1], cp = t[px == 0 ? n - 1 : px - 1];
                missing[i] += (cs != ps[h] && cs != pp[h]) + (cp != ps[h] && cp != pp[h]);
            }
        }
#pragma unroll
        for (std::uint32_t i = 0; i < kArchive; ++i)
            for (int o = 16; o; o >>= 1) missing[i] += __shfl_xor_sync(kFull, missing[i], o);
        std::uint32_t alt = kArchive, largest = 0;
        for (std::uint32_t i = 0; i < size; ++i) {
            const TourRef ri{archive_tour(cv, side, i), archive_tour(cv, side, i) + cv.n_pad, ctl.archive_p0[i]};
            if (fp_equal(ctl.archive_id[i], ctl.active_id) && warp_canonical_compare(ri, parent, n, lane) == 0)
                continue;
            bool better_tie = false;
            if (alt != kArchive && missing[i] == largest) {
                const long long ci = ctl.archive_cost[i], ca = ctl.archive_cost[alt];
                const Fingerprint fi = ctl.archive_id[i], fa = ctl.archive_id[alt];
                const TourRef ra{archive_tour(cv, side, alt), archive_tour(cv, side, alt) + cv.n_pad,
                                 ctl.archive_p0[alt]};
                better_tie = ci < ca || (ci == ca && (fp_less(fi, fa) ||
                                                      (fp_equal(fi, fa) && warp_canonical_compare(ri, ra, n, lane) < 0)));
            }
            if (alt == kArchive || missing[i] > largest || better_tie) { alt = i; largest = missing[i]; }
        }
        if (lane == 0) {
            sh.alternative = alt;
            sh.largest = largest;
            sh.gap[0] = (float)unit_clip(((double)st.parent_cost / (double)st.global_cost - 1) / kArchiveBand);
            sh.gap[1] = alt < kArchive ? (float)unit_clip(((double)ctl.archive_cost[alt] / (double)st.global_cost - 1) /
                                                          kArchiveBand)
                                       : 0.0f;
            sh.difference = alt < kArchive ? (float)largest / (float)(2 * in.sample_count) : 0.0f;
            sh.mask = cv.action_mask & (alt < kArchive ? 0xFFFFFFFFu : 0xFFFFu);
            sh.elapsed = (float)unit_clip((double)((unsigned long long)batch * P.ants) /
                                          (double)((unsigned long long)P.total_iterations * P.ants));
            const unsigned long long stag = ctl.stagnant_batches;
            sh.stagnation = (float)(stag < 32 ? (double)stag / 32.0 : 1.0);
        }
    }
    __syncthreads();
    const std::uint32_t alt = sh.alternative, count = n < kRegionNodes ? n : kRegionNodes;
    for (std::uint32_t w = warp; w < 8; w += warps) {
        // start region (mode, region) and its 4 features (region_features,
        // control_ops.hpp:192-214); lane 2i + s takes node i and its
        // predecessor (s = 0) or successor (s = 1); sums in node order
        const std::uint32_t mode = w >> 2, region = w & 3u;
        const bool valid = mode == 0 || alt < kArchive;
        node_t* nodes = sh.regions[w];
        const node_t* rtour = mode == 0 ? cv.parent : archive_tour(cv, side, alt < kArchive ? alt : 0);
        if (valid) {
            warp_build_region(rtour, n, in.primary, k, cv.key, batch, mode, region, nodes, lane);
        } else {
            if (lane < kRegionNodes) nodes[lane] = 0;
            __syncwarp();
        }
        float regional[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (valid) {
            const std::uint32_t i = lane >> 1, s = lane & 1u;
            const bool active = i < count;
            double half = 0.0, strength_v = 0.0;
            std::uint32_t dis = 0, disp = 0;
            std::uint32_t xn = 0, y = 0;
            if (active) {
                xn = nodes[i];
                if (mode == 0) {
                    const std::uint32_t nb = cv.parent_nbr[xn];
                    y = s ? nb & 0xffffu : nb >> 16;
                } else {
                    const std::uint32_t px = rtour[cv.n_pad + xn];
                    y = s ? rtour[px + 1 == n ? 0 : px + 1] : rtour[px == 0 ? n - 1 : px - 1];
                }
                std::uint32_t pj[kArchive];
#pragma unroll
                for (std::uint32_t j = 0; j < kArchive; ++j) pj[j] = j < size ? archive_tour(cv, side, j)[cv.n_pad + xn] : 0u;
                const int2 a = in.xy[xn], b = in.xy[y];
                half = 0.5 * (double)euc2d(a, b);
                float tau = st.default_trail;
                for (std::uint32_t t = 0; t < k; ++t)
                    if (in.primary[(size_t)xn * k + t] == y) { tau = cv.trails[(size_t)xn * k + t]; break; }
#pragma unroll
                for (std::uint32_t j = 0; j < kArchive; ++j) {
                    if (j >= size) continue;
                    const node_t* t = archive_tour(cv, side, j);
                    const std::uint32_t sj = t[pj[j] + 1 == n ? 0 : pj[j] + 1], qj = t[pj[j] == 0 ? n - 1 : pj[j] - 1];
                    dis += sj != y && qj != y;
                }
                const double lo = (double)st.tau_min, hi = (double)st.tau_max;
                strength_v = lo == hi ? 1.0 : unit_clip(((double)tau - lo) / (hi - lo));
                disp = !has_node(nodes, count, y);
            }
            const double other = __shfl_down_sync(kFull, half, 1);
            double ex = 0.0;
            if (active && s == 0) {
                const double scale = in.local_scale[xn] < in.scale_epsilon ? in.scale_epsilon : in.local_scale[xn];
                ex = unit_clip(((half + other) / scale - 1) / 3);
            }
            double excess = 0, strength = 0;
            for (std::uint32_t q = 0; q < count; ++q) {
                excess += __shfl_sync(kFull, ex, 2 * q);
                strength += __shfl_sync(kFull, strength_v, 2 * q);
                strength += __shfl_sync(kFull, strength_v, 2 * q + 1);
            }
            for (int o = 16; o; o >>= 1) {
                dis += __shfl_xor_sync(kFull, dis, o);
                disp += __shfl_xor_sync(kFull, disp, o);
            }
            // a ratio of small integers rounds to the same float directly as
            // through double; division by 16 or 32 is an exact scaling
            if (count == kRegionNodes) {
                regional[0] = (float)(excess * (1.0 / kRegionNodes));
                regional[2] = (float)(strength * (0.5 / kRegionNodes));
            } else {
                regional[0] = (float)(excess / count);
                regional[2] = (float)(strength / (double)(2 * count));
            }
            regional[1] = __fdiv_rn((float)dis, (float)(2 * count * size));
            regional[3] = __fdiv_rn((float)disp, (float)(2 * count));
        }
        if (lane < 4) {
            const std::uint32_t level = lane, a = mode * 16 + region * 4 + level;
            sh.feat[0][a] = sh.elapsed;
            sh.feat[1][a] = sh.stagnation;
            sh.feat[2][a] = ctl.return_rate;
            sh.feat[3][a] = ctl.ls_work;
            sh.feat[4][a] = (float)mode;
            sh.feat[5][a] = (float)(level + 1) * 0.25f;
            sh.feat[6][a] = sh.gap[mode];
            sh.feat[7][a] = mode ? sh.difference : 0.0f;
            for (int f = 0; f < 4; ++f) sh.feat[8 + f][a] = regional[f];
        }
    }
    __syncthreads();
    if (warp == 0) {
        const std::uint32_t mask = sh.mask;
        std::uint32_t a;
        if (cv.controller_kind == 1) {
            sh.scores[lane] = 0.0f;
            __syncwarp();
            a = choose_conditional(cv.program, [&](int i, std::uint32_t act) { return sh.feat[i][act]; }, mask, lane,
                                   sh.scores);
        } else {
            const float value = eval_program(*cv.program, [&](int i) { return sh.feat[i][lane]; });
            sh.scores[lane] = value;
            a = choose_action(value, (mask >> lane) & 1u, lane);
        }
        __syncwarp();
        const std::uint32_t chosen = a < 32 ? a : 0;
        const DecisionCapture& cap = P.capture;
        for (std::uint32_t i = 0; i < cap.count; ++i) {
            if (cap.points[i] != batch + 1) continue;
            const size_t slot = (size_t)i * colony_count + colony;
            for (std::uint32_t f = 0; f < 12; ++f) cap.features[(slot * 12 + f) * 32 + lane] = sh.feat[f][lane];
            cap.scores[slot * 32 + lane] = sh.scores[lane];
            if (lane == 0) {
                cap.masks[slot] = mask;
                cap.actions[slot] = (std::int32_t)chosen;
            }
        }
        if (lane == 0) {
            sh.action = chosen;
            st.action = (std::int32_t)chosen;
            st.mne_target = 2u << (chosen & 3u);
            st.region = 5;
            ctl.alternative = alt;
            ctl.legal_mask = mask;
            ctl.start_count = count;
            if (chosen >= 16) {
                // restart from the alternative reference (control_state.cuh:302-336)
                st.epoch_cost = st.parent_cost = ctl.archive_cost[alt];
                trail_limits(st.epoch_cost, P.retention, P.p_root, k, st.tau_min, st.tau_max);
                st.default_trail = st.tau_max;
                st.source_is_epoch = 0;
                st.iteration_best = 0;
                ctl.tracked_epoch = st.epoch_cost;
                ctl.active_id = ctl.epoch_id = ctl.archive_id[alt];
                ctl.return_rate = ctl.ls_work = 0.0f;
                ctl.epoch_batches = 0;
                if (ctl.restarts != ~0ull) ++ctl.restarts;
            }
        }
        if (lane < kRegionNodes)
            ctl.start_nodes[lane] = sh.regions[(chosen >> 4) * 4 + ((chosen >> 2) & 3u)][lane];
    }
    __syncthreads();
    if (sh.action >= 16) {
        const node_t* tour = archive_tour(cv, side, alt);
        for (std::uint32_t i = threadIdx.x; i < n; i += blockDim.x) cv.parent[i] = cv.epoch[i] = tour[i];
        __syncthreads();
        for (std::uint32_t i = threadIdx.x; i < n; i += blockDim.x)
            cv.parent_nbr[cv.parent[i]] = (std::uint32_t)cv.parent[i + 1 == n ? 0 : i + 1] |
                                          ((std::uint32_t)cv.parent[i == 0 ? n - 1 : i - 1] << 16);
        const float tmax = st.tau_max;
        for (std::uint32_t i = threadIdx.x; i < n * k; i += blockDim.x) {
            cv.trails[i] = tmax;
            cv.products[i] = tmax * cv.eta[i];
        }
    }
    __syncthreads();
}

// Departure-only prior products (departure_rows) of the colonies whose mode
// is 1, one block per colony: run after the prior's heuristic is applied.
__global__ void __launch_bounds__(256) prior_rows_kernel(const InstanceView* instances, const ColonyView* colonies,
                                                         const std::uint32_t* modes) {
    const std::uint32_t c = blockIdx.x;
    if (!modes[c]) return;
    const ColonyView cv = colonies[c];
    const InstanceView in = instances[cv.instance];
    departure_rows(in, cv, threadIdx.x, blockDim.x, in.n);
}

// Fingerprints (and node-0 positions) of every ant's tour of a batch, one
// warp per ant over the colonies of `list` (all colonies when null)
// (fingerprint_ants, control_state.cuh:45-64); `zero` forces every
// fingerprint to 0 (the collision diagnostic).
__global__ void __launch_bounds__(256) fingerprint_kernel(const ColonyView* colonies, const std::uint32_t* list,
                                                          std::uint32_t ants, std::uint32_t colony_count,
                                                          std::uint32_t zero) {
    const std::uint32_t job = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (job >= ants * colony_count) return;
    const std::uint32_t slot = job / ants, ant = job % ants;
    const std::uint32_t colony = list ? list[slot] : slot;
    const ColonyView& cv = colonies[colony];
    std::uint32_t p0;
    const Fingerprint f = warp_fingerprint(cv.ant_tours + (size_t)ant * cv.n_pad, cv.n, lane, p0);
    if (lane == 0) {
        cv.ant_ids[2 * ant] = zero ? 0ull : f.first;
        cv.ant_ids[2 * ant + 1] = zero ? 0ull : f.second;
        cv.ant_p0[ant] = p0;
    }
}

__global__ void colony_init_kernel(const InstanceView* instances, const ColonyView* colonies, ColonyState* states,
                                   ColonyParams P, std::uint32_t colony_count) {
    const std::uint32_t c = blockIdx.x;
    const ColonyView cv = colonies[c];
    const InstanceView in = instances[cv.instance];
    const std::uint32_t n = in.n, k = in.k;
    __shared__ float s_tmax;
    __shared__ ColonyState s_st;
    if (threadIdx.x == 0) {
        ColonyState st{};
        st.epoch_cost = st.global_cost = st.parent_cost = st.iteration_best_cost = in.initial_cost;
        trail_limits(in.initial_cost, P.retention, P.p_root, k, st.tau_min, st.tau_max);
        st.default_trail = st.tau_max;
        st.mne_target = P.mne_target;
        st.action = -1;
        st.region = 4;
        states[c] = st;
        s_st = st;
        s_tmax = st.tau_max;
    }
    for (std::uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const node_t v = in.initial[i];
        cv.parent[i] = cv.epoch[i] = cv.global[i] = v;
        cv.parent_nbr[v] = (std::uint32_t)in.initial[i + 1 == n ? 0 : i + 1] |
                           ((std::uint32_t)in.initial[i == 0 ? n - 1 : i - 1] << 16);
    }
    __syncthreads();
    const float tmax = s_tmax;
    for (std::uint32_t i = threadIdx.x; i < n * k; i += blockDim.x) {
        cv.trails[i] = tmax;
        cv.eta[i] = in.eta[i];
        cv.products[i] = tmax * in.eta[i];
    }
    if (P.ref_control && cv.control) {
        // the archive holds the initial tour (initialize_control,
        // control_state.cuh:21-43); then the decision before batch 0
        __shared__ RefShared s_ref;
        node_t* a0 = archive_tour(cv, 0, 0);
        for (std::uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            a0[i] = in.initial[i];
            a0[cv.n_pad + in.initial[i]] = (node_t)i;
        }
        __shared__ std::uint32_t s_p0;
        if (threadIdx.x < 32) {
            std::uint32_t p0;
            Fingerprint f = warp_fingerprint(in.initial, n, threadIdx.x, p0);
            if (P.zero_fingerprints) f = Fingerprint{0, 0};
            if (threadIdx.x == 0) {
                s_p0 = p0;
                RefControl ctl{};
                ctl.archive_size = 1;
                ctl.archive_cost[0] = in.initial_cost;
                ctl.archive_id[0] = f;
                ctl.archive_p0[0] = p0;
                ctl.active_id = ctl.epoch_id = f;
                ctl.tracked_global = ctl.tracked_epoch = in.initial_cost;
                ctl.alternative = kArchive;
                s_ref.ctl = ctl;
            }
        }
        __syncthreads();
        ref_decide(cv, in, s_st, P, c, colony_count, 0, s_p0, s_ref);
        if (threadIdx.x == 0) {
            states[c] = s_st;
            *cv.control = s_ref.ctl;
        }
    }
}

__device__ __forceinline__ void write_trace(TraceRow& row, const ColonyState& st, std::uint32_t mne,
                                            std::int32_t action, unsigned long long steps, unsigned long long evals) {
    row.iteration_best_cost = st.iteration_best_cost;
    row.global_cost = st.global_cost;
    row.parent_cost = st.parent_cost;
    row.iteration_best = st.iteration_best;
    row.source_is_epoch = st.source_is_epoch;
    row.tau_min = st.tau_min;
    row.tau_max = st.tau_max;
    row.mne_target = mne;
    row.action = action;
    row.construction_steps = steps;
    row.ls_evaluations = evals;
}

// Fused reduce_and_select + update_pheromone for one colony, then (GP-controlled
// evaluations) the controller decision for the next iteration.  Block b
// updates colony list[b] (colony b when `list` is null); `colony_count` is
// the evaluation's colony count.
__global__ void __launch_bounds__(256) colony_update_kernel(const InstanceView* instances,
                                                            const ColonyView* colonies, ColonyState* states,
                                                            ColonyParams P, TraceRow* trace,
                                                            const std::uint32_t* list,
                                                            std::uint32_t colony_count, std::uint32_t trace_cap) {
    const std::uint32_t c = list ? list[blockIdx.x] : blockIdx.x;
    const ColonyView cv = colonies[c];
    const InstanceView in = instances[cv.instance];
    const std::uint32_t n = in.n, k = in.k, A = P.ants;
    const std::uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    __shared__ unsigned long long s_red[6][8];
    __shared__ ColonyState s_st;
    __shared__ std::uint32_t s_best, s_improve_epoch, s_improve_global, s_from_epoch, s_restart;
    __shared__ float s_tmin, s_tmax, s_inc, s_feat[7];
    __shared__ long long s_sum_final, s_sum_cons, s_best_cost;
    __shared__ unsigned long long s_steps, s_evals;
    __shared__ std::uint32_t s_used_mne, s_parent_p0;

    // iteration best: first strict minimum over ants (costs are >= 0); work counters
    unsigned long long best = ~0ull, steps = 0, evals = 0, moved = 0, sum_final = 0, sum_cons = 0;
    for (std::uint32_t a = threadIdx.x; a < A; a += blockDim.x) {
        const unsigned long long key = ((unsigned long long)cv.ant_costs[a] << 16) | a;
        best = key < best ? key : best;
        steps += cv.ant_counts[3 * a];
        evals += cv.ant_counts[3 * a + 1];
        moved += cv.ant_counts[3 * a + 2];
        sum_final += (unsigned long long)cv.ant_costs[a];
        sum_cons += (unsigned long long)cv.ant_ccosts[a];
    }
    for (int o = 16; o; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(kFull, best, o);
        best = other < best ? other : best;
        steps += __shfl_xor_sync(kFull, steps, o);
        evals += __shfl_xor_sync(kFull, evals, o);
        moved += __shfl_xor_sync(kFull, moved, o);
        sum_final += __shfl_xor_sync(kFull, sum_final, o);
        sum_cons += __shfl_xor_sync(kFull, sum_cons, o);
    }
    if (lane == 0) {
        s_red[0][warp] = best; s_red[1][warp] = steps; s_red[2][warp] = evals;
        s_red[3][warp] = moved; s_red[4][warp] = sum_final; s_red[5][warp] = sum_cons;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (std::uint32_t w = 1; w < warps; ++w) {
            best = s_red[0][w] < best ? s_red[0][w] : best;
            steps += s_red[1][w]; evals += s_red[2][w]; moved += s_red[3][w];
            sum_final += s_red[4][w]; sum_cons += s_red[5][w];
        }
        ColonyState st = states[c];
        const std::uint32_t ib = (std::uint32_t)(best & 0xffffu);
        const long long cost = (long long)(best >> 16);
        const bool ie = cost < st.epoch_cost, ig = cost < st.global_cost;
        if (ie) st.epoch_cost = cost;
        if (ig) { st.global_cost = cost; st.last_improvement = st.iteration + 1; }
        trail_limits(st.epoch_cost, P.retention, P.p_root, k, st.tau_min, st.tau_max);
        const bool from_epoch = source_uniform(cv.key, st.iteration) < P.epoch_source_probability;
        st.parent_cost = from_epoch ? st.epoch_cost : cost;
        st.iteration_best = ib;
        st.iteration_best_cost = cost;
        st.source_is_epoch = from_epoch;
        st.construction_steps += steps;
        st.ls_evaluations += evals;
        st.reversed_elements += moved;
        st.default_trail = fmaxf(st.tau_min, st.default_trail * P.retention_f);
        s_st = st;
        s_best = ib; s_improve_epoch = ie; s_improve_global = ig; s_from_epoch = from_epoch;
        s_tmin = st.tau_min; s_tmax = st.tau_max;
        s_inc = (float)(1.0 / (double)st.parent_cost);
        s_sum_final = (long long)sum_final; s_sum_cons = (long long)sum_cons; s_best_cost = cost;
        s_steps = steps; s_evals = evals; s_used_mne = st.mne_target;
        s_restart = 0;
    }
    __syncthreads();
    const node_t* best_tour = cv.ant_tours + (size_t)s_best * cv.n_pad;
    const bool ie = s_improve_epoch, ig = s_improve_global, fe = s_from_epoch;
    for (std::uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const node_t v = best_tour[i];
        if (ie) cv.epoch[i] = v;
        if (ig) cv.global[i] = v;
        const node_t p = fe ? cv.epoch[i] : v;
        cv.parent[i] = p;
        if (p == 0) s_parent_p0 = i;
    }
    __syncthreads();
    for (std::uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        cv.parent_nbr[cv.parent[i]] = (std::uint32_t)cv.parent[i + 1 == n ? 0 : i + 1] |
                                      ((std::uint32_t)cv.parent[i == 0 ? n - 1 : i - 1] << 16);
    __syncthreads();
    if (P.trail_blocks <= 1) {
        trail_update(n, k, in.primary, cv.parent_nbr, P.retention_f, s_tmin, s_tmax, s_inc, cv.eta, cv.trails,
                     cv.products, threadIdx.x, blockDim.x);
        if (P.prior_rows && P.prior_rows[c]) {
            __syncthreads();
            departure_rows(in, cv, threadIdx.x, blockDim.x, n);
        }
    }
    std::int32_t action = -1;
    if (P.ref_control) {
        // the 12-feature controller: the trace row holds the action this
        // batch ran with; archive and feedback; the next batch's decision
        __shared__ RefShared s_ref;
        if (threadIdx.x == 0) {
            s_ref.ctl = *cv.control;
            if (trace && s_st.iteration < trace_cap)
                write_trace(trace[(size_t)s_st.iteration * colony_count + c], s_st, s_used_mne, s_st.action, s_steps,
                            s_evals);
        }
        __syncthreads();
        ref_update(cv, in, s_st, P, s_ref);
        if (s_st.iteration + 1 < P.total_iterations)
            ref_decide(cv, in, s_st, P, c, colony_count, s_st.iteration + 1, s_parent_p0, s_ref);
        if (threadIdx.x == 0) *cv.control = s_ref.ctl;
    } else if (P.controlled && cv.program) {
        // mean normalised entropy of the trail rows (exact integer sum)
        __syncthreads();
        unsigned long long q = 0;
        for (std::uint32_t row = threadIdx.x; row < n; row += blockDim.x)
            q += row_entropy_q(cv.trails + (size_t)row * k, k, P.log2k);
        for (int o = 16; o; o >>= 1) q += __shfl_xor_sync(kFull, q, o);
        if (lane == 0) s_red[0][warp] = q;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (std::uint32_t w = 1; w < warps; ++w) q += s_red[0][w];
            const ColonyState& st = s_st;
            const std::uint32_t t1 = st.iteration + 1, stag = t1 - st.last_improvement, age = t1 - st.last_restart;
            const long long b = s_best_cost;
            s_feat[0] = (float)t1 / (float)P.total_iterations;
            s_feat[1] = (float)stag / (float)(stag + 16);
            s_feat[2] = clamp01((double)(s_sum_final - (long long)A * b) / ((double)A * (double)b));
            s_feat[3] = clamp01((double)q * (1.0 / 1048576.0) / (double)n);
            s_feat[4] = (float)st.restarts / (float)(st.restarts + 1);
            s_feat[5] = clamp01((double)(s_sum_cons - s_sum_final) / (double)s_sum_cons * 10.0);
            s_feat[6] = (float)age / (float)(age + 16);
        }
        __syncthreads();
        if (warp == 0) {
            // features of action a: the 7 colony features, then its MNE level,
            // start region and restart flag
            auto feature_of = [&](int i, std::uint32_t a) {
                return i < 7 ? s_feat[i] : i == 7 ? (float)(a & 3u) / 3.0f : i == 8 ? (float)((a >> 2) & 3u) / 3.0f
                                                   : i == 9 ? (a >= 16u ? 1.0f : 0.0f) : 0.0f;
            };
            std::uint32_t a;
            if (cv.controller_kind == 1) {
                a = choose_conditional(cv.program, feature_of, cv.action_mask, lane, nullptr);
            } else {
                const float value = eval_program(*cv.program, [&](int i) { return feature_of(i, lane); });
                a = choose_action(value, (cv.action_mask >> lane) & 1u, lane);
            }
            if (lane == 0) {
                const std::uint32_t chosen = a < 32 ? a : 0;
                s_st.action = (std::int32_t)chosen;
                s_st.mne_target = 2u << (chosen & 3u);
                s_st.region = (chosen >> 2) & 3u;
                if (chosen >= 16) {
                    s_restart = 1;
                    ++s_st.restarts;
                    s_st.last_restart = s_st.iteration + 1;
                    s_st.epoch_cost = s_st.global_cost;
                    s_st.parent_cost = s_st.global_cost;
                    trail_limits(s_st.epoch_cost, P.retention, P.p_root, k, s_st.tau_min, s_st.tau_max);
                    s_st.default_trail = s_st.tau_max;
                }
            }
        }
        __syncthreads();
        action = s_st.action;
        if (s_restart) {
            // restart: parent and epoch <- global best, trails <- tau_max
            for (std::uint32_t i = threadIdx.x; i < n; i += blockDim.x) cv.parent[i] = cv.epoch[i] = cv.global[i];
            __syncthreads();
            for (std::uint32_t i = threadIdx.x; i < n; i += blockDim.x)
                cv.parent_nbr[cv.parent[i]] = (std::uint32_t)cv.parent[i + 1 == n ? 0 : i + 1] |
                                              ((std::uint32_t)cv.parent[i == 0 ? n - 1 : i - 1] << 16);
            const float tmax = s_st.tau_max;
            for (std::uint32_t i = threadIdx.x; i < n * k; i += blockDim.x) {
                cv.trails[i] = tmax;
                cv.products[i] = tmax * cv.eta[i];
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        ColonyState st = s_st;
        if (trace && st.iteration < trace_cap && !P.ref_control)
            write_trace(trace[(size_t)st.iteration * colony_count + c], st, s_used_mne, action, s_steps, s_evals);
        ++st.iteration;
        states[c] = st;
    }
}

// The trail update of large candidate matrices, after the colony update has
// chosen the parent and the trail limits (it leaves the trails alone when
// P.trail_blocks > 1): block (x, y) updates rows [n x / X, n (x+1) / X) of
// colony y of the launch (of `list`, or all when null) -- evaporation,
// deposit on the parent's edges, bounds and products exactly as the colony
// update would -- then, for a colony whose prior re-ranks departures, those
// rows' products.  One block per colony streams a large matrix at a small
// fraction of the memory bandwidth; X blocks per colony fill the GPU.
__global__ void __launch_bounds__(256) colony_trails_kernel(const InstanceView* instances,
                                                            const ColonyView* colonies, const ColonyState* states,
                                                            ColonyParams P, const std::uint32_t* list) {
    const std::uint32_t c = list ? list[blockIdx.y] : blockIdx.y;
    const ColonyView cv = colonies[c];
    const InstanceView in = instances[cv.instance];
    const std::uint32_t n = in.n, k = in.k;
    const std::uint32_t r0 = (std::uint32_t)((unsigned long long)n * blockIdx.x / gridDim.x);
    const std::uint32_t r1 = (std::uint32_t)((unsigned long long)n * (blockIdx.x + 1) / gridDim.x);
    if (r0 >= r1) return;
    const ColonyState& st = states[c];
    const float tmin = st.tau_min, tmax = st.tau_max, inc = (float)(1.0 / (double)st.parent_cost);
    const std::size_t off = (std::size_t)r0 * k;
    trail_update(r1 - r0, k, in.primary + off, cv.parent_nbr + r0, P.retention_f, tmin, tmax, inc, cv.eta + off,
                 cv.trails + off, cv.products + off, threadIdx.x, blockDim.x);
    if (P.prior_rows && P.prior_rows[c]) {
        __syncthreads();
        departure_rows(in, cv, r0 + threadIdx.x, blockDim.x, r1);
    }
}

__global__ void pheromone_step_kernel(std::uint32_t n, std::uint32_t k, const node_t* primary,
                                      const std::uint32_t* parent_nbr, float ret, float tmin, float tmax, float inc,
                                      const float* eta, float* trails, float* products) {
    trail_update(n, k, primary, parent_nbr, ret, tmin, tmax, inc, eta, trails, products,
                 blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// ---------------------------------------------------------------------------
// GP scoring: one warp per colony, lane = action (cuda/gp_score.cuh:64-102).
// ---------------------------------------------------------------------------
// Controllers (3 tree slots each, kinds[i]): joint ones score all 32 lanes,
// conditional ones write their role scores to slots 0-9 of the colony's row.
__global__ void score_controllers_kernel(const Program* trees, const std::uint32_t* kinds, std::uint32_t replicas,
                                         const float* features, const std::uint32_t* masks, float* scores,
                                         std::int32_t* actions, std::uint32_t colonies) {
    const std::uint32_t colony = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (colony >= colonies) return;
    const std::uint32_t controller = colony / replicas;
    const Program* slots = trees + 3 * (size_t)controller;
    auto feature_of = [&](int i, std::uint32_t a) { return features[((size_t)i * colonies + colony) * 32 + a]; };
    std::uint32_t chosen;
    if (kinds[controller] == 1) {
        chosen = choose_conditional(slots, feature_of, masks[colony], lane, scores + (size_t)colony * 32);
    } else {
        const float value = eval_program(slots[0], [&](int i) { return feature_of(i, lane); });
        scores[(size_t)colony * 32 + lane] = value;
        chosen = choose_action(value, (masks[colony] >> lane) & 1u, lane);
    }
    if (lane == 0) actions[colony] = (std::int32_t)chosen;
}

__global__ void score_kernel(const Program* programs, std::uint32_t replicas, const float* features,
                             const std::uint32_t* masks, float* scores, std::int32_t* actions,
                             std::uint32_t colonies) {
    const std::uint32_t colony = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (colony >= colonies) return;
    const Program& p = programs[colony / replicas];
    const float value =
        eval_program(p, [&](int i) { return features[((size_t)i * colonies + colony) * 32 + lane]; });
    scores[(size_t)colony * 32 + lane] = value;
    const std::uint32_t chosen = choose_action(value, (masks[colony] >> lane) & 1u, lane);
    if (lane == 0) actions[colony] = (std::int32_t)chosen;
}

}  // namespace faco

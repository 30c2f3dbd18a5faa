// faco_kernels.cu -- the FACO iteration kernels for sm_103a.
//
//   ant_kernel<mode>        construction + local search, one warp per ant
//   colony_init_kernel      reset_colony + initialize_products
//                           (cuda/colony_state.cuh:72-110)
//   colony_update_kernel    reduce_and_select + update_pheromone fused, one
//                           block per colony (cuda/colony_state.cuh:148-229)
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
    constexpr bool kEngine = engine_mode(MODE), kGlobalWs = MODE == kModeEngineGlobal;
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
        if (kEngine) current = region_start(key, batch, ant, in_ptr, region);
        else if (MODE == kModeVisits) current = L.task_visits[(size_t)task * n];
        else current = L.task_starts[task];
        if (L.out_selected && lane == 0) L.out_selected[(size_t)task * n] = (node_t)current;
        if (lane == 0) s.visited[current >> 5] |= 1u << (current & 31u);
        __syncwarp();
        const float* products = kEngine ? cv.products : L.task_products;
        const std::uint32_t k = in.k, b = in.b;
        const unsigned long long loop_cap = 2ull * n + 2;
        unsigned long long guard = 0;
        while (r.mne < target && r.steps + 1 < n) {
            if (++guard > loop_cap) { if (lane == 0) atomicOr(L.error, kErrLoopCap); break; }
            const std::uint32_t step = r.steps + 1;
            // loads that depend only on `current`, issued first
            const std::uint32_t pnbr = __ldg(parent_nbr + current);
            std::uint32_t cand = n;
            float p = 0.0f;
            if (MODE != kModeVisits && lane < k) {
                cand = __ldg(in.primary + (size_t)current * k + lane);
                p = __ldg(products + (size_t)current * k + lane);
            }
            std::uint32_t selected = n;
            if (MODE == kModeVisits) {
                selected = L.task_visits[(size_t)task * n + step];
            } else {
                std::uint32_t rhi = 0, rlo = 0;
                double u_given = 0.0;
                float uf;
                if (kEngine) {
                    const uint4v rb = philox4x32(step, ant, batch, 0, (std::uint32_t)key, (std::uint32_t)(key >> 32));
                    rhi = rb.x;
                    rlo = rb.y;
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
            const std::uint32_t npos = s.pos[selected], tpos = s.pos[current];
            const std::uint32_t previous = s.tour[npos == 0 ? n - 1 : npos - 1];
            const std::uint32_t after = s.tour[npos + 1 == n ? 0 : npos + 1];
            const std::uint32_t target_after = s.tour[tpos + 1 == n ? 0 : tpos + 1];
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
                relocate_shift(s, lane, tpos, npos, selected);
                r.moved += tpos < npos ? npos - tpos : tpos - npos + 1;
            }
            if ((pnbr & 0xffffu) != selected && (pnbr >> 16) != selected) {
                ++r.mne;
                push_absent(s, q, n, current, lane, log, log_cap);
                push_absent(s, q, n, selected, lane, log, log_cap);
                push_absent(s, q, n, previous, lane, log, log_cap);
            }
            current = selected;
            __syncwarp();
        }
        r.construction_cost = cost;
        if (L.out_construction)
            for (std::uint32_t i = lane; i < n; i += 32) L.out_construction[(size_t)task * n + i] = s.tour[i];
        __syncwarp();
    }
    // ---------------- local search ----------------
    long long gain_sum = 0;
    if (L.ls_mode == 1) checklist_ls_first(s, xy, in, n, lane, q, L.ls_limit, r, gain_sum, log, log_cap);
    else checklist_two_opt(s, xy, in, n, lane, q, L.ls_limit, r, gain_sum, log, log_cap);
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

__global__ void colony_init_kernel(const InstanceView* instances, const ColonyView* colonies, ColonyState* states,
                                   ColonyParams P) {
    const std::uint32_t c = blockIdx.x;
    const ColonyView cv = colonies[c];
    const InstanceView in = instances[cv.instance];
    const std::uint32_t n = in.n, k = in.k;
    __shared__ float s_tmax;
    if (threadIdx.x == 0) {
        ColonyState st{};
        st.epoch_cost = st.global_cost = st.parent_cost = st.iteration_best_cost = in.initial_cost;
        trail_limits(in.initial_cost, P.retention, P.p_root, k, st.tau_min, st.tau_max);
        st.default_trail = st.tau_max;
        st.mne_target = P.mne_target;
        st.action = -1;
        st.region = 4;
        states[c] = st;
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

// Fused reduce_and_select + update_pheromone for one colony, then (GP-controlled
// evaluations) the controller decision for the next iteration.
__global__ void __launch_bounds__(256) colony_update_kernel(const InstanceView* instances,
                                                            const ColonyView* colonies, ColonyState* states,
                                                            ColonyParams P, TraceRow* trace,
                                                            std::uint32_t colony_count, std::uint32_t trace_cap) {
    const std::uint32_t c = blockIdx.x;
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
    __shared__ std::uint32_t s_used_mne;

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
        cv.parent[i] = fe ? cv.epoch[i] : v;
    }
    __syncthreads();
    for (std::uint32_t i = threadIdx.x; i < n; i += blockDim.x)
        cv.parent_nbr[cv.parent[i]] = (std::uint32_t)cv.parent[i + 1 == n ? 0 : i + 1] |
                                      ((std::uint32_t)cv.parent[i == 0 ? n - 1 : i - 1] << 16);
    __syncthreads();
    trail_update(n, k, in.primary, cv.parent_nbr, P.retention_f, s_tmin, s_tmax, s_inc, cv.eta, cv.trails,
                 cv.products, threadIdx.x, blockDim.x);
    std::int32_t action = -1;
    if (P.controlled && cv.program) {
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
        if (trace && st.iteration < trace_cap) {
            TraceRow& row = trace[(size_t)st.iteration * colony_count + c];
            row.iteration_best_cost = st.iteration_best_cost;
            row.global_cost = st.global_cost;
            row.parent_cost = st.parent_cost;
            row.iteration_best = st.iteration_best;
            row.source_is_epoch = st.source_is_epoch;
            row.tau_min = st.tau_min;
            row.tau_max = st.tau_max;
            row.mne_target = s_used_mne;
            row.action = action;
            row.construction_steps = s_steps;
            row.ls_evaluations = s_evals;
        }
        ++st.iteration;
        states[c] = st;
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

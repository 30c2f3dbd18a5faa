// faco_engine.cu -- the batch engine behind the C ABI (include/faco_gb300.h).
//
// Replaces the reference's FacoBatchEngine / FixedFacoGpu host drivers
// (cuda/batch_engine.cu:78-1192, cuda/fixed_faco.cu:105-177) and the pybind11
// boundary (cpp/src/bindings.cpp).  One engine owns one CUDA stream and all
// device memory of its evaluations; instances are prepared once at
// registration and stay resident.  The iteration loop -- ant kernel, fused
// colony update -- is captured once per evaluation into a CUDA graph of
// several iterations and replayed; the batch index lives on the device, so
// replays need no parameter changes.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <optional>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/faco_gb300.h"
#include "faco_host.h"
#include "faco_kernels.h"
#include "noalloc_kernels.h"
#include "prior_kernels.h"

namespace {

thread_local std::string g_error;

// Iterations captured per CUDA graph (replayed until the budget is spent).
constexpr std::uint32_t kGraphIterations = 16;
// Batched steps chosen per stretch of iterations (FACO_FOLLOW_AUTO on panels
// beyond one wave of ant warps): every kAdaptIterations iterations the
// colonies' step counters are read back, and the following replays take the
// batched-step graph once the stretch averaged at least kBatchOnSteps
// construction steps per ant and iteration, the one-step graph again below
// kBatchOffSteps.  Measured on the N=1000 throughput panel: batches lose up
// to 1.9x on the short walks of early iterations (11-30 steps), break even
// near 70 and win 19-26 % from 110 steps on.
// With the global-memory ant workspace (large instances) the crossover is
// later: on the large clustered panel (N 5,750-9,650) batches lose up to 17 %
// below 50 steps and win 6-11 % from 150 on.
constexpr std::uint32_t kAdaptIterations = 32;   // 64 switched one stretch later: 3 % slower on iterations 0-320
constexpr double kBatchOnSteps = 72.0, kBatchOffSteps = 60.0;
constexpr double kBatchOnStepsGlobal = 96.0, kBatchOffStepsGlobal = 80.0;
// Automatic chain count: one chain per kColoniesPerChain colonies, at most kMaxChains.
// Trail updates of more than 2 x kTrailCellsPerBlock entries per colony run in
// colony_trails_kernel, one block per kTrailCellsPerBlock entries (at most
// kMaxTrailBlocks per colony).
constexpr std::uint64_t kTrailCellsPerBlock = 16384;
constexpr std::uint64_t kMaxTrailBlocks = 64;
constexpr std::uint32_t kColoniesPerChain = 16;
constexpr std::uint32_t kMaxChains = 8;

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void require(bool ok, const std::string& message) {
    if (!ok) throw Error(FACO_EINVAL, message);
}
void cuda_check(cudaError_t status, const char* what) {
    if (status != cudaSuccess) throw Error(FACO_ECUDA, std::string(what) + ": " + cudaGetErrorString(status));
}

template <class F>
int guarded(F&& body) {
    try {
        body();
        return FACO_OK;
    } catch (const Error& e) {
        g_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_error = "host allocation failed";
        return FACO_ENOMEM;
    } catch (const std::exception& e) {
        g_error = e.what();
        return FACO_EINVAL;
    }
}

template <class T>
class DeviceBuffer {
public:
    DeviceBuffer() = default;
    explicit DeviceBuffer(std::size_t count) { resize(count); }
    ~DeviceBuffer() { release(); }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    DeviceBuffer(DeviceBuffer&& o) noexcept : ptr_(o.ptr_), count_(o.count_) { o.ptr_ = nullptr; o.count_ = 0; }
    void resize(std::size_t count) {
        if (count <= count_ && ptr_) return;
        release();
        if (count) cuda_check(cudaMalloc(reinterpret_cast<void**>(&ptr_), count * sizeof(T)), "cudaMalloc");
        count_ = count;
    }
    void upload(const T* host, std::size_t count, cudaStream_t s) {
        resize(count);
        if (count) cuda_check(cudaMemcpyAsync(ptr_, host, count * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
    }
    void upload(const std::vector<T>& v, cudaStream_t s) { upload(v.data(), v.size(), s); }
    void download(T* host, std::size_t count, cudaStream_t s) const {
        if (count) cuda_check(cudaMemcpyAsync(host, ptr_, count * sizeof(T), cudaMemcpyDeviceToHost, s), "download");
    }
    T* get() const { return ptr_; }
    std::size_t size() const { return count_; }
    std::size_t bytes() const { return count_ * sizeof(T); }

private:
    void release() {
        if (ptr_) cudaFree(ptr_);
        ptr_ = nullptr;
        count_ = 0;
    }
    T* ptr_ = nullptr;
    std::size_t count_ = 0;
};

std::uint64_t mix64(std::uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

using Clock = std::chrono::steady_clock;
double seconds_since(Clock::time_point t) { return std::chrono::duration<double>(Clock::now() - t).count(); }

// Below a 2^24 span per axis every EUC_2D length is < 2^25, where the
// reference's floor(sqrt(dx^2 + dy^2) + 0.5) in double precision equals the
// exactly rounded integer the device computes; wider spans could round the
// two differently at half-integer boundaries, so they are refused.
void require_euc2d_span(const std::int32_t* xy, std::uint32_t n) {
    std::int32_t lo[2] = {xy[0], xy[1]}, hi[2] = {xy[0], xy[1]};
    for (std::size_t i = 0; i < 2ull * n; ++i) {
        lo[i & 1] = std::min(lo[i & 1], xy[i]);
        hi[i & 1] = std::max(hi[i & 1], xy[i]);
    }
    require(static_cast<std::int64_t>(hi[0]) - lo[0] < (1 << 24) && static_cast<std::int64_t>(hi[1]) - lo[1] < (1 << 24),
            "coordinate spans must be below 2^24 per axis (exact EUC_2D lengths)");
}

std::vector<std::int32_t> integer_coordinates(const double* xy, std::uint32_t n) {
    std::vector<std::int32_t> out(2ull * n);
    for (std::size_t i = 0; i < 2ull * n; ++i) {
        const double v = xy[i];
        require(std::isfinite(v) && v == std::floor(v) && std::fabs(v) < 67108864.0,
                "coordinates must be finite integers with |x| < 2^26 (EUC_2D)");
        out[i] = static_cast<std::int32_t>(v);
    }
    require_euc2d_span(out.data(), n);
    return out;
}

// Warps (ants) per block: the largest that keeps the block's shared memory
// within the opt-in limit and at least two blocks per SM when possible.
std::uint32_t choose_warps(std::uint32_t n_max, std::uint32_t ants) {
    constexpr std::uint32_t kSmemLimit = 227u * 1024u;
    std::uint32_t best = 1;
    for (std::uint32_t w = 1; w <= faco::kMaxWarpsPerBlock; w *= 2) {
        if (faco::block_smem_bytes(n_max, w) <= kSmemLimit && w <= std::max(1u, ants)) best = w;
    }
    while (best > 1 && faco::block_smem_bytes(n_max, best) * 2 > kSmemLimit &&
           faco::block_smem_bytes(n_max, best / 2) * 2 <= kSmemLimit)
        best /= 2;
    return std::min<std::uint32_t>(best, 4);
}

struct Instance {
    std::uint64_t key = 0;
    std::uint32_t n = 0, k = 0, b = 0, w = 0;
    std::vector<std::int32_t> xy;
    std::vector<double> source_xy;  // coordinates as registered (identity check on re-registration)
    faco_registration info{};
    std::vector<std::uint32_t> initial;
    std::vector<std::uint16_t> primary, backup, ls;
    std::int64_t initial_cost = 0;
    DeviceBuffer<int2> d_xy;
    DeviceBuffer<faco::node_t> d_primary, d_backup, d_ls, d_initial;
    DeviceBuffer<int> d_ls_dist;
    DeviceBuffer<float> d_eta, d_alpha;
    DeviceBuffer<faco::node_t> d_regions;
    std::uint32_t region_offsets[5] = {0, 0, 0, 0, 0};
    float mean_nn = 1.0f;
    // 12-feature controller data (prepared_problem.cpp:66-86, control_ops.hpp:103-107)
    DeviceBuffer<faco::node_t> d_samples;
    DeviceBuffer<double> d_local_scale;
    std::uint32_t sample_count = 0;
    double scale_epsilon = 0.0;
    faco::InstanceView view() const {
        faco::InstanceView v{n, k, b, w, d_xy.get(), d_primary.get(), d_backup.get(), d_ls.get(), d_ls_dist.get(),
                             d_eta.get(), d_initial.get(), static_cast<long long>(initial_cost), d_regions.get(),
                             {0, 0, 0, 0, 0}};
        for (int r = 0; r < 5; ++r) v.region_offsets[r] = region_offsets[r];
        v.mean_nn = mean_nn;
        v.samples = d_samples.get();
        v.sample_count = sample_count;
        v.local_scale = d_local_scale.get();
        v.scale_epsilon = scale_epsilon;
        v.alpha = d_alpha.get();
        return v;
    }
};

// Sample nodes and per-node scale of the 12-feature controller: the scale of
// a node is the mean of its min(8, n-1) nearest EUC_2D lengths, each divided
// by that count and summed nearest first (prepared_problem.cpp:66-86);
// epsilon = 1e-12 * max(x span, y span, 1).  The LS rows hold the nearest
// lengths in order when they are at least that wide.
void upload_control_data(Instance& in, const std::vector<std::int32_t>& ls_dist, cudaStream_t s) {
    const std::uint32_t n = in.n, width = std::min<std::uint32_t>(8, n - 1);
    std::vector<double> scale(n, 0.0);
    std::vector<std::int32_t> row;
    for (std::uint32_t a = 0; a < n; ++a) {
        const std::int32_t* nearest = ls_dist.data() + static_cast<std::size_t>(a) * in.w;
        if (in.w < width) {
            row.clear();
            for (std::uint32_t b = 0; b < n; ++b)
                if (b != a)
                    row.push_back(faco::host_euc2d(in.xy[2 * a], in.xy[2 * a + 1], in.xy[2 * b], in.xy[2 * b + 1]));
            std::partial_sort(row.begin(), row.begin() + width, row.end());
            nearest = row.data();
        }
        double sum = 0.0;
        for (std::uint32_t j = 0; j < width; ++j) sum += static_cast<double>(nearest[j]) / width;
        scale[a] = sum;
    }
    std::int64_t minx = in.xy[0], maxx = minx, miny = in.xy[1], maxy = miny;
    for (std::uint32_t i = 0; i < n; ++i) {
        minx = std::min<std::int64_t>(minx, in.xy[2 * i]); maxx = std::max<std::int64_t>(maxx, in.xy[2 * i]);
        miny = std::min<std::int64_t>(miny, in.xy[2 * i + 1]); maxy = std::max<std::int64_t>(maxy, in.xy[2 * i + 1]);
    }
    in.scale_epsilon = 1e-12 * std::max({static_cast<double>(maxx - minx), static_cast<double>(maxy - miny), 1.0});
    in.sample_count = std::min<std::uint32_t>(n, faco::kSamples);
    std::vector<faco::node_t> samples(in.sample_count);
    faco::sample_nodes(n, in.key, samples.data());
    in.d_samples.upload(samples, s);
    in.d_local_scale.upload(scale, s);
}

// Packed parent neighbours: successor | predecessor << 16, indexed by node.
std::vector<std::uint32_t> parent_neighbours(const std::uint32_t* tour, std::uint32_t n) {
    std::vector<std::uint32_t> nbr(n);
    for (std::uint32_t i = 0; i < n; ++i)
        nbr[tour[i]] = tour[i + 1 == n ? 0 : i + 1] | (tour[i == 0 ? n - 1 : i - 1] << 16);
    return nbr;
}

void launch_ants(int mode, const faco::AntLaunch& L, std::uint32_t blocks, std::uint32_t warps, cudaStream_t s) {
    const std::uint32_t smem = faco::block_smem_bytes(L.n_max, warps);
    cuda_check(faco::prepare_ant_kernel(mode, smem), "cudaFuncSetAttribute");
    cuda_check(faco::launch_ant_kernel(mode, L, blocks, warps, smem, s), "ant kernel launch");
}

}  // namespace

struct faco_engine {
    faco_settings settings{};
    std::uint32_t dimension = 0, capacity = 0, ants = 0;
    int device = 0;
    int sm_count = 152;                         // multiprocessors of the device (queried at creation)
    cudaStream_t stream = nullptr;
    std::mutex busy;
    std::map<std::uint64_t, std::unique_ptr<Instance>> instances;
    std::vector<std::uint64_t> instance_order;  // device table index -> key
    DeviceBuffer<faco::InstanceView> d_instances;
    // evaluation buffers (grow-only)
    DeviceBuffer<float> trails, products, colony_eta;
    DeviceBuffer<faco::node_t> parent, epoch, global, ant_tours;
    DeviceBuffer<std::uint32_t> parent_nbr;
    DeviceBuffer<long long> ant_costs, ant_ccosts;
    DeviceBuffer<faco::Program> programs;
    DeviceBuffer<unsigned> ant_counts, error;
    DeviceBuffer<faco::ColonyState> states;
    DeviceBuffer<faco::ColonyView> colonies;
    DeviceBuffer<uint2> work;
    DeviceBuffer<std::uint32_t> chain_colonies;
    DeviceBuffer<faco::TraceRow> trace;
    DeviceBuffer<faco::node_t> checkpoints;
    // 12-feature controller (feature spec 2)
    DeviceBuffer<faco::RefControl> ref_controls;
    DeviceBuffer<faco::node_t> archives;          // per colony [2][4][2][n_pad]
    DeviceBuffer<unsigned long long> ant_ids;     // per ant [2]
    DeviceBuffer<std::uint32_t> ant_p0, decision_points, decision_masks;
    DeviceBuffer<float> decision_features, decision_scores;
    DeviceBuffer<std::int32_t> decision_actions;
    // learned edge prior
    DeviceBuffer<faco::MlpParams> prior_params;
    DeviceBuffer<faco::MlpOperands> prior_ops;
    DeviceBuffer<std::uint8_t> prior_enabled;
    DeviceBuffer<std::uint32_t> prior_modes;   // per colony: 1 = the prior re-ranks departures only
    float prior_floor = 0.05f;
    int prior_gamma = 1;
    bool prior_loaded = false;
    DeviceBuffer<std::uint32_t> prior_gnbr, prior_offsets;

    // the evaluation in progress (begin .. finish)
    // One ant-kernel launch per instance size class (n rounded up to a power
    // of two, at least 256): shared memory is sized for the class's largest
    // instance, and the classes run as parallel branches of each iteration.
    struct AntClass {
        std::uint32_t n_max = 0, warps = 1, smem = 0, blocks = 0, first_job = 0;
        int mode = faco::kModeEngine;   // or kModeEngineGlobal (tour/inverse in global memory), or
                                        // either's batched-step variant
        faco::AntLaunch L{};
    };
    // A chain: a subset of the colonies of one size class, whose iterations
    // depend only on one another.  In the evaluation's graph each chain runs
    // its own sequence of ant launches and updates, so one chain's slowest
    // ants overlap the other chains' work instead of idling the GPU at every
    // iteration.
    struct Chain {
        std::uint32_t first = 0, count = 0;   // colonies chain_colonies[first, first + count)
        std::uint32_t cls = 0, first_job = 0, blocks = 0;   // its ant launch: class, jobs
        faco::AntLaunch L{};
    };
    struct EvalState {
        bool active = false;
        bool follow = false;                    // the ant launches take parent-following steps in batches
        std::uint32_t count = 0, n_max = 0, trace_cap = 0, done = 0;
        std::size_t node_total = 0, tau_total = 0;
        std::vector<std::uint32_t> sizes;
        std::vector<std::uint64_t> keys, seeds;
        std::vector<faco_program> programs;     // host copy of the controller slots (snapshots)
        std::vector<std::uint32_t> kinds;
        std::uint32_t action_mask = 0xFFFFFFFFu;
        std::uint32_t feature_spec = 0;         // 2 or 3 for controlled evaluations
        std::vector<std::uint32_t> decision_points;
        std::vector<AntClass> classes;
        std::vector<Chain> chains;
        faco::ColonyParams P{};
        faco::AntLaunch L{};
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        // batched steps chosen per stretch of iterations: the batched-step
        // graph beside the one-step one, the variant of the next replays and
        // the step counters at the last reading
        bool adaptive = false, batched = false;
        double batch_on = kBatchOnSteps, batch_off = kBatchOffSteps;
        cudaGraph_t graph_batched = nullptr;
        cudaGraphExec_t exec_batched = nullptr;
        unsigned long long steps_seen = 0;
        std::uint32_t done_seen = 0;
        bool rebase = false;                    // the next reading only sets the baseline (restored runs)
    } eval;
    std::vector<cudaStream_t> branch_streams;
    std::vector<cudaEvent_t> branch_events;   // [0] fork, [1 + i] join of branch i
    // (class, n_max, ants, blocks, LS mode) -> (warps, kernel mode)
    std::map<std::uint64_t, std::pair<std::uint32_t, int>> tuned_warps;
    DeviceBuffer<faco::node_t> ant_workspace;  // kModeEngineGlobal: tour + inverse per ant

    ~faco_engine() {
        if (eval.exec) cudaGraphExecDestroy(eval.exec);
        if (eval.graph) cudaGraphDestroy(eval.graph);
        if (eval.exec_batched) cudaGraphExecDestroy(eval.exec_batched);
        if (eval.graph_batched) cudaGraphDestroy(eval.graph_batched);
        for (auto st : branch_streams) cudaStreamDestroy(st);
        for (auto ev : branch_events) cudaEventDestroy(ev);
        if (stream) {
            cudaSetDevice(device);
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }

    std::uint32_t index_of(std::uint64_t key) const {
        const auto it = std::find(instance_order.begin(), instance_order.end(), key);
        return static_cast<std::uint32_t>(it - instance_order.begin());
    }

    void upload_instance_table() {
        std::vector<faco::InstanceView> views;
        for (const auto key : instance_order) views.push_back(instances.at(key)->view());
        d_instances.upload(views, stream);
    }

    unsigned read_error() {
        unsigned word = 0;
        error.download(&word, 1, stream);
        cuda_check(cudaStreamSynchronize(stream), "synchronize");
        return word;
    }
    void reset_error() { cuda_check(cudaMemsetAsync(error.get(), 0, sizeof(unsigned), stream), "memset"); }
};

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* faco_last_error(void) { return g_error.c_str(); }

void faco_default_settings(faco_settings* s) {
    if (!s) return;
    std::memset(s, 0, sizeof(*s));
    s->ants = 0;
    s->primary_width = 16;
    s->backup_width = 64;
    s->ls_width = 20;
    s->beta = 1.0;
    s->retention = 0.5;
    s->p_best = 0.1;
    s->epoch_source_probability = 0.01;
    s->ls_evaluation_limit = 100000;
    s->initial_ls_evaluation_limit = 100000;
    s->ls_mode = FACO_LS_TWO_OPT;
    s->autotune = 1;
    s->workspace = FACO_WORKSPACE_AUTO;
    s->force_fingerprint_collisions = 0;
}

int faco_engine_create(uint32_t dimension, uint32_t colonies, const faco_settings* settings, int device,
                       faco_engine** out) {
    return guarded([&] {
        require(out && settings, "null argument");
        *out = nullptr;
        const faco_settings& c = *settings;
        require(dimension >= 3 && dimension <= 10000, "dimension must be in [3, 10000]");
        require(colonies >= 1 && colonies <= 65536, "colonies must be in [1, 65536]");
        require(c.ants <= 4096 && c.primary_width >= 2 && c.ls_width > 0 && std::isfinite(c.beta) && c.beta > 0 &&
                    c.retention >= 0 && c.retention < 1 && c.p_best > 0 && c.p_best < 1 &&
                    c.epoch_source_probability >= 0 && c.epoch_source_probability <= 1,
                "invalid FACO settings");
        require(c.primary_width <= 32 && c.ls_width <= 32, "primary and LS widths are limited to 32 (one warp)");
        require(c.ls_mode == FACO_LS_TWO_OPT || c.ls_mode == FACO_LS_TWO_OPT_OR_OPT, "unknown local-search mode");
        require(c.follow <= FACO_FOLLOW_ON, "unknown follow setting");
        require(c.workspace <= FACO_WORKSPACE_GLOBAL, "unknown ant workspace placement");
        require(c.force_fingerprint_collisions <= 1, "force_fingerprint_collisions must be 0 or 1");
        require(c.chains <= 64, "chains must be in [0, 64]");
        auto e = std::make_unique<faco_engine>();
        e->settings = c;
        e->dimension = dimension;
        e->capacity = colonies;
        e->device = device;
        if (c.ants == 0) {
            std::uint32_t groups = 1;
            while (256ull * groups * groups < dimension) ++groups;
            e->ants = 64 * groups;  // normalized_settings (prepared_problem.cpp:68-73)
        } else {
            e->ants = c.ants;
        }
        e->settings.ants = e->ants;
        cuda_check(cudaSetDevice(device), "cudaSetDevice");
        cuda_check(cudaDeviceGetAttribute(&e->sm_count, cudaDevAttrMultiProcessorCount, device), "SM count");
        cuda_check(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        e->error.resize(1);
        e->reset_error();
        *out = e.release();
    });
}

void faco_engine_destroy(faco_engine* engine) { delete engine; }

int faco_register_problem(faco_engine* e, uint64_t instance_key, const double* xy, uint32_t n,
                          faco_registration* info) {
    return guarded([&] {
        require(e && xy, "null argument");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        require(!e->eval.active, "cannot register while an evaluation is active");
        require(n >= 3 && n <= e->dimension, "instance size must be in [3, dimension]");
        const auto existing = e->instances.find(instance_key);
        if (existing != e->instances.end()) {
            const Instance& known = *existing->second;
            require(known.n == n && std::equal(xy, xy + 2 * std::size_t(n), known.source_xy.begin()),
                    "instance key already registered with different coordinates");
            if (info) *info = known.info;
            return;
        }
        cuda_check(cudaSetDevice(e->device), "cudaSetDevice");
        const auto started = Clock::now();
        auto inst = std::make_unique<Instance>();
        inst->key = instance_key;
        inst->n = n;
        inst->xy = integer_coordinates(xy, n);
        inst->source_xy.assign(xy, xy + 2 * std::size_t(n));
        const faco_settings& c = e->settings;
        inst->k = std::min(c.primary_width, n - 1);
        inst->b = std::min(c.backup_width, n - 1 - inst->k);
        inst->w = std::min(c.ls_width, n - 1);
        // cheap solution: identity tour (make_cheap_problem, prepared_problem.cpp:90-105)
        std::vector<std::uint32_t> identity(n);
        for (std::uint32_t i = 0; i < n; ++i) identity[i] = i;
        const std::int64_t cheap = faco::host_tour_length(inst->xy, identity.data(), n);
        const double cheap_seconds = seconds_since(started);
        std::vector<std::int32_t> ls_dist;
        std::vector<float> eta;
        // device-resident instance; candidate rows from the GPU near lists
        // (prepared_problem.cpp:58-91), the host sort only for rows wider
        // than the kernel's list
        cudaStream_t s = e->stream;
        inst->d_xy.upload(reinterpret_cast<const int2*>(inst->xy.data()), n, s);
        const std::uint32_t needed = std::max(inst->k + inst->b, inst->w);
        std::vector<std::uint32_t> nn;
        if (needed <= faco::kKnnMaxNeeded) {
            DeviceBuffer<faco::node_t> d_near(static_cast<std::size_t>(n) * needed);
            DeviceBuffer<std::int32_t> d_near_dist(static_cast<std::size_t>(n) * needed);
            cuda_check(faco::launch_knn(inst->d_xy.get(), n, needed, d_near.get(), d_near_dist.get(), s),
                       "candidate rows");
            std::vector<std::uint16_t> near(static_cast<std::size_t>(n) * needed);
            std::vector<std::int32_t> near_dist(near.size());
            d_near.download(near.data(), near.size(), s);
            d_near_dist.download(near_dist.data(), near_dist.size(), s);
            cuda_check(cudaStreamSynchronize(s), "candidate rows");
            faco::host_rows_from_near(near, near_dist, n, needed, inst->k, inst->b, inst->w, c.beta, inst->primary,
                                      inst->backup, inst->ls, ls_dist, eta);
            nn = faco::host_nearest_neighbour_tour_near(inst->xy, n, near, needed);
        } else {
            faco::host_candidates(inst->xy, n, inst->k, inst->b, inst->w, inst->primary, inst->backup, inst->ls,
                                  ls_dist, eta, c.beta);
            nn = faco::host_nearest_neighbour_tour(inst->xy, n);
        }
        inst->d_primary.upload(inst->primary, s);
        inst->d_backup.resize(std::max<std::size_t>(inst->backup.size(), 1));
        inst->d_backup.upload(inst->backup, s);
        inst->d_ls.upload(inst->ls, s);
        inst->d_ls_dist.upload(ls_dist, s);
        inst->d_eta.upload(eta, s);
        std::vector<float> alpha;
        faco::host_alpha(inst->xy, n, inst->k, inst->primary, inst->b, inst->backup, inst->w, inst->ls, alpha);
        inst->d_alpha.upload(alpha, s);
        std::vector<std::uint16_t> regions;
        faco::host_regions(inst->xy, n, inst->region_offsets, regions);
        inst->d_regions.upload(regions, s);
        double nn_sum = 0.0;
        for (std::uint32_t a = 0; a < n; ++a) nn_sum += ls_dist[static_cast<std::size_t>(a) * inst->w];
        inst->mean_nn = static_cast<float>(std::max(1.0, nn_sum / n));
        upload_control_data(*inst, ls_dist, s);
        // initial checklist 2-opt over the NN tour on the GPU (prepared_problem.cpp:159-162)
        std::vector<faco::node_t> tour16(nn.begin(), nn.end());
        const long long nn_cost = faco::host_tour_length(inst->xy, nn.data(), n);
        DeviceBuffer<faco::node_t> d_tour, d_out;
        DeviceBuffer<std::uint32_t> d_nbr;
        DeviceBuffer<long long> d_cost, d_costs;
        d_tour.upload(tour16, s);
        d_nbr.upload(parent_neighbours(nn.data(), n), s);
        d_cost.upload(&nn_cost, 1, s);
        d_out.resize(n);
        d_costs.resize(2);
        DeviceBuffer<faco::InstanceView> d_view;
        inst->d_initial.resize(n);
        const faco::InstanceView v = inst->view();
        d_view.upload(&v, 1, s);
        faco::AntLaunch L{};
        L.instances = d_view.get();
        L.warps = 1;
        L.n_max = n;
        L.ls_limit = c.initial_ls_evaluation_limit;
        L.tasks = 1;
        L.task_tours = d_tour.get();
        L.task_nbr = d_nbr.get();
        L.task_costs = d_cost.get();
        L.out_tours = d_out.get();
        L.out_costs = d_costs.get();
        L.error = e->error.get();
        e->reset_error();
        launch_ants(faco::kModePrepare, L, 1, 1, s);
        std::vector<faco::node_t> improved(n);
        long long costs[2] = {0, 0};
        d_out.download(improved.data(), n, s);
        d_costs.download(costs, 2, s);
        const unsigned err = e->read_error();
        if (err) throw Error(FACO_EDEVICE, "device error word " + std::to_string(err) + " during registration");
        inst->initial.assign(improved.begin(), improved.end());
        inst->initial_cost = costs[1];
        require(faco::host_tour_length(inst->xy, inst->initial.data(), n) == inst->initial_cost,
                "initial tour length mismatch");
        if (cheap <= inst->initial_cost) {
            inst->initial = identity;
            inst->initial_cost = cheap;
        }
        std::vector<faco::node_t> init16(inst->initial.begin(), inst->initial.end());
        inst->d_initial.upload(init16, s);
        cuda_check(cudaStreamSynchronize(s), "synchronize");
        inst->info.cheap_seconds = cheap_seconds;
        inst->info.preparation_seconds = seconds_since(started);
        inst->info.initial_cost = inst->initial_cost;
        inst->info.n = n;
        if (info) *info = inst->info;
        e->instance_order.push_back(instance_key);
        e->instances.emplace(instance_key, std::move(inst));
        e->upload_instance_table();
        cuda_check(cudaStreamSynchronize(s), "synchronize");
    });
}

int faco_problem_rows(faco_engine* e, uint64_t key, uint32_t* initial, uint32_t* primary, uint32_t* backup,
                      uint32_t* ls) {
    return guarded([&] {
        require(e != nullptr, "null engine");
        const auto it = e->instances.find(key);
        require(it != e->instances.end(), "instance not registered");
        const Instance& in = *it->second;
        if (initial) std::copy(in.initial.begin(), in.initial.end(), initial);
        if (primary) std::copy(in.primary.begin(), in.primary.end(), primary);
        if (backup) std::copy(in.backup.begin(), in.backup.end(), backup);
        if (ls) std::copy(in.ls.begin(), in.ls.end(), ls);
    });
}

}  // extern "C"

// ---- evaluation: begin / step / finish ------------------------------------
namespace {

void destroy_graph(faco_engine* e) {
    if (e->eval.exec) cudaGraphExecDestroy(e->eval.exec);
    if (e->eval.graph) cudaGraphDestroy(e->eval.graph);
    if (e->eval.exec_batched) cudaGraphExecDestroy(e->eval.exec_batched);
    if (e->eval.graph_batched) cudaGraphDestroy(e->eval.graph_batched);
    e->eval.exec = nullptr;
    e->eval.graph = nullptr;
    e->eval.exec_batched = nullptr;
    e->eval.graph_batched = nullptr;
}

// All ant launches of one iteration: class 0 on `st`, the others on branch
// streams forked from and joined back into `st` (parallel graph branches).
void enqueue_ants(faco_engine* e, cudaStream_t st) {
    auto& v = e->eval;
    const std::size_t branches = v.classes.size();
    if (branches > 1) cuda_check(cudaEventRecord(e->branch_events[0], st), "fork");
    for (std::size_t i = 0; i < branches; ++i) {
        const auto& c = v.classes[i];
        cudaStream_t bs = i == 0 ? st : e->branch_streams[i - 1];
        if (i > 0) cuda_check(cudaStreamWaitEvent(bs, e->branch_events[0], 0), "fork wait");
        cuda_check(faco::launch_ant_kernel(c.mode, c.L, c.blocks, c.warps, c.smem, bs), "ant launch");
        if (i > 0) cuda_check(cudaEventRecord(e->branch_events[i], bs), "join");
    }
    for (std::size_t i = 1; i < branches; ++i) cuda_check(cudaStreamWaitEvent(st, e->branch_events[i], 0), "join wait");
}

// The colony update of one iteration for `colonies` colonies (those of
// `list`, or all when null); with the 12-feature controller the ants'
// fingerprints first, one warp per ant.
void enqueue_update(faco_engine* e, cudaStream_t st, const std::uint32_t* list, std::uint32_t colonies) {
    auto& v = e->eval;
    if (v.P.ref_control) {
        const std::uint32_t warps = colonies * v.P.ants;
        faco::fingerprint_kernel<<<(warps + 7) / 8, 256, 0, st>>>(e->colonies.get(), list, v.P.ants, colonies,
                                                                 v.P.zero_fingerprints);
    }
    faco::colony_update_kernel<<<colonies, 256, 0, st>>>(e->d_instances.get(), e->colonies.get(), e->states.get(),
                                                          v.P, v.trace_cap ? e->trace.get() : nullptr, list,
                                                          v.count, v.trace_cap);
    if (v.P.trail_blocks > 1)
        faco::colony_trails_kernel<<<dim3(v.P.trail_blocks, colonies), 256, 0, st>>>(
            e->d_instances.get(), e->colonies.get(), e->states.get(), v.P, list);
    cuda_check(cudaGetLastError(), "update launch");
}

void enqueue_update(faco_engine* e, cudaStream_t st) { enqueue_update(e, st, nullptr, e->eval.count); }

void enqueue_iteration(faco_engine* e, cudaStream_t st) {
    enqueue_ants(e, st);
    enqueue_update(e, st);
}

// One iteration of chain `g`: its ant launch, then its colonies' update,
// both on `st`.
void enqueue_chain_iteration(faco_engine* e, std::size_t g, cudaStream_t st) {
    auto& v = e->eval;
    const auto& ch = v.chains[g];
    const auto& c = v.classes[ch.cls];
    cuda_check(faco::launch_ant_kernel(c.mode, ch.L, ch.blocks, c.warps, c.smem, st), "ant launch");
    enqueue_update(e, st, e->chain_colonies.get() + ch.first, ch.count);
}

// Streams and events for `branches` parallel graph branches besides `st`.
void ensure_branches(faco_engine* e, std::size_t branches) {
    while (e->branch_streams.size() < branches) {
        cudaStream_t bs;
        cuda_check(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking), "branch stream");
        e->branch_streams.push_back(bs);
    }
    while (e->branch_events.size() < branches + 2) {
        cudaEvent_t ev;
        cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "branch event");
        e->branch_events.push_back(ev);
    }
}

// `iterations` iterations of every colony; with more than one chain, each
// chain's iterations run on their own stream, forked from and joined back
// into `st` (independent branches when captured into a graph).
void enqueue_iterations(faco_engine* e, cudaStream_t st, std::uint32_t iterations) {
    auto& v = e->eval;
    const std::size_t chains = v.chains.size();
    if (chains <= 1) {
        for (std::uint32_t i = 0; i < iterations; ++i) enqueue_iteration(e, st);
        return;
    }
    cuda_check(cudaEventRecord(e->branch_events[0], st), "fork");
    for (std::size_t g = 1; g < chains; ++g)
        cuda_check(cudaStreamWaitEvent(e->branch_streams[g - 1], e->branch_events[0], 0), "fork wait");
    for (std::uint32_t i = 0; i < iterations; ++i)
        for (std::size_t g = 0; g < chains; ++g) enqueue_chain_iteration(e, g, g == 0 ? st : e->branch_streams[g - 1]);
    for (std::size_t g = 1; g < chains; ++g) {
        cuda_check(cudaEventRecord(e->branch_events[g], e->branch_streams[g - 1]), "join");
        cuda_check(cudaStreamWaitEvent(st, e->branch_events[g], 0), "join wait");
    }
}

// The evaluation's graph: kGraphIterations iterations, replayed.  A failed
// enqueue ends the capture (discarding the partial graph) before the error
// propagates, so the stream is usable again.
void capture_one(faco_engine* e, cudaStream_t st, cudaGraph_t& graph, cudaGraphExec_t& exec) {
    cuda_check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    try {
        enqueue_iterations(e, st, kGraphIterations);
    } catch (...) {
        cudaGraph_t partial = nullptr;
        if (cudaStreamEndCapture(st, &partial) == cudaSuccess && partial) cudaGraphDestroy(partial);
        cudaGetLastError();
        throw;
    }
    cuda_check(cudaStreamEndCapture(st, &graph), "end capture");
    cuda_check(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate");
    // upload now, so that the first replay costs what every other one does
    cuda_check(cudaGraphUpload(exec, st), "graph upload");
}

// While alive, every class of an adaptive evaluation launches its
// batched-step variant (the build for panels beyond one wave); the
// one-step modes come back when it ends, an exception included.
class BatchedModes {
  public:
    explicit BatchedModes(faco_engine::EvalState& v) : v_(v) {
        for (auto& cl : v_.classes) {
            modes_.push_back(cl.mode);
            cl.mode = faco::with_follow(cl.mode, true);
        }
    }
    ~BatchedModes() {
        for (std::size_t i = 0; i < modes_.size(); ++i) v_.classes[i].mode = modes_[i];
    }
    BatchedModes(const BatchedModes&) = delete;
    BatchedModes& operator=(const BatchedModes&) = delete;

  private:
    faco_engine::EvalState& v_;
    std::vector<int> modes_;
};

void capture_graph(faco_engine* e, cudaStream_t st) {
    auto& v = e->eval;
    destroy_graph(e);
    capture_one(e, st, v.graph, v.exec);
    if (v.adaptive) {
        // the same iterations with every class's batched-step variant
        BatchedModes batched(v);
        capture_one(e, st, v.graph_batched, v.exec_batched);
    }
    // a fresh evaluation starts with every counter at zero
    v.batched = false;
    v.steps_seen = 0;
    v.done_seen = 0;
    v.rebase = false;
}

// Kernel variant of a size class: the global-memory workspace (tour and
// inverse in global memory, coordinates read from global) lets large classes
// run a full block per SM slot instead of one or two shared-memory-bound ants.
constexpr std::uint32_t kGlobalWorkspaceFrom = 2048;   // auto: n_max above this may use it

bool may_use_global(const faco_settings& c, std::uint32_t n_max) {
    return c.workspace == FACO_WORKSPACE_GLOBAL ||
           (c.workspace == FACO_WORKSPACE_AUTO && n_max > kGlobalWorkspaceFrom);
}
bool may_use_shared(const faco_settings& c, std::uint32_t n_max) {
    return c.workspace != FACO_WORKSPACE_GLOBAL && faco::block_smem_bytes(n_max, 1) <= 227u * 1024u;
}
std::uint32_t class_smem(int mode, std::uint32_t n_max, std::uint32_t warps) {
    return faco::global_mode(mode) ? faco::block_smem_bytes_global(n_max, warps)
                                           : faco::block_smem_bytes(n_max, warps);
}

// Work tables of the size classes: jobs (colony, first ant) of W = warps
// ants each.  With autotuning, every candidate (W, workspace placement) of a
// class is timed on the freshly initialised colonies (the ant kernel alone,
// which changes no colony state: its outputs are rewritten by the first real
// iteration) and the fastest is kept, cached per (class, size, ants, blocks,
// LS mode).  Without it, the default is the shared-memory kernel with
// choose_warps, or the global workspace with 4 warps where only that fits
// or the settings ask for it.
void build_work_tables(faco_engine* e, const std::vector<std::vector<std::uint32_t>>& members,
                       const std::vector<std::uint32_t>& class_ids) {
    auto& v = e->eval;
    const std::uint32_t A = v.L.ants;
    cudaStream_t s = e->stream;
    const faco_settings& c = e->settings;
    auto jobs_for = [&](const std::vector<std::uint32_t>& cols, std::uint32_t warps) {
        std::vector<uint2> jobs;
        for (const std::uint32_t col : cols)
            for (std::uint32_t a = 0; a < A; a += warps) jobs.push_back(make_uint2(col, a));
        return jobs;
    };
    bool need_workspace = false;
    for (const auto& cl : v.classes) need_workspace = need_workspace || may_use_global(c, cl.n_max);
    if (need_workspace) e->ant_workspace.resize(2 * e->ant_tours.size());
    for (auto& cl : v.classes) {
        const bool shared_ok = may_use_shared(c, cl.n_max);
        require(shared_ok || may_use_global(c, cl.n_max), "instance too large for a shared-memory ant block");
        if (shared_ok && !(c.workspace == FACO_WORKSPACE_AUTO && !c.autotune && may_use_global(c, cl.n_max))) {
            cl.mode = faco::kModeEngine;
        } else {
            cl.mode = faco::kModeEngineGlobal;
            cl.warps = std::min<std::uint32_t>(faco::kMaxWarpsPerBlock, std::max(1u, A));
        }
    }
    auto launch_of = [&](std::uint32_t first_job, std::uint32_t warps, std::uint32_t n_max) {
        faco::AntLaunch L = v.L;
        L.work = e->work.get() + first_job;
        L.warps = warps;
        L.n_max = n_max;
        L.workspace = need_workspace ? e->ant_workspace.get() : nullptr;
        L.ant_tours_base = e->ant_tours.get();
        return L;
    };
    if (c.autotune) {
        cudaEvent_t t0, t1;
        cuda_check(cudaEventCreate(&t0), "event");
        cuda_check(cudaEventCreate(&t1), "event");
        for (std::size_t i = 0; i < members.size(); ++i) {
            auto& cl = v.classes[i];
            const std::uint64_t key = (static_cast<std::uint64_t>(class_ids[i]) << 56) ^
                                      (static_cast<std::uint64_t>(cl.n_max) << 40) ^
                                      (static_cast<std::uint64_t>(A) << 24) ^
                                      (static_cast<std::uint64_t>(members[i].size()) << 4) ^
                                      (static_cast<std::uint64_t>(c.workspace) << 2) ^ c.ls_mode;
            const auto hit = e->tuned_warps.find(key);
            if (hit != e->tuned_warps.end()) {
                cl.warps = hit->second.first;
                cl.mode = hit->second.second;
                continue;
            }
            float best_ms = 0.0f;
            for (const int mode : {static_cast<int>(faco::kModeEngine), static_cast<int>(faco::kModeEngineGlobal)}) {
                if (mode == faco::kModeEngine && !may_use_shared(c, cl.n_max)) continue;
                if (mode == faco::kModeEngineGlobal && !may_use_global(c, cl.n_max)) continue;
                for (std::uint32_t w = 1; w <= faco::kMaxWarpsPerBlock && w <= A; w *= 2) {
                    const std::uint32_t smem = class_smem(mode, cl.n_max, w);
                    if (smem > 227u * 1024u) break;
                    const auto jobs = jobs_for(members[i], w);
                    e->work.upload(jobs, s);
                    const faco::AntLaunch L = launch_of(0, w, cl.n_max);
                    cuda_check(faco::prepare_ant_kernel(mode, smem), "attribute");
                    float ms = 0.0f;
                    for (int rep = 0; rep < 3; ++rep) {
                        cuda_check(cudaEventRecord(t0, s), "event");
                        cuda_check(faco::launch_ant_kernel(mode, L, static_cast<std::uint32_t>(jobs.size()), w, smem, s),
                                   "tuning launch");
                        cuda_check(cudaEventRecord(t1, s), "event");
                        cuda_check(cudaEventSynchronize(t1), "tuning");
                        float one = 0.0f;
                        cuda_check(cudaEventElapsedTime(&one, t0, t1), "elapsed");
                        if (rep > 0) ms += one;   // first launch warms caches
                    }
                    if (best_ms == 0.0f || ms < best_ms) {
                        best_ms = ms;
                        cl.warps = w;
                        cl.mode = mode;
                    }
                }
            }
            e->tuned_warps[key] = {cl.warps, cl.mode};
        }
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
    }
    std::vector<uint2> all;
    for (std::size_t i = 0; i < members.size(); ++i) {
        auto& cl = v.classes[i];
        const auto jobs = jobs_for(members[i], cl.warps);
        cl.first_job = static_cast<std::uint32_t>(all.size());
        cl.blocks = static_cast<std::uint32_t>(jobs.size());
        cl.smem = class_smem(cl.mode, cl.n_max, cl.warps);
        all.insert(all.end(), jobs.begin(), jobs.end());
    }
    // chains: each size class split into pieces in proportion to its
    // colony count (G pieces over all classes), its colonies dealt
    // round-robin (largest instances first) so that the pieces are alike;
    // each chain's jobs are a second copy of the work table
    const std::uint32_t count = v.count;
    const std::uint32_t G = std::min(c.chains ? c.chains : std::clamp(count / kColoniesPerChain, 1u, kMaxChains), count);
    v.chains.clear();
    if (G > 1) {
        std::vector<std::uint32_t> list;
        for (std::size_t i = 0; i < members.size(); ++i) {
            const std::uint32_t m = static_cast<std::uint32_t>(members[i].size());
            const std::uint32_t pieces = std::clamp((G * m + count / 2) / count, 1u, m);
            for (std::uint32_t j = 0; j < pieces; ++j) {
                std::vector<std::uint32_t> piece;
                for (std::uint32_t t = j; t < m; t += pieces) piece.push_back(members[i][t]);
                const auto jobs = jobs_for(piece, v.classes[i].warps);
                faco_engine::Chain ch;
                ch.first = static_cast<std::uint32_t>(list.size());
                ch.count = static_cast<std::uint32_t>(piece.size());
                ch.cls = static_cast<std::uint32_t>(i);
                ch.first_job = static_cast<std::uint32_t>(all.size());
                ch.blocks = static_cast<std::uint32_t>(jobs.size());
                v.chains.push_back(ch);
                all.insert(all.end(), jobs.begin(), jobs.end());
                list.insert(list.end(), piece.begin(), piece.end());
            }
        }
        if (v.chains.size() == 1) v.chains.clear();
        else e->chain_colonies.upload(list, s);
    }
    e->work.upload(all, s);
    // batched parent-following steps (the same results): on request, or
    // when every ant warp of the evaluation fits in one wave of the GPU
    const std::uint64_t ant_warps = static_cast<std::uint64_t>(v.count) * A;
    const bool one_wave = ant_warps <= 32ull * static_cast<std::uint64_t>(e->sm_count);
    v.follow = c.follow == FACO_FOLLOW_ON || (c.follow == FACO_FOLLOW_AUTO && one_wave);
    // beyond one wave the automatic choice is made per stretch of iterations
    // from the walk length (step_evaluation), with the later crossover of
    // the global-memory workspace when a class uses it
    bool any_global = false;
    for (const auto& cl : v.classes) any_global = any_global || faco::global_mode(cl.mode);
    v.adaptive = c.follow == FACO_FOLLOW_AUTO && !one_wave;
    v.batch_on = any_global ? kBatchOnStepsGlobal : kBatchOnSteps;
    v.batch_off = any_global ? kBatchOffStepsGlobal : kBatchOffSteps;
    // (beyond one wave, the batched build that favours throughput over one
    // ant's latency)
    if (v.follow)
        for (auto& cl : v.classes) cl.mode = faco::with_follow(cl.mode, !one_wave);
    // the dynamic shared-memory limit is a property of each kernel variant,
    // shared by every class that uses it: it must admit the largest one
    std::map<int, std::uint32_t> smem_max;
    for (auto& cl : v.classes) {
        cl.L = launch_of(cl.first_job, cl.warps, cl.n_max);
        auto& m = smem_max[cl.mode];
        m = std::max(m, cl.smem);
    }
    for (auto& ch : v.chains) ch.L = launch_of(ch.first_job, v.classes[ch.cls].warps, v.classes[ch.cls].n_max);
    for (const auto& [mode, smem] : smem_max) {
        if (smem) cuda_check(faco::prepare_ant_kernel(mode, smem), "cudaFuncSetAttribute");
        if (smem && v.adaptive)
            cuda_check(faco::prepare_ant_kernel(faco::with_follow(mode, true), smem), "cudaFuncSetAttribute");
    }
}

// Controller programs of a GP-controlled evaluation (null: plain FACO).
// Controllers of a GP-controlled evaluation (null: plain FACO): three tree
// slots per controller and its kind (0 joint_single: slot 0 scores all 32
// actions; 1 conditional_three: slots 0-2 are the restart, start-region and
// MNE-level roles).
struct Control {
    const faco_program* programs = nullptr;   // [n_programs][3]
    const std::uint32_t* kinds = nullptr;     // [n_programs]
    std::uint32_t n_programs = 0;
    std::uint32_t action_mask = 0xFFFFFFFFu;
    std::uint32_t total_iterations = 1;
    const std::uint32_t* decision_points = nullptr;   // feature spec 2: decisions to capture
    std::uint32_t n_decisions = 0;
};

// Slots and kinds of plain joint programs (one tree each).
struct JointSlots {
    std::vector<faco_program> slots;
    std::vector<std::uint32_t> kinds;
    JointSlots(const faco_program* programs, std::uint32_t n) : slots(3ull * n), kinds(n, 0) {
        for (std::uint32_t i = 0; i < n; ++i) slots[3ull * i] = programs[i];
    }
};

// Validation of one controller (validate_controller, cpp/src/program_cpu.cpp:11-24,
// python/gp_faco/controller.py:8-33): every used tree valid and of one
// feature spec (2, the reference's 12 features, or 3, this engine's), at most
// 63 nodes over the roles, and a role reads no feature of a decision taken
// after it.  Spec 2 (ROLE_FEATURES): the restart role reads features
// 0-4, 6, 7, the region role all but 5 (the MNE level); spec 3: role 0
// neither the MNE level (7) nor the start region (8), role 1 not the MNE level.
// Returns the feature spec.
std::uint32_t validate_controller(const faco_program* slots, std::uint32_t kind) {
    require(kind <= 1, "unknown controller kind");
    std::uint32_t total = 0;
    const std::uint32_t spec = slots[0].feature_spec_id;
    require(spec == 2 || spec == 3, "controllers use feature spec 2 or 3");
    for (std::uint32_t role = 0; role < (kind ? 3u : 1u); ++role) {
        const faco_program& p = slots[role];
        if (faco_validate_program(&p) != FACO_OK) throw Error(FACO_EINVAL, g_error);
        require(p.feature_spec_id == spec, "the trees of a controller use one feature spec");
        total += p.length;
        for (std::uint32_t i = 0; kind && i < p.length; ++i) {
            const std::uint32_t f = p.operand[i];
            if (p.opcode[i] != 0) continue;
            const bool later = spec == 2 ? (role == 0 && (f == 5 || f >= 8)) || (role == 1 && f == 5)
                                         : (role == 0 && (f == 7 || f == 8)) || (role == 1 && f == 7);
            require(!later, "a role tree reads the features of a later decision");
        }
    }
    require(total <= 63, "a controller has more than 63 nodes");
    return spec;
}

void begin_evaluation(faco_engine* e, const uint64_t* keys, const uint64_t* seeds, uint32_t count,
                      uint32_t mne_target, uint32_t trace_iterations, const Control& control = Control{}) {
    require(e && keys && seeds, "null argument");
    require(!e->eval.active, "an evaluation is already active on this engine");
    cuda_check(cudaSetDevice(e->device), "cudaSetDevice");
    const std::uint32_t A = e->ants;
    require(count >= 1 && count <= e->capacity, "task count must be in [1, colonies]");
    require(mne_target > 0, "MNE target must be positive");
    auto& v = e->eval;
    v.sizes.assign(count, 0);
    v.keys.assign(keys, keys + count);
    v.seeds.assign(seeds, seeds + count);
    v.programs.assign(control.programs, control.programs + (control.programs ? 3ull * control.n_programs : 0));
    v.kinds.assign(control.kinds, control.kinds + (control.programs ? control.n_programs : 0));
    v.action_mask = control.action_mask;
    std::vector<faco::ColonyView> views(count);
    std::size_t tau_total = 0, node_total = 0, ant_total = 0;
    std::uint32_t n_max = 3, k_common = 0;
    for (std::uint32_t c = 0; c < count; ++c) {
        const auto it = e->instances.find(keys[c]);
        require(it != e->instances.end(), "task instance not registered");
        const Instance& in = *it->second;
        require(k_common == 0 || k_common == in.k, "instances of one evaluation must share the primary width");
        k_common = in.k;
        v.sizes[c] = in.n;
        tau_total += (static_cast<std::size_t>(in.n) * in.k + 3) & ~std::size_t{3};
        node_total += faco::pad8(in.n);
        ant_total += static_cast<std::size_t>(A) * faco::pad8(in.n);
        n_max = std::max(n_max, in.n);
    }
    cudaStream_t s = e->stream;
    v.tau_total = tau_total;
    // HBM layout: per colony, trails and products [n][k] (16-byte aligned),
    // node arrays padded to 8 nodes so that every row starts 16-byte aligned
    e->trails.resize(tau_total);
    e->products.resize(tau_total);
    e->colony_eta.resize(tau_total);
    e->parent.resize(node_total);
    e->parent_nbr.resize(node_total);
    e->epoch.resize(node_total);
    e->global.resize(node_total);
    e->ant_tours.resize(ant_total);
    e->ant_costs.resize(static_cast<std::size_t>(A) * count);
    e->ant_ccosts.resize(static_cast<std::size_t>(A) * count);
    std::uint32_t replicas = 1, spec = 0;
    if (control.programs) {
        require(control.n_programs >= 1 && count % control.n_programs == 0,
                "colonies must be a whole number of replicas per program");
        require(control.action_mask != 0, "the action mask leaves no legal action");
        require(control.kinds != nullptr, "controller kinds missing");
        for (std::uint32_t i = 0; i < control.n_programs; ++i) {
            const std::uint32_t si = validate_controller(control.programs + 3ull * i, control.kinds[i]);
            require(spec == 0 || si == spec, "the controllers of one evaluation use one feature spec");
            spec = si;
        }
        if (spec == 2) {
            // the first batch has no alternative reference (batch_engine.cu:599-600)
            require((control.action_mask & 0xFFFFu) != 0, "the action mask keeps no action of mode 0");
            require(A <= faco::kCtlMaxAnts, "the 12-feature controller takes at most 1024 ants per colony");
        }
        replicas = count / control.n_programs;
        static_assert(sizeof(faco::Program) == sizeof(faco_program), "program layout");
        e->programs.upload(reinterpret_cast<const faco::Program*>(control.programs), 3ull * control.n_programs,
                           e->stream);
    }
    require(control.n_decisions == 0 || spec == 2, "decision captures need controllers of feature spec 2");
    if (spec == 2) {
        e->ref_controls.resize(count);
        e->archives.resize(16ull * node_total);
        e->ant_ids.resize(2ull * A * count);
        e->ant_p0.resize(static_cast<std::size_t>(A) * count);
    }
    v.feature_spec = spec;
    v.decision_points.assign(control.decision_points, control.decision_points + control.n_decisions);
    if (control.n_decisions) {
        e->decision_points.upload(v.decision_points, s);
        const std::size_t slots = static_cast<std::size_t>(control.n_decisions) * count;
        e->decision_features.resize(slots * 12 * 32);
        e->decision_scores.resize(slots * 32);
        e->decision_masks.resize(slots);
        e->decision_actions.resize(slots);
    }
    e->ant_counts.resize(3ull * A * count);
    e->states.resize(count);
    std::size_t tau_off = 0, node_off = 0, ant_off = 0;
    for (std::uint32_t c = 0; c < count; ++c) {
        const Instance& in = *e->instances.at(keys[c]);
        faco::ColonyView& cv = views[c];
        cv.instance = e->index_of(keys[c]);
        cv.n = in.n;
        cv.n_pad = faco::pad8(in.n);
        cv.key = mix64(seeds[c] ^ mix64(keys[c]));
        cv.trails = e->trails.get() + tau_off;
        cv.products = e->products.get() + tau_off;
        cv.eta = e->colony_eta.get() + tau_off;
        cv.parent = e->parent.get() + node_off;
        cv.parent_nbr = e->parent_nbr.get() + node_off;
        cv.epoch = e->epoch.get() + node_off;
        cv.global = e->global.get() + node_off;
        cv.ant_tours = e->ant_tours.get() + ant_off;
        cv.ant_costs = e->ant_costs.get() + static_cast<std::size_t>(c) * A;
        cv.ant_ccosts = e->ant_ccosts.get() + static_cast<std::size_t>(c) * A;
        cv.program = control.programs ? e->programs.get() + 3ull * (c / replicas) : nullptr;
        cv.action_mask = control.action_mask;
        cv.controller_kind = control.programs ? control.kinds[c / replicas] : 0u;
        cv.ant_counts = e->ant_counts.get() + 3ull * c * A;
        if (spec == 2) {
            cv.control = e->ref_controls.get() + c;
            cv.archive = e->archives.get() + 16ull * node_off;
            cv.ant_ids = e->ant_ids.get() + 2ull * A * c;
            cv.ant_p0 = e->ant_p0.get() + static_cast<std::size_t>(A) * c;
        }
        tau_off += (static_cast<std::size_t>(in.n) * in.k + 3) & ~std::size_t{3};
        node_off += cv.n_pad;
        ant_off += static_cast<std::size_t>(A) * cv.n_pad;
    }
    e->colonies.upload(views, s);
    v.count = count;
    v.node_total = node_total;
    v.n_max = n_max;
    // size classes, largest instances first inside each class so that the
    // longest ants start in the first wave
    std::vector<std::uint32_t> order(count);
    for (std::uint32_t c = 0; c < count; ++c) order[c] = c;
    std::stable_sort(order.begin(), order.end(),
                     [&](std::uint32_t x, std::uint32_t y) { return v.sizes[x] > v.sizes[y]; });
    auto class_of = [](std::uint32_t n) {
        std::uint32_t c = 0;
        while ((256u << c) < n) ++c;
        return c;
    };
    std::vector<std::vector<std::uint32_t>> members;
    std::vector<std::uint32_t> class_ids;
    for (const std::uint32_t c : order) {
        const std::uint32_t id = class_of(v.sizes[c]);
        if (class_ids.empty() || class_ids.back() != id) {
            class_ids.push_back(id);
            members.emplace_back();
        }
        members.back().push_back(c);
    }
    v.classes.assign(members.size(), faco_engine::AntClass{});
    for (std::size_t i = 0; i < members.size(); ++i) {
        auto& cl = v.classes[i];
        cl.n_max = v.sizes[members[i].front()];
        cl.warps = choose_warps(cl.n_max, A);
    }
    v.trace_cap = trace_iterations;
    if (trace_iterations) e->trace.resize(static_cast<std::size_t>(trace_iterations) * count);
    v.P = faco::ColonyParams{};
    v.P.ants = A;
    v.P.mne_target = mne_target;
    v.P.retention = e->settings.retention;
    v.P.retention_f = static_cast<float>(e->settings.retention);
    v.P.epoch_source_probability = e->settings.epoch_source_probability;
    v.P.controlled = control.programs != nullptr;
    v.P.total_iterations = std::max<std::uint32_t>(1, control.total_iterations);
    v.P.log2k = faco::host_log2(static_cast<float>(k_common));
    v.P.ref_control = spec == 2;
    v.P.zero_fingerprints = e->settings.force_fingerprint_collisions;
    v.P.ls_limit = e->settings.ls_evaluation_limit;
    e->prior_modes.resize(count);
    cuda_check(cudaMemsetAsync(e->prior_modes.get(), 0, count * sizeof(std::uint32_t), s), "memset");
    v.P.prior_rows = e->prior_modes.get();
    if (control.n_decisions) {
        v.P.capture = faco::DecisionCapture{e->decision_points.get(), control.n_decisions, e->decision_features.get(),
                                            e->decision_scores.get(), e->decision_masks.get(),
                                            e->decision_actions.get()};
    }
    v.P.p_root = std::pow(e->settings.p_best, 1.0 / static_cast<double>(k_common));
    // large candidate matrices: the trail update in a kernel of its own with
    // one block per kTrailCellsPerBlock entries of the largest colony (the
    // controllers read the updated trails inside the colony update, so
    // controlled evaluations keep it there)
    {
        const std::uint64_t cells = static_cast<std::uint64_t>(n_max) * k_common;
        v.P.trail_blocks = !v.P.controlled && !v.P.ref_control && cells >= 2 * kTrailCellsPerBlock
                               ? static_cast<std::uint32_t>(std::min<std::uint64_t>(
                                     kMaxTrailBlocks, (cells + kTrailCellsPerBlock - 1) / kTrailCellsPerBlock))
                               : 0u;
    }
    v.L = faco::AntLaunch{};
    v.L.instances = e->d_instances.get();
    v.L.colonies = e->colonies.get();
    v.L.states = e->states.get();
    v.L.ants = A;
    v.L.ls_limit = e->settings.ls_evaluation_limit;
    v.L.ls_mode = e->settings.ls_mode;
    v.L.error = e->error.get();
    e->reset_error();
    faco::colony_init_kernel<<<count, 256, 0, s>>>(e->d_instances.get(), e->colonies.get(), e->states.get(), v.P,
                                                   count);
    cuda_check(cudaGetLastError(), "init launch");
    build_work_tables(e, members, class_ids);
    ensure_branches(e, std::max(v.classes.size(), v.chains.size()));
    // one graph of kGraphIterations iterations, replayed; the batch index is device state
    capture_graph(e, s);
    v.done = 0;
    v.active = true;
}

// The batched or one-step graph for the next replays, from the average
// construction steps per ant and iteration since the last reading (the
// colonies' counters, read after the stream drains: one synchronisation per
// kAdaptIterations iterations).  Results do not depend on the choice.
void choose_variant(faco_engine* e) {
    auto& v = e->eval;
    std::vector<faco::ColonyState> states(v.count);
    e->states.download(states.data(), v.count, e->stream);
    cuda_check(cudaStreamSynchronize(e->stream), "step counters");
    unsigned long long steps = 0;
    for (const auto& st : states) steps += st.construction_steps;
    if (!v.rebase && v.done > v.done_seen && steps >= v.steps_seen) {
        const double per_ant = static_cast<double>(steps - v.steps_seen) /
                               (static_cast<double>(v.done - v.done_seen) * v.count * std::max(1u, v.L.ants));
        if (!v.batched && per_ant >= v.batch_on) v.batched = true;
        else if (v.batched && per_ant < v.batch_off) v.batched = false;
    }
    v.steps_seen = steps;
    v.done_seen = v.done;
    v.rebase = false;
}

void step_evaluation(faco_engine* e, std::uint32_t iterations) {
    auto& v = e->eval;
    require(v.active, "no active evaluation");
    const auto adapt = [&] {
        if (v.adaptive && (v.rebase || v.done >= v.done_seen + kAdaptIterations)) choose_variant(e);
    };
    std::uint32_t left = iterations;
    while (left >= kGraphIterations) {
        adapt();
        cuda_check(cudaGraphLaunch(v.adaptive && v.batched ? v.exec_batched : v.exec, e->stream), "graph launch");
        left -= kGraphIterations;
        v.done += kGraphIterations;
    }
    // the rest as direct launches, of the same variant the graphs would run
    if (left) {
        adapt();
        if (v.adaptive && v.batched) {
            BatchedModes batched(v);
            enqueue_iterations(e, e->stream, left);
        } else {
            enqueue_iterations(e, e->stream, left);
        }
    }
    v.done += left;
}

void finish_evaluation(faco_engine* e, faco_outputs* out, std::uint32_t dimension) {
    auto& v = e->eval;
    require(v.active, "no active evaluation");
    v.active = false;
    destroy_graph(e);
    cudaStream_t s = e->stream;
    cuda_check(cudaStreamSynchronize(s), "evaluation");
    const unsigned err = e->read_error();
    if (err) throw Error(FACO_EDEVICE, "device error word " + std::to_string(err));
    if (!out) return;
    std::vector<faco::node_t> global(v.node_total);
    e->global.download(global.data(), v.node_total, s);
    std::vector<faco::ColonyState> states(v.count);
    e->states.download(states.data(), v.count, s);
    std::vector<faco::RefControl> refs;
    if (v.feature_spec == 2) {
        refs.resize(v.count);
        e->ref_controls.download(refs.data(), v.count, s);
    }
    if (!v.decision_points.empty()) {
        require(out->n_decisions == v.decision_points.size() && out->decision_features && out->decision_scores &&
                    out->decision_masks && out->decision_actions,
                "decision outputs missing");
        const std::size_t slots = v.decision_points.size() * v.count;
        e->decision_features.download(out->decision_features, slots * 12 * 32, s);
        e->decision_scores.download(out->decision_scores, slots * 32, s);
        e->decision_masks.download(out->decision_masks, slots, s);
        e->decision_actions.download(reinterpret_cast<std::int32_t*>(out->decision_actions), slots, s);
    }
    if (out->trace && v.trace_cap) {
        static_assert(sizeof(faco::TraceRow) == sizeof(faco_trace_row), "trace row layout");
        e->trace.download(reinterpret_cast<faco::TraceRow*>(out->trace),
                          static_cast<std::size_t>(std::min(v.trace_cap, v.done)) * v.count, s);
    }
    cuda_check(cudaStreamSynchronize(s), "download");
    std::uint64_t steps = 0, evals = 0, reversed = 0;
    std::size_t node_off = 0;
    // Final verification of every incumbent on the host (batch_engine.cu:1075-1089):
    // a complete permutation whose recomputed length equals the device cost.
    // Colonies are split over host threads; the first failure is reported.
    {
        std::vector<std::size_t> offsets(v.count);
        for (std::uint32_t c = 0; c < v.count; ++c) {
            offsets[c] = node_off;
            node_off += faco::pad8(v.sizes[c]);
        }
        std::vector<const std::vector<std::int32_t>*> coords(v.count);
        for (std::uint32_t c = 0; c < v.count; ++c) coords[c] = &e->instances.at(v.keys[c])->xy;
        std::vector<int> verdict(v.count, 0);
        auto verify = [&](std::uint32_t first, std::uint32_t stride) {
            std::vector<std::uint32_t> tour;
            std::vector<std::uint8_t> seen;
            for (std::uint32_t c = first; c < v.count; c += stride) {
                const std::uint32_t n = v.sizes[c];
                tour.assign(global.begin() + offsets[c], global.begin() + offsets[c] + n);
                seen.assign(n, 0);
                bool permutation = true;
                for (const std::uint32_t node : tour) {
                    if (node >= n || seen[node]) { permutation = false; break; }
                    seen[node] = 1;
                }
                verdict[c] = !permutation ? 1
                           : faco::host_tour_length(*coords[c], tour.data(), n) != states[c].global_cost ? 2 : 0;
            }
        };
        const std::size_t total_nodes = node_off;
        const std::uint32_t workers = static_cast<std::uint32_t>(std::min<std::size_t>(
            std::max(1u, std::min(16u, std::thread::hardware_concurrency())), 1 + total_nodes / 65536));
        std::vector<std::thread> pool;
        for (std::uint32_t t = 1; t < workers; ++t) pool.emplace_back(verify, t, workers);
        verify(0, workers);
        for (auto& th : pool) th.join();
        for (std::uint32_t c = 0; c < v.count; ++c) {
            require(verdict[c] != 1, "device incumbent is not a complete permutation");
            require(verdict[c] != 2, "device incumbent cost differs from its full recomputation");
        }
    }
    node_off = 0;
    for (std::uint32_t c = 0; c < v.count; ++c) {
        const std::uint32_t n = v.sizes[c];
        if (out->tours)
            for (std::uint32_t i = 0; i < dimension; ++i)
                out->tours[static_cast<std::size_t>(c) * dimension + i] = i < n ? global[node_off + i] : UINT32_MAX;
        if (out->costs) out->costs[c] = states[c].global_cost;
        if (out->colony_work) {
            out->colony_work[3 * c] = states[c].construction_steps;
            out->colony_work[3 * c + 1] = states[c].ls_evaluations;
            out->colony_work[3 * c + 2] = states[c].reversed_elements;
        }
        if (out->control_states) {
            faco_control_state& row = out->control_states[c];
            row = faco_control_state{};
            if (v.feature_spec == 2) {
                const faco::RefControl& r = refs[c];
                row.restarts = r.restarts;
                row.stagnant_batches = r.stagnant_batches;
                row.epoch_batches = r.epoch_batches;
                row.return_rate = r.return_rate;
                row.ls_work = r.ls_work;
                row.archive_size = r.archive_size;
            } else {
                row.restarts = states[c].restarts;
                row.stagnant_batches = states[c].iteration - states[c].last_improvement;
                row.epoch_batches = states[c].iteration - states[c].last_restart;
            }
            row.start_region = states[c].region;
            row.mne_target = states[c].mne_target;
        }
        steps += states[c].construction_steps;
        evals += states[c].ls_evaluations;
        reversed += states[c].reversed_elements;
        node_off += faco::pad8(n);
    }
    out->completed_batches = v.done;
    out->construction_steps = steps;
    out->ls_evaluations = evals;
    out->reversed_elements = reversed;
}

}  // namespace

extern "C" {

void* faco_engine_stream(faco_engine* e) { return e ? static_cast<void*>(e->stream) : nullptr; }

}  // extern "C"

namespace {

// ---- colony snapshots (counted_state.hpp:23-38, batch_engine.cu:207-261) ----
// A snapshot is the whole persistent state of a stepwise evaluation: the
// panel, the controllers, every ColonyState and the per-colony trails,
// products, eta and parent/epoch/global tours, framed by a header and closed
// by an FNV-1a checksum.  Ant tours are scratch of one iteration and are not
// kept.  The Philox streams are keyed by the iteration counter kept in the
// colony states, so a restored evaluation continues bit for bit.
constexpr char kSnapshotMagic[8] = {'F', 'A', 'C', 'O', 'S', 'N', 'P', '1'};
constexpr std::uint32_t kSnapshotVersion = 3;
static_assert(sizeof(faco::ColonyState) == 104, "snapshot layout (the Python reader's ColonyState size)");

struct SnapshotHeader {
    char magic[8];
    std::uint32_t version, count, ants, k_common;
    std::uint32_t mne_target, n_programs, action_mask, total_iterations;
    std::uint32_t controlled, done, feature_spec, reserved1;
    std::uint64_t settings_digest, tau_total, node_total;
};

std::uint64_t fnv1a(const void* data, std::size_t bytes, std::uint64_t h = 1469598103934665603ull) {
    const auto* p = static_cast<const unsigned char*>(data);
    for (std::size_t i = 0; i < bytes; ++i) h = (h ^ p[i]) * 1099511628211ull;
    return h;
}

// Everything in the settings that changes the search after registration.
std::uint64_t settings_digest(const faco_settings& c, std::uint32_t ants) {
    std::uint64_t h = fnv1a(&ants, sizeof ants);
    const std::uint32_t u[5] = {c.primary_width, c.backup_width, c.ls_width, c.ls_mode,
                                c.force_fingerprint_collisions};
    const double d[4] = {c.beta, c.retention, c.p_best, c.epoch_source_probability};
    h = fnv1a(u, sizeof u, h);
    h = fnv1a(d, sizeof d, h);
    return fnv1a(&c.ls_evaluation_limit, sizeof c.ls_evaluation_limit, h);
}

std::uint64_t coordinate_digest(const Instance& in) { return fnv1a(in.xy.data(), in.xy.size() * sizeof(std::int32_t)); }

struct SnapshotWriter {
    unsigned char* out;
    std::uint64_t capacity, used = 0;
    void put(const void* data, std::size_t bytes) {
        if (out && used + bytes <= capacity) std::memcpy(out + used, data, bytes);
        used += bytes;
    }
};

template <class T>
std::vector<T> fetch(const DeviceBuffer<T>& d, std::size_t count, cudaStream_t s) {
    std::vector<T> h(count);
    d.download(h.data(), count, s);
    return h;
}

}  // namespace

extern "C" {

int faco_begin_programs(faco_engine* e, const uint64_t* keys, const uint64_t* seeds, uint32_t count,
                        const struct faco_program* programs, uint32_t n_programs, uint32_t action_mask,
                        uint32_t initial_mne, uint32_t total_iterations, uint32_t trace_iterations) {
    return guarded([&] {
        require(e != nullptr && programs != nullptr, "null argument");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        require(total_iterations >= 1, "total_iterations must be positive");
        require(n_programs >= 1, "controller programs missing");
        const JointSlots joint(programs, n_programs);
        Control control;
        control.programs = joint.slots.data();
        control.kinds = joint.kinds.data();
        control.n_programs = n_programs;
        control.action_mask = action_mask;
        control.total_iterations = total_iterations;
        begin_evaluation(e, keys, seeds, count, initial_mne, trace_iterations, control);
    });
}

int faco_snapshot(faco_engine* e, void* buffer, uint64_t capacity, uint64_t* bytes) {
    return guarded([&] {
        require(e && bytes, "null argument");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        auto& v = e->eval;
        require(v.active, "no active evaluation");
        cudaStream_t s = e->stream;
        cuda_check(cudaStreamSynchronize(s), "snapshot");
        const unsigned err = e->read_error();
        if (err) throw Error(FACO_EDEVICE, "device error word " + std::to_string(err));
        SnapshotHeader h{};
        std::memcpy(h.magic, kSnapshotMagic, 8);
        h.version = kSnapshotVersion;
        h.count = v.count;
        h.ants = e->ants;
        h.k_common = e->instances.at(v.keys[0])->k;
        h.mne_target = v.P.mne_target;
        h.n_programs = static_cast<std::uint32_t>(v.kinds.size());
        h.action_mask = v.action_mask;
        h.total_iterations = v.P.total_iterations;
        h.controlled = v.P.controlled;
        h.done = v.done;
        h.feature_spec = v.feature_spec;
        h.settings_digest = settings_digest(e->settings, e->ants);
        h.tau_total = v.tau_total;
        h.node_total = v.node_total;
        SnapshotWriter w{static_cast<unsigned char*>(buffer), buffer ? capacity : 0};
        w.put(&h, sizeof h);
        w.put(v.keys.data(), v.count * sizeof(std::uint64_t));
        w.put(v.seeds.data(), v.count * sizeof(std::uint64_t));
        for (std::uint32_t c = 0; c < v.count; ++c) {
            const std::uint64_t d = coordinate_digest(*e->instances.at(v.keys[c]));
            w.put(&d, sizeof d);
        }
        w.put(v.programs.data(), v.programs.size() * sizeof(faco_program));   // 3 slots per controller
        w.put(v.kinds.data(), v.kinds.size() * sizeof(std::uint32_t));
        if (buffer) {
            const auto states = fetch(e->states, v.count, s);
            const auto trails = fetch(e->trails, v.tau_total, s);
            const auto products = fetch(e->products, v.tau_total, s);
            const auto eta = fetch(e->colony_eta, v.tau_total, s);
            const auto parent = fetch(e->parent, v.node_total, s);
            const auto nbr = fetch(e->parent_nbr, v.node_total, s);
            const auto epoch = fetch(e->epoch, v.node_total, s);
            const auto global = fetch(e->global, v.node_total, s);
            std::vector<faco::RefControl> refs;
            std::vector<faco::node_t> archives;
            if (v.feature_spec == 2) {
                refs = fetch(e->ref_controls, v.count, s);
                archives = fetch(e->archives, 16 * v.node_total, s);
            }
            cuda_check(cudaStreamSynchronize(s), "snapshot download");
            w.put(states.data(), states.size() * sizeof(faco::ColonyState));
            w.put(trails.data(), trails.size() * sizeof(float));
            w.put(products.data(), products.size() * sizeof(float));
            w.put(eta.data(), eta.size() * sizeof(float));
            w.put(parent.data(), parent.size() * sizeof(faco::node_t));
            w.put(nbr.data(), nbr.size() * sizeof(std::uint32_t));
            w.put(epoch.data(), epoch.size() * sizeof(faco::node_t));
            w.put(global.data(), global.size() * sizeof(faco::node_t));
            w.put(refs.data(), refs.size() * sizeof(faco::RefControl));
            w.put(archives.data(), archives.size() * sizeof(faco::node_t));
        } else {
            w.used += v.count * sizeof(faco::ColonyState) + 3 * v.tau_total * sizeof(float) +
                      v.node_total * (3 * sizeof(faco::node_t) + sizeof(std::uint32_t));
            if (v.feature_spec == 2)
                w.used += v.count * sizeof(faco::RefControl) + 16 * v.node_total * sizeof(faco::node_t);
        }
        const std::uint64_t total = w.used + sizeof(std::uint64_t);
        *bytes = total;
        if (!buffer) return;
        require(capacity >= total, "snapshot buffer too small");
        const std::uint64_t sum = fnv1a(buffer, w.used);
        std::memcpy(static_cast<unsigned char*>(buffer) + w.used, &sum, sizeof sum);
    });
}

int faco_restore(faco_engine* e, const void* buffer, uint64_t bytes, uint32_t trace_iterations) {
    return guarded([&] {
        require(e && buffer, "null argument");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        const auto* p = static_cast<const unsigned char*>(buffer);
        require(bytes >= sizeof(SnapshotHeader) + sizeof(std::uint64_t), "snapshot too short");
        std::uint64_t sum;
        std::memcpy(&sum, p + bytes - sizeof sum, sizeof sum);
        require(fnv1a(p, bytes - sizeof sum) == sum, "snapshot checksum mismatch");
        SnapshotHeader h;
        std::memcpy(&h, p, sizeof h);
        require(std::memcmp(h.magic, kSnapshotMagic, 8) == 0 && h.version == kSnapshotVersion,
                "not a snapshot of this engine version");
        require(h.ants == e->ants && h.settings_digest == settings_digest(e->settings, e->ants),
                "snapshot settings differ from the engine's");
        require(h.count >= 1 && h.count <= e->capacity, "snapshot panel exceeds the engine's colonies");
        std::size_t off = sizeof h;
        auto take = [&](std::size_t n) {
            require(off + n + sizeof sum <= bytes, "snapshot truncated");
            const unsigned char* at = p + off;
            off += n;
            return at;
        };
        std::vector<std::uint64_t> keys(h.count), seeds(h.count), digests(h.count);
        std::memcpy(keys.data(), take(h.count * 8ull), h.count * 8ull);
        std::memcpy(seeds.data(), take(h.count * 8ull), h.count * 8ull);
        std::memcpy(digests.data(), take(h.count * 8ull), h.count * 8ull);
        for (std::uint32_t c = 0; c < h.count; ++c) {
            const auto it = e->instances.find(keys[c]);
            require(it != e->instances.end(), "snapshot instance not registered");
            require(coordinate_digest(*it->second) == digests[c], "snapshot instance coordinates differ");
        }
        std::vector<faco_program> programs(3ull * h.n_programs);
        std::vector<std::uint32_t> kinds(h.n_programs);
        std::memcpy(programs.data(), take(programs.size() * sizeof(faco_program)), programs.size() * sizeof(faco_program));
        std::memcpy(kinds.data(), take(kinds.size() * sizeof(std::uint32_t)), kinds.size() * sizeof(std::uint32_t));
        require(static_cast<bool>(h.controlled) == (h.n_programs > 0), "snapshot controller fields inconsistent");
        const unsigned char* states = take(h.count * sizeof(faco::ColonyState));
        const unsigned char* trails = take(h.tau_total * sizeof(float));
        const unsigned char* products = take(h.tau_total * sizeof(float));
        const unsigned char* eta = take(h.tau_total * sizeof(float));
        const unsigned char* parent = take(h.node_total * sizeof(faco::node_t));
        const unsigned char* nbr = take(h.node_total * sizeof(std::uint32_t));
        const unsigned char* epoch = take(h.node_total * sizeof(faco::node_t));
        const unsigned char* global = take(h.node_total * sizeof(faco::node_t));
        require(h.feature_spec == 0 || h.feature_spec == 2 || h.feature_spec == 3, "snapshot feature spec unknown");
        const bool ref = h.feature_spec == 2;
        const unsigned char* refs = ref ? take(h.count * sizeof(faco::RefControl)) : nullptr;
        const unsigned char* archives = ref ? take(16 * h.node_total * sizeof(faco::node_t)) : nullptr;
        require(off + sizeof sum == bytes, "snapshot has trailing bytes");
        Control control;
        if (h.n_programs) {
            control.programs = programs.data();
            control.kinds = kinds.data();
            control.n_programs = h.n_programs;
            control.action_mask = h.action_mask;
        }
        control.total_iterations = h.total_iterations;
        begin_evaluation(e, keys.data(), seeds.data(), h.count, h.mne_target, trace_iterations, control);
        auto& v = e->eval;
        try {
            require(v.tau_total == h.tau_total && v.node_total == h.node_total &&
                        e->instances.at(keys[0])->k == h.k_common,
                    "snapshot layout differs from the engine's");
            cudaStream_t s = e->stream;
            auto put = [&](void* dst, const unsigned char* src, std::size_t n) {
                cuda_check(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, s), "snapshot upload");
            };
            put(e->states.get(), states, h.count * sizeof(faco::ColonyState));
            put(e->trails.get(), trails, h.tau_total * sizeof(float));
            put(e->products.get(), products, h.tau_total * sizeof(float));
            put(e->colony_eta.get(), eta, h.tau_total * sizeof(float));
            put(e->parent.get(), parent, h.node_total * sizeof(faco::node_t));
            put(e->parent_nbr.get(), nbr, h.node_total * sizeof(std::uint32_t));
            put(e->epoch.get(), epoch, h.node_total * sizeof(faco::node_t));
            put(e->global.get(), global, h.node_total * sizeof(faco::node_t));
            require(v.feature_spec == h.feature_spec, "snapshot controller spec differs");
            if (ref) {
                put(e->ref_controls.get(), refs, h.count * sizeof(faco::RefControl));
                put(e->archives.get(), archives, 16 * h.node_total * sizeof(faco::node_t));
            }
            cuda_check(cudaStreamSynchronize(s), "snapshot upload");
            v.done = h.done;
            v.done_seen = v.done;   // the restored counters run from iteration 0: rebase first
            v.rebase = true;
        } catch (...) {
            v.active = false;
            destroy_graph(e);
            cudaStreamSynchronize(e->stream);
            throw;
        }
    });
}

int faco_begin(faco_engine* e, const uint64_t* keys, const uint64_t* seeds, uint32_t count, uint32_t mne_target,
               uint32_t trace_iterations) {
    return guarded([&] {
        require(e != nullptr, "null engine");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        begin_evaluation(e, keys, seeds, count, mne_target, trace_iterations);
    });
}

int faco_step(faco_engine* e, uint32_t iterations) {
    return guarded([&] {
        require(e != nullptr, "null engine");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        step_evaluation(e, iterations);
    });
}

int faco_step_timed(faco_engine* e, uint32_t iterations, double* ant_ms, double* update_ms) {
    return guarded([&] {
        require(e && ant_ms && update_ms, "null argument");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        auto& v = e->eval;
        require(v.active, "no active evaluation");
        cudaStream_t s = e->stream;
        std::vector<cudaEvent_t> ev(3 * iterations);
        for (auto& x : ev) cuda_check(cudaEventCreate(&x), "event");
        for (std::uint32_t i = 0; i < iterations; ++i) {
            // the variant step_evaluation would run (its check falls between
            // iterations, outside the timed kernels)
            if (v.adaptive && (v.rebase || v.done >= v.done_seen + kAdaptIterations)) choose_variant(e);
            std::optional<BatchedModes> batched;
            if (v.adaptive && v.batched) batched.emplace(v);
            cuda_check(cudaEventRecord(ev[3 * i], s), "event");
            enqueue_ants(e, s);
            cuda_check(cudaEventRecord(ev[3 * i + 1], s), "event");
            enqueue_update(e, s);
            cuda_check(cudaEventRecord(ev[3 * i + 2], s), "event");
            v.done += 1;
        }
        cuda_check(cudaStreamSynchronize(s), "timed step");
        double a = 0, u = 0;
        for (std::uint32_t i = 0; i < iterations; ++i) {
            float x = 0, y = 0;
            cuda_check(cudaEventElapsedTime(&x, ev[3 * i], ev[3 * i + 1]), "elapsed");
            cuda_check(cudaEventElapsedTime(&y, ev[3 * i + 1], ev[3 * i + 2]), "elapsed");
            a += x;
            u += y;
        }
        for (auto& x : ev) cudaEventDestroy(x);
        *ant_ms = a;
        *update_ms = u;
    });
}

int faco_get_launch_plan(faco_engine* e, faco_launch_plan* plan) {
    return guarded([&] {
        require(e && plan, "null argument");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        const auto& v = e->eval;
        const std::uint32_t per_update = (v.P.ref_control ? 2u : 1u) + (v.P.trail_blocks > 1 ? 1u : 0u);   // fingerprints + update + trails
        const auto chains = static_cast<std::uint32_t>(v.chains.size());
        plan->size_classes = static_cast<std::uint32_t>(v.classes.size());
        plan->chains = chains;
        plan->graph_iterations = kGraphIterations;
        plan->launches_per_iteration = chains ? chains * (1 + per_update) : plan->size_classes + per_update;
        plan->follow = v.adaptive ? 2u : v.follow ? 1u : 0u;
    });
}

int faco_finish(faco_engine* e, faco_outputs* out) {
    return guarded([&] {
        require(e != nullptr, "null engine");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        finish_evaluation(e, out, e->dimension);
    });
}

}  // extern "C"

namespace {
int evaluate_impl(faco_engine* e, const uint64_t* keys, const uint64_t* seeds, uint32_t count,
                  uint64_t evaluation_limit, uint32_t mne_target, const uint64_t* checkpoint_iterations,
                  uint32_t n_checkpoints, faco_outputs* out, Control control) {
    return guarded([&] {
        require(e && keys && seeds && out, "null argument");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "only one active evaluation per engine");
        const auto started = Clock::now();
        const std::uint32_t A = e->ants;
        require(evaluation_limit % A == 0 && evaluation_limit / A <= UINT32_MAX,
                "evaluation limit must be a whole number of ant batches");
        const std::uint32_t T = static_cast<std::uint32_t>(evaluation_limit / A);
        for (std::uint32_t i = 0; i < n_checkpoints; ++i) {
            require(checkpoint_iterations[i] <= T, "checkpoint beyond the budget");
            require(i == 0 || checkpoint_iterations[i] > checkpoint_iterations[i - 1],
                    "checkpoints must be strictly increasing");
        }
        require(n_checkpoints == 0 || out->checkpoint_tours, "checkpoint output missing");
        for (std::uint32_t i = 0; i < out->n_decisions; ++i) {
            require(out->decision_iterations, "decision iterations missing");
            const std::uint32_t p = out->decision_iterations[i];
            require(p >= 1 && p <= T && (i == 0 || p > out->decision_iterations[i - 1]),
                    "decision iterations must be strictly increasing batch numbers within the budget");
        }
        control.total_iterations = T;
        control.decision_points = out->decision_iterations;
        control.n_decisions = out->n_decisions;
        begin_evaluation(e, keys, seeds, count, mne_target, out->trace ? T : 0, control);
        auto& v = e->eval;
        try {
            if (n_checkpoints) e->checkpoints.resize(static_cast<std::size_t>(n_checkpoints) * v.node_total);
            cudaStream_t s = e->stream;
            cudaEvent_t ev0, ev1;
            cuda_check(cudaEventCreate(&ev0), "event");
            cuda_check(cudaEventCreate(&ev1), "event");
            std::uint32_t cp = 0;
            auto checkpoint = [&]() {
                while (cp < n_checkpoints && checkpoint_iterations[cp] == v.done) {
                    cuda_check(cudaMemcpyAsync(e->checkpoints.get() + static_cast<std::size_t>(cp) * v.node_total,
                                               e->global.get(), v.node_total * sizeof(faco::node_t),
                                               cudaMemcpyDeviceToDevice, s),
                               "checkpoint copy");
                    ++cp;
                }
            };
            cuda_check(cudaEventRecord(ev0, s), "event record");
            checkpoint();
            while (v.done < T) {
                const std::uint32_t stop = cp < n_checkpoints ? static_cast<std::uint32_t>(checkpoint_iterations[cp]) : T;
                step_evaluation(e, stop - v.done);
                checkpoint();
            }
            cuda_check(cudaEventRecord(ev1, s), "event record");
            cuda_check(cudaStreamSynchronize(s), "evaluation");
            float ms = 0;
            cuda_check(cudaEventElapsedTime(&ms, ev0, ev1), "event time");
            cudaEventDestroy(ev0);
            cudaEventDestroy(ev1);
            std::vector<faco::node_t> cps;
            if (n_checkpoints) {
                cps.resize(static_cast<std::size_t>(n_checkpoints) * v.node_total);
                e->checkpoints.download(cps.data(), cps.size(), s);
            }
            const std::vector<std::uint32_t> sizes = v.sizes;
            const std::size_t node_total = v.node_total;
            finish_evaluation(e, out, e->dimension);
            const std::uint32_t D = e->dimension;
            std::size_t node_off = 0;
            for (std::uint32_t c = 0; c < count; ++c) {
                for (std::uint32_t p = 0; p < n_checkpoints; ++p)
                    for (std::uint32_t i = 0; i < D; ++i)
                        out->checkpoint_tours[(static_cast<std::size_t>(p) * count + c) * D + i] =
                            i < sizes[c] ? cps[static_cast<std::size_t>(p) * node_total + node_off + i] : UINT32_MAX;
                node_off += faco::pad8(sizes[c]);
            }
            out->kernel_milliseconds = ms;
            out->solve_seconds = seconds_since(started);
        } catch (...) {
            if (v.active) {
                v.active = false;
                destroy_graph(e);
                cudaStreamSynchronize(e->stream);
            }
            throw;
        }
    });
}


}  // namespace

extern "C" {

int faco_evaluate(faco_engine* e, const uint64_t* keys, const uint64_t* seeds, uint32_t count,
                  uint64_t evaluation_limit, uint32_t mne_target, const uint64_t* checkpoint_iterations,
                  uint32_t n_checkpoints, faco_outputs* out) {
    return evaluate_impl(e, keys, seeds, count, evaluation_limit, mne_target, checkpoint_iterations, n_checkpoints,
                         out, Control{});
}

int faco_evaluate_programs(faco_engine* e, const uint64_t* keys, const uint64_t* seeds, uint32_t count,
                           uint64_t evaluation_limit, const faco_program* programs, uint32_t n_programs,
                           uint32_t action_mask, uint32_t initial_mne, const uint64_t* checkpoint_iterations,
                           uint32_t n_checkpoints, faco_outputs* out) {
    if (!programs || n_programs == 0) {
        g_error = "controller programs missing";
        return FACO_EINVAL;
    }
    const JointSlots joint(programs, n_programs);
    Control control;
    control.programs = joint.slots.data();
    control.kinds = joint.kinds.data();
    control.n_programs = n_programs;
    control.action_mask = action_mask;
    return evaluate_impl(e, keys, seeds, count, evaluation_limit, initial_mne, checkpoint_iterations, n_checkpoints,
                         out, control);
}

int faco_evaluate_controllers(faco_engine* e, const uint64_t* keys, const uint64_t* seeds, uint32_t count,
                              uint64_t evaluation_limit, const faco_program* trees, const uint32_t* kinds,
                              uint32_t n_controllers, uint32_t action_mask, uint32_t initial_mne,
                              const uint64_t* checkpoint_iterations, uint32_t n_checkpoints, faco_outputs* out) {
    if (!trees || !kinds || n_controllers == 0) {
        g_error = "controllers missing";
        return FACO_EINVAL;
    }
    Control control;
    control.programs = trees;
    control.kinds = kinds;
    control.n_programs = n_controllers;
    control.action_mask = action_mask;
    return evaluate_impl(e, keys, seeds, count, evaluation_limit, initial_mne, checkpoint_iterations, n_checkpoints,
                         out, control);
}

int faco_validate_controller(const faco_program* trees, uint32_t kind) {
    return guarded([&] {
        require(trees != nullptr, "null controller");
        validate_controller(trees, kind);
    });
}

int faco_validate_program(const faco_program* p) {
    return guarded([&] {
        require(p != nullptr, "null program");
        const bool extended = p->numeric_spec_id == 2;
        require(p->ir_version == 1 && (p->numeric_spec_id == 1 || extended) &&
                    p->feature_spec_id >= 1 && p->feature_spec_id <= 3 && p->length >= 1 && p->length <= 63 &&
                    p->constants_count <= 63,
                "unknown version or program size out of range");
        for (int i = 0; i < p->constants_count; ++i)
            require(std::isfinite(p->constants[i]) && std::fabs(p->constants[i]) <= 2.0f,
                    "ERC must be finite and in [-2, 2]");
        int depth[64], top = 0;
        const int max_op = extended ? 10 : 8, max_depth = extended ? 6 : 5, max_stack = extended ? 16 : 6;
        for (int i = 0; i < p->length; ++i) {
            const int op = p->opcode[i], operand = p->operand[i];
            if (op == 0 || op == 1) {
                require(!((op == 0 && operand >= 12) || (op == 1 && operand >= p->constants_count)),
                        "terminal index out of range");
                depth[top++] = 0;
            } else {
                require(op >= 2 && op <= max_op, "unknown opcode");
                const int arity = op == 7 ? 1 : op == 10 ? 3 : 2;
                require(operand == 0 && top >= arity, "function operand non-zero or stack underflow");
                int dmax = 0;
                for (int j = top - arity; j < top; ++j) dmax = std::max(dmax, depth[j]);
                top -= arity;
                require(dmax + 1 <= max_depth, "tree too deep");
                depth[top++] = dmax + 1;
            }
            require(top <= max_stack, "stack peak too high");
        }
        require(top == 1, "final stack is not a single value");
    });
}

int faco_score(const faco_program* programs, uint32_t n_programs, const float* features, uint32_t features_count,
               const uint32_t* masks, uint32_t colonies, float* scores, int32_t* actions) {
    return guarded([&] {
        require(programs && features && masks && scores && actions, "null argument");
        require(n_programs >= 1 && colonies >= 1 && colonies % n_programs == 0,
                "colonies must be a multiple of the program count");
        require(features_count == 12, "features must be [12, colonies, 32]");
        for (std::uint32_t i = 0; i < n_programs; ++i)
            if (faco_validate_program(programs + i) != FACO_OK) throw Error(FACO_EINVAL, g_error);
        const std::size_t nf = static_cast<std::size_t>(features_count) * colonies * 32;
        for (std::size_t i = 0; i < nf; ++i)
            require(std::isfinite(features[i]) && features[i] >= 0.0f && features[i] <= 1.0f,
                    "features must be finite and in [0, 1]");
        for (std::uint32_t c = 0; c < colonies; ++c) require(masks[c] != 0, "a colony has no legal action");
        static_assert(sizeof(faco::Program) == sizeof(faco_program), "program layout");
        DeviceBuffer<faco::Program> d_prog;
        DeviceBuffer<float> d_feat, d_scores;
        DeviceBuffer<std::uint32_t> d_masks;
        DeviceBuffer<std::int32_t> d_actions;
        cudaStream_t s = nullptr;
        d_prog.upload(reinterpret_cast<const faco::Program*>(programs), n_programs, s);
        d_feat.upload(features, nf, s);
        d_masks.upload(masks, colonies, s);
        d_scores.resize(static_cast<std::size_t>(colonies) * 32);
        d_actions.resize(colonies);
        const std::uint32_t blocks = (colonies * 32 + 127) / 128;
        faco::score_kernel<<<blocks, 128, 0, s>>>(d_prog.get(), colonies / n_programs, d_feat.get(), d_masks.get(),
                                                  d_scores.get(), d_actions.get(), colonies);
        cuda_check(cudaGetLastError(), "score launch");
        d_scores.download(scores, static_cast<std::size_t>(colonies) * 32, s);
        d_actions.download(actions, colonies, s);
        cuda_check(cudaStreamSynchronize(s), "score");
    });
}

int faco_score_controllers(const faco_program* trees, const uint32_t* kinds, uint32_t n_controllers,
                           const float* features, uint32_t features_count, const uint32_t* masks, uint32_t colonies,
                           float* scores, int32_t* actions) {
    return guarded([&] {
        require(trees && kinds && features && masks && scores && actions, "null argument");
        require(n_controllers >= 1 && colonies >= 1 && colonies % n_controllers == 0,
                "colonies must be a multiple of the controller count");
        require(features_count == 12, "features must be [12, colonies, 32]");
        for (std::uint32_t i = 0; i < n_controllers; ++i) validate_controller(trees + 3ull * i, kinds[i]);
        const std::size_t nf = static_cast<std::size_t>(features_count) * colonies * 32;
        for (std::size_t i = 0; i < nf; ++i)
            require(std::isfinite(features[i]) && features[i] >= 0.0f && features[i] <= 1.0f,
                    "features must be finite and in [0, 1]");
        for (std::uint32_t c = 0; c < colonies; ++c) require(masks[c] != 0, "a colony has no legal action");
        DeviceBuffer<faco::Program> d_trees;
        DeviceBuffer<std::uint32_t> d_kinds, d_masks;
        DeviceBuffer<float> d_feat, d_scores;
        DeviceBuffer<std::int32_t> d_actions;
        cudaStream_t s = nullptr;
        d_trees.upload(reinterpret_cast<const faco::Program*>(trees), 3ull * n_controllers, s);
        d_kinds.upload(kinds, n_controllers, s);
        d_feat.upload(features, nf, s);
        d_masks.upload(masks, colonies, s);
        d_scores.resize(static_cast<std::size_t>(colonies) * 32);
        cuda_check(cudaMemsetAsync(d_scores.get(), 0, static_cast<std::size_t>(colonies) * 32 * sizeof(float), s),
                   "memset");
        d_actions.resize(colonies);
        faco::score_controllers_kernel<<<(colonies * 32 + 127) / 128, 128, 0, s>>>(
            d_trees.get(), d_kinds.get(), colonies / n_controllers, d_feat.get(), d_masks.get(), d_scores.get(),
            d_actions.get(), colonies);
        cuda_check(cudaGetLastError(), "score launch");
        d_scores.download(scores, static_cast<std::size_t>(colonies) * 32, s);
        d_actions.download(actions, colonies, s);
        cuda_check(cudaStreamSynchronize(s), "score");
    });
}

int faco_ant_diagnostic(const int32_t* xy, uint32_t n, const uint32_t* ls_rows, uint32_t w, const uint32_t* tours,
                        const uint32_t* visits, const double* uniforms, const uint32_t* starts,
                        const uint32_t* primary, const float* products, uint32_t k, const uint32_t* backup,
                        uint32_t b, const uint32_t* mne_targets, uint32_t tasks, uint64_t evaluation_limit,
                        uint32_t ls_mode, faco_ant_outputs* out) {
    return guarded([&] {
        require(xy && ls_rows && tours && mne_targets && out, "null argument");
        require(n >= 3 && n <= faco::kMaxNodes && tasks >= 1, "invalid sizes");
        require(faco::block_smem_bytes(n, 1) <= 227u * 1024u, "instance too large for one warp-ant block");
        require(w >= 1 && w <= 32 && w <= n - 1, "LS width must be in [1, min(32, n-1)]");
        require(ls_mode == FACO_LS_TWO_OPT || ls_mode == FACO_LS_TWO_OPT_OR_OPT, "unknown local-search mode");
        require((visits != nullptr) != (uniforms != nullptr), "give exactly one of visits or uniforms");
        if (uniforms) require(starts && primary && products && k >= 1 && k <= 32 && k <= n - 1, "roulette inputs missing");
        std::vector<std::int32_t> hxy(xy, xy + 2ull * n);
        for (auto v : hxy) require(std::abs(v) < (1 << 26), "coordinates must satisfy |x| < 2^26");
        require_euc2d_span(hxy.data(), n);
        std::vector<std::uint16_t> ls;
        std::vector<std::int32_t> ls_dist;
        faco::host_distance_order(hxy, n, w, ls_rows, ls, ls_dist);
        std::vector<std::uint16_t> prim16, back16;
        if (uniforms) {
            prim16.assign(primary, primary + static_cast<std::size_t>(n) * k);
            for (auto v : prim16) require(v < n, "primary candidate out of range");
            if (b) {
                require(backup != nullptr, "backup rows missing");
                back16.assign(backup, backup + static_cast<std::size_t>(n) * b);
            }
        }
        std::vector<faco::node_t> t16(static_cast<std::size_t>(tasks) * n);
        std::vector<std::uint32_t> nbr(t16.size());
        std::vector<long long> costs(tasks);
        for (std::uint32_t t = 0; t < tasks; ++t) {
            std::vector<std::uint8_t> seen(n, 0);
            for (std::uint32_t i = 0; i < n; ++i) {
                const std::uint32_t v = tours[static_cast<std::size_t>(t) * n + i];
                require(v < n && !seen[v], "task tour is not a permutation");
                seen[v] = 1;
                t16[static_cast<std::size_t>(t) * n + i] = static_cast<faco::node_t>(v);
            }
            const auto tn = parent_neighbours(tours + static_cast<std::size_t>(t) * n, n);
            std::copy(tn.begin(), tn.end(), nbr.begin() + static_cast<std::size_t>(t) * n);
            costs[t] = faco::host_tour_length(hxy, tours + static_cast<std::size_t>(t) * n, n);
            if (visits) {
                std::fill(seen.begin(), seen.end(), 0);
                for (std::uint32_t i = 0; i < n; ++i) {
                    const std::uint32_t v = visits[static_cast<std::size_t>(t) * n + i];
                    require(v < n && !seen[v], "visit order is not a permutation");
                    seen[v] = 1;
                }
            } else {
                require(starts[t] < n, "start node out of range");
            }
        }
        cudaStream_t s = nullptr;
        DeviceBuffer<int2> d_xy;
        DeviceBuffer<faco::node_t> d_ls, d_prim, d_back, d_tours, d_visits, d_cons, d_out, d_outpos, d_sel;
        DeviceBuffer<int> d_lsd;
        DeviceBuffer<long long> d_costs, d_outcosts;
        DeviceBuffer<double> d_uni;
        DeviceBuffer<std::uint32_t> d_starts, d_targets, d_check, d_nbr;
        DeviceBuffer<float> d_products;
        DeviceBuffer<unsigned long long> d_counters;
        DeviceBuffer<unsigned> d_err(1);
        DeviceBuffer<faco::InstanceView> d_view;
        d_xy.upload(reinterpret_cast<const int2*>(hxy.data()), n, s);
        d_ls.upload(ls, s);
        d_lsd.upload(ls_dist, s);
        faco::InstanceView v{n, uniforms ? k : 0, uniforms ? b : 0, w, d_xy.get(), nullptr, nullptr, d_ls.get(),
                             d_lsd.get(), nullptr, nullptr, 0};
        if (uniforms) {
            d_prim.upload(prim16, s);
            d_back.resize(std::max<std::size_t>(1, back16.size()));
            d_back.upload(back16, s);
            d_products.upload(products, static_cast<std::size_t>(n) * k, s);
            v.primary = d_prim.get();
            v.backup = d_back.get();
            d_uni.upload(uniforms, static_cast<std::size_t>(tasks) * n, s);
            d_starts.upload(starts, tasks, s);
        } else {
            std::vector<faco::node_t> vis(visits, visits + static_cast<std::size_t>(tasks) * n);
            d_visits.upload(vis, s);
        }
        d_view.upload(&v, 1, s);
        d_tours.upload(t16, s);
        d_nbr.upload(nbr, s);
        d_costs.upload(costs, s);
        d_targets.upload(mne_targets, tasks, s);
        const std::size_t tn = static_cast<std::size_t>(tasks) * n;
        d_cons.resize(tn); d_out.resize(tn); d_outpos.resize(tn); d_sel.resize(tn);
        d_outcosts.resize(2ull * tasks);
        d_counters.resize(10ull * tasks);
        const std::uint32_t cap = out->checklists ? out->checklist_capacity : 0;
        if (cap) d_check.resize(static_cast<std::size_t>(tasks) * cap);
        cuda_check(cudaMemsetAsync(d_err.get(), 0, sizeof(unsigned), s), "memset");
        cuda_check(cudaMemsetAsync(d_sel.get(), 0xff, tn * sizeof(faco::node_t), s), "memset");
        faco::AntLaunch L{};
        L.instances = d_view.get();
        L.warps = choose_warps(n, tasks);
        L.n_max = n;
        L.ls_limit = evaluation_limit;
        L.ls_mode = ls_mode;
        L.tasks = tasks;
        L.task_tours = d_tours.get();
        L.task_nbr = d_nbr.get();
        L.task_costs = d_costs.get();
        L.task_visits = d_visits.get();
        L.task_uniforms = d_uni.get();
        L.task_starts = d_starts.get();
        L.task_targets = d_targets.get();
        L.task_products = d_products.get();
        L.out_construction = d_cons.get();
        L.out_tours = d_out.get();
        L.out_pos = d_outpos.get();
        L.out_selected = d_sel.get();
        L.out_checklist = cap ? d_check.get() : nullptr;
        L.checklist_cap = cap;
        L.out_costs = d_outcosts.get();
        L.out_counters = d_counters.get();
        L.error = d_err.get();
        const std::uint32_t blocks = (tasks + L.warps - 1) / L.warps;
        launch_ants(visits ? faco::kModeVisits : faco::kModeUniforms, L, blocks, L.warps, s);
        std::vector<faco::node_t> h(tn);
        auto widen = [&](const DeviceBuffer<faco::node_t>& d, std::uint32_t* dst) {
            if (!dst) return;
            d.download(h.data(), tn, s);
            cuda_check(cudaStreamSynchronize(s), "download");
            for (std::size_t i = 0; i < tn; ++i) dst[i] = h[i] == 0xffff ? UINT32_MAX : h[i];
        };
        widen(d_cons, out->construction_tours);
        widen(d_out, out->tours);
        widen(d_outpos, out->positions);
        widen(d_sel, out->selected);
        std::vector<long long> oc(2ull * tasks);
        d_outcosts.download(oc.data(), oc.size(), s);
        std::vector<unsigned long long> counters(10ull * tasks);
        d_counters.download(counters.data(), counters.size(), s);
        if (cap) d_check.download(out->checklists, static_cast<std::size_t>(tasks) * cap, s);
        unsigned err = 0;
        d_err.download(&err, 1, s);
        cuda_check(cudaStreamSynchronize(s), "diagnostic");
        for (std::uint32_t t = 0; t < tasks; ++t) {
            if (out->construction_costs) out->construction_costs[t] = oc[2ull * t];
            if (out->final_costs) out->final_costs[t] = oc[2ull * t + 1];
        }
        if (out->counters) std::copy(counters.begin(), counters.end(), out->counters);
        if (err & ~static_cast<unsigned>(faco::kErrQueueOverflow))
            throw Error(FACO_EDEVICE, "device error word " + std::to_string(err));
        if (err) throw Error(FACO_EINVAL, "checklist capacity too small for the recorded pushes");
    });
}

int faco_pheromone_step(uint32_t n, uint32_t k, const uint32_t* primary, const uint32_t* parent, float retention,
                        float minimum, float maximum, float increment, const float* eta, float* trails,
                        float* products) {
    return guarded([&] {
        require(primary && parent && eta && trails && products && n >= 3 && n <= faco::kMaxNodes && k >= 1,
                "invalid arguments");
        std::vector<std::uint8_t> seen(n, 0);
        for (std::uint32_t i = 0; i < n; ++i) {
            require(parent[i] < n && !seen[parent[i]], "parent is not a permutation");
            seen[parent[i]] = 1;
        }
        cudaStream_t s = nullptr;
        const std::size_t cells = static_cast<std::size_t>(n) * k;
        std::vector<faco::node_t> prim16(cells);
        for (std::size_t i = 0; i < cells; ++i) {
            require(primary[i] < n, "primary candidate out of range");
            prim16[i] = static_cast<faco::node_t>(primary[i]);
        }
        DeviceBuffer<faco::node_t> d_prim;
        DeviceBuffer<std::uint32_t> d_nbr;
        DeviceBuffer<float> d_eta, d_tr, d_pr;
        d_prim.upload(prim16, s);
        d_nbr.upload(parent_neighbours(parent, n), s);
        d_eta.upload(eta, cells, s);
        d_tr.upload(trails, cells, s);
        d_pr.resize(cells);
        faco::pheromone_step_kernel<<<static_cast<unsigned>((cells + 1023) / 1024), 256, 0, s>>>(
            n, k, d_prim.get(), d_nbr.get(), retention, minimum, maximum, increment, d_eta.get(), d_tr.get(),
            d_pr.get());
        cuda_check(cudaGetLastError(), "pheromone launch");
        d_tr.download(trails, cells, s);
        d_pr.download(products, cells, s);
        cuda_check(cudaStreamSynchronize(s), "pheromone");
    });
}


// ---------------------------------------------------------------------------
// Learned edge prior: the MLP on its own (training and checks) and its use
// inside a stepwise evaluation.
// ---------------------------------------------------------------------------
int faco_mlp_param_count(void) { return faco::kMlpParamCount; }

static void upload_mlp(DeviceBuffer<faco::MlpParams>& P, DeviceBuffer<faco::MlpOperands>& O, const float* params,
                       cudaStream_t s) {
    P.resize(1);
    O.resize(1);
    P.upload(reinterpret_cast<const faco::MlpParams*>(params), 1, s);
    faco::refresh_operands_kernel<<<4, 256, 0, s>>>(P.get(), O.get());
    cuda_check(cudaGetLastError(), "operand refresh");
}

// The tcgen05 kernels ask for tc::kLaunchSmemBytes of dynamic shared memory
// (above the 48 KB default), which caps them at tc::kCtasPerSm CTAs per SM.
static cudaError_t prepare_tensor_kernels() {
    cudaError_t err = cudaFuncSetAttribute(faco::mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(faco::tc::kLaunchSmemBytes));
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(faco::prior_apply_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(faco::tc::kLaunchSmemBytes));
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(faco::mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(faco::tc::kGradSmemBytes));
    return err;
}
static std::uint32_t tensor_grid(std::uint64_t tiles) {
    return static_cast<std::uint32_t>(std::max<std::uint64_t>(1, std::min<std::uint64_t>(tiles, 152u * faco::tc::kCtasPerSm)));
}

// Gradient CTAs for `rows` rows: one per 128-row tile, at most
// tc::kGradCtasPerSm per SM (every CTA gets at least one tile).
static std::uint32_t grad_blocks(std::uint64_t rows) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        sms = 152;
    const std::uint64_t tiles = (rows + faco::tc::kRows - 1) / faco::tc::kRows;
    return static_cast<std::uint32_t>(
        std::max<std::uint64_t>(1, std::min<std::uint64_t>(tiles, static_cast<std::uint64_t>(sms) * faco::tc::kGradCtasPerSm)));
}

int faco_mlp_forward(const float* params, const uint16_t* x, uint32_t count, float* prob) {
    return guarded([&] {
        require(params && x && prob && count > 0, "invalid arguments");
        cudaStream_t s = nullptr;
        DeviceBuffer<faco::MlpParams> P;
        DeviceBuffer<faco::MlpOperands> O;
        upload_mlp(P, O, params, s);
        DeviceBuffer<__nv_bfloat16> dx;
        dx.upload(reinterpret_cast<const __nv_bfloat16*>(x), static_cast<std::size_t>(count) * faco::kMlpIn, s);
        DeviceBuffer<float> dp(count);
        DeviceBuffer<unsigned> derr(1);
        cuda_check(cudaMemsetAsync(derr.get(), 0, sizeof(unsigned), s), "memset");
        cuda_check(prepare_tensor_kernels(), "tcgen05 kernel attributes");
        faco::mlp_forward_kernel<<<tensor_grid((count + faco::tc::kRows - 1) / faco::tc::kRows), 128,
                                   faco::tc::kLaunchSmemBytes, s>>>(P.get(), O.get(), dx.get(), count, dp.get(),
                                                                    derr.get());
        cuda_check(cudaGetLastError(), "mlp forward");
        unsigned err = 0;
        dp.download(prob, count, s);
        derr.download(&err, 1, s);
        cuda_check(cudaStreamSynchronize(s), "mlp forward");
        if (err) throw Error(FACO_EDEVICE, "device error word " + std::to_string(err) + " in the MLP forward pass");
    });
}

int faco_mlp_gradient(const float* params, const uint16_t* x, const float* y, uint32_t count, float* grad,
                      float* loss) {
    return guarded([&] {
        require(params && x && y && grad && loss && count > 0, "invalid arguments");
        cudaStream_t s = nullptr;
        DeviceBuffer<faco::MlpParams> P, G;
        DeviceBuffer<faco::MlpOperands> O;
        upload_mlp(P, O, params, s);
        DeviceBuffer<__nv_bfloat16> dx;
        dx.upload(reinterpret_cast<const __nv_bfloat16*>(x), static_cast<std::size_t>(count) * faco::kMlpIn, s);
        DeviceBuffer<float> dy, dl(1);
        dy.upload(y, count, s);
        G.resize(1);
        cuda_check(cudaMemsetAsync(dl.get(), 0, sizeof(float), s), "memset");
        cuda_check(prepare_tensor_kernels(), "tcgen05 kernel attributes");
        const std::uint32_t blocks = grad_blocks(count);
        DeviceBuffer<faco::MlpParams> partials(blocks);
        DeviceBuffer<float> loss_partials(blocks);
        DeviceBuffer<unsigned> derr(1);
        cuda_check(cudaMemsetAsync(derr.get(), 0, sizeof(unsigned), s), "memset");
        faco::mlp_grad_kernel<<<blocks, 128, faco::tc::kGradSmemBytes, s>>>(
            P.get(), O.get(), dx.get(), dy.get(), count, 1.0f / count, partials.get(), loss_partials.get(), derr.get());
        faco::mlp_grad_reduce_kernel<<<20, 256, 0, s>>>(partials.get(), loss_partials.get(), blocks, G.get(),
                                                        dl.get());
        cuda_check(cudaGetLastError(), "mlp gradient");
        unsigned err = 0;
        G.download(reinterpret_cast<faco::MlpParams*>(grad), 1, s);
        dl.download(loss, 1, s);
        derr.download(&err, 1, s);
        cuda_check(cudaStreamSynchronize(s), "mlp gradient");
        if (err) throw Error(FACO_EDEVICE, "device error word " + std::to_string(err) + " in the MLP gradient");
    });
}

int faco_mlp_train(float* params, const uint16_t* x, const float* y, uint32_t count, uint32_t epochs,
                   uint32_t batch, float lr, float* epoch_losses) {
    return guarded([&] {
        require(params && x && y && count > 0 && batch > 0 && epochs > 0 && lr > 0, "invalid arguments");
        cudaStream_t s = nullptr;
        DeviceBuffer<faco::MlpParams> P, G, M, V;
        DeviceBuffer<faco::MlpOperands> O;
        upload_mlp(P, O, params, s);
        G.resize(1); M.resize(1); V.resize(1);
        cuda_check(cudaMemsetAsync(M.get(), 0, sizeof(faco::MlpParams), s), "memset");
        cuda_check(cudaMemsetAsync(V.get(), 0, sizeof(faco::MlpParams), s), "memset");
        DeviceBuffer<__nv_bfloat16> dx;
        dx.upload(reinterpret_cast<const __nv_bfloat16*>(x), static_cast<std::size_t>(count) * faco::kMlpIn, s);
        DeviceBuffer<float> dy, dl(epochs);
        dy.upload(y, count, s);
        cuda_check(cudaMemsetAsync(dl.get(), 0, sizeof(float) * epochs, s), "memset");
        const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
        std::uint64_t step = 0;
        cuda_check(prepare_tensor_kernels(), "tcgen05 kernel attributes");
        const std::uint32_t max_blocks = grad_blocks(std::min(batch, count));
        DeviceBuffer<faco::MlpParams> partials(max_blocks);
        DeviceBuffer<float> loss_partials(max_blocks);
        DeviceBuffer<unsigned> derr(1);
        cuda_check(cudaMemsetAsync(derr.get(), 0, sizeof(unsigned), s), "memset");
        for (std::uint32_t ep = 0; ep < epochs; ++ep) {
            for (std::uint32_t first = 0; first < count; first += batch) {
                const std::uint32_t size = std::min(batch, count - first);
                const std::uint32_t blocks = grad_blocks(size);
                ++step;
                faco::mlp_grad_kernel<<<blocks, 128, faco::tc::kGradSmemBytes, s>>>(
                    P.get(), O.get(), dx.get() + static_cast<std::size_t>(first) * faco::kMlpIn, dy.get() + first,
                    size, 1.0f / size, partials.get(), loss_partials.get(), derr.get());
                faco::mlp_grad_reduce_kernel<<<20, 256, 0, s>>>(partials.get(), loss_partials.get(), blocks, G.get(),
                                                                dl.get() + ep);
                const float b1 = 1.0f - std::pow(beta1, static_cast<float>(step));
                const float b2 = 1.0f - std::pow(beta2, static_cast<float>(step));
                faco::adam_kernel<<<20, 256, 0, s>>>(P.get(), G.get(), M.get(), V.get(), lr, beta1, beta2, eps, b1, b2);
                faco::refresh_operands_kernel<<<4, 256, 0, s>>>(P.get(), O.get());
                cuda_check(cudaGetLastError(), "training step");
            }
        }
        std::vector<float> losses(epochs);
        dl.download(losses.data(), epochs, s);
        unsigned err = 0;
        derr.download(&err, 1, s);
        cuda_check(cudaStreamSynchronize(s), "mlp training");
        if (err) throw Error(FACO_EDEVICE, "device error word " + std::to_string(err) + " in the MLP gradient");
        P.download(reinterpret_cast<faco::MlpParams*>(params), 1, s);
        cuda_check(cudaStreamSynchronize(s), "mlp training");
        if (epoch_losses)
            for (std::uint32_t ep = 0; ep < epochs; ++ep) epoch_losses[ep] = losses[ep] / count;
    });
}

int faco_edge_data(faco_engine* e, uint16_t* x_out, float* y_out, uint64_t capacity_rows, uint64_t* rows) {
    return guarded([&] {
        require(e != nullptr, "null engine");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        auto& v = e->eval;
        require(v.active, "no active evaluation");
        std::vector<std::uint64_t> offsets(v.count);
        std::uint64_t total = 0;
        for (std::uint32_t c = 0; c < v.count; ++c) {
            offsets[c] = total;
            total += static_cast<std::uint64_t>(v.sizes[c]) * e->instances.at(v.keys[c])->k;
        }
        if (rows) *rows = total;
        if (!x_out && !y_out) return;
        require(total <= capacity_rows, "output capacity too small");
        cudaStream_t s = e->stream;
        DeviceBuffer<std::uint64_t> d_off;
        d_off.upload(offsets, s);
        DeviceBuffer<__nv_bfloat16> dx;
        DeviceBuffer<float> dy;
        if (x_out) dx.resize(total * faco::kMlpIn);
        if (y_out) dy.resize(total);
        const std::uint32_t smem = 4u * v.n_max;
        cuda_check(cudaFuncSetAttribute(faco::edge_features_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        static_cast<int>(smem)), "attribute");
        faco::edge_features_kernel<<<v.count, 256, smem, s>>>(e->d_instances.get(), e->colonies.get(),
                                                              e->states.get(), 0, d_off.get(),
                                                              x_out ? dx.get() : nullptr, y_out ? dy.get() : nullptr);
        cuda_check(cudaGetLastError(), "edge features");
        if (x_out) dx.download(reinterpret_cast<__nv_bfloat16*>(x_out), total * faco::kMlpIn, s);
        if (y_out) dy.download(y_out, total, s);
        cuda_check(cudaStreamSynchronize(s), "edge data");
    });
}

int faco_colony_rows(faco_engine* e, uint32_t colony, float* trails, float* eta, float* products,
                     uint64_t capacity) {
    return guarded([&] {
        require(e != nullptr, "null engine");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        auto& v = e->eval;
        require(v.active, "no active evaluation");
        require(colony < v.count, "colony index out of range");
        std::size_t offset = 0;
        for (std::uint32_t c = 0; c < colony; ++c)
            offset += (static_cast<std::size_t>(v.sizes[c]) * e->instances.at(v.keys[c])->k + 3) & ~std::size_t{3};
        const std::size_t cells = static_cast<std::size_t>(v.sizes[colony]) * e->instances.at(v.keys[colony])->k;
        require((!trails && !eta && !products) || capacity >= cells, "output capacity too small");
        cudaStream_t s = e->stream;
        const std::pair<const DeviceBuffer<float>*, float*> rows[3] = {
            {&e->trails, trails}, {&e->colony_eta, eta}, {&e->products, products}};
        for (const auto& r : rows)
            if (r.second)
                cuda_check(cudaMemcpyAsync(r.second, r.first->get() + offset, cells * sizeof(float),
                                           cudaMemcpyDeviceToHost, s), "colony rows");
        cuda_check(cudaStreamSynchronize(s), "colony rows");
    });
}

static void apply_prior(faco_engine* e) {
    auto& v = e->eval;
    std::vector<std::uint32_t> offsets(v.count);
    std::uint32_t total = 0, max_cells = 0;
    for (std::uint32_t c = 0; c < v.count; ++c) {
        offsets[c] = total;
        total += faco::pad8(v.sizes[c]);
        max_cells = std::max(max_cells, v.sizes[c] * e->instances.at(v.keys[c])->k);
    }
    e->prior_offsets.upload(offsets, e->stream);
    e->prior_gnbr.resize(total);
    faco::global_neighbours_kernel<<<v.count, 256, 0, e->stream>>>(e->colonies.get(), e->prior_gnbr.get(),
                                                                    e->prior_offsets.get());
    // enough chunk blocks per colony to fill the GPU about four times over
    // 128-entry tiles; about one resident wave of CTAs (4 per SM) over all colonies
    const std::uint32_t tiles = (max_cells + faco::tc::kRows - 1) / faco::tc::kRows;
    const std::uint32_t wave = 152u * faco::tc::kCtasPerSm;
    const std::uint32_t per_colony = std::max<std::uint32_t>(1, std::min(tiles, (wave + v.count - 1) / v.count));
    const dim3 grid(per_colony, v.count);
    cuda_check(prepare_tensor_kernels(), "tcgen05 kernel attributes");
    faco::prior_apply_kernel<<<grid, 128, faco::tc::kLaunchSmemBytes, e->stream>>>(
        e->d_instances.get(), e->colonies.get(), e->states.get(), e->prior_enabled.get(), e->prior_params.get(),
        e->prior_ops.get(), e->prior_floor, e->prior_gamma, e->prior_gnbr.get(), e->prior_offsets.get(),
        e->error.get());
    cuda_check(cudaGetLastError(), "prior apply");
    faco::prior_rows_kernel<<<v.count, 256, 0, e->stream>>>(e->d_instances.get(), e->colonies.get(),
                                                            e->prior_modes.get());
    cuda_check(cudaGetLastError(), "prior rows");
}

int faco_prior_set(faco_engine* e, const float* params, float floor, int gamma, const uint8_t* enabled,
                   uint32_t departures) {
    return guarded([&] {
        require(e && enabled, "null argument");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        auto& v = e->eval;
        require(v.active, "no active evaluation");
        require(std::isfinite(floor) && floor > 0.0f, "the prior floor must be positive (no candidate removed)");
        if (params) {
            for (int i = 0; i < faco::kMlpParamCount; ++i) require(std::isfinite(params[i]), "non-finite parameter");
            upload_mlp(e->prior_params, e->prior_ops, params, e->stream);
            e->prior_loaded = true;
        }
        require(e->prior_loaded, "no prior parameters loaded");
        require(gamma == 1 || gamma == 2, "the prior exponent must be 1 or 2");
        e->prior_floor = floor;
        e->prior_gamma = gamma;
        require(departures <= 1, "departures must be 0 or 1");
        e->prior_enabled.upload(enabled, v.count, e->stream);
        std::vector<std::uint32_t> modes(v.count);
        for (std::uint32_t c = 0; c < v.count; ++c) modes[c] = enabled[c] && departures ? 1u : 0u;
        e->prior_modes.upload(modes, e->stream);
        apply_prior(e);
    });
}

int faco_prior_refresh(faco_engine* e) {
    return guarded([&] {
        require(e != nullptr, "null engine");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        require(e->eval.active && e->prior_loaded && e->prior_enabled.size() >= e->eval.count, "no prior set");
        apply_prior(e);
    });
}

int faco_current_costs(faco_engine* e, int64_t* costs, uint32_t* iterations) {
    return guarded([&] {
        require(e && costs, "null argument");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        auto& v = e->eval;
        require(v.active, "no active evaluation");
        std::vector<faco::ColonyState> st(v.count);
        e->states.download(st.data(), v.count, e->stream);
        cuda_check(cudaStreamSynchronize(e->stream), "costs");
        for (std::uint32_t c = 0; c < v.count; ++c) costs[c] = st[c].global_cost;
        if (iterations) *iterations = st[0].iteration;
    });
}

int faco_set_mne_targets(faco_engine* e, const uint32_t* targets, uint32_t count) {
    return guarded([&] {
        require(e && targets, "null argument");
        std::unique_lock<std::mutex> lock(e->busy, std::try_to_lock);
        if (!lock.owns_lock()) throw Error(FACO_EBUSY, "engine is busy with another call");
        auto& v = e->eval;
        require(v.active, "no active evaluation");
        require(!v.P.controlled, "controlled evaluations choose their MNE targets by action");
        require(count == v.count, "one target per colony");
        for (std::uint32_t c = 0; c < count; ++c) require(targets[c] >= 1, "MNE targets must be positive");
        std::vector<faco::ColonyState> st(v.count);
        e->states.download(st.data(), v.count, e->stream);
        cuda_check(cudaStreamSynchronize(e->stream), "states");
        for (std::uint32_t c = 0; c < count; ++c) st[c].mne_target = targets[c];
        e->states.upload(st, e->stream);
        cuda_check(cudaStreamSynchronize(e->stream), "states");
    });
}

// The pheromone step on caller-owned device buffers; its only scratch is a
// fixed per-device array (faco_noalloc.cu), so the success path allocates no
// device or host memory.  Checks are written without building strings until
// one fails.
int faco_pheromone_step_noalloc(uint32_t n, uint32_t k, const uint32_t* primary, const uint32_t* parent,
                                float retention, float minimum, float maximum, float increment, const float* eta,
                                float* trails, float* products, void* stream) {
    return guarded([&] {
        if (!(primary && parent && eta && trails && products)) throw Error(FACO_EINVAL, "null argument");
        if (n < 3 || k < 1) throw Error(FACO_EINVAL, "invalid sizes: n >= 3 and k >= 1 are required");
        if (n > faco::kNoAllocMaxNodes)
            throw Error(FACO_EINVAL, "n exceeds the 65535 nodes the fixed scratch of "
                                     "faco_pheromone_step_noalloc holds");
        if (static_cast<std::uint64_t>(n) * k >= (1ull << 31))
            throw Error(FACO_EINVAL, "n * k must be below 2^31 candidate entries");
        int device = 0;
        cuda_check(cudaGetDevice(&device), "cudaGetDevice");
        const void* pointers[5] = {primary, parent, eta, trails, products};
        for (const void* p : pointers) {
            cudaPointerAttributes a{};
            cuda_check(cudaPointerGetAttributes(&a, p), "cudaPointerGetAttributes");
            if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
                throw Error(FACO_EINVAL, "faco_pheromone_step_noalloc takes device pointers only");
            // managed memory is reachable from every device, wherever it was allocated
            if (a.type == cudaMemoryTypeDevice && a.device != device)
                throw Error(FACO_EINVAL, "a buffer lives on another device than the current one");
        }
        std::uint32_t bits = 0;
        cuda_check(faco::pheromone_step_noalloc(n, k, primary, parent, retention, minimum, maximum, increment, eta,
                                                trails, products, static_cast<cudaStream_t>(stream), &bits),
                   "pheromone step (no allocation)");
        if (bits & faco::kNoAllocParentRange) throw Error(FACO_EINVAL, "parent node out of range");
        if (bits & faco::kNoAllocParentRepeat) throw Error(FACO_EINVAL, "parent is not a permutation");
        if (bits & faco::kNoAllocPrimaryRange) throw Error(FACO_EINVAL, "primary candidate out of range");
    });
}

}  // extern "C"

/*
 * faco_gb300.h -- C ABI of the GB300 Focused-ACO batch engine.
 *
 * Plain pointers and sizes only.  Every call returns FACO_OK (0) or a
 * negative status; faco_last_error() then holds a message for the calling
 * thread.  No call aborts, traps or throws across the boundary.
 *
 * Each entry point replaces one interface of LinHuanli/GPLSACO's pybind11
 * module gp_faco_ext (cpp/src/bindings.cpp); the file:line it replaces is
 * given beside it.  Host buffers are copied in before a call returns.
 */
#ifndef FACO_GB300_H
#define FACO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FACO_OK 0
#define FACO_EINVAL (-1)   /* invalid argument: ValueError in the reference        */
#define FACO_ECUDA (-2)    /* CUDA runtime error: RuntimeError in the reference    */
#define FACO_EBUSY (-3)    /* a second evaluation on one engine (try_lock failure) */
#define FACO_EDEVICE (-4)  /* a kernel raised its device error word                */
#define FACO_ENOMEM (-5)

/* Local-search variants. */
#define FACO_LS_TWO_OPT 0       /* checklist 2-opt, best gain per node (reference) */
#define FACO_LS_TWO_OPT_OR_OPT 1 /* 2-opt + Or-opt (segments <= 3), first improvement */

/* Ant workspace placement.  Shared memory is fastest per access but holds
 * few large-instance ants per SM; the global-memory workspace (L1/L2-cached)
 * holds a full block per SM slot at any size. */
#define FACO_WORKSPACE_AUTO 0   /* shared; above 2048 nodes the autotuner may pick global */
#define FACO_WORKSPACE_SHARED 1
#define FACO_WORKSPACE_GLOBAL 2

/* FixedFacoSettings (cpp/include/gp_faco/fixed_faco_gpu.hpp:10-21;
 * bindings.cpp:508-519).  ants == 0 selects 64*ceil(sqrt(n)/16). */
typedef struct faco_settings {
    uint32_t ants;
    uint32_t primary_width;
    uint32_t backup_width;
    uint32_t ls_width;
    double beta;
    double retention;
    double p_best;
    double epoch_source_probability;
    uint64_t ls_evaluation_limit;
    uint64_t initial_ls_evaluation_limit;
    uint32_t ls_mode; /* FACO_LS_* */
    uint32_t autotune; /* 1: pick ants per block (and workspace placement) per size class by timing */
    uint32_t workspace; /* FACO_WORKSPACE_*: where an ant keeps its tour and inverse */
    uint32_t force_fingerprint_collisions; /* diagnostic (batch_engine.hpp:66): every tour fingerprint
                                              of the 12-feature controller is 0, so its archive
                                              compares whole tours; 0 in production */
    uint32_t chains; /* independent colony chains in the evaluation's graph (0: one per 16
                        colonies, at most 8); results do not depend on it */
    uint32_t follow; /* FACO_FOLLOW_*: construction steps along the parent tour taken 16-32 at a
                        time, one lane per step; results do not depend on it */
} faco_settings;

/* Batched parent-following steps: AUTO uses them always when the
 * evaluation's ant warps fit in one wave of the GPU (at most 32 per SM),
 * where an iteration lasts as long as its longest walk.  On fuller panels
 * AUTO chooses every 32 iterations from the walk length of the last 32:
 * batches from 72 construction steps per ant and iteration on, steps one at
 * a time again below 60 (96 and 80 with the global-memory ant workspace of
 * large instances); short walks take more instructions in batches than one
 * at a time.  Beyond one wave the batches run a build of the same steps
 * tuned for throughput (fewer registers per thread, more warps per SM)
 * rather than for one ant's latency. */
enum { FACO_FOLLOW_AUTO = 0, FACO_FOLLOW_OFF = 1, FACO_FOLLOW_ON = 2 };

void faco_default_settings(faco_settings* s);

/* Returns the message of the last failed call on this thread. */
const char* faco_last_error(void);

typedef struct faco_engine faco_engine;
struct faco_program;

/* FacoBatchEngine(dimension, colonies, settings) (bindings.cpp:558-573).
 * `dimension` is the largest instance size the engine accepts; instances of
 * different sizes up to it may share one evaluation (uneven batching).
 * `colonies` is the capacity of one evaluation; `device` the CUDA ordinal. */
int faco_engine_create(uint32_t dimension, uint32_t colonies, const faco_settings* settings, int device,
                       faco_engine** engine);
void faco_engine_destroy(faco_engine* engine);

typedef struct faco_registration {
    double cheap_seconds;
    double preparation_seconds;
    int64_t initial_cost;
    uint32_t n;
    uint32_t reserved;
} faco_registration;

/* register_problem(instance_key, coordinates f64[n,2]) (bindings.cpp:623-638).
 * Coordinates must be finite integers with |x| < 2^26 and a span below 2^24
 * per axis, the range in which the TSPLIB EUC_2D formula in double precision
 * rounds every length exactly.  A registered identity is immutable
 * (batch_engine.cu:285-289): registering a key again with the same
 * coordinates returns the first registration's info and does no work; other
 * coordinates under a registered key are FACO_EINVAL. */
int faco_register_problem(faco_engine* engine, uint64_t instance_key, const double* xy, uint32_t n,
                          faco_registration* info);

/* Initial tour and candidate rows of a registered instance (u32 [n], [n][k],
 * [n][b], [n][w]; any pointer may be NULL). */
int faco_problem_rows(faco_engine* engine, uint64_t instance_key, uint32_t* initial_tour, uint32_t* primary,
                      uint32_t* backup, uint32_t* ls);

/* Per-iteration colony trace row. */
typedef struct faco_trace_row {
    int64_t iteration_best_cost;
    int64_t global_cost;
    int64_t parent_cost;
    uint32_t iteration_best;
    uint32_t source_is_epoch;
    float tau_min;
    float tau_max;
    uint32_t mne_target;
    int32_t action;
    uint64_t construction_steps;
    uint64_t ls_evaluations;
} faco_trace_row;

/* Controller feedback of one colony after its last batch (the control_states
 * rows of bindings.cpp:395-407).  Feature spec 2 fills every field; spec 3
 * the restarts, stagnant batches, start region and MNE target. */
typedef struct faco_control_state {
    uint64_t restarts;
    uint64_t stagnant_batches;  /* batches since the last global improvement */
    uint64_t epoch_batches;     /* batches since the last restart (spec 2)    */
    float return_rate;          /* spec 2: EMA of ants returning the parent   */
    float ls_work;              /* spec 2: EMA of the LS budget used          */
    uint32_t archive_size;      /* spec 2: reference tours held (1-4)         */
    uint32_t start_region;      /* start region of the next batch (spec 3: 0-3, 4 = all
                                   nodes; spec 2: 5 = the controller's start list) */
    uint32_t mne_target;        /* MNE target of the next batch               */
    uint32_t reserved;
} faco_control_state;

typedef struct faco_outputs {
    uint32_t* tours;          /* [count][dimension] global-best tours (u32)       */
    int64_t* costs;           /* [count] integer EUC_2D lengths                   */
    faco_trace_row* trace;    /* [iterations][count], may be NULL                 */
    uint32_t* checkpoint_tours; /* [n_checkpoints][count][dimension], may be NULL */
    uint64_t completed_batches;
    uint64_t construction_steps;
    uint64_t ls_evaluations;
    uint64_t reversed_elements; /* tour elements moved by relocations/reversals */
    double kernel_milliseconds; /* device time of the iteration loop             */
    double solve_seconds;
    uint64_t* colony_work;      /* [count][3] per colony: construction steps, LS
                                   evaluations, reversed elements; may be NULL */
    faco_control_state* control_states; /* [count], may be NULL */
    /* Decision captures of feature-spec-2 controllers (decision_iterations,
     * bindings.cpp:323-346): for each 1-based batch number p in
     * decision_iterations (strictly increasing, <= the batches run) the
     * decision taken before batch p-1 -- its 12 x 32 features, the 32
     * scores (conditional controllers: role scores in slots 0-9), the legal
     * mask and the action -- per colony.  n_decisions 0: none. */
    const uint32_t* decision_iterations;
    uint32_t n_decisions;
    float* decision_features;   /* [n_decisions][count][12][32] */
    float* decision_scores;     /* [n_decisions][count][32]     */
    uint32_t* decision_masks;   /* [n_decisions][count]         */
    int32_t* decision_actions;  /* [n_decisions][count]         */
} faco_outputs;

/* evaluate_faco_evaluations(keys, seeds, evaluation_limit_per_colony, mne,
 * checkpoint_iterations=...) (bindings.cpp:701-720; engine
 * cuda/batch_engine.cu:362-365, loop :875-1135).  Plain FACO with a constant
 * MNE target.  The budget must be a whole number of ant batches; instance
 * keys may name instances of different sizes (uneven batching). */
int faco_evaluate(faco_engine* engine, const uint64_t* instance_keys, const uint64_t* seeds, uint32_t count,
                  uint64_t evaluation_limit_per_colony, uint32_t mne_target, const uint64_t* checkpoint_iterations,
                  uint32_t n_checkpoints, faco_outputs* out);

/* evaluate_program_evaluations / evaluate_population_evaluations
 * (bindings.cpp:721-757,776-817; engine cuda/batch_engine.cu:379-437,
 * per-batch control :884-950): colony c is driven by programs[c / (count /
 * n_programs)].  All programs of one call share one feature spec:
 *
 * spec 2, the reference's 12-feature controller (control_state.cuh:45-364,
 * control_cpu.cpp:72-118): before every batch the 32 actions (mode x start
 * region x MNE level) are scored on elapsed fraction, stagnation, return
 * rate, LS work, mode, level, reference gap, sampled difference and four
 * features of the action's 16-node start region; the best legal action sets
 * the MNE target 2<<(a&3) and the start nodes, and a >= 16 restarts from
 * the alternative archive tour.  Actions >= 16 are legal only while the
 * archive holds an alternative; action_mask & 0xffff must be non-zero.
 * Traces record the target and action each batch ran with.
 *
 * spec 3, this engine's compact controller: after every iteration the
 * actions are scored from 7 colony features (iteration fraction,
 * stagnation, mean/best gap, trail-row entropy, restarts, LS gain,
 * reference-tour age) and 3 action descriptors; the action sets the next MNE
 * target 2<<(a&3), the start quadrant (a>>2)&3 and, for a >= 16, a restart
 * from the global best with trails reset to tau_max.  initial_mne is the
 * target of the first iteration.  Traces record the target used and the
 * action chosen after the iteration. */
int faco_evaluate_programs(faco_engine* engine, const uint64_t* instance_keys, const uint64_t* seeds,
                           uint32_t count, uint64_t evaluation_limit_per_colony, const struct faco_program* programs,
                           uint32_t n_programs, uint32_t action_mask, uint32_t initial_mne,
                           const uint64_t* checkpoint_iterations, uint32_t n_checkpoints, faco_outputs* out);

/* Controllers (read_controller / validate_controller, bindings.cpp:58-73,
 * cpp/src/program_cpu.cpp:11-24): three program slots per controller and its
 * kind -- 0 joint_single (slot 0 scores all 32 actions, as
 * faco_evaluate_programs), 1 conditional_three (slots 0-2 are role trees
 * that pick, in turn, restart or not (actions 0-15 / 16-31), the start
 * region (stride 4) and the MNE level (stride 1), each from the features of
 * its candidate actions, python/gp_faco/controller.py:60-84).  A role tree
 * may not read the descriptor of a later decision (role 0: features 7, 8;
 * role 1: feature 7); a controller has at most 63 nodes over its roles.
 * Colony c is driven by controller c / (count / n_controllers). */
int faco_evaluate_controllers(faco_engine* engine, const uint64_t* instance_keys, const uint64_t* seeds,
                              uint32_t count, uint64_t evaluation_limit_per_colony, const struct faco_program* trees,
                              const uint32_t* kinds, uint32_t n_controllers, uint32_t action_mask,
                              uint32_t initial_mne, const uint64_t* checkpoint_iterations, uint32_t n_checkpoints,
                              faco_outputs* out);
int faco_validate_controller(const struct faco_program* trees, uint32_t kind);
/* score_controller_cuda (gp_score.cu:32-47): features f32[12][C][32], masks
 * u32[C]; joint controllers write 32 scores per colony, conditional ones the
 * role scores in slots 0-1, 2-5, 6-9 (the rest 0); actions i32[C]. */
int faco_score_controllers(const struct faco_program* trees, const uint32_t* kinds, uint32_t n_controllers,
                           const float* features, uint32_t features_count, const uint32_t* masks, uint32_t colonies,
                           float* scores, int32_t* actions);

/* The same evaluation in explicit steps (the reference's per-batch loop,
 * cuda/batch_engine.cu:875-1135, driven by the caller): faco_begin uploads the
 * panel and resets every colony; faco_step enqueues `iterations` ant batches
 * on the engine's stream (asynchronous); faco_step_timed runs them, with the
 * kernel variants faco_step would run, as single launches with a CUDA event
 * around every kernel and returns the summed device milliseconds of the ant
 * kernel and of the colony update (synchronous); faco_finish waits
 * and fills tours, costs, counters and up to trace_iterations trace rows. */
int faco_begin(faco_engine* engine, const uint64_t* instance_keys, const uint64_t* seeds, uint32_t count,
               uint32_t mne_target, uint32_t trace_iterations);
int faco_step(faco_engine* engine, uint32_t iterations);
int faco_step_timed(faco_engine* engine, uint32_t iterations, double* ant_milliseconds,
                    double* update_milliseconds);
int faco_finish(faco_engine* engine, faco_outputs* out);
/* The launch plan of the active or most recent evaluation (no counterpart
 * in the reference; zeros before the first): its size classes, its colony chains (independent branches of
 * the graph; 0 when the colonies run as one), the iterations captured per
 * graph (faco_step of that many iterations replays the graph once) and the
 * kernel launches per iteration. */
typedef struct faco_launch_plan {
    uint32_t size_classes;
    uint32_t chains;
    uint32_t graph_iterations;
    uint32_t launches_per_iteration;
    uint32_t follow; /* 1: the ant launches take parent-following steps in batches; 2: chosen
                        every 32 iterations from the walk length */
} faco_launch_plan;
int faco_get_launch_plan(faco_engine* engine, faco_launch_plan* plan);
/* The engine's cudaStream_t (for events recorded by the caller). */
void* faco_engine_stream(faco_engine* engine);

/* faco_begin for GP-controlled colonies: the programs, action mask and
 * initial MNE of faco_evaluate_programs; total_iterations is the budget T
 * that the iteration-fraction feature divides by. */
int faco_begin_programs(faco_engine* engine, const uint64_t* instance_keys, const uint64_t* seeds, uint32_t count,
                        const struct faco_program* programs, uint32_t n_programs, uint32_t action_mask,
                        uint32_t initial_mne, uint32_t total_iterations, uint32_t trace_iterations);

/* Colony snapshot and resume (CountedState capture/restore,
 * cpp/include/gp_faco/counted_state.hpp:23-38, cuda/batch_engine.cu:207-261).
 * faco_snapshot writes the whole persistent state of the active stepwise
 * evaluation (panel, controllers, colony states, trails, products, eta and
 * parent/epoch/global tours; versioned, checksummed) into `buffer`; with
 * buffer NULL it only reports the size in *bytes.  faco_restore begins a
 * stepwise evaluation from such a snapshot on an engine with the same
 * settings and the same instances registered (coordinates are checked);
 * stepping it continues the saved run bit for bit.  Trace rows are indexed
 * by absolute iteration. */
int faco_snapshot(faco_engine* engine, void* buffer, uint64_t capacity, uint64_t* bytes);
int faco_restore(faco_engine* engine, const void* buffer, uint64_t bytes, uint32_t trace_iterations);

/* ---- GP programs -------------------------------------------------------- */
/* Program (cpp/include/gp_faco/program.hpp:10-19). numeric_spec_id 1 is the
 * reference IR (opcodes 0-8, depth <= 5); 2 adds protected division (9) and
 * if>0 (10, three operands), depth <= 6. */
typedef struct faco_program {
    uint16_t ir_version;
    uint16_t numeric_spec_id;
    uint16_t feature_spec_id;
    uint16_t length;
    uint16_t constants_count;
    uint8_t opcode[63];
    uint8_t operand[63];
    float constants[63];
} faco_program;

int faco_validate_program(const faco_program* program);

/* score_cuda(program, features f32[F,C,32], masks u32[C]) (bindings.cpp:
 * 504-506,1007-1009; kernel cuda/gp_score.cuh:64-102).  `programs` holds
 * n_programs programs; colony c uses programs[c / (colonies / n_programs)].
 * Host buffers. */
int faco_score(const faco_program* programs, uint32_t n_programs, const float* features, uint32_t features_count,
               const uint32_t* masks, uint32_t colonies, float* scores, int32_t* actions);

/* ---- diagnostics (parity hooks) ---------------------------------------- */
/* cuda_faco_diagnostic (cpp/include/gp_faco/faco_cuda_diagnostic.hpp:36-39,
 * cuda/faco_operations.cu:60-134): one warp-ant per task runs focused
 * construction from tours[t] then checklist LS.  Choices come from visit
 * orders (visits != NULL, [tasks][n]) or from a roulette over `products`
 * ([n][k] FP32) driven by injected uniforms ([tasks][n], step s uses [s]) with
 * starts[t] as the first node.  ls_rows [n][w] in any order (the engine
 * builds the distance-ordered view).  Outputs (u32/i64) may be NULL. */
typedef struct faco_ant_outputs {
    uint32_t* construction_tours; /* [tasks][n]                                 */
    uint32_t* tours;              /* [tasks][n]                                 */
    uint32_t* positions;          /* [tasks][n]                                 */
    uint32_t* selected;           /* [tasks][n] node chosen at each step        */
    uint32_t* checklists;         /* [tasks][checklist_capacity]                */
    uint32_t checklist_capacity;
    int64_t* construction_costs;  /* [tasks]                                    */
    int64_t* final_costs;         /* [tasks]                                    */
    uint64_t* counters;           /* [tasks][10]: mne, steps, nonidentity,
                                     processed, checks, evaluations, accepted,
                                     reactivations, limit_reached, checklist   */
} faco_ant_outputs;

int faco_ant_diagnostic(const int32_t* xy, uint32_t n, const uint32_t* ls_rows, uint32_t w, const uint32_t* tours,
                        const uint32_t* visits, const double* uniforms, const uint32_t* starts,
                        const uint32_t* primary, const float* products, uint32_t k, const uint32_t* backup,
                        uint32_t b, const uint32_t* mne_targets, uint32_t tasks, uint64_t evaluation_limit,
                        uint32_t ls_mode, faco_ant_outputs* out);

/* ---- learned edge prior ----------------------------------------------------
 * No counterpart in the reference (its only candidate prior is an external
 * LKH export, python/gp_faco/candidate_prior.py:20-36).  An 8 -> 64 -> 64 -> 1
 * MLP (ReLU, sigmoid output) scores every directed candidate edge from
 * [normalised distance, k-rank, angle to the nearest neighbour, ratio to the
 * k-th neighbour distance, normalised trail, in-global-best flag, mutual
 * rank, alpha-nearness]; BF16
 * operands, FP32 accumulation on the tensor cores.  Parameters are one FP32
 * array of faco_mlp_param_count() values: w1[64][8],
 * b1[64], w2[64][64], b2[64], w3[64], b3, 3 padding.  Edge rows x are
 * [count][8] BF16 bit patterns. */
int faco_mlp_param_count(void);
int faco_mlp_forward(const float* params, const uint16_t* x, uint32_t count, float* probabilities);
/* Gradient of the mean binary cross-entropy over `count` rows (labels y). */
int faco_mlp_gradient(const float* params, const uint16_t* x, const float* y, uint32_t count, float* gradient,
                      float* loss_sum);
/* Adam over `epochs` passes of minibatches of `batch` consecutive rows
 * (shuffle the rows first); params updated in place; mean loss per epoch. */
int faco_mlp_train(float* params, const uint16_t* x, const float* y, uint32_t count, uint32_t epochs,
                   uint32_t batch, float learning_rate, float* epoch_losses);
/* During a stepwise evaluation: features (and labels: edge of the colony's
 * global-best tour) of every candidate entry of every colony, rows ordered
 * (colony, node, rank); `rows` receives the row count (pass NULL outputs to
 * query it). */
int faco_edge_data(faco_engine* engine, uint16_t* x, float* y, uint64_t capacity_rows, uint64_t* rows);
/* Enables the prior on colonies with enabled[c] != 0 (params may be NULL to
 * keep the loaded ones): eta' = eta * (floor + p)^gamma (gamma 1 or 2),
 * products refreshed; floor > 0 so that no candidate is removed.  Colonies
 * with enabled[c] == 0 get the plain heuristic back (the per-instance
 * fallback).  departures = 1: the prior re-ranks only the departures from
 * the parent tour -- per node, parent-tour entries keep the plain heuristic
 * and the other entries' prior weights are scaled to the plain total, so an
 * ant leaves the parent tour as often as a plain ant (every batch, after
 * the trail update). */
int faco_prior_set(faco_engine* engine, const float* params, float floor, int gamma, const uint8_t* enabled,
                   uint32_t departures);
/* Recomputes the prior from the colonies' current trails and best tours. */
int faco_prior_refresh(faco_engine* engine);
/* During a stepwise evaluation: one colony's trails, heuristic (the
 * instance's eta, or the prior-reweighted one) and products, [n][k] FP32
 * each, copied out after the work queued so far (synchronises).  Any output
 * may be NULL; `capacity` is the entries each non-NULL output holds.  The
 * parity hook of the reference's trail trace (FixedFacoTrace,
 * cpp/include/gp_faco/fixed_faco_gpu.hpp:23-33, which records the trails
 * before and after each batch). */
int faco_colony_rows(faco_engine* engine, uint32_t colony, float* trails, float* eta, float* products,
                     uint64_t capacity);
/* Current global-best lengths of the colonies (synchronises). */
int faco_current_costs(faco_engine* engine, int64_t* costs, uint32_t* iterations);
/* Per-colony MNE targets (maximum new edges per ant) of the active plain
 * stepwise evaluation from the next batch on, targets[count] >= 1
 * (synchronises).  GP-controlled evaluations choose their targets by action. */
int faco_set_mne_targets(faco_engine* engine, const uint32_t* targets, uint32_t count);

/* One MMAS evaporate/deposit step (cuda/colony_state.cuh:210-229) on FP32
 * trails [n][k] along `parent`; refreshes products = trails * eta. */
int faco_pheromone_step(uint32_t n, uint32_t k, const uint32_t* primary, const uint32_t* parent, float retention,
                        float minimum, float maximum, float increment, const float* eta, float* trails,
                        float* products);

/* The same pheromone step on buffers that already live in device memory,
 * allocating nothing: no device memory (no cudaMalloc/cudaFree) and no host
 * memory on the success path.  No counterpart in the reference.
 *
 * For callers that cannot allocate per call: a loop that keeps trails, eta
 * and candidate lists resident in memory it manages itself (a caching
 * allocator such as PyTorch's, or one fixed arena).  A cudaFree inside the
 * library would synchronise the whole device on every step and a cudaMalloc
 * would compete with the caller's pool for memory it has already reserved.
 *
 * Arguments mean what they mean in faco_pheromone_step, but every array is
 * a device pointer on the current device: primary [n*k] u32 candidate ids,
 * parent [n] u32 tour, eta/trails/products [n*k] f32 (trails in/out,
 * products out).  `stream` is a cudaStream_t (NULL: the legacy default
 * stream); the call enqueues its work there and returns when it is done.
 *
 * Limit: n <= 65535 nodes.  The only scratch is one fixed device array per
 * device (256 KiB of packed parent neighbours, an 8 KiB permutation bitmap
 * and an error word), declared at file scope in the library; larger n is
 * rejected with FACO_EINVAL before any work is enqueued.  The bitmap and the
 * error word must start at zero: every call clears them on `stream` itself
 * before use.  An invalid parent (out of range or repeated node) or
 * candidate id is found on the device and returns FACO_EINVAL with trails
 * and products untouched.
 *
 * Every call looks the scratch address up for the current device
 * (cudaGetSymbolAddress, which allocates nothing), so a cudaDeviceReset or
 * another context between calls is harmless.  Calls must not overlap: two
 * calls in flight at once on one device (from two host threads of one
 * process) race on the single scratch and corrupt each other's result.
 * Calls from one thread never overlap, since each returns only after its
 * work is complete. */
int faco_pheromone_step_noalloc(uint32_t n, uint32_t k, const uint32_t* primary, const uint32_t* parent,
                                float retention, float minimum, float maximum, float increment, const float* eta,
                                float* trails, float* products, void* stream);

#ifdef __cplusplus
}
#endif
#endif

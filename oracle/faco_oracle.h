/*
 * faco_oracle.h -- CPU restatement of the GPLSACO Focused-ACO path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this code; it is the checker that the CUDA engine is compared with
 * (tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg only).
 *
 * Every routine restates one function of the reference, cited by file:line
 * inside LinHuanli/GPLSACO.  Two numeric domains are covered:
 *   - "reference" semantics: FP64 trails and products, exactly as
 *     cpp/src/faco_cpu.cpp and cuda/colony_state.cuh compute them;
 *   - "engine" semantics: the same algorithm with FP32 trails/products
 *     (the arithmetic the GB300 engine uses), restated bit-for-bit.
 * Distances are TSPLIB EUC_2D integers: d = floor(sqrt(dx^2 + dy^2) + 0.5),
 * so every tour length is an exact int64.
 */
#ifndef FACO_ORACLE_H
#define FACO_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

struct orc_program;

/* ---- distances ---------------------------------------------------------- */
typedef struct {
    uint32_t n;
    const int32_t* xy;      /* [n][2] integer coordinates, or NULL           */
    const int32_t* matrix;  /* [n][n] explicit distances (used when non-NULL) */
} orc_dist_t;

int32_t orc_euc2d(int64_t x0, int64_t y0, int64_t x1, int64_t y1);
int32_t orc_distance(const orc_dist_t* d, uint32_t a, uint32_t b);

/* ---- tour (order + inverse positions + exact cost) ---------------------- */
typedef struct {
    uint32_t n;
    uint32_t* order;
    uint32_t* pos;
    int64_t cost;
} orc_tour_t;

/* Fills pos[] and cost from order[]; returns 0 when order is a permutation. */
int orc_tour_reset(orc_tour_t* t, const orc_dist_t* d);
int64_t orc_tour_length(const uint32_t* order, uint32_t n, const orc_dist_t* d);
int orc_relocate(orc_tour_t* t, const orc_dist_t* d, uint32_t target, uint32_t node);
void orc_flip(orc_tour_t* t, uint32_t start, uint32_t end);

/* ---- checklist (FIFO with "pending" flags) ------------------------------ */
typedef struct {
    uint32_t* items;     /* every push in order (capacity cap)               */
    uint32_t cap, head, len;
    uint8_t* queued;     /* queued[v] == 1 iff v is in items[head..len)      */
    int overflow;
} orc_queue_t;

void orc_queue_push_absent(orc_queue_t* q, uint32_t v, uint64_t* pushed);

typedef struct {
    uint64_t processed_nodes, candidate_checks, move_evaluations, accepted_moves, reactivations;
    uint32_t evaluation_limit_reached;
} orc_ls_stats_t;

/* Checklist 2-opt, best gain per popped node (reference semantics).
 * rows: [n][w] LS rows, each ordered by (distance, insertion order); entries
 * >= n are right padding. */
void orc_checklist_two_opt(orc_tour_t* t, const orc_dist_t* d, const uint32_t* rows, uint32_t w,
                           orc_queue_t* q, uint64_t max_evaluations, orc_ls_stats_t* st);
/* First-improvement 2-opt + Or-opt (segments of 1-3 nodes); see the .c file. */
void orc_checklist_ls_first(orc_tour_t* t, const orc_dist_t* d, const uint32_t* rows, uint32_t w,
                            orc_queue_t* q, uint64_t max_evaluations, orc_ls_stats_t* st);

typedef struct {
    uint32_t mne, steps, nonidentity_relocations, legal_exhausted;
} orc_cons_stats_t;

enum { ORC_PRIMARY = 0, ORC_ZERO_WEIGHT = 1, ORC_BACKUP = 2, ORC_GLOBAL = 3, ORC_EXHAUSTED = 4 };

/* Roulette over unvisited primary candidates, weights given as doubles. */
uint32_t orc_select_next(uint32_t current, const uint32_t* primary, const double* products, uint32_t k,
                         const uint32_t* backup, uint32_t b, const uint8_t* visited,
                         const orc_dist_t* d, double uniform, int* stage);

/* ---- one ant: focused construction from a parent tour, then 2-opt ------- */
typedef struct {
    /* choice source: either an explicit visit order (visit[0] = start) ... */
    const uint32_t* visit;
    /* ... or a roulette driven by the given uniforms (uniform[s] for step s) */
    const double* uniforms;
    uint32_t start;
    const uint32_t* primary;   /* [n][k]                                     */
    const float* products32;   /* [n][k] engine products (FP32)              */
    const double* products64;  /* [n][k] reference products (FP64)          */
    uint32_t k;
    const uint32_t* backup;    /* [n][b]                                     */
    uint32_t b;
} orc_choices_t;

typedef struct {
    int64_t construction_cost, final_cost;
    orc_cons_stats_t cons;
    orc_ls_stats_t ls;
    uint32_t start_node, checklist_len;
} orc_ant_info_t;

/* construction_tour, tour, pos: [n]; checklist: capacity 8n+8 (may be NULL);
 * selected (optional, [n]): node chosen at each step, [0] = start. */
int orc_ant(const uint32_t* parent, const orc_dist_t* d, const uint32_t* ls_rows, uint32_t w,
            const orc_choices_t* ch, uint32_t mne_target, uint64_t max_evaluations, uint32_t ls_mode,
            uint32_t* construction_tour, uint32_t* tour, uint32_t* pos, uint32_t* checklist,
            uint32_t* selected, orc_ant_info_t* info);

/* ---- trails ------------------------------------------------------------- */
void orc_trail_limits(uint32_t width, double p_root, double retention, double cost,
                      double* minimum, double* maximum);
/* p_root = pow(p_best, 1/width) -- computed once by the caller. */

/* FP64 evaporate + symmetric deposit along `parent` (reference semantics).
 * trails: [n][k] for rows primary. */
void orc_pheromone64(uint32_t n, uint32_t k, const uint32_t* primary, const uint32_t* parent,
                     double retention, double minimum, double maximum, double increment,
                     double* trails, double* default_trail);
/* FP32 engine update: also refreshes products = trail * eta. */
void orc_pheromone32(uint32_t n, uint32_t k, const uint32_t* primary, const uint32_t* parent,
                     float retention, float minimum, float maximum, float increment,
                     const float* eta, float* trails, float* products, float* default_trail);

/* ---- random stream (Philox4x32-10, Salmon et al. SC'11) ----------------- */
void orc_philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                    uint32_t out[4]);
double orc_uniform(uint64_t key, uint32_t batch, uint32_t ant, uint32_t step);
uint32_t orc_start_node(uint64_t key, uint32_t batch, uint32_t ant, uint32_t n);
double orc_source_uniform(uint64_t key, uint32_t batch);
uint64_t orc_colony_key(uint64_t seed, uint64_t instance_key);

/* ---- instance preparation ----------------------------------------------- */
typedef struct {
    uint32_t k, b, w;        /* primary / backup / LS widths (already clipped) */
    uint64_t initial_ls_evaluation_limit;
} orc_prep_cfg_t;

/* primary [n][k], backup [n][b], ls [n][w], initial tour [n]; returns cost. */
int64_t orc_prepare(uint32_t n, const int32_t* xy, const orc_prep_cfg_t* cfg, uint32_t* primary,
                    uint32_t* backup, uint32_t* ls, uint32_t* initial);

/* ---- the reference's 12-feature controller (feature spec 2) -------------- */
#define ORC_ARCHIVE_CAPACITY 4u
#define ORC_REGION_CAPACITY 16u
#define ORC_SAMPLE_CAPACITY 64u
#define ORC_ARCHIVE_BAND 0.02

typedef struct { uint64_t first, second; } orc_fp_t;

typedef struct {
    float return_rate, ls_work;
    uint64_t stagnant_batches, epoch_batches, restarts;
} orc_feedback_t;

/* Up to 4 reference tours: [4][n] orders and positions, costs, fingerprints. */
typedef struct {
    uint32_t n, size;
    uint32_t* tours;
    uint32_t* pos;
    int64_t cost[ORC_ARCHIVE_CAPACITY];
    orc_fp_t id[ORC_ARCHIVE_CAPACITY];
    uint32_t zero_ids;    /* forced collisions: every fingerprint is 0 */
} orc_archive_t;

/* Everything one decision reads. */
typedef struct {
    uint32_t n;
    const int32_t* xy;
    const uint32_t* primary;      /* [n][k] */
    uint32_t k;
    const uint32_t* samples;      /* min(n, 64) sample nodes */
    uint32_t sample_count;
    const double* local_scale;    /* [n] mean of the 8 nearest lengths */
    double epsilon;
    const uint32_t* active_tour;  /* the parent tour (and its positions) */
    const uint32_t* active_pos;
    int64_t active_cost;
    orc_fp_t active_id;
    const orc_archive_t* archive;
    orc_feedback_t feedback;
    const double* trails;         /* [n][k] */
    double default_trail, tau_min, tau_max;
    double elapsed_ratio;
    uint64_t solve_key;
    uint32_t batch;
    uint32_t experiment_mask;
} orc_control_in_t;

uint64_t orc_ctl_mix(uint64_t v);
orc_fp_t orc_fingerprint_edge(uint32_t a, uint32_t b);
orc_fp_t orc_fingerprint(const uint32_t* tour, uint32_t n);
int orc_canonical_compare(const uint32_t* ta, const uint32_t* pa, const uint32_t* tb, const uint32_t* pb,
                          uint32_t n);
void orc_sample_nodes(uint32_t n, uint64_t instance_key, uint32_t* out);
void orc_build_region(const uint32_t* tour, uint32_t n, const uint32_t* primary, uint32_t k, uint64_t key,
                      uint32_t batch, uint32_t mode, uint32_t region, uint32_t* nodes);
uint32_t orc_sampled_difference(const uint32_t* ct, const uint32_t* cp, const uint32_t* at, const uint32_t* ap,
                                uint32_t n, const uint32_t* samples, uint32_t count);
void orc_update_feedback(orc_feedback_t* s, int improved, double returned_fraction, double work_fraction,
                         uint32_t ants);
void orc_restart_feedback(orc_feedback_t* s);
int orc_archive_update(orc_archive_t* ar, const uint32_t* global_tour, int64_t global_cost,
                       const uint32_t* cand_tours, const int64_t* cand_costs, uint32_t m);
uint32_t orc_archive_alternative(const orc_archive_t* ar, const uint32_t* at, const uint32_t* ap, orc_fp_t active_id,
                                 const uint32_t* samples, uint32_t sample_count);
/* features [12][32], regions [2][4][16]; returns the legal mask. */
uint32_t orc_control_features(const orc_control_in_t* in, float* features, uint32_t* regions,
                              uint32_t* alternative);
/* Per-node scale: sum of the min(8, n-1) nearest EUC_2D lengths, each divided
 * by that count (prepared_problem.cpp:66-86); epsilon = 1e-12 * max span. */
void orc_local_scale(uint32_t n, const int32_t* xy, double* scale, double* epsilon);

/* Decisions captured at the given 1-based batch numbers (the decision made
 * before batch point-1), and the final controller state. */
typedef struct {
    uint64_t instance_key;
    const uint32_t* points;
    uint32_t count;
    float* features;       /* [count][12][32] */
    float* scores;         /* [count][32] (conditional: role scores in 0-9) */
    uint32_t* masks;       /* [count] */
    int32_t* actions;      /* [count] */
    uint32_t archive_size; /* out */
    orc_feedback_t feedback; /* out */
    uint32_t force_collisions; /* every tour fingerprint 0 (batch_engine.hpp:66) */
} orc_control_io_t;

/* ---- a whole plain-FACO colony run in engine arithmetic ------------------ */
typedef struct {
    uint32_t ants, k, b, w, mne_target;
    double beta, retention, p_best, epoch_source_probability;
    uint64_t ls_evaluation_limit;
    uint32_t threads;        /* OpenMP threads over ants (1 = serial)       */
    uint32_t ls_mode;        /* 0 best-gain 2-opt, 1 first-improvement 2-opt + Or-opt */
} orc_run_cfg_t;

typedef struct {
    int64_t iteration_best_cost, global_cost, parent_cost;
    uint32_t iteration_best, source_is_epoch;
    float tau_min, tau_max;
    uint32_t mne_target;
    int32_t action;
    uint64_t construction_steps, ls_evaluations;
} orc_iter_trace_t;

/* Runs `iterations` batches of one colony.  global_tour [n]; trace
 * [iterations] (may be NULL); trails_out/products_out [n][k] (may be NULL).
 * A program of feature spec 2 runs the reference's 12-feature controller
 * (control_oracle.c; `control` carries the instance key, decision captures
 * and the final controller state); spec 3 the engine's own. */
int orc_run_colony(uint32_t n, const int32_t* xy, const uint32_t* primary, const uint32_t* backup,
                   const uint32_t* ls, const uint32_t* initial, int64_t initial_cost,
                   const orc_run_cfg_t* cfg, uint64_t key, uint32_t iterations,
                   uint32_t* global_tour, int64_t* global_cost, orc_iter_trace_t* trace,
                   float* trails_out, float* products_out, const struct orc_program* program, uint32_t mask,
                   uint32_t total_iterations, uint32_t controller_kind, orc_control_io_t* control);

/* ---- learned edge prior (no reference counterpart) ---------------------- */
typedef struct orc_prior_schedule {
    uint32_t count;              /* entries, in batch order */
    const uint32_t* at;          /* [count] batch before which the entry applies */
    const float* etas;           /* [count][n*k] colony heuristic from then on */
    const uint32_t* departures;  /* [count] 1: products by the departure rule */
} orc_prior_schedule_t;
void orc_prior_eta(size_t cells, const float* eta, const float* prob, float floor, int gamma, float* out);
void orc_departure_rows(uint32_t n, uint32_t k, const uint32_t* primary, const uint32_t* parent,
                        const float* trails, const float* eta, const float* prior_eta, float* products);
int orc_run_colony_prior(uint32_t n, const int32_t* xy, const uint32_t* primary, const uint32_t* backup,
                         const uint32_t* ls, const uint32_t* initial, int64_t initial_cost,
                         const orc_run_cfg_t* cfg, uint64_t key, uint32_t iterations,
                         uint32_t* global_tour, int64_t* global_cost, orc_iter_trace_t* trace,
                         float* trails_out, float* products_out, const struct orc_program* program, uint32_t mask,
                         uint32_t total_iterations, uint32_t controller_kind, orc_control_io_t* control,
                         const orc_prior_schedule_t* prior);

/* ---- GP controller scoring (postfix IR) --------------------------------- */
typedef struct orc_program {
    uint16_t ir_version, numeric_spec_id, feature_spec_id, length, constants_count;
    uint8_t opcode[63];
    uint8_t operand[63];
    float constants[63];
} orc_program_t;

float orc_apply_operation(int opcode, float left, float right, float third);
int orc_validate_program(const orc_program_t* p);
/* features [F][C][32] (feature-major), masks [C] -> scores [C][32], actions [C]. */
void orc_score(const orc_program_t* p, uint32_t features_count, const float* features,
               const uint32_t* masks, uint32_t colonies, float* scores, int32_t* actions);

/* ---- the engine's GP controller (feature spec 3; see the .c file) -------- */
float orc_log2(float x);
uint32_t orc_row_entropy_q(const float* tau, uint32_t k, float log2k);
void orc_regions(uint32_t n, const int32_t* xy, uint32_t* offsets, uint32_t* list);
uint32_t orc_region_start(uint64_t key, uint32_t batch, uint32_t ant, uint32_t n, const uint32_t* offsets,
                          const uint32_t* list, uint32_t region);
int32_t orc_control_choose(const orc_program_t* p, const float colony[7], uint32_t mask, float* scores);
/* conditional_three controllers: trees[3] = the restart, start-region and
 * MNE-level roles; role_scores[10] (slots 0-1, 2-5, 6-9) may be NULL. */
int32_t orc_control_choose_conditional(const orc_program_t* trees, const float colony[7], uint32_t mask,
                                       float* role_scores);
/* score_controller (controller.py:60-84) over features [12][C][32]:
 * scores [C][32] (role scores in slots 0-9, the rest 0), actions [C]. */
void orc_score_conditional(const orc_program_t* trees, const float* features, const uint32_t* masks,
                           uint32_t colonies, float* scores, int32_t* actions);

#ifdef __cplusplus
}
#endif
#endif

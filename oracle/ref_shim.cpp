// ref_shim.cpp -- C entry points over the reference's own CPU FACO core.
//
// TEST INFRASTRUCTURE ONLY.  Compiled together with the unmodified reference
// sources cpp/src/faco_cpu.cpp and cpp/src/program_cpu.cpp (LinHuanli/GPLSACO)
// by oracle/build_ref.sh into oracle/_ref/libgplsaco_ref.so.  The tests use it
// to pin the C restatement in oracle/faco_oracle.c to the reference's own code.
// Each entry point composes the reference API the way its own tests do
// (tests/cpp/test_cuda_faco.cpp:68-98, tests/cpp/test_fixed_faco.cpp:235-282,
// tests/python/test_native_scoring.py:23-46); the controller entries compose
// cpp/src/control_cpu.cpp and cpp/include/gp_faco/control_ops.hpp as
// make_action_snapshot does.
#include "gp_faco/control_cpu.hpp"
#include "gp_faco/faco_cpu.hpp"
#include "gp_faco/program.hpp"

#include <cstring>
#include <exception>
#include <limits>
#include <random>
#include <vector>

using gp_faco::Node;

namespace {
gp_faco::DistanceFunction matrix_distance(const double* m, Node n) {
    return [m, n](Node a, Node b) { return m[static_cast<std::size_t>(a) * n + b]; };
}
gp_faco::CandidateRows rows_of(const std::uint32_t* flat, Node n, Node w) {
    gp_faco::CandidateRows rows(n);
    for (Node a = 0; a < n; ++a) rows[a].assign(flat + static_cast<std::size_t>(a) * w, flat + (a + 1ull) * w);
    return rows;
}
}  // namespace

extern "C" {

// FocusedConstruction with an explicit visit order, then checklist_two_opt.
// stats[0..9] = mne, steps, nonidentity, processed, checks, evaluations,
// accepted, reactivations, limit_reached, checklist length.
int ref_ant(std::uint32_t n, const double* matrix, const std::uint32_t* ls_rows, std::uint32_t w,
            const std::uint32_t* parent, const std::uint32_t* visit, std::uint32_t mne_target,
            std::uint64_t cap, std::uint32_t* construction_tour, double* construction_cost,
            std::uint32_t* tour, std::uint32_t* positions, double* final_cost, std::uint32_t* checklist,
            std::uint32_t checklist_capacity, std::uint64_t* stats) {
    try {
        const auto distance = matrix_distance(matrix, n);
        gp_faco::DistanceOrderedCandidates candidates(rows_of(ls_rows, n, w), distance);
        gp_faco::CpuTour reference(std::vector<Node>(parent, parent + n), distance);
        gp_faco::FocusedConstruction cpu(reference, visit[0], mne_target);
        Node next = 1;
        while (!cpu.done()) cpu.step(visit[next++]);
        std::memcpy(construction_tour, cpu.tour().order().data(), n * sizeof(Node));
        *construction_cost = cpu.tour().cost();
        const auto ls = cpu.tour().checklist_two_opt(candidates, cpu.checklist(), cap);
        std::memcpy(tour, cpu.tour().order().data(), n * sizeof(Node));
        std::memcpy(positions, cpu.tour().positions().data(), n * sizeof(Node));
        *final_cost = cpu.tour().cost();
        const auto& list = cpu.checklist();
        if (list.size() > checklist_capacity) return -3;
        std::memcpy(checklist, list.data(), list.size() * sizeof(Node));
        const auto& cs = cpu.stats();
        const std::uint64_t values[10] = {cs.mne, cs.steps, cs.nonidentity_relocations, ls.processed_nodes,
            ls.candidate_checks, ls.move_evaluations, ls.accepted_moves, ls.reactivations,
            ls.evaluation_limit_reached ? 1u : 0u, list.size()};
        std::memcpy(stats, values, sizeof(values));
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// select_next over one row; returns the node, writes the stage code
// (0 primary, 1 zero-weight, 2 backup, 3 global, 4 exhausted).
int ref_select_next(std::uint32_t n, const double* matrix, std::uint32_t current, const std::uint32_t* primary,
                    const double* products, std::uint32_t k, const std::uint32_t* backup, std::uint32_t b,
                    const std::uint8_t* visited, double uniform, std::uint32_t* node, int* stage) {
    try {
        const auto s = gp_faco::select_next(current, std::vector<Node>(primary, primary + k),
            std::vector<double>(products, products + k), std::vector<Node>(backup, backup + b),
            std::vector<std::uint8_t>(visited, visited + n), matrix_distance(matrix, n), uniform);
        *node = s.node;
        *stage = static_cast<int>(s.stage);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

int ref_trail_limits(std::uint32_t count, double p_best, double retention, double cost, double* minimum,
                     double* maximum) {
    try {
        const auto limits = gp_faco::candidate_trail_limits(count, p_best, retention, cost);
        *minimum = limits.minimum;
        *maximum = limits.maximum;
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// SparsePheromone seeded with `trails` (all rows the given width), then
// evaporate + symmetric deposit along every edge of `parent`
// (tests/cpp/test_fixed_faco.cpp:277-281).  Writes the updated stored trails.
int ref_pheromone(std::uint32_t n, std::uint32_t k, const std::uint32_t* primary, const std::uint32_t* parent,
                  double initial, double retention, double minimum, double maximum, double increment,
                  std::uint32_t rounds, double* trails_out, double* default_out) {
    try {
        gp_faco::SparsePheromone pheromone(rows_of(primary, n, k), initial, true);
        for (std::uint32_t r = 0; r < rounds; ++r) {
            pheromone.evaporate(retention, minimum);
            for (Node i = 0; i < n; ++i) pheromone.deposit(parent[(i + n - 1) % n], parent[i], increment, maximum);
        }
        std::memcpy(trails_out, pheromone.stored().data(), sizeof(double) * n * k);
        *default_out = pheromone.default_value();
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// score_cpu for a reference-IR program (features [12][colonies][32]).
int ref_score(std::uint16_t ir_version, std::uint16_t numeric_spec_id, std::uint16_t feature_spec_id,
              std::uint16_t length, const std::uint8_t* opcode, const std::uint8_t* operand,
              std::uint16_t constants_count, const float* constants, const float* features,
              const std::uint32_t* masks, std::uint32_t colonies, float* scores, std::int32_t* actions) {
    try {
        gp_faco::Program p;
        p.ir_version = ir_version; p.numeric_spec_id = numeric_spec_id; p.feature_spec_id = feature_spec_id;
        p.length = length; p.constants_count = constants_count;
        if (length > 63 || constants_count > 63) return -2;
        std::memcpy(p.opcode, opcode, length);
        std::memcpy(p.operand, operand, length);
        std::memcpy(p.constants, constants, constants_count * sizeof(float));
        const auto out = gp_faco::score_cpu(p, std::vector<float>(features, features + 12ull * 32 * colonies),
                                            std::vector<std::uint32_t>(masks, masks + colonies));
        std::memcpy(scores, out.scores.data(), out.scores.size() * sizeof(float));
        std::memcpy(actions, out.actions.data(), out.actions.size() * sizeof(std::int32_t));
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// A whole plain-FACO colony run from the reference's CPU pieces, composed the
// way tests/cpp/test_fixed_faco.cpp:58-119 replays the GPU engine (the
// reduce/select/update order of cuda/colony_state.cuh:148-229): per
// iteration, products = trails x 1/d^beta (SparsePheromone::product_cache);
// every ant starts at a uniform node, builds by FocusedConstruction +
// select_next and runs checklist_two_opt; the first strictly shortest ant is
// the iteration best; the global best improves only strictly; the parent is
// the global best with probability epoch_source_probability, else the
// iteration best; trails evaporate to the new limits and take 1/cost of the
// source along the parent.  Draws come from std::mt19937_64(seed): the start
// node, one uniform per construction step, one per iteration for the source.
int ref_colony(std::uint32_t n, const double* matrix, const std::uint32_t* primary, std::uint32_t k,
               const std::uint32_t* backup, std::uint32_t b, const std::uint32_t* ls_rows, std::uint32_t w,
               const std::uint32_t* initial, double initial_cost, std::uint32_t ants, std::uint32_t mne,
               std::uint32_t iterations, double beta, double retention, double p_best, double source_probability,
               std::uint64_t ls_limit, std::uint64_t seed, std::uint32_t* tour_out, double* cost_out) {
    try {
        const auto distance = matrix_distance(matrix, n);
        const auto primary_rows = rows_of(primary, n, k);
        const auto backup_rows = b ? rows_of(backup, n, b) : gp_faco::CandidateRows(n);
        gp_faco::DistanceOrderedCandidates ls(rows_of(ls_rows, n, w), distance);
        std::mt19937_64 random(seed);
        std::uniform_real_distribution<double> uniform(0, 1);
        std::uniform_int_distribution<Node> start(0, n - 1);
        std::vector<Node> parent(initial, initial + n), best(parent);
        double best_cost = initial_cost;
        const auto initial_limits = gp_faco::candidate_trail_limits(k, p_best, retention, best_cost);
        gp_faco::SparsePheromone pheromone(primary_rows, initial_limits.maximum, true);
        for (std::uint32_t it = 0; it < iterations; ++it) {
            const auto products = pheromone.product_cache(distance, beta);
            gp_faco::CpuTour reference(parent, distance);
            std::vector<Node> iteration_tour;
            double iteration_cost = std::numeric_limits<double>::infinity();
            for (std::uint32_t ant = 0; ant < ants; ++ant) {
                gp_faco::FocusedConstruction cpu(reference, start(random), mne);
                while (!cpu.done()) {
                    const Node current = cpu.current();
                    const std::vector<double> row(products.begin() + static_cast<std::size_t>(current) * k,
                                                  products.begin() + static_cast<std::size_t>(current + 1) * k);
                    const auto chosen = gp_faco::select_next(current, primary_rows[current], row,
                                                             backup_rows[current], cpu.visited(), distance,
                                                             uniform(random));
                    cpu.step(chosen.node);
                }
                cpu.tour().checklist_two_opt(ls, cpu.checklist(), ls_limit);
                if (cpu.tour().cost() < iteration_cost) {
                    iteration_cost = cpu.tour().cost();
                    iteration_tour = cpu.tour().order();
                }
            }
            if (iteration_cost < best_cost) {
                best_cost = iteration_cost;
                best = iteration_tour;
            }
            const bool from_best = uniform(random) < source_probability;
            parent = from_best ? best : iteration_tour;
            const double deposit_cost = from_best ? best_cost : iteration_cost;
            const auto limits = gp_faco::candidate_trail_limits(k, p_best, retention, best_cost);
            pheromone.evaporate(retention, limits.minimum);
            for (Node i = 0; i < n; ++i)
                pheromone.deposit(parent[(i + n - 1) % n], parent[i], 1.0 / deposit_cost, limits.maximum);
        }
        std::memcpy(tour_out, best.data(), n * sizeof(Node));
        *cost_out = gp_faco::CpuTour(best, distance).recomputed_cost();
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// ---- the 12-feature controller (cpp/src/control_cpu.cpp, control_ops.hpp) ----

void ref_fingerprint(const std::uint32_t* tour, std::uint32_t n, std::uint64_t* out) {
    std::vector<Node> positions(n);
    for (Node i = 0; i < n; ++i) positions[tour[i]] = i;
    const auto f = gp_faco::fingerprint({tour, positions.data(), n});
    out[0] = f.first;
    out[1] = f.second;
}

void ref_sample_nodes(std::uint32_t n, std::uint64_t instance_key, std::uint32_t* out) {
    gp_faco::sample_nodes(n, instance_key, out);
}

void ref_build_region(const std::uint32_t* tour, std::uint32_t n, const std::uint32_t* primary, std::uint32_t k,
                      std::uint64_t key, std::uint32_t batch, std::uint32_t mode, std::uint32_t region,
                      std::uint32_t* nodes) {
    std::vector<Node> positions(n);
    for (Node i = 0; i < n; ++i) positions[tour[i]] = i;
    gp_faco::build_region({tour, positions.data(), n}, primary, k, key, batch, mode, region, nodes);
}

// ReferenceArchive seeded with entries[0], updated with global = entries[0]
// and completed = entries[1..m) (one update), then updated once more with
// `global` and `completed`.  Writes the final entries' tours, costs and
// fingerprints.
int ref_archive_update(std::uint32_t n, const double* matrix, const std::uint32_t* entries, std::uint32_t m,
                       const std::uint32_t* global, const std::uint32_t* completed, std::uint32_t c,
                       std::uint32_t* out_tours, double* out_costs, std::uint64_t* out_ids, std::uint32_t* count) {
    try {
        const auto distance = matrix_distance(matrix, n);
        const auto record = [&](const std::uint32_t* t) { return gp_faco::TourRecord(std::vector<Node>(t, t + n), distance); };
        gp_faco::ReferenceArchive archive(record(entries));
        std::vector<gp_faco::TourRecord> first;
        for (std::uint32_t i = 1; i < m; ++i) first.push_back(record(entries + static_cast<std::size_t>(i) * n));
        archive.update(record(entries), first);
        std::vector<gp_faco::TourRecord> batch;
        for (std::uint32_t i = 0; i < c; ++i) batch.push_back(record(completed + static_cast<std::size_t>(i) * n));
        archive.update(record(global), batch);
        const auto& e = archive.entries();
        *count = static_cast<std::uint32_t>(e.size());
        for (std::size_t i = 0; i < e.size(); ++i) {
            std::memcpy(out_tours + i * n, e[i].order.data(), n * sizeof(Node));
            out_costs[i] = e[i].cost;
            out_ids[2 * i] = e[i].identity.first;
            out_ids[2 * i + 1] = e[i].identity.second;
        }
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// make_action_snapshot on an archive built as in ref_archive_update (global =
// entries[0], completed = entries[1..m)), an active tour, feedback
// {return_rate, ls_work, stagnant, epoch_batches, restarts} and the trails of
// a SparsePheromone(initial) evaporated to `minimum` and deposited along
// `parent` for `rounds` rounds.  Writes features [12][32], regions [2][4][16],
// the alternative slot, the legal mask and the trails used.
int ref_action_snapshot(std::uint32_t n, const double* matrix, const std::uint32_t* primary, std::uint32_t k,
                        const std::uint32_t* samples, std::uint32_t sample_count, const double* local_scale,
                        double epsilon, const std::uint32_t* active, const std::uint32_t* entries, std::uint32_t m,
                        const double* feedback, const std::uint32_t* parent, double initial, double retention,
                        double minimum, double maximum, double increment, std::uint32_t rounds, double elapsed,
                        std::uint64_t solve_key, std::uint32_t batch, std::uint32_t experiment_mask,
                        float* features, std::uint32_t* regions, std::uint32_t* alternative, std::uint32_t* legal,
                        double* trails_out, double* default_out) {
    try {
        const auto distance = matrix_distance(matrix, n);
        const auto record = [&](const std::uint32_t* t) { return gp_faco::TourRecord(std::vector<Node>(t, t + n), distance); };
        gp_faco::ReferenceArchive archive(record(entries));
        std::vector<gp_faco::TourRecord> first;
        for (std::uint32_t i = 1; i < m; ++i) first.push_back(record(entries + static_cast<std::size_t>(i) * n));
        archive.update(record(entries), first);
        gp_faco::SparsePheromone pheromone(rows_of(primary, n, k), initial, true);
        for (std::uint32_t r = 0; r < rounds; ++r) {
            pheromone.evaporate(retention, minimum);
            for (Node i = 0; i < n; ++i) pheromone.deposit(parent[(i + n - 1) % n], parent[i], increment, maximum);
        }
        gp_faco::ControlStaticData problem{n, k, std::vector<Node>(primary, primary + static_cast<std::size_t>(n) * k),
            std::vector<Node>(samples, samples + sample_count), std::vector<double>(local_scale, local_scale + n),
            epsilon};
        gp_faco::FeedbackState state;
        state.return_rate = static_cast<float>(feedback[0]);
        state.ls_work = static_cast<float>(feedback[1]);
        state.stagnant_batches = static_cast<std::uint64_t>(feedback[2]);
        state.epoch_batches = static_cast<std::uint64_t>(feedback[3]);
        state.restarts = static_cast<std::uint64_t>(feedback[4]);
        const auto snapshot = gp_faco::make_action_snapshot(problem, record(active), archive, state, pheromone,
            {minimum, maximum}, distance, elapsed, solve_key, batch, experiment_mask);
        std::memcpy(features, snapshot.features.data(), sizeof(float) * 12 * 32);
        for (Node mode = 0; mode < 2; ++mode)
            for (Node region = 0; region < 4; ++region)
                std::memcpy(regions + (mode * 4 + region) * 16, snapshot.regions.nodes[mode][region], 16 * sizeof(Node));
        *alternative = snapshot.alternative_slot;
        *legal = snapshot.legal_mask;
        std::memcpy(trails_out, pheromone.stored().data(), sizeof(double) * n * k);
        *default_out = pheromone.default_value();
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

}  // extern "C"

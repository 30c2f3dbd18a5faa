/*
 * faco_oracle.c -- CPU restatement of the GPLSACO Focused-ACO path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA engine, never linked
 * into the shipped library.  Each function names the reference routine it
 * follows (paths inside LinHuanli/GPLSACO).  Built with -ffp-contract=off so
 * that every FP32/FP64 operation rounds exactly once, as on the GPU.
 */
#include "faco_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------------- */
/* Distances.  TSPLIB EUC_2D (python/gp_faco/distance.py:40-52):           */
/* floor(sqrt(dx^2+dy^2)+0.5).  For |coords| < 2^26 the square sum is exact */
/* in a double and sqrt is correctly rounded, so this is the exact integer */
/* nearest to the true length (a half-integer is never a square root).    */
/* ---------------------------------------------------------------------- */
int32_t orc_euc2d(int64_t x0, int64_t y0, int64_t x1, int64_t y1) {
    const int64_t dx = x0 - x1, dy = y0 - y1;
    const double s = (double)(dx * dx + dy * dy);
    return (int32_t)floor(sqrt(s) + 0.5);
}

int32_t orc_distance(const orc_dist_t* d, uint32_t a, uint32_t b) {
    if (d->matrix) return d->matrix[(size_t)a * d->n + b];
    return orc_euc2d(d->xy[2 * (size_t)a], d->xy[2 * (size_t)a + 1], d->xy[2 * (size_t)b],
                     d->xy[2 * (size_t)b + 1]);
}

/* ---------------------------------------------------------------------- */
/* Tour primitives -- cpp/src/faco_cpu.cpp:47-146 (CpuTour).               */
/* ---------------------------------------------------------------------- */
static inline uint32_t succ(const orc_tour_t* t, uint32_t v) {
    const uint32_t p = t->pos[v] + 1;
    return t->order[p == t->n ? 0 : p];
}
static inline uint32_t pred(const orc_tour_t* t, uint32_t v) {
    const uint32_t p = t->pos[v];
    return t->order[p == 0 ? t->n - 1 : p - 1];
}

int64_t orc_tour_length(const uint32_t* order, uint32_t n, const orc_dist_t* d) {
    int64_t sum = 0;
    uint32_t previous = order[n - 1];
    for (uint32_t i = 0; i < n; ++i) {
        sum += orc_distance(d, previous, order[i]);
        previous = order[i];
    }
    return sum;
}

int orc_tour_reset(orc_tour_t* t, const orc_dist_t* d) {
    for (uint32_t i = 0; i < t->n; ++i) t->pos[i] = UINT32_MAX;
    for (uint32_t i = 0; i < t->n; ++i) {
        const uint32_t v = t->order[i];
        if (v >= t->n || t->pos[v] != UINT32_MAX) return -1;
        t->pos[v] = i;
    }
    t->cost = orc_tour_length(t->order, t->n, d);
    return 0;
}

/* CpuTour::relocate (faco_cpu.cpp:82-112): move `node` right after `target`. */
int orc_relocate(orc_tour_t* t, const orc_dist_t* d, uint32_t target, uint32_t node) {
    if (succ(t, target) == node) return 0;
    const uint32_t before = pred(t, node), after = succ(t, node), target_after = succ(t, target);
    const uint32_t p = t->pos[node], tp = t->pos[target];
    if (tp < p) {
        for (uint32_t i = p; i > tp + 1; --i) t->order[i] = t->order[i - 1];
        t->order[tp + 1] = node;
    } else {
        for (uint32_t i = p; i < tp; ++i) t->order[i] = t->order[i + 1];
        t->order[tp] = node;
    }
    const uint32_t lo = p < tp ? p : tp, hi = p < tp ? tp : p;
    for (uint32_t i = lo; i <= hi; ++i) t->pos[t->order[i]] = i;
    t->cost += -(int64_t)orc_distance(d, before, node) - orc_distance(d, node, after) -
               orc_distance(d, target, target_after) + orc_distance(d, before, after) +
               orc_distance(d, target, node) + orc_distance(d, node, target_after);
    return 1;
}

/* CpuTour::flip_without_cost (faco_cpu.cpp:114-135).  Positions first<last
 * of the two endpoints; the shorter side is reversed, except that first==0
 * always reverses [0,last) (the reference's wrap loop goes round once more
 * and undoes the complement, leaving exactly that). */
void orc_flip(orc_tour_t* t, uint32_t start, uint32_t end) {
    uint32_t first = t->pos[start], last = t->pos[end];
    if (first > last) { const uint32_t s = first; first = last; last = s; }
    const uint32_t n = t->n, length = last - first;
    const int straight = length <= n - length || first == 0;
    const uint32_t count = straight ? length : n - length, begin = straight ? first : last;
    for (uint32_t o = 0; o < count / 2; ++o) {
        const uint32_t l = (begin + o) % n, r = (begin + count - 1 - o) % n;
        const uint32_t a = t->order[l], b = t->order[r];
        t->order[l] = b; t->order[r] = a;
        t->pos[b] = l; t->pos[a] = r;
    }
}

void orc_queue_push_absent(orc_queue_t* q, uint32_t v, uint64_t* pushed) {
    if (q->queued[v]) return;
    q->queued[v] = 1;
    if (q->len < q->cap) q->items[q->len] = v;
    else q->overflow = 1;
    ++q->len;
    if (pushed) ++*pushed;
}

/* CpuTour::checklist_two_opt (faco_cpu.cpp:148-217), the device variant's
 * right-padding rule (cuda/faco_device.cuh:320) and integer gains. */
void orc_checklist_two_opt(orc_tour_t* t, const orc_dist_t* d, const uint32_t* rows, uint32_t w,
                           orc_queue_t* q, uint64_t cap, orc_ls_stats_t* st) {
    int64_t accumulated = 0;
    while (q->head < q->len && st->accepted_moves < t->n) {
        if (st->move_evaluations >= cap) { st->evaluation_limit_reached = 1; break; }
        const uint32_t a = q->items[q->head++];
        q->queued[a] = 0;
        const uint32_t an = succ(t, a), ap = pred(t, a);
        ++st->processed_nodes;
        const int64_t to_next = orc_distance(d, a, an), to_prev = orc_distance(d, ap, a);
        int64_t best = -1;
        uint32_t move[4] = {0, 0, 0, 0};
        int interrupted = 0;
        for (int kind = 0; kind < 2 && !interrupted; ++kind) {
            const int64_t current = kind == 0 ? to_next : to_prev;
            const uint32_t closing_end = kind == 0 ? an : ap;
            for (uint32_t j = 0; j < w; ++j) {
                const uint32_t b = rows[(size_t)a * w + j];
                ++st->candidate_checks;
                if (b >= t->n) break;
                const int64_t ab = orc_distance(d, a, b);
                if (!(current > ab)) break;
                if (st->move_evaluations == cap) { interrupted = 1; break; }
                ++st->move_evaluations;
                const uint32_t nb = kind == 0 ? succ(t, b) : pred(t, b);
                const int64_t other = orc_distance(d, b, nb);
                const int64_t closing = orc_distance(d, closing_end, nb);
                const int64_t gain = (nb == a || b == closing_end) ? 0 : current + other - ab - closing;
                if (gain > best) {
                    best = gain;
                    if (kind == 0) { move[0] = an; move[1] = nb; move[2] = a; move[3] = b; }
                    else { move[0] = a; move[1] = b; move[2] = ap; move[3] = nb; }
                }
            }
        }
        if (interrupted) { st->evaluation_limit_reached = 1; break; }
        if (best > 0) {
            orc_flip(t, move[0], move[1]);
            for (int i = 0; i < 4; ++i) orc_queue_push_absent(q, move[i], &st->reactivations);
            ++st->accepted_moves;
            accumulated -= best;
        }
    }
    t->cost += accumulated;
}

/* Relocation without the cost update (used to apply Or-opt moves). */
static void relocate_order(orc_tour_t* t, uint32_t target, uint32_t node) {
    const uint32_t p = t->pos[node], tp = t->pos[target];
    if (tp < p) {
        for (uint32_t i = p; i > tp + 1; --i) t->order[i] = t->order[i - 1];
        t->order[tp + 1] = node;
    } else {
        for (uint32_t i = p; i < tp; ++i) t->order[i] = t->order[i + 1];
        t->order[tp] = node;
    }
    const uint32_t lo = p < tp ? p : tp, hi = p < tp ? tp : p;
    for (uint32_t i = lo; i <= hi; ++i) t->pos[t->order[i]] = i;
}

/* Checklist local search with first-improvement 2-opt and Or-opt.  The
 * reference has no Or-opt (its LS is the best-gain 2-opt above); this is the
 * engine's own variant, defined here:
 *  - a popped node a first scans 2-opt moves in the same (kind, j) order and
 *    with the same pruning and cap rules as the best-gain search, applying
 *    the FIRST move with positive gain;
 *  - if none, Or-opt: for L = 1, 2, 3 (n >= L + 3) the segment a..e of L
 *    nodes following a in tour order, p = pred(a), q = succ(e), removal gain
 *    G = d(p,a) + d(e,q) - d(p,q); candidates c of a's LS row while
 *    d(a,c) < G, each counted as one move evaluation, c outside the segment;
 *    (i) insert between c and c2 = succ(c) as c,a..e,c2 (c2 outside the
 *    segment), gain G + d(c,c2) - d(c,a) - d(e,c2); then (ii) insert between
 *    c0 = pred(c) and c as c0,e..a,c (c0 outside), gain G + d(c0,c) -
 *    d(c0,e) - d(a,c); the first positive gain in (L, j, variant) order is
 *    applied by successive relocations (c<-a<-...<-e, or c0<-e<-...<-a) and
 *    p, a, e, q and the two insertion neighbours are queued. */
void orc_checklist_ls_first(orc_tour_t* t, const orc_dist_t* d, const uint32_t* rows, uint32_t w,
                            orc_queue_t* q, uint64_t cap, orc_ls_stats_t* st) {
    int64_t accumulated = 0;
    const uint32_t n = t->n;
    while (q->head < q->len && st->accepted_moves < n) {
        if (st->move_evaluations >= cap) { st->evaluation_limit_reached = 1; break; }
        const uint32_t a = q->items[q->head++];
        q->queued[a] = 0;
        const uint32_t an = succ(t, a), ap = pred(t, a);
        ++st->processed_nodes;
        int interrupted = 0, found = 0;
        int64_t gain = 0;
        uint32_t move[6] = {0, 0, 0, 0, 0, 0};
        for (int kind = 0; kind < 2 && !interrupted && !found; ++kind) {
            const int64_t current = kind == 0 ? orc_distance(d, a, an) : orc_distance(d, ap, a);
            const uint32_t closing_end = kind == 0 ? an : ap;
            for (uint32_t j = 0; j < w; ++j) {
                const uint32_t b = rows[(size_t)a * w + j];
                ++st->candidate_checks;
                if (b >= n) break;
                const int64_t ab = orc_distance(d, a, b);
                if (!(current > ab)) break;
                if (st->move_evaluations == cap) { interrupted = 1; break; }
                ++st->move_evaluations;
                const uint32_t nb = kind == 0 ? succ(t, b) : pred(t, b);
                const int64_t g = (nb == a || b == closing_end)
                    ? 0 : current + orc_distance(d, b, nb) - ab - orc_distance(d, closing_end, nb);
                if (g > 0) {
                    gain = g; found = 1;
                    if (kind == 0) { move[0] = an; move[1] = nb; move[2] = a; move[3] = b; }
                    else { move[0] = a; move[1] = b; move[2] = ap; move[3] = nb; }
                    break;
                }
            }
        }
        if (interrupted) { st->evaluation_limit_reached = 1; break; }
        if (found) {
            orc_flip(t, move[0], move[1]);
            for (int i = 0; i < 4; ++i) orc_queue_push_absent(q, move[i], &st->reactivations);
            ++st->accepted_moves;
            accumulated -= gain;
            continue;
        }
        uint32_t seg[3] = {a, 0, 0}, variant = 0, L = 0, cj = 0, cn = 0;
        for (uint32_t len = 1; len <= 3 && !found && !interrupted; ++len) {
            if (n < len + 3) break;
            if (len > 1) seg[len - 1] = succ(t, seg[len - 2]);
            const uint32_t e = seg[len - 1], qn = succ(t, e);
            const int64_t G = orc_distance(d, ap, a) + orc_distance(d, e, qn) - orc_distance(d, ap, qn);
            for (uint32_t j = 0; j < w; ++j) {
                const uint32_t c = rows[(size_t)a * w + j];
                ++st->candidate_checks;
                if (c >= n) break;
                const int64_t ac = orc_distance(d, a, c);
                if (!(G > ac)) break;
                if (st->move_evaluations == cap) { interrupted = 1; break; }
                ++st->move_evaluations;
                int inside = 0;
                for (uint32_t i = 0; i < len; ++i) inside |= seg[i] == c;
                if (inside) continue;
                const uint32_t c2 = succ(t, c), c0 = pred(t, c);
                int c2_in = 0, c0_in = 0;
                for (uint32_t i = 0; i < len; ++i) { c2_in |= seg[i] == c2; c0_in |= seg[i] == c0; }
                if (!c2_in) {
                    const int64_t g = G + orc_distance(d, c, c2) - ac - orc_distance(d, e, c2);
                    if (g > 0) { gain = g; found = 1; variant = 1; L = len; cj = c; cn = c2; break; }
                }
                if (!c0_in) {
                    const int64_t g = G + orc_distance(d, c0, c) - orc_distance(d, c0, e) - ac;
                    if (g > 0) { gain = g; found = 1; variant = 2; L = len; cj = c; cn = c0; break; }
                }
            }
        }
        if (interrupted) { st->evaluation_limit_reached = 1; break; }
        if (found) {
            const uint32_t e = seg[L - 1], qn = succ(t, e);
            if (variant == 1) {
                relocate_order(t, cj, seg[0]);
                for (uint32_t i = 1; i < L; ++i) relocate_order(t, seg[i - 1], seg[i]);
            } else {
                relocate_order(t, cn, e);
                for (uint32_t i = L - 1; i > 0; --i) relocate_order(t, seg[i], seg[i - 1]);
            }
            const uint32_t order6[6] = {ap, a, e, qn, variant == 1 ? cj : cn, variant == 1 ? cn : cj};
            for (int i = 0; i < 6; ++i) orc_queue_push_absent(q, order6[i], &st->reactivations);
            ++st->accepted_moves;
            accumulated -= gain;
        }
    }
    t->cost += accumulated;
}

/* select_next (faco_cpu.cpp:247-294) with the device's visiting order
 * (cuda/faco_choices.cuh:86-142): ordered FP64 prefix sums. */
uint32_t orc_select_next(uint32_t current, const uint32_t* primary, const double* products, uint32_t k,
                         const uint32_t* backup, uint32_t b, const uint8_t* visited,
                         const orc_dist_t* d, double uniform, int* stage) {
    uint32_t available = 0, last = UINT32_MAX;
    double sum = 0;
    for (uint32_t j = 0; j < k; ++j) {
        const uint32_t v = primary[j];
        if (v < d->n && !visited[v]) { ++available; sum += products[j]; last = v; }
    }
    if (available) {
        if (sum == 0) {
            uint32_t target = (uint32_t)(uniform * available);
            if (target >= available) target = available - 1;
            for (uint32_t j = 0; j < k; ++j) {
                const uint32_t v = primary[j];
                if (v < d->n && !visited[v] && target-- == 0) { if (stage) *stage = ORC_ZERO_WEIGHT; return v; }
            }
        }
        const double threshold = uniform * sum;
        double prefix = 0;
        for (uint32_t j = 0; j < k; ++j) {
            const uint32_t v = primary[j];
            if (v < d->n && !visited[v]) {
                prefix += products[j];
                if (threshold < prefix) { if (stage) *stage = ORC_PRIMARY; return v; }
            }
        }
        if (stage) *stage = ORC_PRIMARY;
        return last;
    }
    for (uint32_t j = 0; j < b; ++j) {
        const uint32_t v = backup[j];
        if (v < d->n && !visited[v]) { if (stage) *stage = ORC_BACKUP; return v; }
    }
    uint32_t chosen = current;
    int64_t minimum = INT64_MAX;
    for (uint32_t v = 0; v < d->n; ++v) {
        if (visited[v]) continue;
        const int64_t value = orc_distance(d, current, v);
        if (value < minimum) { minimum = value; chosen = v; }
    }
    if (stage) *stage = chosen == current ? ORC_EXHAUSTED : ORC_GLOBAL;
    return chosen;
}

/* One ant: FocusedConstruction (faco_cpu.cpp:219-245) then the checklist
 * 2-opt on the construction's checklist (tests/cpp/test_fixed_faco.cpp:235-256). */
int orc_ant(const uint32_t* parent, const orc_dist_t* d, const uint32_t* ls_rows, uint32_t w,
            const orc_choices_t* ch, uint32_t mne_target, uint64_t max_evaluations, uint32_t ls_mode,
            uint32_t* construction_tour, uint32_t* tour, uint32_t* pos, uint32_t* checklist,
            uint32_t* selected, orc_ant_info_t* info) {
    const uint32_t n = d->n;
    memset(info, 0, sizeof(*info));
    uint32_t* ppos = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint8_t* visited = (uint8_t*)calloc(n, 1);
    uint8_t* queued = (uint8_t*)calloc(n, 1);
    const uint32_t cap = 8 * n + 8;
    uint32_t* items = checklist ? checklist : (uint32_t*)malloc(sizeof(uint32_t) * cap);
    double* row = (double*)malloc(sizeof(double) * (ch->k ? ch->k : 1));
    if (!ppos || !visited || !queued || !items || !row) return -1;
    for (uint32_t i = 0; i < n; ++i) ppos[parent[i]] = i;
    memcpy(tour, parent, sizeof(uint32_t) * n);
    orc_tour_t t = {n, tour, pos, 0};
    orc_tour_reset(&t, d);
    orc_queue_t q = {items, cap, 0, 0, queued, 0};
    uint32_t current = ch->visit ? ch->visit[0] : ch->start;
    info->start_node = current;
    if (selected) selected[0] = current;
    visited[current] = 1;
    orc_cons_stats_t* cs = &info->cons;
    while (cs->mne < mne_target && cs->steps + 1 < n) {
        const uint32_t step = cs->steps + 1;
        uint32_t chosen;
        if (ch->visit) {
            chosen = ch->visit[step];
        } else {
            const uint32_t* prow = ch->primary + (size_t)current * ch->k;
            for (uint32_t j = 0; j < ch->k; ++j)
                row[j] = ch->products64 ? ch->products64[(size_t)current * ch->k + j]
                                        : (double)ch->products32[(size_t)current * ch->k + j];
            chosen = orc_select_next(current, prow, row, ch->k, ch->backup + (size_t)current * ch->b, ch->b,
                                     visited, d, ch->uniforms[step], NULL);
        }
        if (chosen >= n || visited[chosen]) { cs->legal_exhausted = 1; break; }
        if (selected) selected[step] = chosen;
        const uint32_t previous = pred(&t, chosen);
        visited[chosen] = 1;
        ++cs->steps;
        if (orc_relocate(&t, d, current, chosen)) ++cs->nonidentity_relocations;
        const uint32_t pp = ppos[current];
        const uint32_t ps = parent[pp + 1 == n ? 0 : pp + 1], pq = parent[pp == 0 ? n - 1 : pp - 1];
        if (ps != chosen && pq != chosen) {
            ++cs->mne;
            orc_queue_push_absent(&q, current, NULL);
            orc_queue_push_absent(&q, chosen, NULL);
            orc_queue_push_absent(&q, previous, NULL);
        }
        current = chosen;
    }
    if (construction_tour) memcpy(construction_tour, tour, sizeof(uint32_t) * n);
    info->construction_cost = t.cost;
    if (ls_mode == 1) orc_checklist_ls_first(&t, d, ls_rows, w, &q, max_evaluations, &info->ls);
    else orc_checklist_two_opt(&t, d, ls_rows, w, &q, max_evaluations, &info->ls);
    info->final_cost = t.cost;
    info->checklist_len = q.len;
    const int overflow = q.overflow;
    free(ppos); free(visited); free(queued); free(row);
    if (!checklist) free(items);
    return overflow ? -2 : 0;
}

/* ---------------------------------------------------------------------- */
/* Trails -- candidate_trail_limits (faco_cpu.cpp:296-304), bounds()      */
/* (cuda/colony_state.cuh:66-70), SparsePheromone evaporate/deposit       */
/* (faco_cpu.cpp:322-343) and update_pheromone (colony_state.cuh:210-229). */
/* ---------------------------------------------------------------------- */
void orc_trail_limits(uint32_t width, double p_root, double retention, double cost, double* minimum,
                      double* maximum) {
    const double mx = 1.0 / (cost * (1.0 - retention));
    const double mn = mx * (1.0 - p_root) / (((double)width - 1.0) * p_root);
    *maximum = mx;
    *minimum = mn < mx ? mn : mx;
}

static inline int parent_edge(const uint32_t* parent, const uint32_t* ppos, uint32_t n, uint32_t from,
                              uint32_t to) {
    const uint32_t p = ppos[from];
    return parent[p + 1 == n ? 0 : p + 1] == to || parent[p == 0 ? n - 1 : p - 1] == to;
}

void orc_pheromone64(uint32_t n, uint32_t k, const uint32_t* primary, const uint32_t* parent,
                     double retention, double minimum, double maximum, double increment, double* trails,
                     double* default_trail) {
    uint32_t* ppos = (uint32_t*)malloc(sizeof(uint32_t) * n);
    for (uint32_t i = 0; i < n; ++i) ppos[parent[i]] = i;
    for (uint32_t from = 0; from < n; ++from)
        for (uint32_t j = 0; j < k; ++j) {
            const size_t i = (size_t)from * k + j;
            double v = trails[i] * retention;
            v = v > minimum ? v : minimum;
            if (primary[i] < n && parent_edge(parent, ppos, n, from, primary[i])) {
                v = v + increment;
                v = v < maximum ? v : maximum;
            }
            trails[i] = v;
        }
    const double dv = *default_trail * retention;
    *default_trail = dv > minimum ? dv : minimum;
    free(ppos);
}

void orc_pheromone32(uint32_t n, uint32_t k, const uint32_t* primary, const uint32_t* parent,
                     float retention, float minimum, float maximum, float increment, const float* eta,
                     float* trails, float* products, float* default_trail) {
    uint32_t* ppos = (uint32_t*)malloc(sizeof(uint32_t) * n);
    for (uint32_t i = 0; i < n; ++i) ppos[parent[i]] = i;
    for (uint32_t from = 0; from < n; ++from)
        for (uint32_t j = 0; j < k; ++j) {
            const size_t i = (size_t)from * k + j;
            float v = fmaxf(minimum, trails[i] * retention);
            if (primary[i] < n && parent_edge(parent, ppos, n, from, primary[i])) v = fminf(maximum, v + increment);
            trails[i] = v;
            products[i] = v * eta[i];
        }
    *default_trail = fmaxf(minimum, *default_trail * retention);
    free(ppos);
}

/* ---------------------------------------------------------------------- */
/* Learned edge prior (no reference counterpart; it reweights the         */
/* heuristic of initialize_products, colony_state.cuh:91-110, and of      */
/* SparsePheromone::product_cache, faco_cpu.cpp:351-363).                 */
/*   eta'[e] = eta[e] * f, f = floor + p[e], squared when gamma == 2,      */
/* in FP32 with one rounding per operation.  p is the network's            */
/* probability for the candidate entry; floor > 0, so no weight is zero.   */
/* ---------------------------------------------------------------------- */
void orc_prior_eta(size_t cells, const float* eta, const float* prob, float floor, int gamma, float* out) {
    for (size_t e = 0; e < cells; ++e) {
        const float f = floor + prob[e];
        out[e] = eta[e] * (gamma == 2 ? f * f : f);
    }
}

/* Products of a colony whose prior re-ranks only the departures from the  */
/* parent tour: per node i, the entries of i's two parent-tour neighbours   */
/* keep the plain heuristic (trail * eta), and the others take the prior's  */
/* (trail * eta') scaled by plain / prior, the two totals summed in         */
/* candidate order over those other entries (scale 1 when the prior total   */
/* is 0), so that their total weight stays the plain one.                   */
void orc_departure_rows(uint32_t n, uint32_t k, const uint32_t* primary, const uint32_t* parent,
                        const float* trails, const float* eta, const float* prior_eta, float* products) {
    uint32_t* succ = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* pred = (uint32_t*)malloc(sizeof(uint32_t) * n);
    for (uint32_t p = 0; p < n; ++p) {
        succ[parent[p]] = parent[p + 1 == n ? 0 : p + 1];
        pred[parent[p]] = parent[p == 0 ? n - 1 : p - 1];
    }
    for (uint32_t i = 0; i < n; ++i) {
        const size_t row = (size_t)i * k;
        float plain = 0.0f, prior = 0.0f;
        for (uint32_t j = 0; j < k; ++j) {
            const uint32_t node = primary[row + j];
            if (node == succ[i] || node == pred[i]) continue;
            const float t = trails[row + j];
            plain += t * eta[row + j];
            prior += t * prior_eta[row + j];
        }
        const float scale = prior > 0.0f ? plain / prior : 1.0f;
        for (uint32_t j = 0; j < k; ++j) {
            const uint32_t node = primary[row + j];
            const float t = trails[row + j];
            products[row + j] = node == succ[i] || node == pred[i] ? t * eta[row + j] : t * prior_eta[row + j] * scale;
        }
    }
    free(succ);
    free(pred);
}

/* ---------------------------------------------------------------------- */
/* Random stream.  Philox4x32 with 10 rounds as published by Salmon,       */
/* Moraes, Dror and Shaw, "Parallel random numbers: as easy as 1, 2, 3"    */
/* (SC'11).  The counter layout is this engine's own:                     */
/*   (step, ant, batch, 0) construction uniform for step >= 1              */
/*   (0, ant, batch, 1)    start node                                      */
/*   (0, 0xffffffff, batch, 2) colony source draw (epoch vs iteration best)*/
/* ---------------------------------------------------------------------- */
void orc_philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                    uint32_t out[4]) {
    for (int round = 0; round < 10; ++round) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0; c1 = lo1; c2 = hi0 ^ c3 ^ k1; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline double u53(uint32_t hi, uint32_t lo) {
    return (double)((((uint64_t)hi << 32) | lo) >> 11) * 0x1.0p-53;
}

double orc_uniform(uint64_t key, uint32_t batch, uint32_t ant, uint32_t step) {
    uint32_t x[4];
    orc_philox4x32(step, ant, batch, 0, (uint32_t)key, (uint32_t)(key >> 32), x);
    return u53(x[0], x[1]);
}

uint32_t orc_start_node(uint64_t key, uint32_t batch, uint32_t ant, uint32_t n) {
    uint32_t x[4];
    orc_philox4x32(0, ant, batch, 1, (uint32_t)key, (uint32_t)(key >> 32), x);
    return (uint32_t)(((uint64_t)x[0] * n) >> 32);
}

double orc_source_uniform(uint64_t key, uint32_t batch) {
    uint32_t x[4];
    orc_philox4x32(0, 0xffffffffu, batch, 2, (uint32_t)key, (uint32_t)(key >> 32), x);
    return u53(x[0], x[1]);
}

/* SplitMix64 finaliser (Steele, Lea, Flood 2014) over seed and instance. */
static uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
uint64_t orc_colony_key(uint64_t seed, uint64_t instance_key) { return mix64(seed ^ mix64(instance_key)); }

/* ---------------------------------------------------------------------- */
/* Preparation -- prepare_problem (cpp/src/prepared_problem.cpp:107-175)  */
/* with EUC_2D integers: rows sorted by (distance, node id), NN tour from */
/* node 0 (first strict minimum), checklist 2-opt over the whole tour,    */
/* identity tour kept when it is no longer.                               */
/* ---------------------------------------------------------------------- */
typedef struct { int64_t d; uint32_t v; } orc_pair_t;
static int pair_less(const void* x, const void* y) {
    const orc_pair_t* a = (const orc_pair_t*)x; const orc_pair_t* b = (const orc_pair_t*)y;
    if (a->d != b->d) return a->d < b->d ? -1 : 1;
    return a->v < b->v ? -1 : (a->v > b->v);
}

int64_t orc_prepare(uint32_t n, const int32_t* xy, const orc_prep_cfg_t* cfg, uint32_t* primary,
                    uint32_t* backup, uint32_t* ls, uint32_t* initial) {
    const orc_dist_t d = {n, xy, NULL};
    orc_pair_t* row = (orc_pair_t*)malloc(sizeof(orc_pair_t) * n);
    for (uint32_t a = 0; a < n; ++a) {
        uint32_t m = 0;
        for (uint32_t b = 0; b < n; ++b) if (b != a) { row[m].d = orc_distance(&d, a, b); row[m].v = b; ++m; }
        qsort(row, m, sizeof(orc_pair_t), pair_less);
        for (uint32_t j = 0; j < cfg->k; ++j) primary[(size_t)a * cfg->k + j] = row[j].v;
        for (uint32_t j = 0; j < cfg->b; ++j) backup[(size_t)a * cfg->b + j] = row[cfg->k + j].v;
        for (uint32_t j = 0; j < cfg->w; ++j) ls[(size_t)a * cfg->w + j] = row[j].v;
    }
    free(row);
    uint8_t* seen = (uint8_t*)calloc(n, 1);
    uint32_t current = 0;
    for (uint32_t i = 0; i < n; ++i) {
        initial[i] = current; seen[current] = 1;
        uint32_t next = n; int64_t shortest = INT64_MAX;
        for (uint32_t b = 0; b < n; ++b) {
            if (seen[b]) continue;
            const int64_t v = orc_distance(&d, current, b);
            if (v < shortest) { shortest = v; next = b; }
        }
        current = next;
    }
    uint32_t* pos = (uint32_t*)malloc(sizeof(uint32_t) * n);
    orc_tour_t t = {n, initial, pos, 0};
    orc_tour_reset(&t, &d);
    const uint32_t cap = 8 * n + 8;
    uint32_t* items = (uint32_t*)malloc(sizeof(uint32_t) * cap);
    memset(seen, 0, n);
    orc_queue_t q = {items, cap, 0, 0, seen, 0};
    for (uint32_t i = 0; i < n; ++i) orc_queue_push_absent(&q, initial[i], NULL);
    orc_ls_stats_t st; memset(&st, 0, sizeof(st));
    orc_checklist_two_opt(&t, &d, ls, cfg->w, &q, cfg->initial_ls_evaluation_limit, &st);
    int64_t cost = orc_tour_length(initial, n, &d);
    uint32_t* identity = items;  /* reuse */
    for (uint32_t i = 0; i < n; ++i) identity[i] = i;
    const int64_t cheap = orc_tour_length(identity, n, &d);
    if (cheap <= cost) { memcpy(initial, identity, sizeof(uint32_t) * n); cost = cheap; }
    free(items); free(pos); free(seen);
    return cost;
}

/* ---------------------------------------------------------------------- */
/* GP controller of the engine (feature spec 3).  The reference scores 32   */
/* actions per colony from 12 features (cuda/control_state.cuh:200-364);  */
/* the engine's own set is 7 colony features + 3 action descriptors:      */
/*  f0 iteration fraction (t+1)/T, f1 stagnation s/(s+16), f2 mean/best gap,*/
/*  f3 mean normalised entropy of the trail rows, f4 restarts r/(r+1),     */
/*  f5 LS gain (10x relative, clipped), f6 reference-tour age a/(a+16);     */
/*  f7 MNE level (a&3)/3, f8 start region ((a>>2)&3)/3, f9 restart flag.    */
/* Action a: MNE target 2<<(a&3), start region (a>>2)&3 (quadrant around  */
/* the bounding-box centre), restart when a >= 16 (parent and epoch <- the */
/* global best, trails <- tau_max).  Everything below is exact or single- */
/* rounding FP32/FP64 arithmetic so that the GPU reproduces it bit for bit.*/
/* ---------------------------------------------------------------------- */
static int arity_of(int op);

float orc_log2(float x) {
    /* x = m 2^e, m in [sqrt(2)/2, sqrt(2)); log2 m = (2/ln 2) atanh((m-1)/(m+1)) */
    uint32_t bits;
    memcpy(&bits, &x, 4);
    int e = (int)((bits >> 23) & 255u) - 127;
    uint32_t mb = (bits & 0x7FFFFFu) | 0x3F800000u;
    float m;
    memcpy(&m, &mb, 4);
    if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e += 1; }
    const float t = (m - 1.0f) / (m + 1.0f), t2 = t * t;
    const float s = t * (1.0f + t2 * (0x1.555556p-2f + t2 * (0x1.99999ap-3f + t2 * 0x1.24924ap-3f)));
    return (float)e + s * 0x1.715476p+1f;
}

uint32_t orc_row_entropy_q(const float* tau, uint32_t k, float log2k) {
    float sum = 0.0f;
    for (uint32_t j = 0; j < k; ++j) sum = sum + tau[j];
    if (!(sum > 0.0f)) return 0;
    float h = 0.0f;
    for (uint32_t j = 0; j < k; ++j) {
        const float p = tau[j] / sum;
        if (p > 0.0f) h = h - p * orc_log2(p);
    }
    float hn = h / log2k;
    hn = hn < 0.0f ? 0.0f : hn > 1.0f ? 1.0f : hn;
    return (uint32_t)(hn * 1048576.0f + 0.5f);
}

void orc_regions(uint32_t n, const int32_t* xy, uint32_t* offsets, uint32_t* list) {
    int64_t minx = xy[0], maxx = xy[0], miny = xy[1], maxy = xy[1];
    for (uint32_t i = 0; i < n; ++i) {
        minx = xy[2 * i] < minx ? xy[2 * i] : minx; maxx = xy[2 * i] > maxx ? xy[2 * i] : maxx;
        miny = xy[2 * i + 1] < miny ? xy[2 * i + 1] : miny; maxy = xy[2 * i + 1] > maxy ? xy[2 * i + 1] : maxy;
    }
    uint32_t count[4] = {0, 0, 0, 0};
    for (uint32_t i = 0; i < n; ++i)
        ++count[(2 * (int64_t)xy[2 * i] >= minx + maxx) + 2 * (2 * (int64_t)xy[2 * i + 1] >= miny + maxy)];
    offsets[0] = 0;
    for (int r = 0; r < 4; ++r) offsets[r + 1] = offsets[r] + count[r];
    uint32_t fill[4] = {offsets[0], offsets[1], offsets[2], offsets[3]};
    for (uint32_t i = 0; i < n; ++i)
        list[fill[(2 * (int64_t)xy[2 * i] >= minx + maxx) + 2 * (2 * (int64_t)xy[2 * i + 1] >= miny + maxy)]++] = i;
}

uint32_t orc_region_start(uint64_t key, uint32_t batch, uint32_t ant, uint32_t n, const uint32_t* offsets,
                          const uint32_t* list, uint32_t region) {
    if (region >= 4 || offsets[region + 1] == offsets[region]) return orc_start_node(key, batch, ant, n);
    uint32_t x[4];
    orc_philox4x32(0, ant, batch, 1, (uint32_t)key, (uint32_t)(key >> 32), x);
    const uint32_t size = offsets[region + 1] - offsets[region];
    return list[offsets[region] + (uint32_t)(((uint64_t)x[0] * size) >> 32)];
}

static float clamp01(double v) { return (float)(v < 0.0 ? 0.0 : v > 1.0 ? 1.0 : v); }

/* Scores the 32 actions of one colony from its 7 colony features and picks
 * the first maximum within 1e-6 among legal actions (score_cpu rule). */
/* One program on the 12 features of one action (postfix evaluation as in
 * score_cpu, cpp/src/program_cpu.cpp:79-116). */
static float orc_eval12(const orc_program_t* p, const float f[12]) {
    float stack[16] = {0};
    int top = 0;
    for (int i = 0; i < p->length; ++i) {
        const int op = p->opcode[i];
        if (op == 0) stack[top++] = f[p->operand[i]];
        else if (op == 1) stack[top++] = p->constants[p->operand[i]];
        else {
            const int ar = arity_of(op);
            const float third = ar == 3 ? stack[--top] : 0.0f;
            const float right = ar >= 2 ? stack[--top] : 0.0f;
            const float left = stack[--top];
            stack[top++] = orc_apply_operation(op, left, right, third);
        }
    }
    return stack[0];
}

/* Feature spec 3 of action a: the 7 colony features, then its MNE level,
 * start region and restart flag. */
static void orc_action_features(const float colony[7], int a, float f[12]) {
    for (int i = 0; i < 7; ++i) f[i] = colony[i];
    f[7] = (float)(a & 3) / 3.0f;
    f[8] = (float)((a >> 2) & 3) / 3.0f;
    f[9] = a >= 16 ? 1.0f : 0.0f;
    f[10] = f[11] = 0.0f;
}

int32_t orc_control_choose(const orc_program_t* p, const float colony[7], uint32_t mask, float* scores) {
    float maximum = -INFINITY;
    for (int a = 0; a < 32; ++a) {
        float f[12];
        orc_action_features(colony, a, f);
        scores[a] = orc_eval12(p, f);
        if ((mask >> a) & 1u) maximum = fmaxf(maximum, scores[a]);
    }
    for (int a = 0; a < 32; ++a)
        if (((mask >> a) & 1u) && maximum - scores[a] <= 1e-6f) return a;
    return 0;
}

/* conditional_three (python/gp_faco/controller.py:60-84): role 0 picks the
 * restart half (2 options, stride 16), role 1 the start region (4, stride
 * 4), role 2 the MNE level (4, stride 1), from the prefix fixed so far; each
 * candidate is scored on the features of action prefix + i * stride and is
 * legal when any action of its stride-wide window is; the first maximum
 * within 1e-6 wins.  values(trees + role, action) gives a score. */
static int32_t orc_conditional(const orc_program_t* trees, uint32_t mask, float* role_scores,
                               float (*value)(const orc_program_t*, int, const void*), const void* ctx) {
    int32_t prefix = 0;
    for (int role = 0; role < 3; ++role) {
        const int width = role == 0 ? 2 : 4, stride = role == 0 ? 16 : role == 1 ? 4 : 1;
        const int slot = role == 0 ? 0 : role == 1 ? 2 : 6;
        float vals[4], maximum = -INFINITY;
        int legal[4];
        for (int i = 0; i < width; ++i) {
            const int a = prefix + i * stride;
            vals[i] = value(trees + role, a, ctx);
            legal[i] = ((mask >> a) & ((1u << stride) - 1u)) != 0u;
            if (legal[i]) maximum = fmaxf(maximum, vals[i]);
            if (role_scores) role_scores[slot + i] = vals[i];
        }
        int chosen = 0;
        for (int i = 0; i < width; ++i)
            if (legal[i] && maximum - vals[i] <= 1e-6f) { chosen = i; break; }
        prefix += chosen * stride;
    }
    return prefix;
}

static float orc_colony_value(const orc_program_t* p, int a, const void* ctx) {
    float f[12];
    orc_action_features((const float*)ctx, a, f);
    return orc_eval12(p, f);
}

int32_t orc_control_choose_conditional(const orc_program_t* trees, const float colony[7], uint32_t mask,
                                       float* role_scores) {
    return orc_conditional(trees, mask, role_scores, orc_colony_value, colony);
}

typedef struct { const float* features; uint32_t colonies, colony; } orc_feature_ctx_t;

static float orc_array_value(const orc_program_t* p, int a, const void* ctx) {
    const orc_feature_ctx_t* c = (const orc_feature_ctx_t*)ctx;
    float f[12];
    for (int i = 0; i < 12; ++i) f[i] = c->features[((size_t)i * c->colonies + c->colony) * 32 + (size_t)a];
    return orc_eval12(p, f);
}

void orc_score_conditional(const orc_program_t* trees, const float* features, const uint32_t* masks,
                           uint32_t colonies, float* scores, int32_t* actions) {
    for (uint32_t c = 0; c < colonies; ++c) {
        const orc_feature_ctx_t ctx = {features, colonies, c};
        for (int j = 0; j < 32; ++j) scores[(size_t)c * 32 + j] = 0.0f;
        actions[c] = orc_conditional(trees, masks[c], scores + (size_t)c * 32, orc_array_value, &ctx);
    }
}

/* ---------------------------------------------------------------------- */
/* Feature spec 2 inside a colony run: the state the reference keeps per   */
/* colony (ControllerState, control_ops.hpp:160-173) and its per-batch     */
/* update (update_control, control_state.cuh:124-245).                     */
/* ---------------------------------------------------------------------- */
typedef struct {
    orc_control_in_t in;
    orc_archive_t archive;
    uint32_t samples[ORC_SAMPLE_CAPACITY];
    double* local_scale;
    double epsilon;
    double* trails64;
    uint32_t* ppos;
    orc_fp_t* ids;
    int64_t* costs;
    orc_feedback_t feedback;
    orc_fp_t active_id, epoch_id;
    int64_t tracked_global, tracked_epoch, parent_cost;
} ctl2_t;

static int ctl2_init(ctl2_t* t, uint32_t n, const int32_t* xy, const uint32_t* primary, uint32_t k,
                     const uint32_t* initial, int64_t initial_cost, uint64_t instance_key, uint32_t zero) {
    (void)primary;
    t->local_scale = (double*)malloc(sizeof(double) * n);
    t->trails64 = (double*)malloc(sizeof(double) * (size_t)n * k);
    t->ppos = (uint32_t*)malloc(sizeof(uint32_t) * n);
    t->archive.tours = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)ORC_ARCHIVE_CAPACITY * n);
    t->archive.pos = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)ORC_ARCHIVE_CAPACITY * n);
    if (!t->local_scale || !t->trails64 || !t->ppos || !t->archive.tours || !t->archive.pos) return -1;
    orc_sample_nodes(n, instance_key, t->samples);
    orc_local_scale(n, xy, t->local_scale, &t->epsilon);
    t->archive.n = n;
    t->archive.size = 1;
    memcpy(t->archive.tours, initial, sizeof(uint32_t) * n);
    for (uint32_t i = 0; i < n; ++i) t->archive.pos[initial[i]] = i;
    t->archive.cost[0] = initial_cost;
    t->archive.zero_ids = zero;
    t->archive.id[0] = zero ? (orc_fp_t){0, 0} : orc_fingerprint(initial, n);
    t->active_id = t->epoch_id = t->archive.id[0];
    t->tracked_global = t->tracked_epoch = t->parent_cost = initial_cost;
    return 0;
}

static void ctl2_free(ctl2_t* t) {
    free(t->local_scale); free(t->trails64); free(t->ppos); free(t->archive.tours); free(t->archive.pos);
    free(t->ids); free(t->costs);
}

static void ctl2_input(ctl2_t* t, uint32_t n, const int32_t* xy, const uint32_t* primary, uint32_t k,
                       const uint32_t* parent, int64_t parent_cost, const float* trails, float dflt, float tmin,
                       float tmax, double elapsed, uint64_t key, uint32_t batch, uint32_t mask) {
    for (uint32_t i = 0; i < n; ++i) t->ppos[parent[i]] = i;
    for (size_t i = 0; i < (size_t)n * k; ++i) t->trails64[i] = (double)trails[i];
    orc_control_in_t* in = &t->in;
    in->n = n; in->xy = xy; in->primary = primary; in->k = k;
    in->samples = t->samples; in->sample_count = n < ORC_SAMPLE_CAPACITY ? n : ORC_SAMPLE_CAPACITY;
    in->local_scale = t->local_scale; in->epsilon = t->epsilon;
    in->active_tour = parent; in->active_pos = t->ppos; in->active_cost = parent_cost; in->active_id = t->active_id;
    in->archive = &t->archive; in->feedback = t->feedback;
    in->trails = t->trails64; in->default_trail = (double)dflt;
    in->tau_min = (double)tmin; in->tau_max = (double)tmax;
    in->elapsed_ratio = elapsed; in->solve_key = key; in->batch = batch; in->experiment_mask = mask;
}

static float ctl2_value(const orc_program_t* p, int a, const void* ctx) {
    const float* f = (const float*)ctx;
    float col[12];
    for (int i = 0; i < 12; ++i) col[i] = f[i * 32 + a];
    return orc_eval12(p, col);
}

/* joint_single: first maximum within 1e-6 among legal actions; conditional
 * controllers: the role rule, role scores in slots 0-9. */
static int32_t ctl2_choose(const orc_program_t* program, uint32_t kind, const float* f, uint32_t legal,
                           float* scores) {
    if (kind == 1) {
        for (int a = 0; a < 32; ++a) scores[a] = 0.0f;
        return orc_conditional(program, legal, scores, ctl2_value, f);
    }
    float maximum = -INFINITY;
    for (int a = 0; a < 32; ++a) {
        scores[a] = ctl2_value(program, a, f);
        if ((legal >> a) & 1u) maximum = fmaxf(maximum, scores[a]);
    }
    for (int a = 0; a < 32; ++a)
        if (((legal >> a) & 1u) && maximum - scores[a] <= 1e-6f) return a;
    return 0;
}

static int ctl2_update(ctl2_t* t, uint32_t n, const uint32_t* tours, const orc_ant_info_t* infos, uint32_t A,
                       uint32_t best, const uint32_t* global_tour, int64_t global_cost, int64_t epoch_cost,
                       int from_epoch, uint64_t ls_limit) {
    if (!t->ids) {
        t->ids = (orc_fp_t*)malloc(sizeof(orc_fp_t) * A);
        t->costs = (int64_t*)malloc(sizeof(int64_t) * A);
        if (!t->ids || !t->costs) return -1;
    }
    for (uint32_t a = 0; a < A; ++a) {
        t->ids[a] = t->archive.zero_ids ? (orc_fp_t){0, 0} : orc_fingerprint(tours + (size_t)a * n, n);
        t->costs[a] = infos[a].final_cost;
    }
    const int improved = global_cost < t->tracked_global;
    if (orc_archive_update(&t->archive, global_tour, global_cost, tours, t->costs, A) != 0) return -1;
    double returned = 0, work = 0;
    for (uint32_t a = 0; a < A; ++a) {
        returned += t->ids[a].first == t->active_id.first && t->ids[a].second == t->active_id.second;
        if (ls_limit) work += (double)infos[a].ls.move_evaluations / (double)ls_limit;
    }
    orc_update_feedback(&t->feedback, improved, returned / A, work / A, A);
    if (epoch_cost < t->tracked_epoch) t->epoch_id = t->ids[best];
    t->active_id = from_epoch ? t->epoch_id : t->ids[best];
    t->tracked_global = global_cost;
    t->tracked_epoch = epoch_cost;
    return 0;
}

/* A start node from a start list (the engine's Philox draw of orc_region_start). */
static uint32_t orc_list_start(uint64_t key, uint32_t batch, uint32_t ant, const uint32_t* list, uint32_t count) {
    uint32_t x[4];
    orc_philox4x32(0, ant, batch, 1, (uint32_t)key, (uint32_t)(key >> 32), x);
    return list[((uint64_t)x[0] * count) >> 32];
}

/* ---------------------------------------------------------------------- */
/* A whole colony in engine arithmetic: reset_colony + initialize_products */
/* (colony_state.cuh:72-110), per batch every ant, reduce_and_select      */
/* (:148-208) and the FP32 trail update.                                  */
/* ---------------------------------------------------------------------- */
int orc_run_colony(uint32_t n, const int32_t* xy, const uint32_t* primary, const uint32_t* backup,
                   const uint32_t* ls, const uint32_t* initial, int64_t initial_cost,
                   const orc_run_cfg_t* c, uint64_t key, uint32_t iterations, uint32_t* global_tour,
                   int64_t* global_cost_out, orc_iter_trace_t* trace, float* trails_out,
                   float* products_out, const orc_program_t* program, uint32_t mask,
                   uint32_t total_iterations, uint32_t controller_kind, orc_control_io_t* control) {
    return orc_run_colony_prior(n, xy, primary, backup, ls, initial, initial_cost, c, key, iterations, global_tour,
                                global_cost_out, trace, trails_out, products_out, program, mask, total_iterations,
                                controller_kind, control, NULL);
}

/* The colony run with a learned prior: before batch prior->at[r] the colony */
/* heuristic becomes prior->etas[r] ([n][k]; the instance's eta to fall back */
/* to plain FACO) and the products are recomputed from the current trails,   */
/* by the departure rule when prior->departures[r] is set, which then also   */
/* follows every trail update.  Entries apply in order; NULL: plain FACO.    */
int orc_run_colony_prior(uint32_t n, const int32_t* xy, const uint32_t* primary, const uint32_t* backup,
                         const uint32_t* ls, const uint32_t* initial, int64_t initial_cost,
                         const orc_run_cfg_t* c, uint64_t key, uint32_t iterations, uint32_t* global_tour,
                         int64_t* global_cost_out, orc_iter_trace_t* trace, float* trails_out,
                         float* products_out, const orc_program_t* program, uint32_t mask,
                         uint32_t total_iterations, uint32_t controller_kind, orc_control_io_t* control,
                         const orc_prior_schedule_t* prior) {
    const orc_dist_t d = {n, xy, NULL};
    const uint32_t k = c->k, A = c->ants;
    const size_t cells = (size_t)n * k;
    float* eta = (float*)malloc(sizeof(float) * cells);
    float* ceta = (float*)malloc(sizeof(float) * cells);   /* the colony's heuristic */
    float* trails = (float*)malloc(sizeof(float) * cells);
    float* products = (float*)malloc(sizeof(float) * cells);
    uint32_t* parent = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* epoch = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* tours = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n * A);
    uint32_t* region_list = (uint32_t*)malloc(sizeof(uint32_t) * n);
    orc_ant_info_t* infos = (orc_ant_info_t*)malloc(sizeof(orc_ant_info_t) * A);
    if (!eta || !ceta || !trails || !products || !parent || !epoch || !tours || !infos || !region_list) return -1;
    for (size_t i = 0; i < cells; ++i) {
        const uint32_t to = primary[i];
        const double dist = to < n ? (double)orc_distance(&d, (uint32_t)(i / k), to) : 0.0;
        eta[i] = to >= n ? 0.0f : (float)(dist > 0 ? (c->beta == 1.0 ? 1.0 / dist : 1.0 / pow(dist, c->beta)) : 1.0);
    }
    memcpy(ceta, eta, sizeof(float) * cells);
    uint32_t prior_next = 0, departures = 0;
    uint32_t region_offsets[5] = {0, 0, 0, 0, 0};
    orc_regions(n, xy, region_offsets, region_list);
    const double p_root = pow(c->p_best, 1.0 / (double)k);
    int64_t epoch_cost = initial_cost, global_cost = initial_cost;
    double tmin, tmax;
    orc_trail_limits(k, p_root, c->retention, (double)epoch_cost, &tmin, &tmax);
    float dflt = (float)tmax;
    for (size_t i = 0; i < cells; ++i) { trails[i] = (float)tmax; products[i] = trails[i] * ceta[i]; }
    memcpy(parent, initial, sizeof(uint32_t) * n);
    memcpy(epoch, initial, sizeof(uint32_t) * n);
    memcpy(global_tour, initial, sizeof(uint32_t) * n);
    uint32_t mne = c->mne_target, region = 4, restarts = 0, last_improvement = 0, last_restart = 0;
    const float log2k = orc_log2((float)k);
    int failed = 0;
    /* the reference's 12-feature controller (feature spec 2) */
    const int spec2 = program && program->feature_spec_id == 2;
    ctl2_t ctl;
    memset(&ctl, 0, sizeof(ctl));
    uint32_t start_list[ORC_REGION_CAPACITY], start_count = 0;
    int32_t used_action = -1;
    uint32_t cursor = 0;
    if (spec2 && ctl2_init(&ctl, n, xy, primary, k, initial, initial_cost, control ? control->instance_key : 0,
                           control ? control->force_collisions : 0) != 0)
        return -1;
    for (uint32_t batch = 0; batch < iterations; ++batch) {
        while (prior && prior_next < prior->count && prior->at[prior_next] == batch) {
            memcpy(ceta, prior->etas + (size_t)prior_next * cells, sizeof(float) * cells);
            departures = prior->departures[prior_next];
            for (size_t i = 0; i < cells; ++i) products[i] = trails[i] * ceta[i];
            if (departures) orc_departure_rows(n, k, primary, parent, trails, eta, ceta, products);
            ++prior_next;
        }
        if (spec2) {
            /* decision before the batch (batch_engine.cu:884-950) */
            float f[12 * 32], scores[32];
            uint32_t regions[2 * 4 * ORC_REGION_CAPACITY], alt = ORC_ARCHIVE_CAPACITY;
            ctl2_input(&ctl, n, xy, primary, k, parent, ctl.parent_cost, trails, dflt, (float)tmin, (float)tmax,
                       (double)((uint64_t)batch * A) / (double)((uint64_t)total_iterations * A), key, batch, mask);
            const uint32_t legal = orc_control_features(&ctl.in, f, regions, &alt);
            if (!legal) { failed = 1; break; }
            const int32_t a = ctl2_choose(program, controller_kind, f, legal, scores);
            if (control && cursor < control->count && batch + 1 == control->points[cursor]) {
                memcpy(control->features + (size_t)cursor * 12 * 32, f, sizeof(f));
                memcpy(control->scores + (size_t)cursor * 32, scores, sizeof(scores));
                control->masks[cursor] = legal;
                control->actions[cursor] = a;
                ++cursor;
            }
            used_action = a;
            mne = 2u << (a & 3);
            start_count = n < ORC_REGION_CAPACITY ? n : ORC_REGION_CAPACITY;
            memcpy(start_list, regions + ((uint32_t)a / 16 * 4 + ((uint32_t)a / 4) % 4) * ORC_REGION_CAPACITY,
                   sizeof(start_list));
            if (a >= 16) {
                /* restart from the alternative reference (control_state.cuh:302-336) */
                const orc_archive_t* ar = &ctl.archive;
                epoch_cost = ar->cost[alt];
                ctl.parent_cost = epoch_cost;
                orc_trail_limits(k, p_root, c->retention, (double)epoch_cost, &tmin, &tmax);
                dflt = (float)tmax;
                ctl.tracked_epoch = epoch_cost;
                ctl.active_id = ctl.epoch_id = ar->id[alt];
                orc_restart_feedback(&ctl.feedback);
                memcpy(parent, ar->tours + (size_t)alt * n, sizeof(uint32_t) * n);
                memcpy(epoch, ar->tours + (size_t)alt * n, sizeof(uint32_t) * n);
                for (size_t i = 0; i < cells; ++i) { trails[i] = (float)tmax; products[i] = trails[i] * ceta[i]; }
            }
        }
#ifdef _OPENMP
#pragma omp parallel num_threads(c->threads > 0 ? (int)c->threads : 1)
#endif
        {
            uint32_t* ptour = (uint32_t*)malloc(sizeof(uint32_t) * n);
            uint32_t* ppos = (uint32_t*)malloc(sizeof(uint32_t) * n);
            double* uni = (double*)malloc(sizeof(double) * n);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
            for (int ant = 0; ant < (int)A; ++ant) {
                for (uint32_t s = 1; s < n; ++s) uni[s] = orc_uniform(key, batch, (uint32_t)ant, s);
                const uint32_t start = spec2 ? orc_list_start(key, batch, (uint32_t)ant, start_list, start_count)
                                             : orc_region_start(key, batch, (uint32_t)ant, n, region_offsets,
                                                                region_list, region);
                const orc_choices_t ch = {NULL, uni, start, primary, products, NULL, k, backup, c->b};
                if (orc_ant(parent, &d, ls, c->w, &ch, mne, c->ls_evaluation_limit, c->ls_mode, NULL, ptour, ppos,
                            NULL, NULL, &infos[ant]) != 0)
                    failed = 1;
                memcpy(tours + (size_t)ant * n, ptour, sizeof(uint32_t) * n);
            }
            free(ptour); free(ppos); free(uni);
        }
        uint32_t best = 0;
        uint64_t steps = 0, evals = 0;
        int64_t sum_final = 0, sum_cons = 0;
        for (uint32_t a = 0; a < A; ++a) {
            steps += infos[a].cons.steps; evals += infos[a].ls.move_evaluations;
            sum_final += infos[a].final_cost; sum_cons += infos[a].construction_cost;
            if (infos[a].final_cost < infos[best].final_cost) best = a;
        }
        const int64_t cost = infos[best].final_cost;
        const uint32_t* best_tour = tours + (size_t)best * n;
        if (cost < epoch_cost) { epoch_cost = cost; memcpy(epoch, best_tour, sizeof(uint32_t) * n); }
        if (cost < global_cost) {
            global_cost = cost;
            memcpy(global_tour, best_tour, sizeof(uint32_t) * n);
            last_improvement = batch + 1;
        }
        orc_trail_limits(k, p_root, c->retention, (double)epoch_cost, &tmin, &tmax);
        const int from_epoch = orc_source_uniform(key, batch) < c->epoch_source_probability;
        int64_t parent_cost = from_epoch ? epoch_cost : cost;
        memcpy(parent, from_epoch ? epoch : best_tour, sizeof(uint32_t) * n);
        orc_pheromone32(n, k, primary, parent, (float)c->retention, (float)tmin, (float)tmax,
                        (float)(1.0 / (double)parent_cost), ceta, trails, products, &dflt);
        if (departures) orc_departure_rows(n, k, primary, parent, trails, eta, ceta, products);
        const uint32_t used_mne = mne;
        int32_t action = -1;
        if (spec2) {
            if (ctl2_update(&ctl, n, tours, infos, A, best, global_tour, global_cost, epoch_cost, from_epoch,
                            c->ls_evaluation_limit) != 0) { failed = 1; break; }
            ctl.parent_cost = parent_cost;
            action = used_action;
        } else if (program) {
            uint64_t sumq = 0;
            for (uint32_t row = 0; row < n; ++row) sumq += orc_row_entropy_q(trails + (size_t)row * k, k, log2k);
            const uint32_t t1 = batch + 1, stag = t1 - last_improvement, age = t1 - last_restart;
            float f[7], scores[32];
            f[0] = (float)t1 / (float)total_iterations;
            f[1] = (float)stag / (float)(stag + 16);
            f[2] = clamp01((double)(sum_final - (int64_t)A * cost) / ((double)A * (double)cost));
            f[3] = clamp01((double)sumq * (1.0 / 1048576.0) / (double)n);
            f[4] = (float)restarts / (float)(restarts + 1);
            f[5] = clamp01((double)(sum_cons - sum_final) / (double)sum_cons * 10.0);
            f[6] = (float)age / (float)(age + 16);
            action = controller_kind == 1 ? orc_control_choose_conditional(program, f, mask, scores)
                                          : orc_control_choose(program, f, mask, scores);
            mne = 2u << (action & 3);
            region = ((uint32_t)action >> 2) & 3u;
            if (action >= 16) {
                ++restarts;
                last_restart = t1;
                memcpy(parent, global_tour, sizeof(uint32_t) * n);
                memcpy(epoch, global_tour, sizeof(uint32_t) * n);
                epoch_cost = global_cost;
                parent_cost = global_cost;
                orc_trail_limits(k, p_root, c->retention, (double)epoch_cost, &tmin, &tmax);
                for (size_t i = 0; i < cells; ++i) { trails[i] = (float)tmax; products[i] = trails[i] * ceta[i]; }
                dflt = (float)tmax;
            }
        }
        if (trace) {
            orc_iter_trace_t* r = &trace[batch];
            r->iteration_best_cost = cost; r->global_cost = global_cost; r->parent_cost = parent_cost;
            r->iteration_best = best; r->source_is_epoch = (uint32_t)from_epoch;
            r->tau_min = (float)tmin; r->tau_max = (float)tmax;
            r->mne_target = used_mne; r->action = action;
            r->construction_steps = steps; r->ls_evaluations = evals;
        }
    }
    if (spec2 && control) {
        control->archive_size = ctl.archive.size;
        control->feedback = ctl.feedback;
    }
    if (spec2) ctl2_free(&ctl);
    *global_cost_out = global_cost;
    if (trails_out) memcpy(trails_out, trails, sizeof(float) * cells);
    if (products_out) memcpy(products_out, products, sizeof(float) * cells);
    free(eta); free(ceta); free(trails); free(products); free(parent); free(epoch); free(tours); free(infos); free(region_list);
    return failed ? -2 : 0;
}

/* ---------------------------------------------------------------------- */
/* GP scoring -- apply_operation (cpp/include/gp_faco/program_ops.hpp:13-30)*/
/* and score_cpu (cpp/src/program_cpu.cpp:79-116).  Opcodes 0-8 are the  */
/* reference IR; 9 (protected division) and 10 (if>0, three operands) are  */
/* the extended grammar (numeric_spec_id 2).                               */
/* ---------------------------------------------------------------------- */
float orc_apply_operation(int opcode, float left, float right, float third) {
    float r = 0.0f;
    switch (opcode) {
        case 2: r = left + right; break;
        case 3: r = left - right; break;
        case 4: r = left * right; break;
        case 5: r = fminf(left, right); break;
        case 6: r = fmaxf(left, right); break;
        case 7: r = fabsf(left); break;
        case 8: { const float q = 1.0f + right * right; r = left * (1.0f / sqrtf(q)); break; }
        case 9: r = fabsf(right) < 1e-6f ? 1.0f : left / right; break;
        case 10: r = left > 0.0f ? right : third; break;
        default: break;
    }
    return fminf(8.0f, fmaxf(-8.0f, r));
}

static int arity_of(int op) { return op == 7 ? 1 : op == 10 ? 3 : 2; }

int orc_validate_program(const orc_program_t* p) {
    const int extended = p->numeric_spec_id == 2;
    if (p->ir_version != 1 || (p->numeric_spec_id != 1 && !extended) ||
        (p->feature_spec_id < 1 || p->feature_spec_id > 3) || p->length == 0 || p->length > 63 ||
        p->constants_count > 63)
        return -1;
    for (int i = 0; i < p->constants_count; ++i)
        if (!isfinite(p->constants[i]) || fabsf(p->constants[i]) > 2.0f) return -2;
    int depth[64], top = 0;
    const int max_op = extended ? 10 : 8, max_depth = extended ? 6 : 5, max_stack = extended ? 16 : 6;
    for (int i = 0; i < p->length; ++i) {
        const int op = p->opcode[i], operand = p->operand[i];
        if (op == 0 || op == 1) {
            if ((op == 0 && operand >= 12) || (op == 1 && operand >= p->constants_count)) return -3;
            depth[top++] = 0;
        } else if (op >= 2 && op <= max_op) {
            const int a = arity_of(op);
            if (operand != 0 || top < a) return -4;
            int dmax = 0;
            for (int j = top - a; j < top; ++j) dmax = depth[j] > dmax ? depth[j] : dmax;
            top -= a;
            if (dmax + 1 > max_depth) return -5;
            depth[top++] = dmax + 1;
        } else {
            return -6;
        }
        if (top > max_stack) return -7;
    }
    return top == 1 ? 0 : -8;
}

void orc_score(const orc_program_t* p, uint32_t features_count, const float* features, const uint32_t* masks,
               uint32_t colonies, float* scores, int32_t* actions) {
    (void)features_count;
    for (uint32_t c = 0; c < colonies; ++c) {
        float maximum = -INFINITY;
        for (int action = 0; action < 32; ++action) {
            float stack[16] = {0};
            int top = 0;
            for (int i = 0; i < p->length; ++i) {
                const int op = p->opcode[i];
                if (op == 0) stack[top++] = features[((size_t)p->operand[i] * colonies + c) * 32 + action];
                else if (op == 1) stack[top++] = p->constants[p->operand[i]];
                else {
                    const int a = arity_of(op);
                    const float third = a == 3 ? stack[--top] : 0.0f;
                    const float right = a >= 2 ? stack[--top] : 0.0f;
                    const float left = stack[--top];
                    stack[top++] = orc_apply_operation(op, left, right, third);
                }
            }
            scores[(size_t)c * 32 + action] = stack[0];
            if ((masks[c] >> action) & 1u) maximum = fmaxf(maximum, stack[0]);
        }
        actions[c] = 32;
        for (int action = 0; action < 32; ++action)
            if (((masks[c] >> action) & 1u) && maximum - scores[(size_t)c * 32 + action] <= 1e-6f) {
                actions[c] = action;
                break;
            }
    }
}

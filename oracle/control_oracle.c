/*
 * control_oracle.c -- CPU restatement of the reference's 12-feature colony
 * controller (feature spec 2): tour fingerprints, the reference-tour archive,
 * controller feedback, sampled tour differences, start regions and the
 * 12 x 32 action features.
 *
 * TEST INFRASTRUCTURE ONLY (see faco_oracle.h).  Follows
 * cpp/include/gp_faco/control_ops.hpp:15-214 (hash, fingerprints, canonical
 * order, ControlRandom, sample nodes, regions, feedback, region features),
 * cpp/src/control_cpu.cpp:12-118 (archive update, alternative reference,
 * action snapshot) and cuda/control_state.cuh:124-364 (per-batch order).
 * Lengths are exact EUC_2D integers; every double expression is evaluated in
 * the order the reference writes it.
 */
#include "faco_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* SplitMix64's output function (Steele, Lea, Flood 2014). */
uint64_t orc_ctl_mix(uint64_t v) {
    v += 0x9e3779b97f4a7c15ULL;
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31);
}

/* Fingerprint of one undirected edge: two independently salted mixes of
 * (min << 32 | max).  A tour's fingerprint XORs its n edges. */
orc_fp_t orc_fingerprint_edge(uint32_t a, uint32_t b) {
    const uint64_t lo = a < b ? a : b, hi = a < b ? b : a, edge = (lo << 32) | hi;
    const orc_fp_t f = {orc_ctl_mix(edge ^ 0xb5ad4eceda1ce2a9ULL), orc_ctl_mix(edge ^ 0xd6e8feb86659fd93ULL)};
    return f;
}

orc_fp_t orc_fingerprint(const uint32_t* tour, uint32_t n) {
    orc_fp_t f = {0, 0};
    for (uint32_t i = 0; i < n; ++i) {
        const orc_fp_t e = orc_fingerprint_edge(tour[i], tour[i + 1 == n ? 0 : i + 1]);
        f.first ^= e.first;
        f.second ^= e.second;
    }
    return f;
}

static int fp_equal(orc_fp_t a, orc_fp_t b) { return a.first == b.first && a.second == b.second; }
static int fp_less(orc_fp_t a, orc_fp_t b) { return a.first < b.first || (a.first == b.first && a.second < b.second); }

static uint32_t t_succ(const uint32_t* t, const uint32_t* p, uint32_t n, uint32_t v) {
    return t[p[v] + 1 == n ? 0 : p[v] + 1];
}
static uint32_t t_pred(const uint32_t* t, const uint32_t* p, uint32_t n, uint32_t v) {
    return t[p[v] == 0 ? n - 1 : p[v] - 1];
}
static int t_contains(const uint32_t* t, const uint32_t* p, uint32_t n, uint32_t a, uint32_t b) {
    return t_succ(t, p, n, a) == b || t_pred(t, p, n, a) == b;
}

/* The tours read from city 0 in their canonical direction (towards the
 * smaller neighbour of 0), compared element by element. */
int orc_canonical_compare(const uint32_t* ta, const uint32_t* pa, const uint32_t* tb, const uint32_t* pb,
                          uint32_t n) {
    const int fa = t_succ(ta, pa, n, 0) < t_pred(ta, pa, n, 0);
    const int fb = t_succ(tb, pb, n, 0) < t_pred(tb, pb, n, 0);
    uint32_t ia = pa[0], ib = pb[0];
    for (uint32_t i = 1; i < n; ++i) {
        ia = fa ? (ia + 1 == n ? 0 : ia + 1) : (ia == 0 ? n - 1 : ia - 1);
        ib = fb ? (ib + 1 == n ? 0 : ib + 1) : (ib == 0 ? n - 1 : ib - 1);
        if (ta[ia] != tb[ib]) return ta[ia] < tb[ib] ? -1 : 1;
    }
    return 0;
}

/* ControlRandom::bounded: rejection below (2^64 - bound) mod bound. */
typedef struct { uint64_t key, counter; } ctl_random_t;
static uint32_t ctl_bounded(ctl_random_t* r, uint32_t bound) {
    const uint64_t threshold = (0 - (uint64_t)bound) % bound;
    uint64_t word;
    do { word = orc_ctl_mix(r->key + r->counter++); } while (word < threshold);
    return (uint32_t)(word % bound);
}

/* The rank-th node not in existing[0..count) (count <= 64). */
static uint32_t remaining_node(uint32_t rank, const uint32_t* existing, uint32_t count) {
    uint32_t sorted[ORC_SAMPLE_CAPACITY];
    for (uint32_t i = 0; i < count; ++i) {
        uint32_t j = i;
        while (j && sorted[j - 1] > existing[i]) { sorted[j] = sorted[j - 1]; --j; }
        sorted[j] = existing[i];
    }
    uint32_t node = rank;
    for (uint32_t i = 0; i < count; ++i) if (sorted[i] <= node) ++node;
    return node;
}

void orc_sample_nodes(uint32_t n, uint64_t instance_key, uint32_t* out) {
    const uint32_t count = n < ORC_SAMPLE_CAPACITY ? n : ORC_SAMPLE_CAPACITY;
    ctl_random_t r = {orc_ctl_mix(instance_key ^ 0x6a09e667f3bcc909ULL), 0};
    for (uint32_t i = 0; i < count; ++i) out[i] = remaining_node(ctl_bounded(&r, n - i), out, i);
}

static int has_node(const uint32_t* nodes, uint32_t count, uint32_t v) {
    for (uint32_t i = 0; i < count; ++i) if (nodes[i] == v) return 1;
    return 0;
}

/* Start region (mode, region) of one batch: regions 0 and 1 are 16
 * consecutive nodes of the reference tour from a random position, region 2
 * a breadth-first walk over the primary candidate rows from a random node,
 * region 3 (and any shortfall of 2) uniformly drawn distinct nodes. */
void orc_build_region(const uint32_t* tour, uint32_t n, const uint32_t* primary, uint32_t k, uint64_t key,
                      uint32_t batch, uint32_t mode, uint32_t region, uint32_t* nodes) {
    const uint32_t count = n < ORC_REGION_CAPACITY ? n : ORC_REGION_CAPACITY;
    ctl_random_t r = {orc_ctl_mix(key ^ 0xbb67ae8584caa73bULL ^ orc_ctl_mix((uint64_t)batch ^ 0x3c6ef372fe94f82bULL) ^
                                  orc_ctl_mix((uint64_t)(mode * 4 + region + 1) ^ 0xa54ff53a5f1d36f1ULL)),
                      0};
    uint32_t used = 0;
    if (region < 2) {
        const uint32_t start = ctl_bounded(&r, n);
        for (uint32_t i = 0; i < count; ++i) nodes[i] = tour[(start + i) % n];
        return;
    }
    if (region == 2) {
        nodes[used++] = ctl_bounded(&r, n);
        for (uint32_t head = 0; head < used && used < count; ++head)
            for (uint32_t j = 0; j < k && used < count; ++j) {
                const uint32_t v = primary[(size_t)nodes[head] * k + j];
                if (v < n && !has_node(nodes, used, v)) nodes[used++] = v;
            }
    }
    while (used < count) {
        const uint32_t v = remaining_node(ctl_bounded(&r, n - used), nodes, used);
        nodes[used++] = v;
    }
}

uint32_t orc_sampled_difference(const uint32_t* ct, const uint32_t* cp, const uint32_t* at, const uint32_t* ap,
                                uint32_t n, const uint32_t* samples, uint32_t count) {
    uint32_t missing = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const uint32_t v = samples[i];
        missing += !t_contains(at, ap, n, v, t_succ(ct, cp, n, v));
        missing += !t_contains(at, ap, n, v, t_pred(ct, cp, n, v));
    }
    return missing;
}

static double unit_clip(double v) { return v < 0 ? 0 : v > 1 ? 1 : v; }

void orc_update_feedback(orc_feedback_t* s, int improved, double returned_fraction, double work_fraction,
                         uint32_t ants) {
    if (!ants) return;
    const float returned = (float)unit_clip(returned_fraction);
    const float work = (float)unit_clip(work_fraction);
    s->return_rate += (returned - s->return_rate) * 0.0625f;
    s->ls_work += (work - s->ls_work) * 0.0625f;
    if (improved) s->stagnant_batches = 0;
    else if (s->stagnant_batches != UINT64_MAX) ++s->stagnant_batches;
    if (s->epoch_batches != UINT64_MAX) ++s->epoch_batches;
}

void orc_restart_feedback(orc_feedback_t* s) {
    s->return_rate = s->ls_work = 0;
    s->epoch_batches = 0;
    if (s->restarts != UINT64_MAX) ++s->restarts;
}

/* ---- archive -------------------------------------------------------------- */

typedef struct {
    const uint32_t* tour;
    const uint32_t* pos;
    int64_t cost;
    orc_fp_t id;
    uint32_t order;      /* position in the pool (stable sort key) */
} pool_entry_t;

static int record_less(const pool_entry_t* a, const pool_entry_t* b, uint32_t n) {
    if (a->cost != b->cost) return a->cost < b->cost;
    if (!fp_equal(a->id, b->id)) return fp_less(a->id, b->id);
    return orc_canonical_compare(a->tour, a->pos, b->tour, b->pos, n) < 0;
}

static int duplicate_record(const pool_entry_t* a, const pool_entry_t* b, uint32_t n) {
    return fp_equal(a->id, b->id) && orc_canonical_compare(a->tour, a->pos, b->tour, b->pos, n) == 0;
}

static uint32_t g_sort_n;
static int pool_cmp(const void* x, const void* y) {
    const pool_entry_t* a = (const pool_entry_t*)x;
    const pool_entry_t* b = (const pool_entry_t*)y;
    if (record_less(a, b, g_sort_n)) return -1;
    if (record_less(b, a, g_sort_n)) return 1;
    return a->order < b->order ? -1 : a->order > b->order ? 1 : 0;
}

/* ReferenceArchive::update (control_cpu.cpp:25-44): the global best first,
 * then the best distinct tours of the old archive and the batch within 2 %
 * of the global cost, at most 4.  tours/pos of the candidates [m][n]. */
int orc_archive_update(orc_archive_t* ar, const uint32_t* global_tour, int64_t global_cost,
                       const uint32_t* cand_tours, const int64_t* cand_costs, uint32_t m) {
    const uint32_t n = ar->n;
    const uint32_t total = ar->size + m;
    pool_entry_t* pool = (pool_entry_t*)malloc(sizeof(pool_entry_t) * (total + 1));
    uint32_t* cand_pos = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)m + 1) * n);
    uint32_t* gpos = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint32_t* new_tours = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)ORC_ARCHIVE_CAPACITY * n);
    uint32_t* new_pos = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)ORC_ARCHIVE_CAPACITY * n);
    if (!pool || !cand_pos || !gpos || !new_tours || !new_pos) return -1;
    for (uint32_t i = 0; i < n; ++i) gpos[global_tour[i]] = i;
    uint32_t count = 0;
    for (uint32_t i = 0; i < ar->size; ++i, ++count) {
        pool_entry_t e = {ar->tours + (size_t)i * n, ar->pos + (size_t)i * n, ar->cost[i], ar->id[i], count};
        pool[count] = e;
    }
    for (uint32_t a = 0; a < m; ++a, ++count) {
        const uint32_t* t = cand_tours + (size_t)a * n;
        uint32_t* p = cand_pos + (size_t)a * n;
        for (uint32_t i = 0; i < n; ++i) p[t[i]] = i;
        const orc_fp_t zero = {0, 0};
        pool_entry_t e = {t, p, cand_costs[a], ar->zero_ids ? zero : orc_fingerprint(t, n), count};
        pool[count] = e;
    }
    g_sort_n = n;
    qsort(pool, total, sizeof(pool_entry_t), pool_cmp);
    pool_entry_t chosen[ORC_ARCHIVE_CAPACITY];
    const orc_fp_t zero_id = {0, 0};
    const pool_entry_t g = {global_tour, gpos, global_cost,
                            ar->zero_ids ? zero_id : orc_fingerprint(global_tour, n), 0};
    chosen[0] = g;
    uint32_t used = 1;
    const double limit = (double)global_cost * (1 + ORC_ARCHIVE_BAND);
    for (uint32_t i = 0; i < total && used < ORC_ARCHIVE_CAPACITY; ++i) {
        if ((double)pool[i].cost > limit) continue;
        int dup = 0;
        for (uint32_t j = 0; j < used && !dup; ++j) dup = duplicate_record(&pool[i], &chosen[j], n);
        if (dup) continue;
        chosen[used++] = pool[i];
    }
    for (uint32_t s = 0; s < used; ++s) {
        memcpy(new_tours + (size_t)s * n, chosen[s].tour, sizeof(uint32_t) * n);
        memcpy(new_pos + (size_t)s * n, chosen[s].pos, sizeof(uint32_t) * n);
    }
    for (uint32_t s = 0; s < ORC_ARCHIVE_CAPACITY; ++s) {
        ar->cost[s] = s < used ? chosen[s].cost : 0;
        const orc_fp_t zero = {0, 0};
        ar->id[s] = s < used ? chosen[s].id : zero;
    }
    memcpy(ar->tours, new_tours, sizeof(uint32_t) * (size_t)used * n);
    memcpy(ar->pos, new_pos, sizeof(uint32_t) * (size_t)used * n);
    ar->size = used;
    free(pool); free(cand_pos); free(gpos); free(new_tours); free(new_pos);
    return 0;
}

/* ReferenceArchive::alternative (control_cpu.cpp:46-63): the archive entry,
 * other than the active tour, that differs most from it on the sampled
 * nodes; ties by cost, fingerprint, canonical order.  4 when none. */
uint32_t orc_archive_alternative(const orc_archive_t* ar, const uint32_t* at, const uint32_t* ap, orc_fp_t active_id,
                                 const uint32_t* samples, uint32_t sample_count) {
    const uint32_t n = ar->n;
    uint32_t selected = ORC_ARCHIVE_CAPACITY, largest = 0;
    for (uint32_t i = 0; i < ar->size; ++i) {
        const uint32_t* ct = ar->tours + (size_t)i * n;
        const uint32_t* cp = ar->pos + (size_t)i * n;
        if (fp_equal(ar->id[i], active_id) && orc_canonical_compare(ct, cp, at, ap, n) == 0) continue;
        const uint32_t diff = orc_sampled_difference(ct, cp, at, ap, n, samples, sample_count);
        int better_tie = 0;
        if (selected != ORC_ARCHIVE_CAPACITY && diff == largest) {
            const pool_entry_t a = {ct, cp, ar->cost[i], ar->id[i], 0};
            const pool_entry_t b = {ar->tours + (size_t)selected * n, ar->pos + (size_t)selected * n,
                                    ar->cost[selected], ar->id[selected], 0};
            better_tie = record_less(&a, &b, n);
        }
        if (selected == ORC_ARCHIVE_CAPACITY || diff > largest || better_tie) { selected = i; largest = diff; }
    }
    return selected;
}

/* ---- features ------------------------------------------------------------- */

static double trail_lookup(const orc_control_in_t* in, uint32_t a, uint32_t b) {
    for (uint32_t j = 0; j < in->k; ++j)
        if (in->primary[(size_t)a * in->k + j] == b) return in->trails[(size_t)a * in->k + j];
    return in->default_trail;
}

/* region_features (control_ops.hpp:192-214) of one region around the
 * reference tour (rt, rp). */
static void region_features(const orc_control_in_t* in, const uint32_t* rt, const uint32_t* rp,
                            const uint32_t* nodes, uint32_t count, float out[4]) {
    const orc_dist_t d = {in->n, in->xy, NULL};
    const orc_archive_t* ar = in->archive;
    const uint32_t n = in->n;
    double excess = 0, disagreement = 0, strength = 0, dispersion = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const uint32_t v = nodes[i], prev = t_pred(rt, rp, n, v), next = t_succ(rt, rp, n, v);
        const double scale = in->local_scale[v] < in->epsilon ? in->epsilon : in->local_scale[v];
        excess += unit_clip(((0.5 * (double)orc_distance(&d, v, prev) + 0.5 * (double)orc_distance(&d, v, next)) /
                             scale - 1) / 3);
        const uint32_t nb[2] = {prev, next};
        for (int s = 0; s < 2; ++s) {
            for (uint32_t j = 0; j < ar->size; ++j)
                disagreement += !t_contains(ar->tours + (size_t)j * n, ar->pos + (size_t)j * n, n, v, nb[s]);
            strength += in->tau_min == in->tau_max ? 1
                        : unit_clip((trail_lookup(in, v, nb[s]) - in->tau_min) / (in->tau_max - in->tau_min));
            dispersion += !has_node(nodes, count, nb[s]);
        }
    }
    out[0] = (float)(excess / count);
    out[1] = (float)(disagreement / (2 * count * ar->size));
    out[2] = (float)(strength / (2 * count));
    out[3] = (float)(dispersion / (2 * count));
}

/* make_action_snapshot (control_cpu.cpp:72-118): the 12 features of each
 * of the 32 actions (features[f * 32 + a]), the start regions, the
 * alternative archive entry and the legal mask.  Returns the mask (0 when no
 * action is legal). */
uint32_t orc_control_features(const orc_control_in_t* in, float* features, uint32_t* regions,
                              uint32_t* alternative) {
    const orc_archive_t* ar = in->archive;
    const uint32_t n = in->n;
    const uint32_t alt = orc_archive_alternative(ar, in->active_tour, in->active_pos, in->active_id, in->samples,
                                                 in->sample_count);
    *alternative = alt;
    const int has_alt = alt < ORC_ARCHIVE_CAPACITY;
    const uint32_t mask = in->experiment_mask & (has_alt ? 0xFFFFFFFFu : 0xFFFFu);
    const uint32_t count = n < ORC_REGION_CAPACITY ? n : ORC_REGION_CAPACITY;
    memset(regions, 0, sizeof(uint32_t) * 2 * 4 * ORC_REGION_CAPACITY);
    for (uint32_t mode = 0; mode < 2; ++mode) {
        const uint32_t* rt = NULL;
        const uint32_t* rp = NULL;
        int64_t rcost = 0;
        if (mode == 0) { rt = in->active_tour; rp = in->active_pos; rcost = in->active_cost; }
        else if (has_alt) { rt = ar->tours + (size_t)alt * n; rp = ar->pos + (size_t)alt * n; rcost = ar->cost[alt]; }
        float gap = 0, difference = 0;
        if (rt) {
            gap = (float)unit_clip(((double)rcost / (double)ar->cost[0] - 1) / ORC_ARCHIVE_BAND);
            if (mode)
                difference = (float)orc_sampled_difference(rt, rp, in->active_tour, in->active_pos, n, in->samples,
                                                           in->sample_count) /
                             (float)(2 * in->sample_count);
        }
        for (uint32_t region = 0; region < 4; ++region) {
            float regional[4] = {0, 0, 0, 0};
            uint32_t* nodes = regions + (mode * 4 + region) * ORC_REGION_CAPACITY;
            if (rt) {
                orc_build_region(rt, n, in->primary, in->k, in->solve_key, in->batch, mode, region, nodes);
                region_features(in, rt, rp, nodes, count, regional);
            }
            for (uint32_t level = 0; level < 4; ++level) {
                const uint32_t a = mode * 16 + region * 4 + level;
                const uint64_t stag = in->feedback.stagnant_batches;
                const float v[12] = {(float)unit_clip(in->elapsed_ratio),
                                     (float)(stag < 32 ? (double)stag / 32.0 : 1), in->feedback.return_rate,
                                     in->feedback.ls_work, (float)mode, (float)(level + 1) * 0.25f, gap, difference,
                                     regional[0], regional[1], regional[2], regional[3]};
                for (int f = 0; f < 12; ++f) features[f * 32 + a] = v[f];
            }
        }
    }
    return mask;
}

void orc_local_scale(uint32_t n, const int32_t* xy, double* scale, double* epsilon) {
    const orc_dist_t d = {n, xy, NULL};
    const uint32_t w = n - 1 < 8 ? n - 1 : 8;
    int64_t minx = xy[0], maxx = xy[0], miny = xy[1], maxy = xy[1];
    for (uint32_t i = 0; i < n; ++i) {
        minx = xy[2 * i] < minx ? xy[2 * i] : minx; maxx = xy[2 * i] > maxx ? xy[2 * i] : maxx;
        miny = xy[2 * i + 1] < miny ? xy[2 * i + 1] : miny; maxy = xy[2 * i + 1] > maxy ? xy[2 * i + 1] : maxy;
    }
    double span = (double)(maxx - minx);
    if ((double)(maxy - miny) > span) span = (double)(maxy - miny);
    if (1.0 > span) span = 1.0;
    *epsilon = 1e-12 * span;
    int32_t best[8];
    for (uint32_t a = 0; a < n; ++a) {
        uint32_t have = 0;
        for (uint32_t b = 0; b < n; ++b) {
            if (b == a) continue;
            const int32_t v = orc_distance(&d, a, b);
            if (have < w) {
                uint32_t j = have++;
                while (j && best[j - 1] > v) { best[j] = best[j - 1]; --j; }
                best[j] = v;
            } else if (v < best[w - 1]) {
                uint32_t j = w - 1;
                while (j && best[j - 1] > v) { best[j] = best[j - 1]; --j; }
                best[j] = v;
            }
        }
        double s = 0;
        for (uint32_t j = 0; j < w; ++j) s += (double)best[j] / w;
        scale[a] = s;
    }
}

// faco_prepare.cpp -- host part of instance registration.
//
// Follows prepare_problem (cpp/src/prepared_problem.cpp:107-175) with TSPLIB
// EUC_2D integer lengths: per node the nearest candidates by (distance,
// node id) -- primary row, backup row, LS row -- and a nearest-neighbour tour
// from node 0.  The initial checklist 2-opt over that tour runs on the GPU
// with the engine's own local-search kernel (faco_engine.cu).
#include "faco_host.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <thread>
#include <vector>

namespace faco {

std::int32_t host_euc2d(std::int64_t x0, std::int64_t y0, std::int64_t x1, std::int64_t y1) {
    const std::int64_t dx = x0 - x1, dy = y0 - y1;
    return static_cast<std::int32_t>(std::floor(std::sqrt(static_cast<double>(dx * dx + dy * dy)) + 0.5));
}

// The engine's log2 (same single-rounding FP32 steps as the device's): the
// exponent plus (2/ln 2) atanh((m-1)/(m+1)) as a 4-term series.
float host_log2(float x) {
    std::uint32_t bits;
    std::memcpy(&bits, &x, 4);
    int e = static_cast<int>((bits >> 23) & 255u) - 127;
    const std::uint32_t mb = (bits & 0x7FFFFFu) | 0x3F800000u;
    float m;
    std::memcpy(&m, &mb, 4);
    if (m > 0x1.6a09e6p+0f) { m = m * 0.5f; e += 1; }
    const float t = (m - 1.0f) / (m + 1.0f), t2 = t * t;
    const float s = t * (1.0f + t2 * (0x1.555556p-2f + t2 * (0x1.99999ap-3f + t2 * 0x1.24924ap-3f)));
    return static_cast<float>(e) + s * 0x1.715476p+1f;
}

// Nodes grouped by quadrant around the bounding-box centre (start regions of
// the controller's actions); offsets[r]..offsets[r+1] index `list`.
void host_regions(const std::vector<std::int32_t>& xy, std::uint32_t n, std::uint32_t offsets[5],
                  std::vector<std::uint16_t>& list) {
    std::int64_t minx = xy[0], maxx = xy[0], miny = xy[1], maxy = xy[1];
    for (std::uint32_t i = 0; i < n; ++i) {
        minx = std::min<std::int64_t>(minx, xy[2 * i]); maxx = std::max<std::int64_t>(maxx, xy[2 * i]);
        miny = std::min<std::int64_t>(miny, xy[2 * i + 1]); maxy = std::max<std::int64_t>(maxy, xy[2 * i + 1]);
    }
    auto quadrant = [&](std::uint32_t i) {
        return (2 * static_cast<std::int64_t>(xy[2 * i]) >= minx + maxx ? 1u : 0u) +
               (2 * static_cast<std::int64_t>(xy[2 * i + 1]) >= miny + maxy ? 2u : 0u);
    };
    std::uint32_t count[4] = {0, 0, 0, 0};
    for (std::uint32_t i = 0; i < n; ++i) ++count[quadrant(i)];
    offsets[0] = 0;
    for (int r = 0; r < 4; ++r) offsets[r + 1] = offsets[r] + count[r];
    std::uint32_t fill[4] = {offsets[0], offsets[1], offsets[2], offsets[3]};
    list.assign(n, 0);
    for (std::uint32_t i = 0; i < n; ++i) list[fill[quadrant(i)]++] = static_cast<std::uint16_t>(i);
}

std::int64_t host_tour_length(const std::vector<std::int32_t>& xy, const std::uint32_t* order, std::uint32_t n) {
    std::int64_t sum = 0;
    std::uint32_t prev = order[n - 1];
    for (std::uint32_t i = 0; i < n; ++i) {
        const std::uint32_t v = order[i];
        sum += host_euc2d(xy[2 * prev], xy[2 * prev + 1], xy[2 * v], xy[2 * v + 1]);
        prev = v;
    }
    return sum;
}

void host_candidates(const std::vector<std::int32_t>& xy, std::uint32_t n, std::uint32_t k, std::uint32_t b,
                     std::uint32_t w, std::vector<std::uint16_t>& primary, std::vector<std::uint16_t>& backup,
                     std::vector<std::uint16_t>& ls, std::vector<std::int32_t>& ls_dist, std::vector<float>& eta,
                     double beta) {
    primary.assign(static_cast<std::size_t>(n) * k, 0);
    backup.assign(static_cast<std::size_t>(n) * b, 0);
    ls.assign(static_cast<std::size_t>(n) * w, 0);
    ls_dist.assign(static_cast<std::size_t>(n) * w, 0);
    eta.assign(static_cast<std::size_t>(n) * k, 0.0f);
    const std::uint32_t needed = std::max(k + b, w);
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const unsigned threads = n >= 2000 ? hw : 1;
    auto work = [&](unsigned t) {
        std::vector<std::pair<std::int32_t, std::uint32_t>> row;
        row.reserve(n);
        for (std::uint32_t a = t; a < n; a += threads) {
            row.clear();
            for (std::uint32_t v = 0; v < n; ++v)
                if (v != a) row.emplace_back(host_euc2d(xy[2 * a], xy[2 * a + 1], xy[2 * v], xy[2 * v + 1]), v);
            std::partial_sort(row.begin(), row.begin() + needed, row.end());
            for (std::uint32_t j = 0; j < k; ++j) {
                primary[static_cast<std::size_t>(a) * k + j] = static_cast<std::uint16_t>(row[j].second);
                const double d = row[j].first;
                eta[static_cast<std::size_t>(a) * k + j] =
                    static_cast<float>(d > 0 ? (beta == 1.0 ? 1.0 / d : 1.0 / std::pow(d, beta)) : 1.0);
            }
            for (std::uint32_t j = 0; j < b; ++j)
                backup[static_cast<std::size_t>(a) * b + j] = static_cast<std::uint16_t>(row[k + j].second);
            for (std::uint32_t j = 0; j < w; ++j) {
                ls[static_cast<std::size_t>(a) * w + j] = static_cast<std::uint16_t>(row[j].second);
                ls_dist[static_cast<std::size_t>(a) * w + j] = row[j].first;
            }
        }
    };
    if (threads == 1) {
        work(0);
    } else {
        std::vector<std::thread> pool;
        for (unsigned t = 0; t < threads; ++t) pool.emplace_back(work, t);
        for (auto& th : pool) th.join();
    }
}

std::vector<std::uint32_t> host_nearest_neighbour_tour(const std::vector<std::int32_t>& xy, std::uint32_t n) {
    std::vector<std::uint32_t> tour;
    tour.reserve(n);
    std::vector<std::uint8_t> seen(n, 0);
    std::uint32_t current = 0;
    for (std::uint32_t i = 0; i < n; ++i) {
        tour.push_back(current);
        seen[current] = 1;
        std::uint32_t next = n;
        std::int32_t shortest = INT32_MAX;
        for (std::uint32_t v = 0; v < n; ++v) {
            if (seen[v]) continue;
            const std::int32_t d = host_euc2d(xy[2 * current], xy[2 * current + 1], xy[2 * v], xy[2 * v + 1]);
            if (d < shortest) { shortest = d; next = v; }
        }
        current = next;
    }
    return tour;
}

// The rows of host_candidates, taken from each node's near list sorted by
// (length, id): primary = the first k, backup = the next b, LS = the first w.
void host_rows_from_near(const std::vector<std::uint16_t>& near, const std::vector<std::int32_t>& near_dist,
                         std::uint32_t n, std::uint32_t needed, std::uint32_t k, std::uint32_t b, std::uint32_t w,
                         double beta, std::vector<std::uint16_t>& primary, std::vector<std::uint16_t>& backup,
                         std::vector<std::uint16_t>& ls, std::vector<std::int32_t>& ls_dist, std::vector<float>& eta) {
    if (k + b > needed || w > needed) throw std::invalid_argument("near lists shorter than the rows");
    primary.assign(static_cast<std::size_t>(n) * k, 0);
    backup.assign(static_cast<std::size_t>(n) * b, 0);
    ls.assign(static_cast<std::size_t>(n) * w, 0);
    ls_dist.assign(static_cast<std::size_t>(n) * w, 0);
    eta.assign(static_cast<std::size_t>(n) * k, 0.0f);
    for (std::uint32_t a = 0; a < n; ++a) {
        const std::size_t row = static_cast<std::size_t>(a) * needed;
        for (std::uint32_t j = 0; j < k; ++j) {
            primary[static_cast<std::size_t>(a) * k + j] = near[row + j];
            const double d = near_dist[row + j];
            eta[static_cast<std::size_t>(a) * k + j] =
                static_cast<float>(d > 0 ? (beta == 1.0 ? 1.0 / d : 1.0 / std::pow(d, beta)) : 1.0);
        }
        for (std::uint32_t j = 0; j < b; ++j) backup[static_cast<std::size_t>(a) * b + j] = near[row + k + j];
        for (std::uint32_t j = 0; j < w; ++j) {
            ls[static_cast<std::size_t>(a) * w + j] = near[row + j];
            ls_dist[static_cast<std::size_t>(a) * w + j] = near_dist[row + j];
        }
    }
}

// The first unvisited node of the current node's near list is the nearest
// unvisited node with the lowest id among equals (every node outside the list
// has a larger (length, id) key than every listed one), which is the choice
// of the full scan in host_nearest_neighbour_tour.
std::vector<std::uint32_t> host_nearest_neighbour_tour_near(const std::vector<std::int32_t>& xy, std::uint32_t n,
                                                            const std::vector<std::uint16_t>& near,
                                                            std::uint32_t needed) {
    std::vector<std::uint32_t> tour;
    tour.reserve(n);
    std::vector<std::uint8_t> seen(n, 0);
    std::uint32_t current = 0;
    for (std::uint32_t i = 0; i < n; ++i) {
        tour.push_back(current);
        seen[current] = 1;
        if (i + 1 == n) break;
        std::uint32_t next = n;
        const std::uint16_t* list = near.data() + static_cast<std::size_t>(current) * needed;
        for (std::uint32_t j = 0; j < needed; ++j)
            if (!seen[list[j]]) { next = list[j]; break; }
        if (next == n) {
            std::int32_t shortest = INT32_MAX;
            for (std::uint32_t v = 0; v < n; ++v) {
                if (seen[v]) continue;
                const std::int32_t d = host_euc2d(xy[2 * current], xy[2 * current + 1], xy[2 * v], xy[2 * v + 1]);
                if (d < shortest) { shortest = d; next = v; }
            }
        }
        current = next;
    }
    return tour;
}

// DistanceOrderedCandidates (cpp/src/faco_cpu.cpp:32-45): stable sort of a
// given row by distance, keeping the input order of ties.
void host_distance_order(const std::vector<std::int32_t>& xy, std::uint32_t n, std::uint32_t w,
                         const std::uint32_t* rows, std::vector<std::uint16_t>& ls,
                         std::vector<std::int32_t>& ls_dist) {
    ls.assign(static_cast<std::size_t>(n) * w, 0);
    ls_dist.assign(static_cast<std::size_t>(n) * w, 0);
    std::vector<std::pair<std::int32_t, std::uint32_t>> row(w);
    for (std::uint32_t a = 0; a < n; ++a) {
        for (std::uint32_t j = 0; j < w; ++j) {
            const std::uint32_t v = rows[static_cast<std::size_t>(a) * w + j];
            if (v >= n || v == a) throw std::invalid_argument("LS candidate out of range or self loop");
            row[j] = {host_euc2d(xy[2 * a], xy[2 * a + 1], xy[2 * v], xy[2 * v + 1]), v};
        }
        std::stable_sort(row.begin(), row.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
        for (std::uint32_t j = 0; j < w; ++j) {
            ls[static_cast<std::size_t>(a) * w + j] = static_cast<std::uint16_t>(row[j].second);
            ls_dist[static_cast<std::size_t>(a) * w + j] = row[j].first;
        }
    }
}

}  // namespace faco

namespace faco {

// Alpha-nearness of every primary candidate entry (Helsgaun, "An effective
// implementation of the Lin-Kernighan traveling salesman heuristic", EJOR
// 126 (2000), after Held and Karp's 1-trees): alpha(i, j) = d(i, j) -
// beta(i, j), beta the longest edge on the path between i and j in a minimum
// spanning tree -- the smallest bottleneck of any path between them, so the
// same for every minimum tree.  The tree here spans the candidate graph (the
// union of the primary, backup and LS rows, undirected); where that graph
// has several components, entries whose ends lie in different components
// get alpha = d(i, j).  Kruskal's algorithm over the edges sorted by (length,
// ends), then path maxima by binary lifting from a root per component.
void host_alpha(const std::vector<std::int32_t>& xy, std::uint32_t n, std::uint32_t k,
                const std::vector<std::uint16_t>& primary, std::uint32_t b, const std::vector<std::uint16_t>& backup,
                std::uint32_t w, const std::vector<std::uint16_t>& ls, std::vector<float>& alpha) {
    struct Edge { std::int32_t d; std::uint32_t a, c; };
    std::vector<Edge> edges;
    edges.reserve(static_cast<std::size_t>(n) * (k + b + w));
    auto dist = [&](std::uint32_t i, std::uint32_t j) {
        return host_euc2d(xy[2 * i], xy[2 * i + 1], xy[2 * j], xy[2 * j + 1]);
    };
    auto add_rows = [&](const std::vector<std::uint16_t>& rows, std::uint32_t width) {
        for (std::uint32_t i = 0; i < n; ++i)
            for (std::uint32_t r = 0; r < width; ++r) {
                const std::uint32_t j = rows[static_cast<std::size_t>(i) * width + r];
                if (j < n && j != i) edges.push_back({dist(i, j), std::min(i, j), std::max(i, j)});
            }
    };
    add_rows(primary, k);
    add_rows(backup, b);
    add_rows(ls, w);
    std::sort(edges.begin(), edges.end(), [](const Edge& x, const Edge& y) {
        return x.d != y.d ? x.d < y.d : x.a != y.a ? x.a < y.a : x.c < y.c;
    });
    std::vector<std::uint32_t> root(n);
    for (std::uint32_t i = 0; i < n; ++i) root[i] = i;
    auto find = [&](std::uint32_t v) {
        while (root[v] != v) v = root[v] = root[root[v]];
        return v;
    };
    std::vector<std::vector<std::pair<std::uint32_t, std::int32_t>>> tree(n);
    for (const Edge& e : edges) {
        const std::uint32_t ra = find(e.a), rc = find(e.c);
        if (ra == rc) continue;
        root[ra] = rc;
        tree[e.a].push_back({e.c, e.d});
        tree[e.c].push_back({e.a, e.d});
    }
    // roots, depths and the lifting tables (ancestor, longest edge to it)
    std::uint32_t levels = 1;
    while ((1u << levels) < n) ++levels;
    std::vector<std::uint32_t> up(static_cast<std::size_t>(levels) * n), comp(n, n), depth(n, 0);
    std::vector<std::int32_t> best(static_cast<std::size_t>(levels) * n, 0);
    std::vector<std::uint32_t> queue;
    queue.reserve(n);
    for (std::uint32_t s = 0; s < n; ++s) {
        if (comp[s] != n) continue;
        comp[s] = s;
        up[s] = s;
        best[s] = 0;
        queue.assign(1, s);
        for (std::size_t h = 0; h < queue.size(); ++h) {
            const std::uint32_t v = queue[h];
            for (const auto& [u, d] : tree[v]) {
                if (comp[u] != n) continue;
                comp[u] = s;
                depth[u] = depth[v] + 1;
                up[u] = v;
                best[u] = d;
                queue.push_back(u);
            }
        }
    }
    for (std::uint32_t l = 1; l < levels; ++l)
        for (std::uint32_t v = 0; v < n; ++v) {
            const std::uint32_t mid = up[static_cast<std::size_t>(l - 1) * n + v];
            up[static_cast<std::size_t>(l) * n + v] = up[static_cast<std::size_t>(l - 1) * n + mid];
            best[static_cast<std::size_t>(l) * n + v] =
                std::max(best[static_cast<std::size_t>(l - 1) * n + v], best[static_cast<std::size_t>(l - 1) * n + mid]);
        }
    auto path_max = [&](std::uint32_t a, std::uint32_t c) {
        std::int32_t m = 0;
        if (depth[a] < depth[c]) std::swap(a, c);
        for (std::uint32_t l = levels; l-- > 0;)
            if (depth[a] - depth[c] >= (1u << l)) {
                m = std::max(m, best[static_cast<std::size_t>(l) * n + a]);
                a = up[static_cast<std::size_t>(l) * n + a];
            }
        if (a == c) return m;
        for (std::uint32_t l = levels; l-- > 0;) {
            const std::uint32_t ua = up[static_cast<std::size_t>(l) * n + a], uc = up[static_cast<std::size_t>(l) * n + c];
            if (ua != uc) {
                m = std::max({m, best[static_cast<std::size_t>(l) * n + a], best[static_cast<std::size_t>(l) * n + c]});
                a = ua;
                c = uc;
            }
        }
        return std::max({m, best[a], best[c]});
    };
    alpha.assign(static_cast<std::size_t>(n) * k, 0.0f);
    for (std::uint32_t i = 0; i < n; ++i)
        for (std::uint32_t r = 0; r < k; ++r) {
            const std::uint32_t j = primary[static_cast<std::size_t>(i) * k + r];
            if (j >= n) continue;
            const std::int32_t d = dist(i, j);
            alpha[static_cast<std::size_t>(i) * k + r] =
                static_cast<float>(comp[i] == comp[j] ? d - path_max(i, j) : d);
        }
}

}  // namespace faco

// faco_host.h -- host-side helpers of the engine (no CUDA types).
#pragma once

#include <cstdint>
#include <vector>

namespace faco {

float host_log2(float x);
void host_regions(const std::vector<std::int32_t>& xy, std::uint32_t n, std::uint32_t offsets[5],
                  std::vector<std::uint16_t>& list);
std::int32_t host_euc2d(std::int64_t x0, std::int64_t y0, std::int64_t x1, std::int64_t y1);
std::int64_t host_tour_length(const std::vector<std::int32_t>& xy, const std::uint32_t* order, std::uint32_t n);
void host_candidates(const std::vector<std::int32_t>& xy, std::uint32_t n, std::uint32_t k, std::uint32_t b,
                     std::uint32_t w, std::vector<std::uint16_t>& primary, std::vector<std::uint16_t>& backup,
                     std::vector<std::uint16_t>& ls, std::vector<std::int32_t>& ls_dist, std::vector<float>& eta,
                     double beta);
std::vector<std::uint32_t> host_nearest_neighbour_tour(const std::vector<std::int32_t>& xy, std::uint32_t n);
// Rows and eta from sorted near lists ([n][needed] ids and lengths).
void host_rows_from_near(const std::vector<std::uint16_t>& near, const std::vector<std::int32_t>& near_dist,
                         std::uint32_t n, std::uint32_t needed, std::uint32_t k, std::uint32_t b, std::uint32_t w,
                         double beta, std::vector<std::uint16_t>& primary, std::vector<std::uint16_t>& backup,
                         std::vector<std::uint16_t>& ls, std::vector<std::int32_t>& ls_dist, std::vector<float>& eta);
// The nearest-neighbour tour using the near lists; a full scan only when
// every listed node is already visited.
std::vector<std::uint32_t> host_nearest_neighbour_tour_near(const std::vector<std::int32_t>& xy, std::uint32_t n,
                                                            const std::vector<std::uint16_t>& near,
                                                            std::uint32_t needed);
// Alpha-nearness (length minus the longest edge on the minimum spanning
// tree path between the ends) of every primary candidate entry, [n][k].
void host_alpha(const std::vector<std::int32_t>& xy, std::uint32_t n, std::uint32_t k,
                const std::vector<std::uint16_t>& primary, std::uint32_t b, const std::vector<std::uint16_t>& backup,
                std::uint32_t w, const std::vector<std::uint16_t>& ls, std::vector<float>& alpha);
void host_distance_order(const std::vector<std::int32_t>& xy, std::uint32_t n, std::uint32_t w,
                         const std::uint32_t* rows, std::vector<std::uint16_t>& ls,
                         std::vector<std::int32_t>& ls_dist);

}  // namespace faco

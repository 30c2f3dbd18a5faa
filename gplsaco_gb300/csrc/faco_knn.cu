// faco_knn.cu -- candidate rows of instance registration on the GPU.
//
// prepare_problem (cpp/src/prepared_problem.cpp:58-91) sorts, per node, all
// other nodes by distance and keeps the first k + b (primary and backup
// rows) and the first w (LS row).  Here one block per node computes every
// EUC_2D length as a 64-bit key (length << 16 | node id, so that ties order
// by id as the reference's partial_sort of (distance, id) pairs does), finds
// the `needed`-th smallest key with a radix select over 8-bit digits
// (warp-aggregated shared-memory histograms), gathers the keys up to it and
// sorts them with a bitonic network.  The result is each node's `needed`
// nearest nodes in (distance, id) order with their lengths.
#include <cuda_runtime.h>

#include <cstdint>

#include "faco_common.cuh"
#include "faco_kernels.h"

namespace faco {
namespace {

constexpr std::uint32_t kKnnThreads = 512;
constexpr unsigned long long kNoKey = ~0ull;

__global__ void __launch_bounds__(kKnnThreads) knn_kernel(const int2* __restrict__ xy, std::uint32_t n,
                                                          std::uint32_t needed, node_t* __restrict__ near_ids,
                                                          std::int32_t* __restrict__ near_dist) {
    extern __shared__ unsigned long long keys[];               // [n]
    __shared__ unsigned hist[256];
    __shared__ unsigned long long picked[kKnnMaxNeeded];
    __shared__ unsigned s_digit, s_rank, s_count;
    const std::uint32_t a = blockIdx.x, tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const int2 pa = xy[a];
    for (std::uint32_t j = tid; j < n; j += kKnnThreads)
        keys[j] = j == a ? kNoKey : ((unsigned long long)euc2d(pa, xy[j]) << 16) | j;
    // radix select of the key of rank needed - 1 (lengths < 2^28, so keys < 2^44)
    unsigned long long prefix = 0, mask = 0;
    unsigned rank = needed - 1;
    for (int shift = 40; shift >= 0; shift -= 8) {
        for (std::uint32_t i = tid; i < 256; i += kKnnThreads) hist[i] = 0;
        __syncthreads();
        for (std::uint32_t base = 0; base < n; base += kKnnThreads) {
            const std::uint32_t j = base + tid;
            const unsigned long long key = j < n ? keys[j] : kNoKey;
            const bool counted = j < n && (key & mask) == prefix;
            const unsigned digit = counted ? (unsigned)(key >> shift) & 255u : 256u;
            const unsigned peers = __match_any_sync(0xffffffffu, digit);
            if (counted && (__ffs(peers) - 1) == (int)lane) atomicAdd(&hist[digit], (unsigned)__popc(peers));
        }
        __syncthreads();
        if (warp == 0) {
            unsigned sum = 0;
#pragma unroll
            for (int t = 0; t < 8; ++t) sum += hist[lane * 8 + t];
            unsigned incl = sum;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const unsigned v = __shfl_up_sync(0xffffffffu, incl, off);
                if ((int)lane >= off) incl += v;
            }
            const unsigned excl = incl - sum;
            if (excl <= rank && rank < incl) {
                unsigned c = excl;
                for (int t = 0; t < 8; ++t) {
                    const unsigned h = hist[lane * 8 + t];
                    if (rank < c + h) {
                        s_digit = lane * 8 + t;
                        s_rank = rank - c;
                        break;
                    }
                    c += h;
                }
            }
        }
        __syncthreads();
        prefix |= (unsigned long long)s_digit << shift;
        mask |= 255ull << shift;
        rank = s_rank;
        __syncthreads();
    }
    // prefix is now the exact key of rank needed - 1 (keys are distinct)
    if (tid == 0) s_count = 0;
    std::uint32_t width = 1;
    while (width < needed) width <<= 1;
    for (std::uint32_t i = needed + tid; i < width; i += kKnnThreads) picked[i] = kNoKey;
    __syncthreads();
    for (std::uint32_t j = tid; j < n; j += kKnnThreads)
        if (keys[j] <= prefix) picked[atomicAdd(&s_count, 1u)] = keys[j];
    __syncthreads();
    for (std::uint32_t k = 2; k <= width; k <<= 1)
        for (std::uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (std::uint32_t i = tid; i < width; i += kKnnThreads) {
                const std::uint32_t p = i ^ j;
                if (p > i) {
                    const unsigned long long x = picked[i], y = picked[p];
                    if ((x > y) == ((i & k) == 0)) {
                        picked[i] = y;
                        picked[p] = x;
                    }
                }
            }
            __syncthreads();
        }
    for (std::uint32_t i = tid; i < needed; i += kKnnThreads) {
        near_ids[(size_t)a * needed + i] = (node_t)(picked[i] & 0xffffu);
        near_dist[(size_t)a * needed + i] = (std::int32_t)(picked[i] >> 16);
    }
}

}  // namespace

std::uint32_t knn_smem_bytes(std::uint32_t n) { return 8u * n; }

cudaError_t launch_knn(const int2* xy, std::uint32_t n, std::uint32_t needed, node_t* near_ids,
                       std::int32_t* near_dist, cudaStream_t stream) {
    if (needed < 1 || needed > kKnnMaxNeeded || needed >= n) return cudaErrorInvalidValue;
    const std::uint32_t smem = knn_smem_bytes(n);
    cudaError_t err = cudaFuncSetAttribute(knn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    knn_kernel<<<n, kKnnThreads, smem, stream>>>(xy, n, needed, near_ids, near_dist);
    return cudaGetLastError();
}

}  // namespace faco

// faco_noalloc.cu -- the MMAS pheromone step on caller-owned device buffers,
// with its only scratch in a fixed file-scope device array: no device or
// host memory is allocated per call.
//
//   noalloc_prepare_kernel   packs the parent tour's neighbours into the
//                            scratch and checks parent/candidate ranges
//   noalloc_update_kernel    evaporate/deposit + products refresh (the same
//                            rule as the engine's colony update,
//                            cuda/colony_state.cuh:210-229), skipped as a
//                            whole when the prepare kernel found a problem
#include <cuda_runtime.h>

#include <cstdint>

#include "noalloc_kernels.h"

namespace faco {
namespace {

// The per-device scratch.  `nbr` needs no initial value: a valid parent
// tour writes every entry 0..n-1 before the update reads it.  `seen` (the
// permutation bitmap) and `error` must start at zero; the host clears their
// first ceil(n/32) words and the error word on the call's stream before the
// prepare kernel runs.
struct PheromoneScratch {
    std::uint32_t nbr[kNoAllocMaxNodes + 1];
    std::uint32_t seen[(kNoAllocMaxNodes + 32) / 32];
    std::uint32_t error;
};

__device__ __align__(256) PheromoneScratch g_pheromone_scratch;

__global__ void noalloc_prepare_kernel(std::uint32_t n, std::uint32_t k, const std::uint32_t* primary,
                                       const std::uint32_t* parent, PheromoneScratch* s) {
    const std::uint32_t stride = gridDim.x * blockDim.x;
    const std::uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
    for (std::uint32_t p = first; p < n; p += stride) {
        const std::uint32_t v = parent[p];
        if (v >= n) {
            atomicOr(&s->error, kNoAllocParentRange);
            continue;
        }
        const std::uint32_t bit = 1u << (v & 31u);
        if (atomicOr(&s->seen[v >> 5], bit) & bit) {
            atomicOr(&s->error, kNoAllocParentRepeat);
            continue;
        }
        const std::uint32_t next = parent[p + 1 == n ? 0 : p + 1], prev = parent[p == 0 ? n - 1 : p - 1];
        s->nbr[v] = (next & 0xffffu) | ((prev & 0xffffu) << 16);
    }
    const std::uint32_t cells = n * k;
    for (std::uint32_t i = first; i < cells; i += stride)
        if (primary[i] >= n) atomicOr(&s->error, kNoAllocPrimaryRange);
}

__device__ __forceinline__ float noalloc_trail(float tau, std::uint32_t to, std::uint32_t nb, float ret, float tmin,
                                               float tmax, float inc) {
    float v = fmaxf(tmin, tau * ret);
    if (to == (nb & 0xffffu) || to == (nb >> 16)) v = fminf(tmax, v + inc);
    return v;
}

template <bool VEC>
__global__ void noalloc_update_kernel(std::uint32_t n, std::uint32_t k, const std::uint32_t* primary, float ret,
                                      float tmin, float tmax, float inc, const float* eta, float* trails,
                                      float* products, const PheromoneScratch* s) {
    if (s->error) return;
    const std::uint32_t cells = n * k;
    const std::uint32_t stride = gridDim.x * blockDim.x;
    const std::uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
    if (VEC) {
        for (std::uint32_t q = first; q * 4 < cells; q += stride) {
            const std::uint32_t idx = q * 4, nb = s->nbr[idx / k];
            const float4 t = *reinterpret_cast<const float4*>(trails + idx);
            const float4 e = *reinterpret_cast<const float4*>(eta + idx);
            const uint4 to = *reinterpret_cast<const uint4*>(primary + idx);
            float4 v;
            v.x = noalloc_trail(t.x, to.x, nb, ret, tmin, tmax, inc);
            v.y = noalloc_trail(t.y, to.y, nb, ret, tmin, tmax, inc);
            v.z = noalloc_trail(t.z, to.z, nb, ret, tmin, tmax, inc);
            v.w = noalloc_trail(t.w, to.w, nb, ret, tmin, tmax, inc);
            *reinterpret_cast<float4*>(trails + idx) = v;
            *reinterpret_cast<float4*>(products + idx) = make_float4(v.x * e.x, v.y * e.y, v.z * e.z, v.w * e.w);
        }
    } else {
        for (std::uint32_t idx = first; idx < cells; idx += stride) {
            const float v = noalloc_trail(trails[idx], primary[idx], s->nbr[idx / k], ret, tmin, tmax, inc);
            trails[idx] = v;
            products[idx] = v * eta[idx];
        }
    }
}

// Address of the scratch in the current context, looked up on every call:
// cudaGetSymbolAddress allocates nothing, and a cached address would dangle
// after a cudaDeviceReset or under another context of the same device.
cudaError_t scratch_address(PheromoneScratch** out) {
    void* p = nullptr;
    const cudaError_t err = cudaGetSymbolAddress(&p, g_pheromone_scratch);
    if (err != cudaSuccess) return err;
    *out = static_cast<PheromoneScratch*>(p);
    return cudaSuccess;
}

// Grid-stride launches: at most 16 blocks of 256 threads per SM of the
// current device (enough to cover the latency of the streaming loops), at
// least one block.
std::uint32_t grid_for(std::uint64_t items, int sms) {
    const std::uint64_t cap = 16ull * static_cast<std::uint64_t>(sms > 0 ? sms : 1);
    const std::uint64_t blocks = (items + 255) / 256;
    return static_cast<std::uint32_t>(blocks < 1 ? 1 : (blocks > cap ? cap : blocks));
}

}  // namespace

cudaError_t pheromone_step_noalloc(std::uint32_t n, std::uint32_t k, const std::uint32_t* primary,
                                   const std::uint32_t* parent, float retention, float minimum, float maximum,
                                   float increment, const float* eta, float* trails, float* products,
                                   cudaStream_t stream, std::uint32_t* error_bits) {
    PheromoneScratch* s = nullptr;
    cudaError_t err = scratch_address(&s);
    if (err != cudaSuccess) return err;
    int device = 0, sms = 0;
    err = cudaGetDevice(&device);
    if (err == cudaSuccess) err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (err != cudaSuccess) return err;
    err = cudaMemsetAsync(s->seen, 0, ((n + 31) / 32) * sizeof(std::uint32_t), stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(&s->error, 0, sizeof(std::uint32_t), stream);
    if (err != cudaSuccess) return err;
    const std::uint64_t cells = static_cast<std::uint64_t>(n) * k;
    noalloc_prepare_kernel<<<grid_for(cells > n ? cells : n, sms), 256, 0, stream>>>(n, k, primary, parent, s);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    const auto aligned = [](const void* p) { return (reinterpret_cast<std::uintptr_t>(p) & 15u) == 0; };
    if ((k & 3u) == 0 && aligned(primary) && aligned(eta) && aligned(trails) && aligned(products))
        noalloc_update_kernel<true><<<grid_for(cells / 4, sms), 256, 0, stream>>>(
            n, k, primary, retention, minimum, maximum, increment, eta, trails, products, s);
    else
        noalloc_update_kernel<false><<<grid_for(cells, sms), 256, 0, stream>>>(
            n, k, primary, retention, minimum, maximum, increment, eta, trails, products, s);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    err = cudaMemcpyAsync(error_bits, &s->error, sizeof(std::uint32_t), cudaMemcpyDeviceToHost, stream);
    if (err != cudaSuccess) return err;
    return cudaStreamSynchronize(stream);
}

}  // namespace faco

// prior_mlp.cu -- forward, backward and Adam kernels of the edge-prior MLP.
#include <cuda_runtime.h>

#include "prior_kernels.h"
#include "prior_mlp.cuh"
#include "prior_mlp_tc.cuh"

namespace faco {

namespace {

__device__ __forceinline__ float sigmoid(float z) { return 1.0f / (1.0f + expf(-z)); }

}  // namespace

// Probabilities for E edges (x: [E][8] BF16) on the tcgen05 tensor cores:
// 128-edge tiles, 128 threads per CTA (one TMEM lane per edge).
__global__ void __launch_bounds__(128) mlp_forward_kernel(const MlpParams* P, const MlpOperands* O,
                                                          const __nv_bfloat16* x, std::uint32_t E, float* prob,
                                                          unsigned* error) {
    extern __shared__ __align__(16) unsigned char smem[];
    tc::forward_rows(
        P, O, E, smem, error,
        [&](std::uint32_t row) { return *reinterpret_cast<const uint4*>(x + (size_t)row * kMlpIn); },
        [&](std::uint32_t row, float z) { prob[row] = sigmoid(z); });
}

// Binary cross-entropy gradients of the mean loss over E edges on the
// tcgen05 tensor cores (tc::gradient_rows): 128-edge tiles strided over the
// grid, weight gradients accumulated in TMEM across a CTA's tiles.  Block b
// writes its partial gradient to partials[b] and its loss sum to
// loss_partials[b]; mlp_grad_reduce_kernel adds the partials in block order,
// and the tensor core's accumulation order is fixed, so every run gives the
// same bits.
__global__ void __launch_bounds__(128) mlp_grad_kernel(const MlpParams* P, const MlpOperands* O,
                                                       const __nv_bfloat16* x, const float* y, std::uint32_t E,
                                                       float inv_count, MlpParams* partials, float* loss_partials,
                                                       unsigned* error) {
    extern __shared__ __align__(16) unsigned char smem[];
    tc::gradient_rows(
        P, O, E, inv_count, smem, error,
        [&](std::uint32_t row) { return *reinterpret_cast<const uint4*>(x + (size_t)row * kMlpIn); },
        [&](std::uint32_t row) { return y[row]; }, partials + blockIdx.x, loss_partials + blockIdx.x);
}

// grad = the block partials summed in block order; *loss += their losses.
__global__ void mlp_grad_reduce_kernel(const MlpParams* partials, const float* loss_partials, std::uint32_t blocks,
                                       MlpParams* grad, float* loss) {
    const float* src = reinterpret_cast<const float*>(partials);
    float* dst = reinterpret_cast<float*>(grad);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpParamCount; i += gridDim.x * blockDim.x) {
        float sum = 0.f;
        for (std::uint32_t b = 0; b < blocks; ++b) sum += src[(size_t)b * kMlpParamCount + i];
        dst[i] = sum;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        float sum = 0.f;
        for (std::uint32_t b = 0; b < blocks; ++b) sum += loss_partials[b];
        *loss += sum;
    }
}

// Adam on the FP32 masters (decoupled from the BF16 operand refresh below).
__global__ void adam_kernel(MlpParams* P, const MlpParams* grad, MlpParams* m, MlpParams* v, float lr, float beta1,
                            float beta2, float eps, float bias1, float bias2) {
    float* p = reinterpret_cast<float*>(P);
    const float* gr = reinterpret_cast<const float*>(grad);
    float* mm = reinterpret_cast<float*>(m);
    float* vv = reinterpret_cast<float*>(v);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpParamCount; i += gridDim.x * blockDim.x) {
        const float gi = gr[i];
        mm[i] = beta1 * mm[i] + (1.0f - beta1) * gi;
        vv[i] = beta2 * vv[i] + (1.0f - beta2) * gi * gi;
        p[i] -= lr * (mm[i] / bias1) / (sqrtf(vv[i] / bias2) + eps);
    }
}

// ---------------------------------------------------------------------------
// Candidate-edge features of a colony state, one row of 8 BF16 per directed
// candidate entry (i, r), j = primary[i][r]:
//   x0 min(d(i,j) / mean nearest-neighbour distance, 8) / 8
//   x1 r / (k-1)                          (k-rank)
//   x2 (1 - cos angle(j-i, nn(i)-i)) / 2  (angle to the nearest neighbour)
//   x3 d(i,j) / d(i, k-th neighbour)
//   x4 (tau - tau_min) / (tau_max - tau_min), clipped to [0,1]
//   x5 1 when (i,j) is an edge of the colony's global-best tour
//   x6 rank of i in j's own candidate row / (k-1), 1 when absent
//   x7 min(alpha(i,j) / mean nearest-neighbour distance, 4) / 4, alpha the
//      alpha-nearness (length minus the longest edge on the minimum
//      spanning tree path between i and j)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void edge_features(const InstanceView& in, const ColonyView& cv, const ColonyState& st,
                                              const std::uint32_t* gnbr, std::uint32_t i, std::uint32_t r,
                                              float x[kMlpFeatures]) {
    const std::uint32_t k = in.k;
    const std::uint32_t j = in.primary[(size_t)i * k + r];
    const int2 pi = in.xy[i], pj = in.xy[j], pn = in.xy[in.primary[(size_t)i * k]];
    const int2 pk = in.xy[in.primary[(size_t)i * k + k - 1]];
    const float dij = (float)euc2d(pi, pj), dik = (float)euc2d(pi, pk);
    x[0] = fminf(dij / in.mean_nn, 8.0f) * 0.125f;
    x[1] = k > 1 ? (float)r / (float)(k - 1) : 0.0f;
    const float ax = (float)(pj.x - pi.x), ay = (float)(pj.y - pi.y);
    const float bx = (float)(pn.x - pi.x), by = (float)(pn.y - pi.y);
    const float na = sqrtf(ax * ax + ay * ay), nb = sqrtf(bx * bx + by * by);
    const float cosv = na > 0.0f && nb > 0.0f ? (ax * bx + ay * by) / (na * nb) : 1.0f;
    x[2] = fminf(fmaxf((1.0f - cosv) * 0.5f, 0.0f), 1.0f);
    x[3] = dik > 0.0f ? fminf(dij / dik, 1.0f) : 1.0f;
    const float span = st.tau_max - st.tau_min;
    const float tau = cv.trails[(size_t)i * k + r];
    x[4] = span > 0.0f ? fminf(fmaxf((tau - st.tau_min) / span, 0.0f), 1.0f) : 1.0f;
    const std::uint32_t nb2 = gnbr[i];
    x[5] = (j == (nb2 & 0xffffu) || j == (nb2 >> 16)) ? 1.0f : 0.0f;
    // mutual nearness: where i sits in j's own candidate row (1 if absent)
    float back = 1.0f;
    for (std::uint32_t t = 0; t < k; ++t)
        if (in.primary[(size_t)j * k + t] == i) {
            back = k > 1 ? (float)t / (float)(k - 1) : 0.0f;
            break;
        }
    x[6] = back;
    x[7] = fminf(in.alpha[(size_t)i * k + r] / in.mean_nn, 4.0f) * 0.25f;
}

// Packed neighbours of the colony's global-best tour in shared memory.
__device__ void global_neighbours(const ColonyView& cv, std::uint32_t n, std::uint32_t* gnbr) {
    for (std::uint32_t p = threadIdx.x; p < n; p += blockDim.x)
        gnbr[cv.global[p]] = (std::uint32_t)cv.global[p + 1 == n ? 0 : p + 1] |
                             ((std::uint32_t)cv.global[p == 0 ? n - 1 : p - 1] << 16);
}

// Features (and optionally labels from the global-best tours) of colonies
// [first, first + gridDim.x); rows start at row_offset[colony].
__global__ void edge_features_kernel(const InstanceView* instances, const ColonyView* colonies,
                                     const ColonyState* states, std::uint32_t first, const std::uint64_t* row_offset,
                                     __nv_bfloat16* x_out, float* y_out) {
    extern __shared__ std::uint32_t gnbr[];
    const std::uint32_t c = first + blockIdx.x;
    const ColonyView cv = colonies[c];
    const InstanceView in = instances[cv.instance];
    const ColonyState st = states[c];
    const std::uint32_t n = in.n, k = in.k;
    global_neighbours(cv, n, gnbr);
    __syncthreads();
    const std::uint64_t base = row_offset[c];
    for (std::uint32_t idx = threadIdx.x; idx < n * k; idx += blockDim.x) {
        const std::uint32_t i = idx / k, r = idx % k;
        if (x_out) {
            float x[kMlpFeatures];
            edge_features(in, cv, st, gnbr, i, r, x);
            __nv_bfloat16* row = x_out + (base + idx) * kMlpIn;
            for (int f = 0; f < kMlpFeatures; ++f) row[f] = __float2bfloat16(x[f]);
        }
        if (y_out) {
            const std::uint32_t j = in.primary[idx], nb = gnbr[i];
            y_out[base + idx] = (j == (nb & 0xffffu) || j == (nb >> 16)) ? 1.0f : 0.0f;
        }
    }
}

// Packed neighbours of every colony's global-best tour into gnbr (rows at
// the colonies' parent_nbr offsets).  One block per colony.
__global__ void global_neighbours_kernel(const ColonyView* colonies, std::uint32_t* gnbr_all,
                                         const std::uint32_t* node_offset) {
    const ColonyView cv = colonies[blockIdx.x];
    std::uint32_t* gnbr = gnbr_all + node_offset[blockIdx.x];
    global_neighbours(cv, cv.n, gnbr);
}

// Applies the prior to the colonies whose flag is set: for every candidate
// entry eta' = eta * (floor + p)^gamma (gamma in {1, 2}), p the MLP
// probability (tcgen05 forward over 128-entry tiles, features computed per
// entry), and products = trails * eta'.  The factor is never zero, so no
// candidate is removed.  Flag clear: eta' = eta (plain FACO).  Grid:
// (CTAs per colony, colonies), 128 threads.
__global__ void __launch_bounds__(128) prior_apply_kernel(const InstanceView* instances, const ColonyView* colonies,
                                                          const ColonyState* states, const std::uint8_t* enabled,
                                                          const MlpParams* P, const MlpOperands* O, float floor,
                                                          int gamma, const std::uint32_t* gnbr_all,
                                                          const std::uint32_t* node_offset, unsigned* error) {
    extern __shared__ __align__(16) unsigned char smem[];
    const std::uint32_t c = blockIdx.y;
    const ColonyView cv = colonies[c];
    const InstanceView in = instances[cv.instance];
    const std::uint32_t k = in.k, cells = in.n * k;
    if (!enabled[c]) {
        for (std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cells; i += gridDim.x * blockDim.x) {
            cv.eta[i] = in.eta[i];
            cv.products[i] = cv.trails[i] * in.eta[i];
        }
        return;
    }
    const ColonyState st = states[c];
    const std::uint32_t* gnbr = gnbr_all + node_offset[c];
    tc::forward_rows(
        P, O, cells, smem, error,
        [&](std::uint32_t e) {
            float x[kMlpFeatures];
            edge_features(in, cv, st, gnbr, e / k, e % k, x);
            return make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], x[5]),
                              pack_bf16(x[6], x[7]));
        },
        [&](std::uint32_t e, float z) {
            const float f = floor + sigmoid(z);
            const float eta = in.eta[e] * (gamma == 2 ? f * f : f);
            cv.eta[e] = eta;
            cv.products[e] = cv.trails[e] * eta;
        });
}

// BF16 operand copies of the masters.
__global__ void refresh_operands_kernel(const MlpParams* P, MlpOperands* O) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kMlpHidden * kMlpHidden; i += gridDim.x * blockDim.x) {
        O->w2[i] = __float2bfloat16(P->w2[i]);
        if (i < kMlpHidden * kMlpIn)
            O->w1[i] = __float2bfloat16(P->w1[i]);
    }
}

}  // namespace faco

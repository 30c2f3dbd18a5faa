// prior_mlp.cu -- forward, backward and Adam kernels of the edge-prior MLP.
#include <cuda_runtime.h>

#include "prior_kernels.h"
#include "prior_mlp.cuh"
#include "prior_mlp_tc.cuh"

namespace faco {

namespace {

constexpr int kWarps = 4;                 // 64 edges per block chunk
constexpr int kChunk = 16 * kWarps;

struct SharedOperands {
    __nv_bfloat16 w1[kMlpHidden * kMlpIn];
    __nv_bfloat16 w2[kMlpHidden * kMlpHidden];
    __nv_bfloat16 w2t[kMlpHidden * kMlpHidden];
    float b1[kMlpHidden], b2[kMlpHidden], w3[kMlpHidden];
    float b3;
};

__device__ void load_operands(SharedOperands& s, const MlpParams* P, const MlpOperands* O) {
    for (int i = threadIdx.x; i < kMlpHidden * kMlpIn; i += blockDim.x) s.w1[i] = O->w1[i];
    for (int i = threadIdx.x; i < kMlpHidden * kMlpHidden; i += blockDim.x) {
        s.w2[i] = O->w2[i];
        s.w2t[i] = O->w2t[i];
    }
    for (int i = threadIdx.x; i < kMlpHidden; i += blockDim.x) {
        s.b1[i] = P->b1[i];
        s.b2[i] = P->b2[i];
        s.w3[i] = P->w3[i];
    }
    if (threadIdx.x == 0) s.b3 = P->b3;
}

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

// Binary cross-entropy gradients of the mean loss over `scale_count` edges.
// Blocks stride over 64-edge chunks; block b writes its partial gradient to
// partials[b] and its summed loss to loss_partials[b] (every entry written by
// one thread, the warps' shares of the vectors summed in warp order), and
// mlp_grad_reduce_kernel adds the partials in block order -- the same bits on
// every run.
__global__ void __launch_bounds__(128) mlp_grad_kernel(const MlpParams* P, const MlpOperands* O,
                                                       const __nv_bfloat16* x, const float* y, std::uint32_t E,
                                                       float inv_count, MlpParams* partials, float* loss_partials) {
    MlpParams* grad = partials + blockIdx.x;
    __shared__ float s_vec[4][3][kMlpHidden];
    __shared__ float s_scalar[4][2];
    __shared__ SharedOperands s;
    __shared__ __align__(16) __nv_bfloat16 xs[kChunk * kMlpIn];
    __shared__ __align__(16) __nv_bfloat16 h1s[kChunk * kMlpHidden];
    __shared__ __align__(16) __nv_bfloat16 dh2s[kChunk * kMlpHidden];
    __shared__ __align__(16) __nv_bfloat16 dh1s[kChunk * kMlpHidden];
    load_operands(s, P, O);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    float gw2[8][4], gw1[4] = {0.f, 0.f, 0.f, 0.f}, gb1[16], gb2[16], gw3[16], gb3 = 0.f, lsum = 0.f;
#pragma unroll
    for (int i = 0; i < 16; ++i) gb1[i] = gb2[i] = gw3[i] = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) gw2[nt][0] = gw2[nt][1] = gw2[nt][2] = gw2[nt][3] = 0.f;
    const std::uint32_t chunks = (E + kChunk - 1) / kChunk;
    for (std::uint32_t chunk = blockIdx.x; chunk < chunks; chunk += gridDim.x) {
        const std::uint32_t c0 = chunk * kChunk;
        for (int i = threadIdx.x; i < kChunk * kMlpIn; i += blockDim.x) {
            const std::uint32_t e = c0 + i / kMlpIn;
            xs[i] = e < E ? x[(size_t)e * kMlpIn + i % kMlpIn] : __float2bfloat16(0.f);
        }
        __syncthreads();
        const int r0 = warp * 16;               // first row of this warp inside the chunk
        MlpTile t;
        mlp_forward_tile(xs + r0 * kMlpIn, s.w1, s.w2, s.b1, s.b2, s.w3, s.b3, lane, t);
        // output layer: dz = (sigmoid(z) - y) / count
        float dz[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const std::uint32_t e = c0 + r0 + g + 8 * h;
            const bool valid = e < E;
            const float z = t.z[h], label = valid ? y[e] : 0.f;
            dz[h] = valid ? (sigmoid(z) - label) * inv_count : 0.f;
            if (valid && q == 0) lsum += fmaxf(z, 0.f) - z * label + log1pf(expf(-fabsf(z)));
        }
        gb3 += q == 0 ? dz[0] + dz[1] : 0.f;
        // dh2 = dz * w3 (where h2 > 0); dW3, db2 partial sums
        float dh2[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int c = nt * 8 + 2 * q;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float w = s.w3[c + (i & 1)];
                dh2[nt][i] = t.h2[nt][i] > 0.f ? dz[i >> 1] * w : 0.f;
            }
            gw3[2 * nt] += dz[0] * t.h2[nt][0] + dz[1] * t.h2[nt][2];
            gw3[2 * nt + 1] += dz[0] * t.h2[nt][1] + dz[1] * t.h2[nt][3];
            gb2[2 * nt] += dh2[nt][0] + dh2[nt][2];
            gb2[2 * nt + 1] += dh2[nt][1] + dh2[nt][3];
        }
        // dh1 = dh2 * W2 (tensor cores), then masked by h1 > 0
        float dh1[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) dh1[nt][0] = dh1[nt][1] = dh1[nt][2] = dh1[nt][3] = 0.f;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const std::uint32_t a[4] = {pack_bf16(dh2[2 * kt][0], dh2[2 * kt][1]),
                                        pack_bf16(dh2[2 * kt][2], dh2[2 * kt][3]),
                                        pack_bf16(dh2[2 * kt + 1][0], dh2[2 * kt + 1][1]),
                                        pack_bf16(dh2[2 * kt + 1][2], dh2[2 * kt + 1][3])};
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
                mma_bf16(dh1[nt], a, ld_pair(s.w2t, nt * 8 + g, kt * 16 + 2 * q, kMlpHidden),
                         ld_pair(s.w2t, nt * 8 + g, kt * 16 + 8 + 2 * q, kMlpHidden));
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
            for (int i = 0; i < 4; ++i) dh1[nt][i] = t.h1[nt][i] > 0.f ? dh1[nt][i] : 0.f;
            gb1[2 * nt] += dh1[nt][0] + dh1[nt][2];
            gb1[2 * nt + 1] += dh1[nt][1] + dh1[nt][3];
            // stage activations and gradients (BF16) for the weight-gradient products
            const int col = nt * 8 + 2 * q;
            *reinterpret_cast<std::uint32_t*>(h1s + (r0 + g) * kMlpHidden + col) = pack_bf16(t.h1[nt][0], t.h1[nt][1]);
            *reinterpret_cast<std::uint32_t*>(h1s + (r0 + g + 8) * kMlpHidden + col) =
                pack_bf16(t.h1[nt][2], t.h1[nt][3]);
            *reinterpret_cast<std::uint32_t*>(dh2s + (r0 + g) * kMlpHidden + col) = pack_bf16(dh2[nt][0], dh2[nt][1]);
            *reinterpret_cast<std::uint32_t*>(dh2s + (r0 + g + 8) * kMlpHidden + col) =
                pack_bf16(dh2[nt][2], dh2[nt][3]);
            *reinterpret_cast<std::uint32_t*>(dh1s + (r0 + g) * kMlpHidden + col) = pack_bf16(dh1[nt][0], dh1[nt][1]);
            *reinterpret_cast<std::uint32_t*>(dh1s + (r0 + g + 8) * kMlpHidden + col) =
                pack_bf16(dh1[nt][2], dh1[nt][3]);
        }
        __syncthreads();
        // weight gradients with the chunk's 64 edges as K: this warp owns
        // output rows 16*warp .. 16*warp+15 of dW2 and dW1
        const int o = warp * 16 + g;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt) {
            const int e = kt * 16 + 2 * q;
            const std::uint32_t a2[4] = {ld_col_pair(dh2s, e, o, kMlpHidden), ld_col_pair(dh2s, e, o + 8, kMlpHidden),
                                         ld_col_pair(dh2s, e + 8, o, kMlpHidden),
                                         ld_col_pair(dh2s, e + 8, o + 8, kMlpHidden)};
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
                mma_bf16(gw2[nt], a2, ld_col_pair(h1s, e, nt * 8 + g, kMlpHidden),
                         ld_col_pair(h1s, e + 8, nt * 8 + g, kMlpHidden));
            const std::uint32_t a1[4] = {ld_col_pair(dh1s, e, o, kMlpHidden), ld_col_pair(dh1s, e, o + 8, kMlpHidden),
                                         ld_col_pair(dh1s, e + 8, o, kMlpHidden),
                                         ld_col_pair(dh1s, e + 8, o + 8, kMlpHidden)};
            mma_bf16(gw1, a1, ld_col_pair(xs, e, g, kMlpIn), ld_col_pair(xs, e + 8, g, kMlpIn));
        }
        __syncthreads();
    }
    // flush: weight matrices (each warp owns 16 rows, each thread its
    // entries), then the vectors
    const int o = warp * 16 + g;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int col = nt * 8 + 2 * q;
        grad->w2[o * kMlpHidden + col] = gw2[nt][0];
        grad->w2[o * kMlpHidden + col + 1] = gw2[nt][1];
        grad->w2[(o + 8) * kMlpHidden + col] = gw2[nt][2];
        grad->w2[(o + 8) * kMlpHidden + col + 1] = gw2[nt][3];
    }
    grad->w1[o * kMlpIn + 2 * q] = gw1[0];
    grad->w1[o * kMlpIn + 2 * q + 1] = gw1[1];
    grad->w1[(o + 8) * kMlpIn + 2 * q] = gw1[2];
    grad->w1[(o + 8) * kMlpIn + 2 * q + 1] = gw1[3];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        // reduce over the 8 row groups (lanes with equal q)
        for (int off = 4; off < 32; off <<= 1) {
            gb1[i] += __shfl_xor_sync(0xffffffffu, gb1[i], off);
            gb2[i] += __shfl_xor_sync(0xffffffffu, gb2[i], off);
            gw3[i] += __shfl_xor_sync(0xffffffffu, gw3[i], off);
        }
    }
    if (g == 0) {
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int c = nt * 8 + 2 * q + j;
                s_vec[warp][0][c] = gb1[2 * nt + j];
                s_vec[warp][1][c] = gb2[2 * nt + j];
                s_vec[warp][2][c] = gw3[2 * nt + j];
            }
    }
    for (int off = 16; off; off >>= 1) {
        gb3 += __shfl_xor_sync(0xffffffffu, gb3, off);
        lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
    }
    if (lane == 0) {
        s_scalar[warp][0] = gb3;
        s_scalar[warp][1] = lsum;
    }
    __syncthreads();
    if (threadIdx.x < kMlpHidden) {
        const int c = threadIdx.x;
        float v0 = 0.f, v1 = 0.f, v2 = 0.f;
        for (int w = 0; w < 4; ++w) {
            v0 += s_vec[w][0][c];
            v1 += s_vec[w][1][c];
            v2 += s_vec[w][2][c];
        }
        grad->b1[c] = v0;
        grad->b2[c] = v1;
        grad->w3[c] = v2;
    }
    if (threadIdx.x == 0) {
        float v0 = 0.f, v1 = 0.f;
        for (int w = 0; w < 4; ++w) {
            v0 += s_scalar[w][0];
            v1 += s_scalar[w][1];
        }
        grad->b3 = v0;
        grad->pad[0] = grad->pad[1] = grad->pad[2] = 0.f;
        loss_partials[blockIdx.x] = v1;
    }
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
        const int r = i / kMlpHidden, c = i % kMlpHidden;
        O->w2[i] = __float2bfloat16(P->w2[i]);
        O->w2t[c * kMlpHidden + r] = __float2bfloat16(P->w2[i]);
        if (i < kMlpHidden * kMlpIn)
            O->w1[i] = __float2bfloat16(P->w1[i]);
    }
}

}  // namespace faco

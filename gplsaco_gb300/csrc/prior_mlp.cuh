// prior_mlp.cuh -- the learned edge prior: an 8 -> 64 -> 64 -> 1 MLP scored
// per candidate edge (8 features), BF16 operands with FP32 accumulation on the tensor
// cores (mma.sync m16n8k16), forward and backward.
//
// The reference has no learned prior (its only prior is an external LKH
// candidate export, python/gp_faco/candidate_prior.py:20-36); this is the
// engine's own component.  Layout of one warp tile: 16 edges (rows); layer 1
// K = 16 (8 features + zero padding), layers 2 and the input gradient K = 64;
// the weight gradients use the edges as the K dimension, staged through
// shared memory by the block (4 warps = 64 edges per chunk).
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

namespace faco {

constexpr int kMlpIn = 8;       // feature slots per edge
constexpr int kMlpFeatures = 8;
constexpr int kMlpHidden = 64;

// FP32 master parameters (4,673 used values) and their BF16 operand copies.
struct MlpParams {
    float w1[kMlpHidden * kMlpIn];      // [out][in]
    float b1[kMlpHidden];
    float w2[kMlpHidden * kMlpHidden];  // [out][in]
    float b2[kMlpHidden];
    float w3[kMlpHidden];
    float b3;
    float pad[3];
};

struct MlpOperands {
    __nv_bfloat16 w1[kMlpHidden * kMlpIn];          // [out][in]
    __nv_bfloat16 w2[kMlpHidden * kMlpHidden];      // [out][in]
    __nv_bfloat16 w2t[kMlpHidden * kMlpHidden];     // [in][out] (input-gradient operand)
};

constexpr int kMlpParamCount = sizeof(MlpParams) / sizeof(float);

__device__ __forceinline__ std::uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const std::uint32_t*>(&v);
}

// D = A(16x16, row) * B(16x8, col) + C, BF16 inputs, FP32 accumulate.
__device__ __forceinline__ void mma_bf16(float (&d)[4], const std::uint32_t (&a)[4], std::uint32_t b0,
                                         std::uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Two consecutive BF16 values of a row-major [rows][ld] array as one 32-bit
// operand register (lower half = lower column).
__device__ __forceinline__ std::uint32_t ld_pair(const __nv_bfloat16* m, int row, int col, int ld) {
    return *reinterpret_cast<const std::uint32_t*>(m + row * ld + col);
}
// Two BF16 values of a column (rows r, r+1) of a row-major array.
__device__ __forceinline__ std::uint32_t ld_col_pair(const __nv_bfloat16* m, int row, int col, int ld) {
    const std::uint16_t lo = *reinterpret_cast<const std::uint16_t*>(m + row * ld + col);
    const std::uint16_t hi = *reinterpret_cast<const std::uint16_t*>(m + (row + 1) * ld + col);
    return (std::uint32_t)lo | ((std::uint32_t)hi << 16);
}

struct MlpTile {
    float h1[8][4];   // layer-1 activations (after ReLU), C fragments of 8 n-tiles
    float h2[8][4];   // layer-2 activations (after ReLU)
    float z[2];       // logits of rows g and g+8
};

// Forward pass of one 16-edge tile.  x: [16][8] BF16 rows of this tile (row
// stride 8).  Operands w1/w2 in shared memory.
__device__ __forceinline__ void mlp_forward_tile(const __nv_bfloat16* x, const __nv_bfloat16* w1,
                                                 const __nv_bfloat16* w2, const float* b1, const float* b2,
                                                 const float* w3, float b3, std::uint32_t lane, MlpTile& t) {
    const int g = lane >> 2, q = lane & 3;
    // layer 1: A = x (K padded to 16 with zeros)
    const std::uint32_t a1[4] = {ld_pair(x, g, 2 * q, kMlpIn), ld_pair(x, g + 8, 2 * q, kMlpIn), 0u, 0u};
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        mma_bf16(d, a1, ld_pair(w1, nt * 8 + g, 2 * q, kMlpIn), 0u);
        const float bb0 = b1[nt * 8 + 2 * q], bb1 = b1[nt * 8 + 2 * q + 1];
        t.h1[nt][0] = fmaxf(d[0] + bb0, 0.f);
        t.h1[nt][1] = fmaxf(d[1] + bb1, 0.f);
        t.h1[nt][2] = fmaxf(d[2] + bb0, 0.f);
        t.h1[nt][3] = fmaxf(d[3] + bb1, 0.f);
    }
    // layer 2: A fragments of k-tile kt come from the C fragments of n-tiles 2kt, 2kt+1
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) t.h2[nt][0] = t.h2[nt][1] = t.h2[nt][2] = t.h2[nt][3] = 0.f;
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        const std::uint32_t a[4] = {pack_bf16(t.h1[2 * kt][0], t.h1[2 * kt][1]),
                                    pack_bf16(t.h1[2 * kt][2], t.h1[2 * kt][3]),
                                    pack_bf16(t.h1[2 * kt + 1][0], t.h1[2 * kt + 1][1]),
                                    pack_bf16(t.h1[2 * kt + 1][2], t.h1[2 * kt + 1][3])};
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
            mma_bf16(t.h2[nt], a, ld_pair(w2, nt * 8 + g, kt * 16 + 2 * q, kMlpHidden),
                     ld_pair(w2, nt * 8 + g, kt * 16 + 8 + 2 * q, kMlpHidden));
    }
    float z0 = 0.f, z1 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int c0 = nt * 8 + 2 * q;
        const float bb0 = b2[c0], bb1 = b2[c0 + 1];
        t.h2[nt][0] = fmaxf(t.h2[nt][0] + bb0, 0.f);
        t.h2[nt][1] = fmaxf(t.h2[nt][1] + bb1, 0.f);
        t.h2[nt][2] = fmaxf(t.h2[nt][2] + bb0, 0.f);
        t.h2[nt][3] = fmaxf(t.h2[nt][3] + bb1, 0.f);
        z0 += t.h2[nt][0] * w3[c0] + t.h2[nt][1] * w3[c0 + 1];
        z1 += t.h2[nt][2] * w3[c0] + t.h2[nt][3] * w3[c0 + 1];
    }
    z0 += __shfl_xor_sync(0xffffffffu, z0, 1);
    z0 += __shfl_xor_sync(0xffffffffu, z0, 2);
    z1 += __shfl_xor_sync(0xffffffffu, z1, 1);
    z1 += __shfl_xor_sync(0xffffffffu, z1, 2);
    t.z[0] = z0 + b3;
    t.z[1] = z1 + b3;
}

}  // namespace faco

// prior_mlp_tc.cuh -- the edge-prior MLP forward pass and its training
// gradient on the 5th-generation tensor cores (tcgen05): 128-edge tiles,
// BF16 operands staged in shared memory and read by the tensor core through
// matrix descriptors, FP32 accumulators in tensor memory (TMEM), epilogues
// from tcgen05.ld.  The gradient is described above gradient_rows.
//
// Forward pass:
//
// Per tile (128 edges = 128 TMEM lanes, one row per thread):
//   layer 1  D1[128][64] = X[128][16] . W1[64][16]^T      (1 MMA, K = 16)
//   epilogue h1 = relu(D1 + b1) as BF16 -> shared memory (A operand)
//   layer 2  D2[128][64] = H1[128][64] . W2[64][64]^T     (4 MMAs, K = 16 each)
//            into the same TMEM columns; meanwhile every thread fetches its
//            row of the next tile
//   epilogue z = w3 . relu(D2 + b2) + b3 per row, p = sigmoid(z)
// One thread issues the MMAs and commits them to an mbarrier; every wait on
// it is bounded and sets the error word when it runs out.
//
// Operand layout (no swizzle, K-major): 8-row x 16-byte core matrices; in a
// K = 16 slab, element (r, k) sits at (r / 8) * 256 + (k / 8) * 128 +
// (r % 8) * 16 + (k % 8) * 2 bytes, i.e. core matrices 128 bytes apart along
// K and 256 bytes apart along the rows; slabs follow each other.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

#include "faco_common.cuh"
#include "prior_mlp.cuh"

namespace faco {
namespace tc {

constexpr std::uint32_t kRows = 128;                 // edges per tile (M)
constexpr std::uint32_t kTmemColumns = 64;           // D1, then D2 over it (D1 is read out first)
constexpr std::uint32_t kXBytes = kRows * 16 * 2;    // one K = 16 slab
constexpr std::uint32_t kHBytes = kRows * 64 * 2;    // four slabs
constexpr std::uint32_t kW1Bytes = 64 * 16 * 2;
constexpr std::uint32_t kW2Bytes = 64 * 64 * 2;
constexpr std::uint32_t kSmemBytes = kXBytes + kHBytes + kW1Bytes + kW2Bytes;   // 30 KB
// Dynamic shared memory per CTA: 30 KB, so at most seven CTAs share an SM
// and their 7 x 64 TMEM columns fit in its 512 (an allocation never waits).
constexpr std::uint32_t kLaunchSmemBytes = kSmemBytes;
constexpr std::uint32_t kCtasPerSm = 7;
constexpr std::uint32_t kWaitLimit = 1u << 20;       // try_wait attempts (about a second)
// No-swizzle K-major layout: core matrices 128 bytes apart along K (leading
// byte offset), 256 bytes apart along the rows (stride byte offset).
constexpr std::uint32_t kLbo = 128, kSbo = 256;

__device__ __forceinline__ std::uint32_t smem_u32(const void* p) {
    return static_cast<std::uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, k) in a K-major no-swizzle operand with `rows`
// rows (rows a multiple of 8, K slabs of 16 elements).
__device__ __forceinline__ std::uint32_t operand_offset(std::uint32_t r, std::uint32_t k, std::uint32_t rows) {
    return (k >> 4) * rows * 32u + (r >> 3) * 256u + ((k >> 3) & 1u) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor: start address, leading (K-direction) and
// stride (row-direction) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ std::uint64_t matrix_desc(std::uint32_t saddr, std::uint32_t lbo, std::uint32_t sbo) {
    return (std::uint64_t)((saddr >> 4) & 0x3FFFu) | ((std::uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((std::uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulate, BF16 A and B, both
// K-major, N = 64, M = 128.
constexpr std::uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma(std::uint32_t d_tmem, std::uint64_t a, std::uint64_t b, std::uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void commit(std::uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// Waits for the barrier's phase `parity` to complete, at most `limit` tries.
__device__ __forceinline__ bool wait_parity(std::uint64_t* bar, std::uint32_t parity, std::uint32_t limit) {
    const std::uint32_t addr = smem_u32(bar);
    for (std::uint32_t i = 0; i < limit; ++i) {
        std::uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void load16(std::uint32_t taddr, float (&v)[16]) {
    std::uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive floats of a 16-byte aligned shared array (4 vector loads).
__device__ __forceinline__ void load_vec16(const float* p, float (&v)[16]) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float4 t = reinterpret_cast<const float4*>(p)[q];
        v[4 * q] = t.x;
        v[4 * q + 1] = t.y;
        v[4 * q + 2] = t.z;
        v[4 * q + 3] = t.w;
    }
}

// Forward pass over rows [0, count): feat(row) gives the row's 8 BF16
// features as a uint4, out(row, z) receives its logit.  Rows are split
// over the CTAs of blockIdx.x / gridDim.x in 128-row tiles.  128 threads;
// `smem` holds kSmemBytes (16-byte aligned).  Returns false (and sets
// kErrTensorWait) if an MMA completion wait ran out.
template <class Feat, class Out>
__device__ bool forward_rows(const MlpParams* P, const MlpOperands* O, std::uint32_t count, unsigned char* smem,
                             unsigned* error, Feat feat, Out out) {
    __shared__ std::uint64_t bar;
    __shared__ std::uint32_t tmem_slot;
    __shared__ __align__(16) float s_b1[64], s_b2[64], s_w3[64];
    const std::uint32_t tid = threadIdx.x, warp = tid >> 5;
    unsigned char* xs = smem;
    unsigned char* hs = xs + kXBytes;
    unsigned char* w1s = hs + kHBytes;
    unsigned char* w2s = w1s + kW1Bytes;
    // weights as B operands (N = 64 rows = output units, K-major); W1's K
    // padded from 8 to 16 with zeros
    for (std::uint32_t i = tid; i < 64 * 16; i += blockDim.x) {
        const std::uint32_t n = i >> 4, k = i & 15u;
        const __nv_bfloat16 v = k < kMlpIn ? O->w1[n * kMlpIn + k] : __float2bfloat16(0.0f);
        *reinterpret_cast<__nv_bfloat16*>(w1s + operand_offset(n, k, 64)) = v;
    }
    for (std::uint32_t i = tid; i < 64 * 64; i += blockDim.x) {
        const std::uint32_t n = i >> 6, k = i & 63u;
        *reinterpret_cast<__nv_bfloat16*>(w2s + operand_offset(n, k, 64)) = O->w2[n * 64 + k];
    }
    for (std::uint32_t i = tid; i < 64; i += blockDim.x) {
        s_b1[i] = P->b1[i];
        s_b2[i] = P->b2[i];
        s_w3[i] = P->w3[i];
    }
    const float b3 = P->b3;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)) : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(kTmemColumns)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const std::uint32_t tmem = tmem_slot;
    const std::uint32_t lane_base = (warp * 32u) << 16;     // this warp's TMEM lane quarter
    const std::uint64_t dx = matrix_desc(smem_u32(xs), kLbo, kSbo);
    const std::uint64_t dw1 = matrix_desc(smem_u32(w1s), kLbo, kSbo);
    std::uint32_t phase = 0;
    bool ok = true;
    const std::uint32_t stride = gridDim.x * kRows;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (blockIdx.x * kRows + tid < count) v = feat(blockIdx.x * kRows + tid);
    for (std::uint32_t first = blockIdx.x * kRows; first < count; first += stride) {
        // X tile: this thread's row, K = 8 features + 8 zeros
        const std::uint32_t row = first + tid;
        *reinterpret_cast<uint4*>(xs + operand_offset(tid, 0, kRows)) = v;
        *reinterpret_cast<uint4*>(xs + operand_offset(tid, 8, kRows)) = make_uint4(0, 0, 0, 0);
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        if (tid == 0) {
            mma(tmem, dx, dw1, 0);
            commit(&bar);
        }
        bool waited = wait_parity(&bar, phase, kWaitLimit);
        if (__syncthreads_or(!waited)) { ok = false; break; }
        phase ^= 1u;
        fence_after();
        // epilogue 1: h1 = relu(D1 + b1) -> BF16 A operand of layer 2
#pragma unroll
        for (std::uint32_t c = 0; c < 64; c += 16) {
            float a[16], bias[16];
            load16(tmem + lane_base + c, a);
            load_vec16(s_b1 + c, bias);
#pragma unroll
            for (int g = 0; g < 2; ++g) {
                uint4 packed;
                std::uint32_t* w = reinterpret_cast<std::uint32_t*>(&packed);
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int i = g * 8 + 2 * t;
                    w[t] = pack_bf16(fmaxf(a[i] + bias[i], 0.f), fmaxf(a[i + 1] + bias[i + 1], 0.f));
                }
                *reinterpret_cast<uint4*>(hs + operand_offset(tid, c + g * 8, kRows)) = packed;
            }
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        if (tid == 0) {
#pragma unroll
            for (std::uint32_t kk = 0; kk < 4; ++kk)
                mma(tmem, matrix_desc(smem_u32(hs + kk * kRows * 32u), kLbo, kSbo),
                    matrix_desc(smem_u32(w2s + kk * 64u * 32u), kLbo, kSbo), kk > 0);
            commit(&bar);
        }
        // the next tile's row while the layer-2 MMAs run
        v = make_uint4(0, 0, 0, 0);
        if (row + stride < count) v = feat(row + stride);
        waited = wait_parity(&bar, phase, kWaitLimit);
        if (__syncthreads_or(!waited)) { ok = false; break; }
        phase ^= 1u;
        fence_after();
        // epilogue 2: z = w3 . relu(D2 + b2) + b3
        float z = 0.f;
#pragma unroll
        for (std::uint32_t c = 0; c < 64; c += 16) {
            float a[16], bias[16], w3[16];
            load16(tmem + lane_base + c, a);
            load_vec16(s_b2 + c, bias);
            load_vec16(s_w3 + c, w3);
#pragma unroll
            for (int t = 0; t < 16; ++t) z += fmaxf(a[t] + bias[t], 0.f) * w3[t];
        }
        if (row < count) out(row, z + b3);
        fence_before();
        __syncthreads();     // TMEM and shared operands are reused by the next tile
        fence_after();
    }
    if (!ok) {
        if (tid == 0) atomicOr(error, kErrTensorWait);
        // give the MMAs of the phase that ran out a bounded second chance to
        // finish before the tensor memory is released
        wait_parity(&bar, phase, kWaitLimit);
    }
    fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemColumns) : "memory");
    return ok;
}

// ---------------------------------------------------------------------------
// Gradient of the mean binary cross-entropy on the tensor cores.
//
// Every per-edge operand of a 128-edge tile is stored with the edge as the
// row and 8-feature core matrices as 2 KB blocks:
//   edge e, feature f at (f / 8) * 2048 + (e / 8) * 128 + (e % 8) * 16 + (f % 8) * 2
// so thread e writes its row as one 16-byte store per block, and the same
// bytes serve two views: K-major with the edges as M (forward products,
// leading byte offset 2048, stride byte offset 128) and MN-major with the
// edges as K (weight-gradient products: core matrices 128 bytes apart along
// the edges, 2048 bytes apart along the features).  The weights use 1 KB
// blocks (64 rows): W2 K-major gives W2^T as B of the forward product, and
// its MN-major view gives W2 as B of the input gradient dH1 = dH2 . W2.
//
// X' holds the 8 features and, in its second block, a 1 (feature 8) and
// the row's dz (feature 9); the forward product never sees them because
// W1's padding columns are zero.  Per tile:
//   S  = X' W1^T            -> h1 = relu(S + b1)            -> H1
//   S  = H1 W2^T            -> h2 = relu(S + b2), z, dz      -> H2, dH2, X'[9]
//   S  = dH2 W2             -> dh1 = S where h1 > 0          -> dH1
//   G3 += [H2 | dH2]^T X'   (N = 16): row c, column 9 = sum dz h2_c  (dw3)
//   GW += [dH2 | dH1]^T [H1 | X'] (N = 80):
//         rows 0-63:  columns 0-63 dW2, column 72 (the ones) db2
//         rows 64-127: columns 64-71 dW1, column 72 db1
// db3 and the loss are per-thread sums reduced over the block at the end.
// TMEM: S at column 0, G3 at 64, GW at 128 (256 columns, so at most two
// CTAs per SM, which is also what the 84 KB of shared memory allows).
// ---------------------------------------------------------------------------
constexpr std::uint32_t kGradBlock = 2048;                        // 8 features x 128 edges
constexpr std::uint32_t kGradH1 = 0;                              // H1  8 blocks
constexpr std::uint32_t kGradX = kGradH1 + 8 * kGradBlock;        // X'  2 blocks (right after H1)
constexpr std::uint32_t kGradH2 = kGradX + 2 * kGradBlock;        // H2  8 blocks
constexpr std::uint32_t kGradDH2 = kGradH2 + 8 * kGradBlock;      // dH2 8 blocks (right after H2)
constexpr std::uint32_t kGradDH1 = kGradDH2 + 8 * kGradBlock;     // dH1 8 blocks (right after dH2)
constexpr std::uint32_t kGradW1 = kGradDH1 + 8 * kGradBlock;      // W1  [64][16] 2 KB
constexpr std::uint32_t kGradW2 = kGradW1 + 2048;                 // W2  [64][64] 8 KB
// 6 KB of slack after W2 keeps every operand window inside the allocation
// even under the other reading of the descriptors' two byte offsets
constexpr std::uint32_t kGradSmemBytes = kGradW2 + 8192 + 6144;   // 86,016 bytes
constexpr std::uint32_t kGradCtasPerSm = 2;
constexpr std::uint32_t kGradTmemColumns = 256;
constexpr std::uint32_t kGradColS = 0, kGradColG3 = 64, kGradColGW = 128;

// Instruction descriptor of kind::f16 (FP32 accumulate, BF16 A and B),
// M = 128; a_mn / b_mn select the MN-major (transposed) operand view.
__host__ __device__ constexpr std::uint32_t idesc_f16(std::uint32_t n, std::uint32_t a_mn, std::uint32_t b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (a_mn << 15) | (b_mn << 16) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma_desc(std::uint32_t d_tmem, std::uint64_t a, std::uint64_t b, std::uint32_t idesc,
                                         std::uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

// Byte offset of (row e, feature f) in a 128-row edge operand and of
// (row o, input f) in a 64-row weight operand.
__device__ __forceinline__ std::uint32_t edge_offset(std::uint32_t e, std::uint32_t f) {
    return (f >> 3) * kGradBlock + (e >> 3) * 128u + (e & 7u) * 16u + (f & 7u) * 2u;
}
__device__ __forceinline__ std::uint32_t weight_offset(std::uint32_t o, std::uint32_t f) {
    return (f >> 3) * 1024u + (o >> 3) * 128u + (o & 7u) * 16u + (f & 7u) * 2u;
}

__device__ __forceinline__ uint4 pack8(const float* a) {
    return make_uint4(pack_bf16(a[0], a[1]), pack_bf16(a[2], a[3]), pack_bf16(a[4], a[5]), pack_bf16(a[6], a[7]));
}

// Partial gradient and loss sum of this CTA's rows (128-row tiles strided
// over the grid) into *grad and *loss_sum.  128 threads, `smem` holds
// kGradSmemBytes (16-byte aligned).  Returns false (and sets
// kErrTensorWait) if an MMA completion wait ran out; the partial is then
// incomplete.
template <class Feat, class Label>
__device__ bool gradient_rows(const MlpParams* P, const MlpOperands* O, std::uint32_t count, float inv_count,
                              unsigned char* smem, unsigned* error, Feat feat, Label label, MlpParams* grad,
                              float* loss_sum) {
    __shared__ std::uint64_t bar;
    __shared__ std::uint32_t tmem_slot;
    __shared__ __align__(16) float s_b1[64], s_b2[64], s_w3[64];
    __shared__ float s_scalar[4][2];
    const std::uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    for (std::uint32_t i = tid; i < 64 * 16; i += blockDim.x) {
        const std::uint32_t o = i >> 4, f = i & 15u;
        const __nv_bfloat16 v = f < kMlpIn ? O->w1[o * kMlpIn + f] : __float2bfloat16(0.0f);
        *reinterpret_cast<__nv_bfloat16*>(smem + kGradW1 + weight_offset(o, f)) = v;
    }
    for (std::uint32_t i = tid; i < 64 * 64; i += blockDim.x) {
        const std::uint32_t o = i >> 6, f = i & 63u;
        *reinterpret_cast<__nv_bfloat16*>(smem + kGradW2 + weight_offset(o, f)) = O->w2[o * 64 + f];
    }
    for (std::uint32_t i = tid; i < 64; i += blockDim.x) {
        s_b1[i] = P->b1[i];
        s_b2[i] = P->b2[i];
        s_w3[i] = P->w3[i];
    }
    const float b3 = P->b3;
    if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)) : "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(kGradTmemColumns)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const std::uint32_t tmem = tmem_slot;
    const std::uint32_t lane_base = (warp * 32u) << 16;
    const std::uint32_t base = smem_u32(smem);
    constexpr std::uint32_t kForward = idesc_f16(64, 0, 0), kInputGrad = idesc_f16(64, 0, 1);
    constexpr std::uint32_t kDw3 = idesc_f16(16, 1, 1), kDw = idesc_f16(80, 1, 1);
    std::uint32_t phase = 0;
    bool ok = true, any = false;
    float db3 = 0.f, lsum = 0.f;
    const std::uint32_t stride = gridDim.x * kRows;
    uint4 v = make_uint4(0, 0, 0, 0);
    float y = 0.f;
    if (blockIdx.x * kRows + tid < count) {
        v = feat(blockIdx.x * kRows + tid);
        y = label(blockIdx.x * kRows + tid);
    }
    for (std::uint32_t first = blockIdx.x * kRows; first < count; first += stride) {
        const std::uint32_t row = first + tid;
        const bool valid = row < count;
        if (any) {
            // the previous tile's weight-gradient products still read the operands
            const bool waited = wait_parity(&bar, phase, kWaitLimit);
            if (__syncthreads_or(!waited)) { ok = false; break; }
            phase ^= 1u;
            fence_after();
        }
        *reinterpret_cast<uint4*>(smem + kGradX + tid * 16u) = v;
        *reinterpret_cast<uint4*>(smem + kGradX + kGradBlock + tid * 16u) = make_uint4(0, 0, 0, 0);
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        if (tid == 0) {
            mma_desc(tmem + kGradColS, matrix_desc(base + kGradX, kGradBlock, 128),
                     matrix_desc(base + kGradW1, 1024, 128), kForward, 0);
            commit(&bar);
        }
        bool waited = wait_parity(&bar, phase, kWaitLimit);
        if (__syncthreads_or(!waited)) { ok = false; break; }
        phase ^= 1u;
        fence_after();
        // h1 = relu(S + b1) -> H1
#pragma unroll
        for (std::uint32_t c = 0; c < 64; c += 16) {
            float a[16], bias[16];
            load16(tmem + lane_base + kGradColS + c, a);
            load_vec16(s_b1 + c, bias);
#pragma unroll
            for (int t = 0; t < 16; ++t) a[t] = fmaxf(a[t] + bias[t], 0.f);
            *reinterpret_cast<uint4*>(smem + kGradH1 + (c / 8) * kGradBlock + tid * 16u) = pack8(a);
            *reinterpret_cast<uint4*>(smem + kGradH1 + (c / 8 + 1) * kGradBlock + tid * 16u) = pack8(a + 8);
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        if (tid == 0) {
#pragma unroll
            for (std::uint32_t kk = 0; kk < 4; ++kk)
                mma_desc(tmem + kGradColS, matrix_desc(base + kGradH1 + kk * 2 * kGradBlock, kGradBlock, 128),
                         matrix_desc(base + kGradW2 + kk * 2 * 1024, 1024, 128), kForward, kk > 0);
            commit(&bar);
        }
        // the next tile's row while the layer-2 products run
        uint4 v_next = make_uint4(0, 0, 0, 0);
        float y_next = 0.f;
        if (row + stride < count) {
            v_next = feat(row + stride);
            y_next = label(row + stride);
        }
        waited = wait_parity(&bar, phase, kWaitLimit);
        if (__syncthreads_or(!waited)) { ok = false; break; }
        phase ^= 1u;
        fence_after();
        // h2 = relu(S + b2), z = w3 . h2 + b3, dz; H2, dH2 = dz w3 where h2 > 0, X'[8..9] = (1, dz)
        float h[64];
        float z = 0.f;
#pragma unroll
        for (std::uint32_t c = 0; c < 64; c += 16) {
            float a[16], bias[16], w3[16];
            load16(tmem + lane_base + kGradColS + c, a);
            load_vec16(s_b2 + c, bias);
            load_vec16(s_w3 + c, w3);
#pragma unroll
            for (int t = 0; t < 16; ++t) {
                h[c + t] = fmaxf(a[t] + bias[t], 0.f);
                z += h[c + t] * w3[t];
            }
        }
        z += b3;
        const float dz = valid ? (1.0f / (1.0f + expf(-z)) - y) * inv_count : 0.f;
        if (valid) lsum += fmaxf(z, 0.f) - z * y + log1pf(expf(-fabsf(z)));
        db3 += dz;
#pragma unroll
        for (std::uint32_t c = 0; c < 64; c += 8) {
            float d[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) d[t] = h[c + t] > 0.f ? dz * s_w3[c + t] : 0.f;
            *reinterpret_cast<uint4*>(smem + kGradH2 + (c / 8) * kGradBlock + tid * 16u) = pack8(h + c);
            *reinterpret_cast<uint4*>(smem + kGradDH2 + (c / 8) * kGradBlock + tid * 16u) = pack8(d);
        }
        *reinterpret_cast<uint4*>(smem + kGradX + kGradBlock + tid * 16u) = make_uint4(pack_bf16(1.0f, dz), 0, 0, 0);
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        const std::uint32_t acc = any ? 1u : 0u;
        if (tid == 0) {
#pragma unroll
            for (std::uint32_t kk = 0; kk < 4; ++kk)
                mma_desc(tmem + kGradColS, matrix_desc(base + kGradDH2 + kk * 2 * kGradBlock, kGradBlock, 128),
                         matrix_desc(base + kGradW2 + kk * 256, 128, 1024), kInputGrad, kk > 0);
            // dw3: A = [H2 | dH2] (the dH2 half unused), B = X'
#pragma unroll
            for (std::uint32_t kk = 0; kk < 8; ++kk)
                mma_desc(tmem + kGradColG3, matrix_desc(base + kGradH2 + kk * 256, 128, kGradBlock),
                         matrix_desc(base + kGradX + kk * 256, 128, kGradBlock), kDw3, acc | (kk > 0));
            commit(&bar);
        }
        waited = wait_parity(&bar, phase, kWaitLimit);
        if (__syncthreads_or(!waited)) { ok = false; break; }
        phase ^= 1u;
        fence_after();
        // dh1 = S where h1 > 0 -> dH1
#pragma unroll
        for (std::uint32_t c = 0; c < 64; c += 16) {
            float a[16];
            load16(tmem + lane_base + kGradColS + c, a);
#pragma unroll
            for (int g = 0; g < 2; ++g) {
                const uint4 hv = *reinterpret_cast<const uint4*>(smem + kGradH1 + (c / 8 + g) * kGradBlock + tid * 16u);
                const std::uint32_t hw[4] = {hv.x, hv.y, hv.z, hv.w};
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    if (!(__uint_as_float(hw[t] << 16) > 0.f)) a[g * 8 + 2 * t] = 0.f;
                    if (!(__uint_as_float(hw[t] & 0xFFFF0000u) > 0.f)) a[g * 8 + 2 * t + 1] = 0.f;
                }
                *reinterpret_cast<uint4*>(smem + kGradDH1 + (c / 8 + g) * kGradBlock + tid * 16u) = pack8(a + g * 8);
            }
        }
        fence_async_smem();
        fence_before();
        __syncthreads();
        fence_after();
        if (tid == 0) {
#pragma unroll
            for (std::uint32_t kk = 0; kk < 8; ++kk)
                mma_desc(tmem + kGradColGW, matrix_desc(base + kGradDH2 + kk * 256, 128, kGradBlock),
                         matrix_desc(base + kGradH1 + kk * 256, 128, kGradBlock), kDw, acc | (kk > 0));
            commit(&bar);
        }
        any = true;
        v = v_next;
        y = y_next;
    }
    if (ok && any) {
        const bool waited = wait_parity(&bar, phase, kWaitLimit);
        if (__syncthreads_or(!waited)) ok = false;
        else phase ^= 1u;
        fence_after();
    }
    if (ok) {
        // lanes 0-63: dW2 row o, db2[o], dw3[o]; lanes 64-127: dW1 row o, db1[o]
        const std::uint32_t o = tid & 63u;
        float a[16];
        if (warp < 2) {
#pragma unroll
            for (std::uint32_t c = 0; c < 64; c += 16) {
                load16(tmem + lane_base + kGradColGW + c, a);
#pragma unroll
                for (int t = 0; t < 16; ++t) grad->w2[o * 64 + c + t] = any ? a[t] : 0.f;
            }
            load16(tmem + lane_base + kGradColGW + 64, a);
            grad->b2[o] = any ? a[8] : 0.f;
            load16(tmem + lane_base + kGradColG3, a);
            grad->w3[o] = any ? a[9] : 0.f;
        } else {
            load16(tmem + lane_base + kGradColGW + 64, a);
#pragma unroll
            for (int t = 0; t < kMlpIn; ++t) grad->w1[o * kMlpIn + t] = any ? a[t] : 0.f;
            grad->b1[o] = any ? a[8] : 0.f;
        }
    }
    for (int off = 16; off; off >>= 1) {
        db3 += __shfl_xor_sync(0xffffffffu, db3, off);
        lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
    }
    if (lane == 0) {
        s_scalar[warp][0] = db3;
        s_scalar[warp][1] = lsum;
    }
    if (!ok) {
        if (tid == 0) atomicOr(error, kErrTensorWait);
        wait_parity(&bar, phase, kWaitLimit);
    }
    fence_before();
    __syncthreads();
    if (tid == 0) {
        grad->b3 = s_scalar[0][0] + s_scalar[1][0] + s_scalar[2][0] + s_scalar[3][0];
        grad->pad[0] = grad->pad[1] = grad->pad[2] = 0.f;
        *loss_sum = s_scalar[0][1] + s_scalar[1][1] + s_scalar[2][1] + s_scalar[3][1];
    }
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kGradTmemColumns)
                     : "memory");
    return ok;
}

}  // namespace tc
}  // namespace faco

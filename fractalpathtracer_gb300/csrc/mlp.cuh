// mlp.cuh -- the learned distance surrogate: layout, features and the
// per-warp bf16 tensor-core forward pass (mma.sync m16n8k16, FP32 accumulate).
//
// Network: 3-D point -> 99 Fourier features (the normalised point and
// sin/cos of pi * f_k * u_i for 16 log-spaced frequencies f_k = 2^(6k/15))
// -> 4 hidden layers of 64 SiLU units -> 1 output (distance / label_scale).
// BF16 weights and activations, FP32 accumulation.  Training evaluates SiLU
// with an f32 tanh; inference takes the sigmoid from a packed f16x2 tanh.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace fpt {
namespace mlp {

constexpr int kFreq = 16;
constexpr int kIn = 3 + 3 * 2 * kFreq;      // 99 features
constexpr int kInPad = 112;                 // K of layer 0, a multiple of 16
constexpr int kHid = 64;
constexpr int kHidden = 4;                  // hidden layers
// Row strides in shared memory (elements): +8 bf16 keeps ldmatrix rows on distinct banks.
constexpr int kStrideIn = kInPad + 8;       // 120
constexpr int kStrideH = kHid + 8;          // 72

// Parameter offsets (floats, master copy): W0[64x112] b0[64] W1[64x64] b1 W2 b2 W3 b3 W4[64] b4[1].
constexpr int kW0 = 0;
constexpr int kB0 = kW0 + kHid * kInPad;
constexpr int kW1 = kB0 + kHid;
constexpr int kB1 = kW1 + kHid * kHid;
constexpr int kW2 = kB1 + kHid;
constexpr int kB2 = kW2 + kHid * kHid;
constexpr int kW3 = kB2 + kHid;
constexpr int kB3 = kW3 + kHid * kHid;
constexpr int kW4 = kB3 + kHid;
constexpr int kB4 = kW4 + kHid;
constexpr int kParams = kB4 + 1;            // 19777 (padded W0 columns stay zero)

__host__ __device__ inline int w_offset(int layer) { return layer == 0 ? kW0 : (layer == 1 ? kW1 : (layer == 2 ? kW2 : kW3)); }
__host__ __device__ inline int b_offset(int layer) { return layer == 0 ? kB0 : (layer == 1 ? kB1 : (layer == 2 ? kB2 : kB3)); }
__host__ __device__ inline int k_of(int layer) { return layer == 0 ? kInPad : kHid; }

// Shared-memory image of the weights: padded rows, bf16.
struct SmemWeights {
    __nv_bfloat16 w0[kHid * kStrideIn];
    __nv_bfloat16 w[3][kHid * kStrideH];
    float b[kHidden][kHid];
    float w4[kHid];
    float b4;
};

// Device view of a trained model used by the surrogate march.
struct Model {
    const __nv_bfloat16 *wbf;   // kParams bf16 (same layout as the master copy)
    const float *params;        // kParams fp32 master copy (biases and W4 read from here)
    float center[3], inv_half[3];
    float label_scale;          // distance = output * label_scale
};

__host__ __device__ inline float frequency(int k) { return exp2f(6.0f * float(k) / 15.0f); }

// Features of one point, written to a bf16 row (kInPad entries, zero padded):
// u, then (sin, cos)(pi f_k u_i) for k = 0..15, i = 0..2.  f_{k+5} = 4 f_k,
// so only k = 0..4 take sin/cos; the rest follow by two double-angle steps
// (sin 2a = 2 sin a cos a, cos 2a = 1 - 2 sin^2 a).
__device__ __forceinline__ void features(const float u[3], __nv_bfloat16 *row) {
    row[0] = __float2bfloat16_rn(u[0]);
    row[1] = __float2bfloat16_rn(u[1]);
    row[2] = __float2bfloat16_rn(u[2]);
#pragma unroll
    for (int r = 0; r < 5; ++r) {
        const float f = 3.14159265358979f * exp2f(0.4f * float(r));
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            float s, c;
            __sincosf(f * u[i], &s, &c);
#pragma unroll
            for (int k = r; k < kFreq; k += 5) {
                row[3 + (k * 3 + i) * 2] = __float2bfloat16_rn(s);
                row[3 + (k * 3 + i) * 2 + 1] = __float2bfloat16_rn(c);
#pragma unroll
                for (int q = 0; q < 2; ++q) {   // angle x 4
                    float s2 = 2.0f * s * c, c2 = 1.0f - 2.0f * s * s;
                    s = s2;
                    c = c2;
                }
            }
        }
    }
#pragma unroll
    for (int j = kIn; j < kInPad; ++j) row[j] = __float2bfloat16_rn(0.0f);
}

// SiLU(z) = z sigmoid(z), sigmoid(z) = (1 + tanh(z/2)) / 2: one MUFU op.
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sigmoid_fast(float z) { return fmaf(0.5f, tanh_approx(0.5f * z), 0.5f); }
__device__ __forceinline__ float silu(float z) { return z * sigmoid_fast(z); }
__device__ __forceinline__ float silu_grad(float z) {
    float s = sigmoid_fast(z);
    return s + z * s * (1.0f - s);
}

// ---------------------------------------------------------------- mma helpers
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void ldmatrix_x4(uint32_t r[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p))
                 : "memory");
}
__device__ __forceinline__ void ldmatrix_x4_trans(uint32_t r[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p))
                 : "memory");
}
__device__ __forceinline__ void ldmatrix_x2(uint32_t r[2], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(smem_addr(p)) : "memory");
}
__device__ __forceinline__ void ldmatrix_x2_trans(uint32_t r[2], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(smem_addr(p)) : "memory");
}
// D = A(16x16 bf16, row) * B(16x8 bf16, col) + D (fp32)
__device__ __forceinline__ void mma16816(float d[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// A fragment (16x16) from a row-major bf16 tile: rows r0.., columns k0..
__device__ __forceinline__ void load_a(uint32_t a[4], const __nv_bfloat16 *base, int stride, int r0, int k0, int lane) {
    const __nv_bfloat16 *p = base + (r0 + (lane & 15)) * stride + k0 + ((lane >> 4) << 3);
    ldmatrix_x4(a, p);
}
// A fragment of the transpose: A(m, k) = S[k][m] with S row-major [K x M].
__device__ __forceinline__ void load_a_trans(uint32_t a[4], const __nv_bfloat16 *base, int stride, int m0, int k0, int lane) {
    int j = lane >> 3, r = lane & 7;
    // matrices: (m0..7,k0..7) (m8..15,k0..7) (m0..7,k8..15) (m8..15,k8..15)
    const __nv_bfloat16 *p = base + (k0 + ((j >> 1) << 3) + r) * stride + m0 + ((j & 1) << 3);
    ldmatrix_x4_trans(a, p);
}
// B fragment (16x8) from W row-major [N x K] (B(k, n) = W[n][k]): rows n0..n0+7, columns k0..k0+15.
__device__ __forceinline__ void load_b_nk(uint32_t b[2], const __nv_bfloat16 *base, int stride, int n0, int k0, int lane) {
    int l = lane & 15;
    const __nv_bfloat16 *p = base + (n0 + (l & 7)) * stride + k0 + ((l >> 3) << 3);
    ldmatrix_x2(b, p);
}
// B fragment from S row-major [K x N] (B(k, n) = S[k][n]).
__device__ __forceinline__ void load_b_kn(uint32_t b[2], const __nv_bfloat16 *base, int stride, int n0, int k0, int lane) {
    int l = lane & 15;
    const __nv_bfloat16 *p = base + (k0 + l) * stride + n0;
    ldmatrix_x2_trans(b, p);
}

// Loads the bf16 weights of a model into shared memory (all threads of the block).
__device__ __forceinline__ void load_weights(SmemWeights &sw, const Model &M) {
    for (int i = threadIdx.x; i < kHid * kInPad; i += blockDim.x) {
        int n = i / kInPad, k = i - n * kInPad;
        sw.w0[n * kStrideIn + k] = M.wbf[kW0 + i];
    }
    for (int l = 1; l < kHidden; ++l)
        for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x) {
            int n = i / kHid, k = i - n * kHid;
            sw.w[l - 1][n * kStrideH + k] = M.wbf[w_offset(l) + i];
        }
    for (int i = threadIdx.x; i < kHidden * kHid; i += blockDim.x) sw.b[i / kHid][i % kHid] = M.params[b_offset(i / kHid) + i % kHid];
    for (int i = threadIdx.x; i < kHid; i += blockDim.x) sw.w4[i] = __bfloat162float(M.wbf[kW4 + i]);
    if (threadIdx.x == 0) sw.b4 = M.params[kB4];
}

// One dense layer for the warp's 32 rows: Z = H * W^T + b.  `hin` holds the
// input rows (row-major, stride sin), `w` the weights [64 x K] (stride swd).
// Writes SiLU(Z) (bf16) to hout (stride kStrideH) and, if zout, Z (bf16,
// row stride zstride; shared or global memory).  All reads of hin happen
// before the first write, so hout may alias hin.
template <int K>
__device__ __forceinline__ void dense_layer(const __nv_bfloat16 *hin, int sin, const __nv_bfloat16 *w, int swd, const float *bias,
                                            __nv_bfloat16 *zout, int zstride, __nv_bfloat16 *hout, int lane) {
    float acc[2][8][4];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int n = 0; n < 8; ++n)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[m][n][q] = 0.0f;
#pragma unroll
    for (int k0 = 0; k0 < K; k0 += 16) {
        uint32_t a[2][4];
        load_a(a[0], hin, sin, 0, k0, lane);
        load_a(a[1], hin, sin, 16, k0, lane);
#pragma unroll
        for (int n = 0; n < 8; ++n) {
            uint32_t b[2];
            load_b_nk(b, w, swd, n * 8, k0, lane);
            mma16816(acc[0][n], a[0], b);
            mma16816(acc[1][n], a[1], b);
        }
    }
    __syncwarp();
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int n = 0; n < 8; ++n)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                int row = m * 16 + g + h * 8, col = n * 8 + t * 2;
                float z0 = acc[m][n][h * 2] + bias[col], z1 = acc[m][n][h * 2 + 1] + bias[col + 1];
                __nv_bfloat162 hz = __floats2bfloat162_rn(silu(z0), silu(z1));
                *reinterpret_cast<__nv_bfloat162 *>(hout + row * kStrideH + col) = hz;
                if (zout) *reinterpret_cast<__nv_bfloat162 *>(zout + size_t(row) * zstride + col) = __floats2bfloat162_rn(z0, z1);
            }
    __syncwarp();
}

// Per-warp scratch of the forward pass: the 32 feature rows (layer 0 reads
// them through ldmatrix; the hidden layers stay in registers).
struct WarpForward {
    __nv_bfloat16 x[32 * kStrideIn];
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

// SiLU of two values for inference, from their halves h = z / 2:
// z sigmoid(z) = h + h tanh(h), with the tanh from one packed f16x2 MUFU op
// (half the MUFU work of two f32 tanh) and h, the product and the rounding
// to BF16 in f32.  A caller that adds a bias first can pass
// fmaf(z, 0.5, b / 2), which equals (z + b) / 2 exactly.
__device__ __forceinline__ uint32_t silu2_bf16_half(float h0, float h1) {
    const __half2 hh = __floats2half2_rn(h0, h1);
    uint32_t t;
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(*reinterpret_cast<const uint32_t *>(&hh)));
    const float2 tf = __half22float2(*reinterpret_cast<const __half2 *>(&t));
    return pack_bf16(fmaf(h0, tf.x, h0), fmaf(h1, tf.y, h1));
}
__device__ __forceinline__ uint32_t silu2_bf16(float z0, float z1) { return silu2_bf16_half(0.5f * z0, 0.5f * z1); }

// SiLU epilogue that turns the accumulators of a 32 x 64 layer output (two
// m16 tiles x eight n8 tiles) into the A fragments of the next layer's
// m16n8k16 products: n-tiles 2kb and 2kb+1 hold exactly the (row, k) pairs of
// k-block kb (row g: c0 c1, row g+8: c2 c3), so no shared memory is needed.
__device__ __forceinline__ void silu_to_fragments(const float acc[2][8][4], const float *bias, uint32_t a[2][4][4], int lane) {
    const int t = lane & 3;
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int n = 0; n < 8; ++n) {
            const int col = n * 8 + t * 2;
            const float b0 = bias[col], b1 = bias[col + 1];
            a[m][n >> 1][(n & 1) * 2 + 0] = silu2_bf16(acc[m][n][0] + b0, acc[m][n][1] + b1);
            a[m][n >> 1][(n & 1) * 2 + 1] = silu2_bf16(acc[m][n][2] + b0, acc[m][n][3] + b1);
        }
}

// acc = A (registers, 32 x 64) x W^T, W [64 x 64] in shared memory.
__device__ __forceinline__ void hidden_product(const uint32_t a[2][4][4], const __nv_bfloat16 *w, float acc[2][8][4], int lane) {
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int n = 0; n < 8; ++n)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[m][n][q] = 0.0f;
#pragma unroll
    for (int kb = 0; kb < 4; ++kb)
#pragma unroll
        for (int n = 0; n < 8; ++n) {
            uint32_t b[2];
            load_b_nk(b, w, kStrideH, n * 8, kb * 16, lane);
            mma16816(acc[0][n], a[0][kb], b);
            mma16816(acc[1][n], a[1][kb], b);
        }
}

// Forward pass of 32 points (one per lane, normalised coordinates u); returns
// this lane's output (in label units).  All lanes of the warp must call it.
__device__ __forceinline__ float forward32(const SmemWeights &sw, WarpForward &wf, const float u[3], int lane) {
    features(u, wf.x + lane * kStrideIn);
    __syncwarp();
    float acc[2][8][4];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int n = 0; n < 8; ++n)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[m][n][q] = 0.0f;
#pragma unroll
    for (int k0 = 0; k0 < kInPad; k0 += 16) {
        uint32_t a0[4], a1[4];
        load_a(a0, wf.x, kStrideIn, 0, k0, lane);
        load_a(a1, wf.x, kStrideIn, 16, k0, lane);
#pragma unroll
        for (int n = 0; n < 8; ++n) {
            uint32_t b[2];
            load_b_nk(b, sw.w0, kStrideIn, n * 8, k0, lane);
            mma16816(acc[0][n], a0, b);
            mma16816(acc[1][n], a1, b);
        }
    }
    __syncwarp();   // the feature rows may be rewritten by the next call
    uint32_t a[2][4][4];
    silu_to_fragments(acc, sw.b[0], a, lane);
#pragma unroll
    for (int l = 0; l < 2; ++l) {
        hidden_product(a, sw.w[l], acc, lane);
        silu_to_fragments(acc, sw.b[l + 1], a, lane);
    }
    hidden_product(a, sw.w[2], acc, lane);
    // Output layer: per-row dot product of the (bf16-rounded) last activations
    // with W4, reduced over the quad that holds the row.
    const int t = lane & 3;
    float part[2][2] = {{0.0f, 0.0f}, {0.0f, 0.0f}};
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int n = 0; n < 8; ++n) {
            const int col = n * 8 + t * 2;
            const float b0 = sw.b[3][col], b1 = sw.b[3][col + 1], w0 = sw.w4[col], w1 = sw.w4[col + 1];
            const uint32_t hlo = silu2_bf16(acc[m][n][0] + b0, acc[m][n][1] + b1);
            const uint32_t hhi = silu2_bf16(acc[m][n][2] + b0, acc[m][n][3] + b1);
            const float h0 = __uint_as_float(hlo << 16), h1 = __uint_as_float(hlo & 0xffff0000u);
            const float h2 = __uint_as_float(hhi << 16), h3 = __uint_as_float(hhi & 0xffff0000u);
            part[m][0] += h0 * w0 + h1 * w1;
            part[m][1] += h2 * w0 + h3 * w1;
        }
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            part[m][h] += __shfl_xor_sync(0xffffffffu, part[m][h], 1);
            part[m][h] += __shfl_xor_sync(0xffffffffu, part[m][h], 2);
        }
    // lane L holds row L: m-tile L / 16, row (L % 16) = g + 8 h, held by lane 4 g
    const int src = (lane & 7) * 4;
    const float v00 = __shfl_sync(0xffffffffu, part[0][0], src), v01 = __shfl_sync(0xffffffffu, part[0][1], src);
    const float v10 = __shfl_sync(0xffffffffu, part[1][0], src), v11 = __shfl_sync(0xffffffffu, part[1][1], src);
    const bool upper = (lane & 8) != 0;
    const float dot = lane < 16 ? (upper ? v01 : v00) : (upper ? v11 : v10);
    return sw.b4 + dot;
}

}  // namespace mlp
}  // namespace fpt

// mlp.cu -- training and inference of the learned distance surrogate on sm_103a.
//
// Training data: points labelled by the scene's exact distance estimator
// (mapSdf), a share uniform in the model's box and the rest within
// `near_band` of the surface (rejection sampling on the GPU).  Loss:
// asymmetric squared error, overestimates weighted by `overestimate_weight`.
// Optimiser: Adam on an FP32 master copy; BF16 weights and activations in the
// tensor-core passes (FP32 accumulate):
//   train_fwd_bwd_kernel   per warp 32 samples (mma.sync m16n8k16): forward
//                          through the 4 hidden layers, loss, backward deltas
//                          (W products through transposed ldmatrix); writes
//                          features, activations, pre-activations and deltas
//                          (bf16), and per warp its output-layer gradient and
//                          loss sums
//   wgrad_tc_kernel        tcgen05: per (layer, 512-row chunk of the batch)
//                          D = H^T dZ, a 128 x 64 FP32 accumulator in tensor
//                          memory; a row of ones in H^T gives the bias
//                          gradient in the same MMAs
//   wgrad_reduce_kernel,   the chunks' and warps' partial sums added in a
//   out_reduce_kernel      fixed order: gradients and loss are deterministic
//   adam_kernel
// The skip march that uses the model is in skip.cuh (one instantiation per
// scene kind).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "bridge_internal.h"
#include "fpt_kernels.h"
#include "fpt_math.cuh"
#include "mlp.cuh"
#include "mlp_tc.cuh"
#include "skip.cuh"

namespace fpt {
namespace mlp {

constexpr int kWarpsTrain = 4;                 // 128 samples per block
constexpr uint32_t kRowsPerBlock = 32u * kWarpsTrain;
constexpr uint32_t kOutPart = kHid + 2;        // per warp of the training kernel: dW4[64], db4, loss

// Shared scratch of one warp in the training kernel.
struct WarpTrain {
    __nv_bfloat16 buf[32 * kStrideIn];         // features, then each layer's activations (in place)
    __nv_bfloat16 d[2][32 * kStrideH];         // deltas (ping-pong)
};

struct TrainArgs {
    const float4 *data;        // xyz point, w label (distance)
    uint32_t n_data;
    uint32_t batch;
    uint32_t step;
    uint32_t seed;
    int identity;              // row r reads data[r] (gradient checks)
    float inv_label_scale;
    float over_weight;
    Model model;
    __nv_bfloat16 *gx;         // [rows x kInPad] features
    __nv_bfloat16 *gh[3];      // H1..H3 [rows x kHid]
    __nv_bfloat16 *gz[4];      // Z1..Z4 [rows x kHid]
    __nv_bfloat16 *gdz[4];     // dZ1..dZ4 [rows x kHid]
    float *grad;               // kParams gradients (accumulated)
    float *loss;               // sum of the batch loss (accumulated)
    float *out_part;           // per warp kOutPart partial sums (output layer and loss)
    float *w_part;             // wgrad_tc_kernel partials
    uint32_t *fail;            // MMA time-out word of the tensor-core passes
};

__device__ __forceinline__ uint32_t hash2(uint32_t a, uint32_t b) { return pcg_hash(a ^ pcg_hash(b)); }

// dZ_l = (dZ_{l+1} W_l) o SiLU'(Z_l) for the warp's 32 rows; Z_l is read from
// global memory (row stride kHid).
__device__ __forceinline__ void backprop_layer(const __nv_bfloat16 *dz_next, const __nv_bfloat16 *w, const __nv_bfloat16 *zg,
                                               __nv_bfloat16 *dz_out, int lane) {
    float acc[2][8][4];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int n = 0; n < 8; ++n)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[m][n][q] = 0.0f;
#pragma unroll
    for (int k0 = 0; k0 < kHid; k0 += 16) {
        uint32_t a[2][4];
        load_a(a[0], dz_next, kStrideH, 0, k0, lane);
        load_a(a[1], dz_next, kStrideH, 16, k0, lane);
#pragma unroll
        for (int n = 0; n < 8; ++n) {
            uint32_t b[2];
            load_b_kn(b, w, kStrideH, n * 8, k0, lane);   // B(k = j, n = i) = W[j][i]
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
            for (int hh = 0; hh < 2; ++hh) {
                int row = m * 16 + g + hh * 8, col = n * 8 + t * 2;
                __nv_bfloat162 zz = *reinterpret_cast<const __nv_bfloat162 *>(zg + size_t(row) * kHid + col);
                float d0 = acc[m][n][hh * 2] * silu_grad(__bfloat162float(zz.x));
                float d1 = acc[m][n][hh * 2 + 1] * silu_grad(__bfloat162float(zz.y));
                *reinterpret_cast<__nv_bfloat162 *>(dz_out + row * kStrideH + col) = __floats2bfloat162_rn(d0, d1);
            }
    __syncwarp();
}

// Copies the warp's 32 rows (cols columns) from shared to global memory.
__device__ __forceinline__ void store_rows(__nv_bfloat16 *g, int gstride, const __nv_bfloat16 *s, int sstride, int cols,
                                           uint32_t row0, int lane) {
    for (int r = 0; r < 32; ++r)
        for (int c = lane * 2; c < cols; c += 64)
            *reinterpret_cast<__nv_bfloat162 *>(g + size_t(row0 + r) * gstride + c) =
                *reinterpret_cast<const __nv_bfloat162 *>(s + r * sstride + c);
}

__global__ void __launch_bounds__(32 * kWarpsTrain, 2) train_fwd_bwd_kernel(TrainArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemWeights &sw = *reinterpret_cast<SmemWeights *>(smem_raw);
    WarpTrain *wt_all = reinterpret_cast<WarpTrain *>(smem_raw + ((sizeof(SmemWeights) + 127) & ~size_t(127)));
    load_weights(sw, A.model);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpTrain &wt = wt_all[warp];
    const uint32_t row0 = (blockIdx.x * kWarpsTrain + warp) * 32u;
    const uint32_t row = row0 + lane;
    const bool valid = row < A.batch;
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) s = A.data[A.identity ? row : hash2(A.seed + A.step * 7919u, row) % A.n_data];
    const Model &M = A.model;
    float u[3] = {(s.x - M.center[0]) * M.inv_half[0], (s.y - M.center[1]) * M.inv_half[1], (s.z - M.center[2]) * M.inv_half[2]};
    features(u, wt.buf + lane * kStrideIn);
    __syncwarp();
    store_rows(A.gx, kInPad, wt.buf, kStrideIn, kInPad, row0, lane);
    // forward: H_{l+1} = SiLU(H_l W_l^T + b_l), Z kept in global memory
    dense_layer<kInPad>(wt.buf, kStrideIn, sw.w0, kStrideIn, sw.b[0], A.gz[0] + size_t(row0) * kHid, kHid, wt.buf, lane);
    store_rows(A.gh[0], kHid, wt.buf, kStrideH, kHid, row0, lane);
    dense_layer<kHid>(wt.buf, kStrideH, sw.w[0], kStrideH, sw.b[1], A.gz[1] + size_t(row0) * kHid, kHid, wt.buf, lane);
    store_rows(A.gh[1], kHid, wt.buf, kStrideH, kHid, row0, lane);
    dense_layer<kHid>(wt.buf, kStrideH, sw.w[1], kStrideH, sw.b[2], A.gz[2] + size_t(row0) * kHid, kHid, wt.buf, lane);
    store_rows(A.gh[2], kHid, wt.buf, kStrideH, kHid, row0, lane);
    dense_layer<kHid>(wt.buf, kStrideH, sw.w[2], kStrideH, sw.b[3], A.gz[3] + size_t(row0) * kHid, kHid, wt.buf, lane);
    const __nv_bfloat16 *h4 = wt.buf + lane * kStrideH;
    float out = sw.b4;
    for (int j = 0; j < kHid; ++j) out += __bfloat162float(h4[j]) * sw.w4[j];
    // asymmetric loss: weight over_weight on overestimates
    const float y = s.w * A.inv_label_scale;
    const float e = out - y;
    const float wgt = e > 0.0f ? A.over_weight : 1.0f;
    const float dout = valid ? 2.0f * wgt * e / float(A.batch) : 0.0f;
    float loss = valid ? wgt * e * e : 0.0f;
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    // output layer: dW4[j] = sum_b dout_b H4[b][j], db4 = sum_b dout_b; the warp's sums go to its
    // partial row (out_reduce_kernel adds the warps in order)
    float *part = A.out_part + size_t(blockIdx.x * kWarpsTrain + warp) * kOutPart;
    for (int j = 0; j < kHid; ++j) {
        float v = dout * __bfloat162float(h4[j]);
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) part[j] = v;
    }
    {
        float v = dout;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) {
            part[kHid] = v;
            part[kHid + 1] = loss;
        }
    }
    __syncwarp();   // Z4 rows written by other lanes are visible from here
    // dZ4 = dout W4 o SiLU'(Z4)
    const __nv_bfloat16 *z4 = A.gz[3] + size_t(row) * kHid;
    for (int j = 0; j < kHid; j += 2) {
        __nv_bfloat162 zz = *reinterpret_cast<const __nv_bfloat162 *>(z4 + j);
        float d0 = dout * sw.w4[j] * silu_grad(__bfloat162float(zz.x));
        float d1 = dout * sw.w4[j + 1] * silu_grad(__bfloat162float(zz.y));
        *reinterpret_cast<__nv_bfloat162 *>(wt.d[0] + lane * kStrideH + j) = __floats2bfloat162_rn(d0, d1);
    }
    __syncwarp();
    store_rows(A.gdz[3], kHid, wt.d[0], kStrideH, kHid, row0, lane);
    // hidden layers 3, 2, 1
    int cur = 0;
    for (int l = 3; l >= 1; --l) {
        backprop_layer(wt.d[cur], sw.w[l - 1], A.gz[l - 1] + size_t(row0) * kHid, wt.d[cur ^ 1], lane);
        cur ^= 1;
        store_rows(A.gdz[l - 1], kHid, wt.d[cur], kStrideH, kHid, row0, lane);
    }
}

// ---------------------------------------------------------------- forward + backward on tcgen05
// The training pass of train_fwd_bwd_kernel with its products on the
// 5th-generation tensor cores: 128 rows per CTA, one row per thread, the
// M = 128, N = 64, K = 16 MMA shape of the inference pass.  Forward: per
// layer H_l x W_l^T into a 128 x 64 FP32 accumulator in tensor memory; each
// thread reads its row, adds the bias, stores Z_l (bf16) and H_{l+1} =
// SiLU(Z_l) (bf16) to global memory and into the next layer's operand tile.
// Backward: dZ_4 = dout W4 o SiLU'(Z_4) per row, then dZ_l = (dZ_{l+1} W_l) o
// SiLU'(Z_l) with B = W_l^T staged at set-up.  Same arithmetic as the
// mma.sync pass (BF16 operands, FP32 accumulation, SiLU and its derivative on
// the FP32 pre-activation / its bf16 copy); only the order of the FP32 sums
// differs.
// Two floats as a packed pair of bf16 (lo in the low half).
__device__ __forceinline__ uint32_t bf16_pair(float lo, float hi) {
    return uint32_t(__bfloat16_as_ushort(__float2bfloat16_rn(lo))) | (uint32_t(__bfloat16_as_ushort(__float2bfloat16_rn(hi))) << 16);
}

struct TrainTcSmem {
    alignas(128) unsigned char act[kTcRows * kInPad * 2];        // operand A: features, activations, then deltas
    alignas(128) unsigned char w0[kHid * kInPad * 2];            // forward B of layer 0: W0[n][k]
    alignas(128) unsigned char w[kHidden - 1][kHid * kHid * 2];  // forward B: W_l[n][k]
    alignas(128) unsigned char wt[kHidden - 1][kHid * kHid * 2]; // backward B: W_l^T, element (k, n) = W_l[n][k]
    float b[kHidden][kHid];
    float w4[kHid];
    float b4;
    uint32_t tmem;
    alignas(8) uint64_t bar;
    unsigned char slack[4096];
};
inline size_t train_tc_smem_bytes() { return sizeof(TrainTcSmem); }

// One round of MMAs (A = the act tile with K = k columns, B at `b`) into the
// accumulator; every thread then holds its row in r.  False when the MMAs did
// not complete within kMmaWaitNs (the same in every thread).
__device__ __forceinline__ bool train_round(TrainTcSmem &sm, uint32_t b, int k, uint32_t &phase, uint32_t r[64]) {
    const int t = threadIdx.x;
    const uint32_t act = umma::smem_u32(sm.act);
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    if (t == 0) {
        umma::fence_after_sync();
        for (int j = 0; j < k / 16; ++j)
            umma::mma_bf16(sm.tmem, umma::smem_desc(act + uint32_t(j) * 2u * kActK, kActK, kCore),
                           umma::smem_desc(b + uint32_t(j) * 2u * kWK, kWK, kCore), kTcIdesc, uint32_t(j));
        umma::mma_commit(&sm.bar);
    }
    const int late = t == 0 ? int(!umma::mbar_wait(&sm.bar, phase, kMmaWaitNs)) : 0;
    phase ^= 1u;
    if (__syncthreads_or(late)) return false;
    umma::fence_after_sync();
    __syncwarp();
    umma::tmem_ld64(sm.tmem + (uint32_t(t & ~31) << 16), r);
    return true;
}

__device__ __forceinline__ void store_row64(__nv_bfloat16 *g, const uint32_t h[32]) {
    uint4 *d = reinterpret_cast<uint4 *>(g);
#pragma unroll
    for (int q = 0; q < 8; ++q) d[q] = make_uint4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
}

__global__ void __launch_bounds__(kTcRows) train_fwd_bwd_tc_kernel(TrainArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainTcSmem &sm = *reinterpret_cast<TrainTcSmem *>(smem_raw);
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const Model &M = A.model;
    if (__syncthreads_or(t == 0 && *reinterpret_cast<volatile uint32_t *>(A.fail) != 0u)) return;   // an earlier launch timed out
    for (int i = t; i < kHid * kInPad; i += kTcRows) {
        const int n = i / kInPad, k = i - n * kInPad;
        *reinterpret_cast<__nv_bfloat16 *>(sm.w0 + w_core_offset(n, k)) = M.wbf[kW0 + i];
    }
    for (int l = 1; l < kHidden; ++l)
        for (int i = t; i < kHid * kHid; i += kTcRows) {
            const int n = i / kHid, k = i - n * kHid;
            *reinterpret_cast<__nv_bfloat16 *>(sm.w[l - 1] + w_core_offset(n, k)) = M.wbf[w_offset(l) + i];
            *reinterpret_cast<__nv_bfloat16 *>(sm.wt[l - 1] + w_core_offset(k, n)) = M.wbf[w_offset(l) + i];
        }
    for (int i = t; i < kHidden * kHid; i += kTcRows) sm.b[i / kHid][i % kHid] = M.params[b_offset(i / kHid) + i % kHid];
    for (int i = t; i < kHid; i += kTcRows) sm.w4[i] = __bfloat162float(M.wbf[kW4 + i]);
    if (t == 0) {
        sm.b4 = M.params[kB4];
        umma::mbar_init(&sm.bar, 1u);
    }
    if (t < 32) {
        __syncwarp();
        umma::tmem_alloc(&sm.tmem, kTcCols);
        umma::tmem_relinquish();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t act = umma::smem_u32(sm.act);
    const uint32_t row = blockIdx.x * kTcRows + uint32_t(t);
    const bool valid = row < A.batch;
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    if (valid) s = A.data[A.identity ? row : hash2(A.seed + A.step * 7919u, row) % A.n_data];
    {
        const float u[3] = {(s.x - M.center[0]) * M.inv_half[0], (s.y - M.center[1]) * M.inv_half[1], (s.z - M.center[2]) * M.inv_half[2]};
        uint32_t f[kInPad / 2];
        feature_pairs(u, f);
#pragma unroll
        for (int kc = 0; kc < kInPad / 8; ++kc) umma::st_shared_v4(act + act_offset(t, kc), f[4 * kc], f[4 * kc + 1], f[4 * kc + 2], f[4 * kc + 3]);
        uint4 *gx = reinterpret_cast<uint4 *>(A.gx + size_t(row) * kInPad);
#pragma unroll
        for (int q = 0; q < kInPad / 8; ++q) gx[q] = make_uint4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
    }
    uint32_t phase = 0, r[64], h[32];
    bool ok = true;
    float dout = 0.0f, loss = 0.0f;
    // forward
    for (int L = 0; L < kHidden && ok; ++L) {
        ok = train_round(sm, umma::smem_u32(L == 0 ? sm.w0 : sm.w[L - 1]), L == 0 ? kInPad : kHid, phase, r);
        if (!ok) break;
        uint32_t z[32];
#pragma unroll
        for (int c = 0; c < kHid; c += 2) {
            const float z0 = __uint_as_float(r[c]) + sm.b[L][c], z1 = __uint_as_float(r[c + 1]) + sm.b[L][c + 1];
            z[c >> 1] = bf16_pair(z0, z1);
            h[c >> 1] = bf16_pair(silu(z0), silu(z1));
        }
        store_row64(A.gz[L] + size_t(row) * kHid, z);
        if (L + 1 < kHidden) {
            store_row64(A.gh[L] + size_t(row) * kHid, h);
#pragma unroll
            for (int kc = 0; kc < kHid / 8; ++kc) umma::st_shared_v4(act + act_offset(t, kc), h[4 * kc], h[4 * kc + 1], h[4 * kc + 2], h[4 * kc + 3]);
        }
    }
    if (ok) {
        // output layer, loss, dZ4 (h holds H4, r + bias the FP32 Z4)
        float out = sm.b4;
#pragma unroll
        for (int c = 0; c < kHid; c += 2) {
            out += __uint_as_float(h[c >> 1] << 16) * sm.w4[c];
            out += __uint_as_float(h[c >> 1] & 0xffff0000u) * sm.w4[c + 1];
        }
        const float y = s.w * A.inv_label_scale;
        const float e = out - y;
        const float wgt = e > 0.0f ? A.over_weight : 1.0f;
        dout = valid ? 2.0f * wgt * e / float(A.batch) : 0.0f;
        loss = valid ? wgt * e * e : 0.0f;
        float *part = A.out_part + size_t(blockIdx.x * (kTcRows / 32) + warp) * kOutPart;
        for (int c = 0; c < kHid; ++c) {
            const uint32_t hb = (c & 1) ? (h[c >> 1] & 0xffff0000u) : (h[c >> 1] << 16);
            float v = dout * __uint_as_float(hb);
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) part[c] = v;
        }
        {
            float v = dout, lv = loss;
            for (int o = 16; o > 0; o >>= 1) {
                v += __shfl_xor_sync(0xffffffffu, v, o);
                lv += __shfl_xor_sync(0xffffffffu, lv, o);
            }
            if (lane == 0) {
                part[kHid] = v;
                part[kHid + 1] = lv;
            }
        }
        uint32_t d[32];
#pragma unroll
        for (int c = 0; c < kHid; c += 2) {
            const float z0 = __bfloat162float(__float2bfloat16_rn(__uint_as_float(r[c]) + sm.b[3][c]));
            const float z1 = __bfloat162float(__float2bfloat16_rn(__uint_as_float(r[c + 1]) + sm.b[3][c + 1]));
            d[c >> 1] = bf16_pair(dout * sm.w4[c] * silu_grad(z0), dout * sm.w4[c + 1] * silu_grad(z1));
        }
        store_row64(A.gdz[3] + size_t(row) * kHid, d);
#pragma unroll
        for (int kc = 0; kc < kHid / 8; ++kc) umma::st_shared_v4(act + act_offset(t, kc), d[4 * kc], d[4 * kc + 1], d[4 * kc + 2], d[4 * kc + 3]);
    }
    // backward through hidden layers 3, 2, 1: dZ_l = (dZ_{l+1} W_l) o SiLU'(Z_l)
    for (int l = kHidden - 1; l >= 1 && ok; --l) {
        ok = train_round(sm, umma::smem_u32(sm.wt[l - 1]), kHid, phase, r);
        if (!ok) break;
        const uint4 *zg = reinterpret_cast<const uint4 *>(A.gz[l - 1] + size_t(row) * kHid);
        uint32_t d[32];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const uint4 zz = zg[q];
            const uint32_t zw[4] = {zz.x, zz.y, zz.z, zz.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int c = q * 8 + e * 2;
                const float z0 = __uint_as_float(zw[e] << 16), z1 = __uint_as_float(zw[e] & 0xffff0000u);
                d[c >> 1] = bf16_pair(__uint_as_float(r[c]) * silu_grad(z0), __uint_as_float(r[c + 1]) * silu_grad(z1));
            }
        }
        store_row64(A.gdz[l - 1] + size_t(row) * kHid, d);
        if (l > 1) {
#pragma unroll
            for (int kc = 0; kc < kHid / 8; ++kc) umma::st_shared_v4(act + act_offset(t, kc), d[4 * kc], d[4 * kc + 1], d[4 * kc + 2], d[4 * kc + 3]);
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (t < 32) {
        __syncwarp();
        umma::fence_after_sync();
        umma::tmem_dealloc(sm.tmem, kTcCols);
    }
    if (!ok && t == 0) atomicOr(A.fail, 2u);
}

// ---------------------------------------------------------------- weight gradients on tcgen05
// For layer l and a 256-row chunk of the batch: D[m][n] = sum_b H_l[b][m] dZ_l[b][n]
// (m < K_l: dW_l[n][m]; m = K_l: a row of ones in H^T, so D[K_l][n] is the
// bias gradient db_l[n]).  A = H^T (128 x 64-row tile of the batch, K-major),
// B = dZ^T (64 x 64), the M = 128, N = 64, K = 16 MMA shape of the forward
// pass, accumulated over the chunk in one 64-column tensor-memory tile.  Each
// CTA writes its 128 x 64 partial; wgrad_reduce_kernel adds the chunks in
// order (no atomics: the same data gives the same bits).
constexpr uint32_t kWgChunk = 256;            // batch rows per CTA
constexpr uint32_t kWgTile = 64;              // batch rows per round of 4 MMAs
struct WgSmem {
    alignas(128) unsigned char a[kTcRows * kWgTile * 2];   // H^T tile, [k chunk][m group][8 m][8 k]
    alignas(128) unsigned char b[kHid * kWgTile * 2];      // dZ^T tile, [k chunk][n group][8 n][8 k]
    uint32_t tmem;
    alignas(8) uint64_t bar;
    unsigned char slack[4096];                             // keeps descriptor reads inside the CTA's shared memory
};
inline size_t wgrad_smem_bytes() { return sizeof(WgSmem); }

struct WgradArgs {
    const __nv_bfloat16 *h[kHidden];     // H_0 = features (kInPad columns), H_1..H_3 (kHid columns)
    const __nv_bfloat16 *dz[kHidden];    // dZ_1..dZ_4 (kHid columns)
    uint32_t batch, chunks;
    float *part;                         // [layer][chunk][128][64] partial sums
    uint32_t *fail;                      // set (bit 2) when an MMA does not complete in time; later launches skip their work
};

// Global tile loads of one round (64 batch rows): H rows as 16-byte vectors
// (8 columns each, at most 7 per thread) and dZ rows (4 per thread).
struct WgLoad {
    uint4 h[(kTcRows * kWgTile / 8 + kTcRows - 1) / kTcRows];
    uint4 dz[kHid * kWgTile / 8 / kTcRows];
};
__device__ __forceinline__ void wg_load(WgLoad &L, const __nv_bfloat16 *H, const __nv_bfloat16 *DZ, int kcols, uint32_t kb, uint32_t b1) {
    const int t = threadIdx.x, nvec = kcols / 8;
#pragma unroll
    for (int q = 0; q < int(sizeof(L.h) / sizeof(uint4)); ++q) {
        const int i = t + q * kTcRows, row = i / nvec, v = i - row * nvec;
        L.h[q] = (row < int(kWgTile) && kb + uint32_t(row) < b1)
                     ? *reinterpret_cast<const uint4 *>(H + size_t(kb + row) * kcols + v * 8)
                     : make_uint4(0u, 0u, 0u, 0u);
    }
#pragma unroll
    for (int q = 0; q < int(sizeof(L.dz) / sizeof(uint4)); ++q) {
        const int i = t + q * kTcRows, row = i >> 3, v = i & 7;
        L.dz[q] = kb + uint32_t(row) < b1 ? *reinterpret_cast<const uint4 *>(DZ + size_t(kb + row) * kHid + v * 8)
                                          : make_uint4(0u, 0u, 0u, 0u);
    }
}
// The loaded vectors into the K-major operand tiles (a transpose: each of a
// vector's 8 values goes to its own row of H^T / dZ^T), and the row of ones.
__device__ __forceinline__ void wg_store(const WgLoad &L, WgSmem &sm, int kcols, uint32_t kb, uint32_t b1) {
    const int t = threadIdx.x, nvec = kcols / 8;
#pragma unroll
    for (int q = 0; q < int(sizeof(L.h) / sizeof(uint4)); ++q) {
        const int i = t + q * kTcRows, row = i / nvec, v = i - row * nvec;
        if (row >= int(kWgTile)) continue;
        const uint32_t w[4] = {L.h[q].x, L.h[q].y, L.h[q].z, L.h[q].w};
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int m = v * 8 + e;
            *reinterpret_cast<uint16_t *>(sm.a + act_offset(m, row >> 3) + (row & 7) * 2) = uint16_t(w[e >> 1] >> ((e & 1) * 16));
        }
    }
#pragma unroll
    for (int q = 0; q < int(sizeof(L.dz) / sizeof(uint4)); ++q) {
        const int i = t + q * kTcRows, row = i >> 3, v = i & 7;
        const uint32_t w[4] = {L.dz[q].x, L.dz[q].y, L.dz[q].z, L.dz[q].w};
#pragma unroll
        for (int e = 0; e < 8; ++e)
            *reinterpret_cast<uint16_t *>(sm.b + w_core_offset(v * 8 + e, row)) = uint16_t(w[e >> 1] >> ((e & 1) * 16));
    }
    if (t < int(kWgTile))   // H^T row kcols: ones on the chunk's rows, so its product with dZ is the bias gradient
        *reinterpret_cast<uint16_t *>(sm.a + act_offset(kcols, t >> 3) + (t & 7) * 2) = kb + uint32_t(t) < b1 ? 0x3F80u : 0u;
}

__global__ void __launch_bounds__(kTcRows) wgrad_tc_kernel(WgradArgs G) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WgSmem &sm = *reinterpret_cast<WgSmem *>(smem_raw);
    const int t = threadIdx.x;
    const int layer = blockIdx.y;
    const int kcols = layer == 0 ? kInPad : kHid;
    const __nv_bfloat16 *H = G.h[layer], *DZ = G.dz[layer];
    float *out = G.part + ((size_t(layer) * G.chunks + blockIdx.x) * kTcRows + uint32_t(t)) * kHid;
    // an earlier launch gave up: no MMA here (one read, the same decision in every thread)
    if (__syncthreads_or(t == 0 && *reinterpret_cast<volatile uint32_t *>(G.fail) != 0u)) {
        for (int n = 0; n < kHid; ++n) out[n] = 0.0f;
        return;
    }
    if (t == 0) umma::mbar_init(&sm.bar, 1u);
    if (t < 32) {
        __syncwarp();
        umma::tmem_alloc(&sm.tmem, kTcCols);
        umma::tmem_relinquish();
    }
    // H^T rows above the ones row stay zero for every round
    for (int i = t; i < (kTcRows - kcols - 1) * int(kWgTile); i += kTcRows) {
        const int m = kcols + 1 + i / int(kWgTile), k = i % int(kWgTile);
        *reinterpret_cast<uint16_t *>(sm.a + act_offset(m, k >> 3) + (k & 7) * 2) = 0u;
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t a = umma::smem_u32(sm.a), bt = umma::smem_u32(sm.b);
    const uint32_t b0 = blockIdx.x * kWgChunk, b1 = min(G.batch, b0 + kWgChunk);
    uint32_t phase = 0;
    bool fail = false, any = false;
    WgLoad L;
    wg_load(L, H, DZ, kcols, b0, b1);
    for (uint32_t kb = b0; kb < b1; kb += kWgTile) {   // the same trips in every thread
        wg_store(L, sm, kcols, kb, b1);
        umma::fence_smem_to_async();
        umma::fence_before_sync();
        __syncthreads();
        if (t == 0) {
            umma::fence_after_sync();
#pragma unroll
            for (uint32_t j = 0; j < kWgTile / 16; ++j)
                umma::mma_bf16(sm.tmem, umma::smem_desc(a + j * 2u * kActK, kActK, kCore), umma::smem_desc(bt + j * 2u * kWK, kWK, kCore),
                               kTcIdesc, (any || j > 0u) ? 1u : 0u);
            umma::mma_commit(&sm.bar);
        }
        if (kb + kWgTile < b1) wg_load(L, H, DZ, kcols, kb + kWgTile, b1);   // the next round's loads overlap the MMAs
        const int late = t == 0 ? int(!umma::mbar_wait(&sm.bar, phase, kMmaWaitNs)) : 0;
        phase ^= 1u;
        any = true;
        if (__syncthreads_or(late)) {
            fail = true;
            break;
        }
        umma::fence_after_sync();
    }
    if (any && !fail) {
        __syncwarp();
        uint32_t r[64];
        umma::tmem_ld64(sm.tmem + (uint32_t(t & ~31) << 16), r);
#pragma unroll
        for (int n = 0; n < kHid; n += 4)
            *reinterpret_cast<float4 *>(out + n) = make_float4(__uint_as_float(r[n]), __uint_as_float(r[n + 1]), __uint_as_float(r[n + 2]),
                                                               __uint_as_float(r[n + 3]));
    } else {
        for (int n = 0; n < kHid; ++n) out[n] = 0.0f;
    }
    umma::fence_before_sync();
    __syncthreads();
    if (t < 32) {
        __syncwarp();
        umma::fence_after_sync();
        umma::tmem_dealloc(sm.tmem, kTcCols);
    }
    if (fail && t == 0) atomicOr(G.fail, 2u);
}

// grad += the chunks' partials, added in chunk order: one thread per (layer, m <= K_l, n).
__global__ void __launch_bounds__(256) wgrad_reduce_kernel(const float *part, uint32_t chunks, float *grad) {
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= uint32_t(kHidden) * kTcRows * kHid) return;
    const int layer = int(idx / (kTcRows * kHid)), m = int((idx / kHid) % kTcRows), n = int(idx % kHid);
    const int kcols = k_of(layer);
    if (m > kcols) return;
    float s = 0.0f;
    for (uint32_t c = 0; c < chunks; ++c) s += part[((size_t(layer) * chunks + c) * kTcRows + m) * kHid + n];
    if (m < kcols) grad[w_offset(layer) + n * kcols + m] += s;
    else grad[b_offset(layer) + n] += s;
}

// Output layer and loss: grad[W4], grad[b4] and the loss += the warps' partial
// sums.  Thread (j, g) adds warps g, g + 8, ... in order; thread (j, 0) then
// adds the 8 group sums in order (a fixed order: the same bits every run).
constexpr int kOutGroups = 8;
__global__ void __launch_bounds__(kOutPart * kOutGroups) out_reduce_kernel(const float *part, uint32_t warps, float *grad, float *loss) {
    __shared__ float sums[kOutGroups][kOutPart];
    const uint32_t j = threadIdx.x % kOutPart, g = threadIdx.x / kOutPart;
    float s = 0.0f;
    for (uint32_t w = g; w < warps; w += kOutGroups) s += part[size_t(w) * kOutPart + j];
    sums[g][j] = s;
    __syncthreads();
    if (g != 0u) return;
    float total = 0.0f;
#pragma unroll
    for (int k = 0; k < kOutGroups; ++k) total += sums[k][j];
    if (j < uint32_t(kHid)) grad[kW4 + j] += total;
    else if (j == uint32_t(kHid)) grad[kB4] += total;
    else *loss += total;
}

__global__ void __launch_bounds__(256) adam_kernel(float *params, float *m, float *v, float *grad, __nv_bfloat16 *wbf, float lr,
                                                   float b1t, float b2t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    const bool pad = i < kB0 && (i % kInPad) >= kIn;   // padded feature columns of W0 stay zero
    const float g = pad ? 0.0f : grad[i];
    const float mi = 0.9f * m[i] + 0.1f * g;
    const float vi = 0.999f * v[i] + 0.001f * g * g;
    m[i] = mi;
    v[i] = vi;
    float p = params[i];
    if (!pad) p -= lr * (mi / (1.0f - b1t)) / (sqrtf(vi / (1.0f - b2t)) + 1e-8f);
    params[i] = p;
    wbf[i] = __float2bfloat16_rn(p);
    grad[i] = 0.0f;
}

__global__ void to_bf16_kernel(const float *params, __nv_bfloat16 *wbf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kParams) wbf[i] = __float2bfloat16_rn(params[i]);
}

// ---------------------------------------------------------------- data generation
__device__ __forceinline__ float unit_float(uint32_t h) { return float(h >> 8) * (1.0f / 16777216.0f); }

__global__ void __launch_bounds__(256) gen_points_kernel(float4 *out, uint32_t n, uint32_t seed, uint32_t offset, float3 bmin,
                                                         float3 bsize) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t h = hash2(seed, offset + i);
    out[i] = make_float4(bmin.x + bsize.x * unit_float(pcg_hash(h)), bmin.y + bsize.y * unit_float(pcg_hash(h + 1u)),
                         bmin.z + bsize.z * unit_float(pcg_hash(h + 2u)), 0.0f);
}

// Appends the labelled candidates with |d| < band to dst (first `target`).
__global__ void __launch_bounds__(256) keep_near_kernel(const float4 *cand, uint32_t n, float band, float4 *dst, uint32_t target,
                                                        uint32_t *counter) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float4 c = i < n ? cand[i] : make_float4(0.f, 0.f, 0.f, 1e30f);
    bool keep = i < n && isfinite(c.w) && fabsf(c.w) < band;
    uint32_t at = warp_append(counter, keep);
    if (keep && at < target) dst[at] = c;
}

// ---------------------------------------------------------------- prediction
__global__ void __launch_bounds__(128) predict_kernel(Model M, const float4 *pts, float *out, uint32_t n) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemWeights &sw = *reinterpret_cast<SmemWeights *>(smem_raw);
    WarpForward *wf = reinterpret_cast<WarpForward *>(smem_raw + ((sizeof(SmemWeights) + 127) & ~size_t(127)));
    load_weights(sw, M);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t base = (blockIdx.x * 4u + warp) * 32u; base < n; base += gridDim.x * 128u) {
        uint32_t i = base + lane;
        float4 p = i < n ? pts[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        float u[3] = {(p.x - M.center[0]) * M.inv_half[0], (p.y - M.center[1]) * M.inv_half[1], (p.z - M.center[2]) * M.inv_half[2]};
        float o = forward32(sw, wf[warp], u, lane);
        if (i < n) out[i] = o * M.label_scale;
    }
}
// The same prediction with the network on tcgen05: 128 points per CTA
// iteration.  *fail_word gets bit 2 if an MMA did not complete.
__global__ void __launch_bounds__(kTcRows, 4) predict_tc_kernel(Model M, const float4 *pts, float *out, uint32_t n, uint32_t *fail_word) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TcSmem &sm = *reinterpret_cast<TcSmem *>(smem_raw);
    tc_setup(sm, M);
    uint32_t phase = 0;
    bool fail = false;
    for (uint32_t base = blockIdx.x * uint32_t(kTcRows); base < n; base += gridDim.x * uint32_t(kTcRows)) {
        const uint32_t i = base + threadIdx.x;
        const float4 p = i < n ? pts[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float u[3] = {(p.x - M.center[0]) * M.inv_half[0], (p.y - M.center[1]) * M.inv_half[1], (p.z - M.center[2]) * M.inv_half[2]};
        const float o = tc_forward(sm, phase, u, fail);
        if (fail) break;   // the same in every thread
        if (i < n) out[i] = o * M.label_scale;
    }
    tc_teardown(sm);
    if (fail && threadIdx.x == 0) atomicOr(fail_word, 2u);
}
// Bounded-wait check (no fault): one CTA holds tensor memory and waits on an
// mbarrier with a 20 ms limit, once after an arrival and once with none.
// out[0] / out[1]: 1 = the phase completed, 2 = the wait ran out; out[2] /
// out[3]: nanoseconds each wait took.  The tensor memory is freed either way.
__global__ void __launch_bounds__(128) bounded_wait_kernel(uint32_t *out) {
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tmem;
    if (threadIdx.x == 0) {
        umma::mbar_init(&bar[0], 1u);
        umma::mbar_init(&bar[1], 1u);
    }
    if (threadIdx.x < 32) {
        __syncwarp();
        umma::tmem_alloc(&tmem, 32u);
        umma::tmem_relinquish();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (threadIdx.x == 0) {
        umma::mbar_arrive(&bar[0]);   // the first barrier's phase completes; nothing arrives on the second
        for (int k = 0; k < 2; ++k) {
            unsigned long long t0, t1;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
            const bool ok = umma::mbar_wait(&bar[k], 0u, 20000000ull);
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
            out[k] = ok ? 1u : 2u;
            out[2 + k] = uint32_t(min(t1 - t0, 0xffffffffull));
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) {
        __syncwarp();
        umma::fence_after_sync();
        umma::tmem_dealloc(tmem, 32u);
    }
}

size_t forward_smem_bytes() { return ((sizeof(SmemWeights) + 127) & ~size_t(127)) + 4 * sizeof(WarpForward); }
size_t train_smem_bytes() { return ((sizeof(SmemWeights) + 127) & ~size_t(127)) + kWarpsTrain * sizeof(WarpTrain); }

// ---------------------------------------------------------------- host model
struct HostModel {
    float *params = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *loss = nullptr;
    __nv_bfloat16 *wbf = nullptr;
    float4 *data = nullptr;
    uint32_t n_data = 0;
    __nv_bfloat16 *act = nullptr;   // gx | gh[3] | gz[4] | gdz[4]
    float *part = nullptr;          // gradient partials: wgrad_tc_kernel chunks, then train-kernel warps, then the fail word
    uint32_t rows_cap = 0;
    float center[3] = {0, 0, 0}, inv_half[3] = {1, 1, 1}, lo[3] = {-1, -1, -1}, hi[3] = {1, 1, 1}, label_scale = 1.0f;
    uint32_t step = 0;
    Model view() const {
        Model M;
        M.wbf = wbf;
        M.params = params;
        for (int k = 0; k < 3; ++k) { M.center[k] = center[k]; M.inv_half[k] = inv_half[k]; }
        M.label_scale = label_scale;
        return M;
    }
};

static std::unordered_map<uint64_t, HostModel *> &models() {
    static std::unordered_map<uint64_t, HostModel *> m;
    return m;
}
static uint64_t g_next_model = 1;

static void free_model(HostModel *hm) {
    cudaFree(hm->params); cudaFree(hm->m); cudaFree(hm->v); cudaFree(hm->grad); cudaFree(hm->loss); cudaFree(hm->wbf);
    cudaFree(hm->data); cudaFree(hm->act); cudaFree(hm->part);
    delete hm;
}

// Partial sums of a batch of `rows`: [4 layers][chunks][128][64] for the
// weight gradients, [warps][kOutPart] for the output layer and loss, and one
// word for MMA time-outs.
static uint32_t wgrad_chunks(uint32_t rows) { return (rows + kWgChunk - 1) / kWgChunk; }
static size_t part_floats(uint32_t rows) {
    return size_t(kHidden) * wgrad_chunks(rows) * kTcRows * kHid + size_t(rows / 32u) * kOutPart + 4;
}

static bool ensure_rows(HostModel &hm, uint32_t batch, char *error, size_t error_len) {
    const uint32_t rows = (batch + kRowsPerBlock - 1) / kRowsPerBlock * kRowsPerBlock;
    if (hm.rows_cap >= rows) return true;
    cudaFree(hm.act);
    hm.act = nullptr;
    hm.rows_cap = 0;
    cudaFree(hm.part);
    hm.part = nullptr;
    const size_t elems = size_t(rows) * (kInPad + 11 * kHid);
    if (!check(cudaMalloc(&hm.act, elems * sizeof(__nv_bfloat16)), "activation buffers", error, error_len)) return false;
    if (!check(cudaMalloc(&hm.part, part_floats(rows) * sizeof(float)), "gradient partials", error, error_len) ||
        !check(cudaMemset(hm.part, 0, part_floats(rows) * sizeof(float)), "gradient partials", error, error_len))
        return false;
    hm.rows_cap = rows;
    return true;
}

// The MMA time-out word of the model's gradient passes (0: none timed out).
static bool gradients_failed(const HostModel &hm, cudaStream_t st, char *error, size_t error_len) {
    if (!hm.part) return false;
    const float *w = hm.part + size_t(kHidden) * wgrad_chunks(hm.rows_cap) * kTcRows * kHid + size_t(hm.rows_cap / 32u) * kOutPart;
    uint32_t f = 0;
    if (!check(cudaMemcpyAsync(&f, w, 4, cudaMemcpyDeviceToHost, st), "gradient status readback", error, error_len) ||
        !check(cudaStreamSynchronize(st), "gradient status readback", error, error_len))
        return true;
    if (f != 0u) {
        set_error(error, error_len, "a weight-gradient MMA did not complete within 1 s (training aborted)");
        return true;
    }
    return false;
}

static void fill_train_args(TrainArgs &A, HostModel &hm, const float4 *data, uint32_t n_data, uint32_t batch, float over_weight) {
    A.data = data; A.n_data = n_data; A.batch = batch; A.step = hm.step; A.seed = 0; A.identity = 0;
    A.inv_label_scale = 1.0f / hm.label_scale;
    A.over_weight = over_weight;
    A.model = hm.view();
    __nv_bfloat16 *p = hm.act;
    const size_t rows = hm.rows_cap;
    A.gx = p; p += rows * kInPad;
    for (int l = 0; l < 3; ++l) { A.gh[l] = p; p += rows * kHid; }
    for (int l = 0; l < 4; ++l) { A.gz[l] = p; p += rows * kHid; }
    for (int l = 0; l < 4; ++l) { A.gdz[l] = p; p += rows * kHid; }
    A.grad = hm.grad;
    A.loss = hm.loss;
    A.w_part = hm.part;
    A.out_part = hm.part + size_t(kHidden) * wgrad_chunks(hm.rows_cap) * kTcRows * kHid;
    A.fail = reinterpret_cast<uint32_t *>(A.out_part + size_t(hm.rows_cap / 32u) * kOutPart);
}

static void set_attributes() {
    static bool done = false;
    if (done) return;
    cudaFuncSetAttribute(train_fwd_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(train_smem_bytes()));
    cudaFuncSetAttribute(predict_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(forward_smem_bytes()));
    cudaFuncSetAttribute(predict_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tc_smem_bytes()));
    cudaFuncSetAttribute(wgrad_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(wgrad_smem_bytes()));
    cudaFuncSetAttribute(train_fwd_bwd_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(train_tc_smem_bytes()));
    done = true;
}

// Forward + backward of one batch: accumulates into A.grad and A.loss.
static void launch_gradients(const TrainArgs &A, cudaStream_t st) {
    set_attributes();
    const uint32_t blocks = (A.batch + kRowsPerBlock - 1) / kRowsPerBlock;
    // forward + backward on the network engine of the inference passes (tcgen05 by default)
    if (ctx().network_engine == FPT_CUDA_NET_MMA_SYNC) train_fwd_bwd_kernel<<<blocks, 32 * kWarpsTrain, train_smem_bytes(), st>>>(A);
    else train_fwd_bwd_tc_kernel<<<blocks, kTcRows, train_tc_smem_bytes(), st>>>(A);
    WgradArgs G;
    G.h[0] = A.gx;
    for (int l = 1; l < kHidden; ++l) G.h[l] = A.gh[l - 1];
    for (int l = 0; l < kHidden; ++l) G.dz[l] = A.gdz[l];
    G.batch = A.batch;
    G.chunks = wgrad_chunks(A.batch);
    G.part = A.w_part;
    G.fail = A.fail;
    wgrad_tc_kernel<<<dim3(G.chunks, kHidden), kTcRows, wgrad_smem_bytes(), st>>>(G);
    wgrad_reduce_kernel<<<(kHidden * kTcRows * kHid + 255) / 256, 256, 0, st>>>(A.w_part, G.chunks, A.grad);
    out_reduce_kernel<<<1, kOutPart * kOutGroups, 0, st>>>(A.out_part, blocks * kWarpsTrain, A.grad, A.loss);
}

static HostModel *find(uint64_t id) {
    auto it = models().find(id);
    return it == models().end() ? nullptr : it->second;
}

}  // namespace mlp

bool surrogate_bind(uint64_t model, DeviceScene &S, char *error, size_t error_len) {
    if (!mlp::find(model)) {
        set_error(error, error_len, "unknown surrogate model handle %llu", (unsigned long long)model);
        return false;
    }
    if (S.formula == 0) {
        set_error(error, error_len, "the surrogate skip needs an extension formula (Mandelbulb, Mandelbox, Menger, hybrid)");
        return false;
    }
    if (S.ground_plane) {
        set_error(error, error_len, "the surrogate skip needs all geometry inside the model's box (no ground plane)");
        return false;
    }
    if (S.translucent) {
        set_error(error, error_len, "the surrogate skip does not support translucent materials");
        return false;
    }
    return true;
}

bool surrogate_args(uint64_t model, const DeviceScene &S, unsigned long long *stats, SkipArgs &A, char *error, size_t error_len) {
    mlp::HostModel *hm = mlp::find(model);
    if (!hm) {
        set_error(error, error_len, "unknown surrogate model handle %llu", (unsigned long long)model);
        return false;
    }
    A.M = hm->view();
    for (int k = 0; k < 3; ++k) { A.lo[k] = hm->lo[k]; A.hi[k] = hm->hi[k]; }
    A.margin = S.surrogate_margin > 0.0f ? S.surrogate_margin : 0.1f;
    A.safety = S.surrogate_safety > 0.0f ? S.surrogate_safety : 0.9f;
    A.max_iters = S.surrogate_max_iters ? S.surrogate_max_iters : 64u;
    A.use_network = S.surrogate == FPT_CUDA_SURROGATE_SKIP ? 1u : 0u;
    A.engine = ctx().network_engine;
    A.guard = nullptr;
    A.cam_step = nullptr;
    A.stats = stats;
    return true;
}

}  // namespace fpt

using namespace fpt;

extern "C" {

int fpt_cuda_mlp_create(const struct FptRenderConfig *config, const struct FptCudaSceneExt *ext, const struct FptCudaMlpConfig *mc,
                        uint64_t *model, struct FptCudaMlpStats *stats, char *error, size_t error_len) {
    if (model) *model = 0;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (!config || !mc || !model) { set_error(error, error_len, "missing surrogate input"); return 1; }
    if (mc->steps > 0 && (mc->points < 1024 || mc->batch < 64 || mc->batch > (1u << 22))) {
        set_error(error, error_len, "training needs points >= 1024 and 64 <= batch <= 4M");
        return 1;
    }
    for (int k = 0; k < 3; ++k)
        if (!(mc->bounds_max[k] > mc->bounds_min[k])) { set_error(error, error_len, "surrogate bounds must be increasing"); return 1; }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    auto *hm = new mlp::HostModel();
    const size_t np = mlp::kParams;
    bool ok = check(cudaMalloc(&hm->params, np * 4), "parameters", error, error_len) &&
              check(cudaMalloc(&hm->m, np * 4), "adam state", error, error_len) &&
              check(cudaMalloc(&hm->v, np * 4), "adam state", error, error_len) &&
              check(cudaMalloc(&hm->grad, np * 4), "gradients", error, error_len) &&
              check(cudaMalloc(&hm->loss, 64), "loss", error, error_len) &&
              check(cudaMalloc(&hm->wbf, np * 2), "bf16 weights", error, error_len);
    if (!ok) { mlp::free_model(hm); return 1; }
    float half_max = 0.0f;
    for (int k = 0; k < 3; ++k) {
        hm->lo[k] = mc->bounds_min[k];
        hm->hi[k] = mc->bounds_max[k];
        hm->center[k] = 0.5f * (mc->bounds_min[k] + mc->bounds_max[k]);
        const float half = 0.5f * (mc->bounds_max[k] - mc->bounds_min[k]);
        hm->inv_half[k] = 1.0f / half;
        half_max = std::max(half_max, half);
    }
    hm->label_scale = half_max;
    // He-uniform initialisation from the seed, zero biases, small output layer.
    std::vector<float> init(np, 0.0f);
    const uint32_t seed = mc->seed;
    auto urand = [&](uint32_t i) { return float(pcg_hash(pcg_hash(seed) ^ i) >> 8) * (2.0f / 16777216.0f) - 1.0f; };
    for (int l = 0; l < mlp::kHidden; ++l) {
        const int K = mlp::k_of(l), fan = l == 0 ? mlp::kIn : mlp::kHid;
        const float bound = std::sqrt(6.0f / float(fan));
        for (int n = 0; n < mlp::kHid; ++n)
            for (int k = 0; k < K; ++k)
                if (l > 0 || k < mlp::kIn) init[mlp::w_offset(l) + n * K + k] = bound * urand(uint32_t(mlp::w_offset(l) + n * K + k));
    }
    for (int j = 0; j < mlp::kHid; ++j) init[mlp::kW4 + j] = 0.03f * urand(uint32_t(mlp::kW4 + j));
    ok = check(cudaMemcpyAsync(hm->params, init.data(), np * 4, cudaMemcpyHostToDevice, c.stream), "init upload", error, error_len) &&
         check(cudaMemsetAsync(hm->m, 0, np * 4, c.stream), "adam reset", error, error_len) &&
         check(cudaMemsetAsync(hm->v, 0, np * 4, c.stream), "adam reset", error, error_len) &&
         check(cudaMemsetAsync(hm->grad, 0, np * 4, c.stream), "grad reset", error, error_len);
    if (ok) {
        mlp::to_bf16_kernel<<<(mlp::kParams + 255) / 256, 256, 0, c.stream>>>(hm->params, hm->wbf);
        ok = check(cudaGetLastError(), "init conversion", error, error_len);
    }
    if (!ok) { mlp::free_model(hm); return 1; }
    auto t0 = std::chrono::steady_clock::now();
    uint32_t near_found = 0;
    if (mc->points > 0) {
        // Training data: uniform share, then near-surface rejection sampling.
        DeviceScene S;
        if (!compile_scene(*config, ext, S, error, error_len)) { mlp::free_model(hm); return 1; }
        S.surrogate = 0;
        if (!upload_scene(S, nullptr, error, error_len)) { mlp::free_model(hm); return 1; }
        if (!check(cudaMalloc(&hm->data, size_t(mc->points) * sizeof(float4)), "training data", error, error_len)) {
            mlp::free_model(hm);
            return 1;
        }
        hm->n_data = mc->points;
        const float nf = std::min(std::max(mc->near_fraction, 0.0f), 1.0f);
        const uint32_t near_target = uint32_t(double(mc->points) * nf);
        const uint32_t uniform = mc->points - near_target;
        const float band = mc->near_band > 0.0f ? mc->near_band : 0.05f;
        const float3 bmin = make_float3(mc->bounds_min[0], mc->bounds_min[1], mc->bounds_min[2]);
        const float3 bsize = make_float3(mc->bounds_max[0] - bmin.x, mc->bounds_max[1] - bmin.y, mc->bounds_max[2] - bmin.z);
        if (uniform) {
            mlp::gen_points_kernel<<<(uniform + 255) / 256, 256, 0, c.stream>>>(hm->data, uniform, seed, 0u, bmin, bsize);
            ok = check(launch_label(S.kind, c.scene, hm->data, uniform, c.stream), "labelling", error, error_len);
        }
        if (ok && near_target) {
            const uint32_t cand = 1u << 22;
            float4 *cbuf = nullptr;
            uint32_t *counter = reinterpret_cast<uint32_t *>(hm->loss) + 8;
            ok = check(cudaMalloc(&cbuf, size_t(cand) * sizeof(float4)), "candidate buffer", error, error_len) &&
                 check(cudaMemsetAsync(counter, 0, 4, c.stream), "counter reset", error, error_len);
            for (uint32_t round = 0; ok && near_found < near_target && round < 1024; ++round) {
                mlp::gen_points_kernel<<<cand / 256, 256, 0, c.stream>>>(cbuf, cand, seed ^ 0x5bd1e995u, round * cand, bmin, bsize);
                ok = check(launch_label(S.kind, c.scene, cbuf, cand, c.stream), "labelling", error, error_len);
                if (!ok) break;
                mlp::keep_near_kernel<<<cand / 256, 256, 0, c.stream>>>(cbuf, cand, band, hm->data + uniform, near_target, counter);
                ok = check(cudaMemcpyAsync(&near_found, counter, 4, cudaMemcpyDeviceToHost, c.stream), "sample count", error, error_len) &&
                     check(cudaStreamSynchronize(c.stream), "training data generation", error, error_len);
            }
            cudaFree(cbuf);
            if (ok && near_found < near_target) {
                set_error(error, error_len, "only %u of %u near-surface samples found: does the box hold the surface?", near_found,
                          near_target);
                ok = false;
            }
            near_found = std::min(near_found, near_target);
        }
        if (!ok) { mlp::free_model(hm); return 1; }
    }
    auto t1 = std::chrono::steady_clock::now();
    float loss_first = 0.0f, loss_last = 0.0f;
    if (mc->steps > 0) {
        if (!mlp::ensure_rows(*hm, mc->batch, error, error_len)) { mlp::free_model(hm); return 1; }
        const float over = mc->overestimate_weight > 0.0f ? mc->overestimate_weight : 10.0f;
        const float lr0 = mc->lr > 0.0f ? mc->lr : 2e-3f;
        for (uint32_t s = 0; s < mc->steps; ++s) {
            const bool probe = s == 0 || s + 1 == mc->steps;
            if (probe) cudaMemsetAsync(hm->loss, 0, 4, c.stream);
            mlp::TrainArgs A;
            mlp::fill_train_args(A, *hm, hm->data, hm->n_data, mc->batch, over);
            A.seed = seed;
            mlp::launch_gradients(A, c.stream);
            hm->step += 1;
            const float lr = std::max(lr0 * 0.5f * (1.0f + std::cos(3.14159265f * float(s) / float(mc->steps))), lr0 * 0.02f);
            const float b1t = std::pow(0.9f, float(hm->step)), b2t = std::pow(0.999f, float(hm->step));
            mlp::adam_kernel<<<(mlp::kParams + 255) / 256, 256, 0, c.stream>>>(hm->params, hm->m, hm->v, hm->grad, hm->wbf, lr, b1t, b2t);
            if (probe) {
                float l = 0.0f;
                if (!check(cudaMemcpyAsync(&l, hm->loss, 4, cudaMemcpyDeviceToHost, c.stream), "loss readback", error, error_len) ||
                    !check(cudaStreamSynchronize(c.stream), "training step", error, error_len)) {
                    mlp::free_model(hm);
                    return 1;
                }
                (s == 0 ? loss_first : loss_last) = l / float(mc->batch);
            }
        }
    }
    if (!check(cudaStreamSynchronize(c.stream), "training", error, error_len)) { mlp::free_model(hm); return 1; }
    if (mc->steps > 0 && mlp::gradients_failed(*hm, c.stream, error, error_len)) { mlp::free_model(hm); return 1; }
    auto t2 = std::chrono::steady_clock::now();
    const uint64_t id = mlp::g_next_model++;
    mlp::models()[id] = hm;
    *model = id;
    if (stats) {
        stats->loss_first = loss_first;
        stats->loss_last = loss_last;
        stats->data_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        stats->train_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
        stats->params = mlp::kParams;
        stats->steps = mc->steps;
        stats->label_scale = hm->label_scale;
        stats->near_points = near_found;
    }
    return 0;
}

int fpt_cuda_mlp_destroy(uint64_t model) {
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(nullptr, 0)) return 1;
    auto it = mlp::models().find(model);
    if (it == mlp::models().end()) return 1;
    cudaStreamSynchronize(ctx().stream);
    mlp::free_model(it->second);
    mlp::models().erase(it);
    return 0;
}

int fpt_cuda_mlp_predict(uint64_t model, const float *points_xyzw, size_t n, float *distances, char *error, size_t error_len) {
    if (!points_xyzw || !distances || n == 0 || n > (size_t(1) << 28)) { set_error(error, error_len, "bad prediction input"); return 1; }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    mlp::HostModel *hm = mlp::find(model);
    if (!hm) { set_error(error, error_len, "unknown surrogate model handle"); return 1; }
    Context &c = ctx();
    if (!ensure_buffer((void **)&c.points, &c.cap_points, n * sizeof(float4), error, error_len) ||
        !ensure_buffer((void **)&c.grads, &c.cap_grads, n * sizeof(float), error, error_len))
        return 1;
    if (!check(cudaMemcpyAsync(c.points, points_xyzw, n * sizeof(float4), cudaMemcpyHostToDevice, c.stream), "point upload", error, error_len))
        return 1;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    mlp::set_attributes();
    const bool tc = c.network_engine == FPT_CUDA_NET_TCGEN05;
    if (tc && (!ensure_buffer((void **)&c.counter, &c.cap_counter, 64, error, error_len) ||
               !check(cudaMemsetAsync(c.counter, 0, 64, c.stream), "counter reset", error, error_len)))
        return 1;
    if (tc) {
        const int per_sm = mlp::tc_blocks_per_sm(reinterpret_cast<const void *>(mlp::predict_tc_kernel));
        const unsigned blocks = unsigned(std::min<size_t>((n + mlp::kTcRows - 1) / mlp::kTcRows, size_t(sms) * size_t(std::max(per_sm, 1))));
        mlp::predict_tc_kernel<<<blocks, mlp::kTcRows, mlp::tc_smem_bytes(), c.stream>>>(hm->view(), c.points, c.grads, uint32_t(n),
                                                                                          c.counter + C_GUARD);
    } else {
        const unsigned blocks = unsigned(std::min<size_t>((n + 127) / 128, size_t(sms) * 8));
        mlp::predict_kernel<<<blocks, 128, mlp::forward_smem_bytes(), c.stream>>>(hm->view(), c.points, c.grads, uint32_t(n));
    }
    if (!check(cudaGetLastError(), "prediction launch", error, error_len) ||
        !check(cudaMemcpyAsync(distances, c.grads, n * sizeof(float), cudaMemcpyDeviceToHost, c.stream), "prediction readback", error, error_len))
        return 1;
    if (!check(cudaStreamSynchronize(c.stream), "prediction", error, error_len)) return 1;
    if (tc) {
        uint32_t guard = 0;
        if (!check(cudaMemcpy(&guard, c.counter + C_GUARD, sizeof(guard), cudaMemcpyDeviceToHost), "guard readback", error, error_len))
            return 1;
        if (guard) { set_error(error, error_len, "a surrogate network MMA did not complete within 1 s"); return 1; }
    }
    return 0;
}

int fpt_test_bounded_waits(uint32_t *result, size_t result_len, char *error, size_t error_len) {
    if (!result || result_len < 4) { set_error(error, error_len, "result needs 4 entries"); return 1; }
    std::memset(result, 0, 4 * sizeof(uint32_t));
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    if (!ensure_buffer((void **)&c.counter, &c.cap_counter, 64, error, error_len) ||
        !check(cudaMemsetAsync(c.counter, 0, 4 * sizeof(uint32_t), c.stream), "result reset", error, error_len))
        return 1;
    mlp::bounded_wait_kernel<<<1, 128, 0, c.stream>>>(c.counter);
    if (!check(cudaGetLastError(), "bounded-wait launch", error, error_len) ||
        !check(cudaMemcpyAsync(result, c.counter, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream), "result readback", error,
               error_len))
        return 1;
    return check(cudaStreamSynchronize(c.stream), "bounded-wait kernel", error, error_len) ? 0 : 1;
}

int fpt_cuda_mlp_get_params(uint64_t model, float *params, size_t len, char *error, size_t error_len) {
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    mlp::HostModel *hm = mlp::find(model);
    if (!hm) { set_error(error, error_len, "unknown surrogate model handle"); return 1; }
    if (!params || len < size_t(mlp::kParams)) { set_error(error, error_len, "parameter buffer too small (need %d)", mlp::kParams); return 1; }
    Context &c = ctx();
    if (!check(cudaMemcpyAsync(params, hm->params, mlp::kParams * 4, cudaMemcpyDeviceToHost, c.stream), "parameter readback", error, error_len))
        return 1;
    return check(cudaStreamSynchronize(c.stream), "parameter readback", error, error_len) ? 0 : 1;
}

int fpt_cuda_mlp_set_params(uint64_t model, const float *params, size_t len, char *error, size_t error_len) {
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    mlp::HostModel *hm = mlp::find(model);
    if (!hm) { set_error(error, error_len, "unknown surrogate model handle"); return 1; }
    if (!params || len < size_t(mlp::kParams)) { set_error(error, error_len, "parameter buffer too small (need %d)", mlp::kParams); return 1; }
    Context &c = ctx();
    if (!check(cudaMemcpyAsync(hm->params, params, mlp::kParams * 4, cudaMemcpyHostToDevice, c.stream), "parameter upload", error, error_len))
        return 1;
    mlp::to_bf16_kernel<<<(mlp::kParams + 255) / 256, 256, 0, c.stream>>>(hm->params, hm->wbf);
    return check(cudaStreamSynchronize(c.stream), "parameter upload", error, error_len) ? 0 : 1;
}

// One forward/backward pass over the given labelled points (xyz, w = label)
// with the current weights, no update: gradients of the mean asymmetric loss
// and the loss itself.
int fpt_cuda_mlp_gradients(uint64_t model, const float *points_xyzw, size_t n, float overestimate_weight, float *gradients,
                           size_t len, float *loss, char *error, size_t error_len) {
    if (!points_xyzw || !gradients || n == 0 || n > (size_t(1) << 22)) { set_error(error, error_len, "bad gradient input"); return 1; }
    if (len < size_t(mlp::kParams)) { set_error(error, error_len, "gradient buffer too small (need %d)", mlp::kParams); return 1; }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    mlp::HostModel *hm = mlp::find(model);
    if (!hm) { set_error(error, error_len, "unknown surrogate model handle"); return 1; }
    Context &c = ctx();
    if (!ensure_buffer((void **)&c.points, &c.cap_points, n * sizeof(float4), error, error_len) ||
        !mlp::ensure_rows(*hm, uint32_t(n), error, error_len))
        return 1;
    mlp::TrainArgs A;
    mlp::fill_train_args(A, *hm, c.points, uint32_t(n), uint32_t(n), overestimate_weight);
    A.identity = 1;
    bool ok = check(cudaMemcpyAsync(c.points, points_xyzw, n * sizeof(float4), cudaMemcpyHostToDevice, c.stream), "point upload", error, error_len) &&
              check(cudaMemsetAsync(hm->grad, 0, mlp::kParams * 4, c.stream), "grad reset", error, error_len) &&
              check(cudaMemsetAsync(hm->loss, 0, 4, c.stream), "loss reset", error, error_len);
    if (!ok) return 1;
    mlp::launch_gradients(A, c.stream);
    float l = 0.0f;
    ok = check(cudaGetLastError(), "gradient launch", error, error_len) &&
         check(cudaMemcpyAsync(gradients, hm->grad, mlp::kParams * 4, cudaMemcpyDeviceToHost, c.stream), "gradient readback", error, error_len) &&
         check(cudaMemcpyAsync(&l, hm->loss, 4, cudaMemcpyDeviceToHost, c.stream), "loss readback", error, error_len) &&
         check(cudaMemsetAsync(hm->grad, 0, mlp::kParams * 4, c.stream), "grad reset", error, error_len) &&
         check(cudaStreamSynchronize(c.stream), "gradient pass", error, error_len) &&
         !mlp::gradients_failed(*hm, c.stream, error, error_len);
    if (loss) *loss = l / float(n);
    return ok ? 0 : 1;
}

int fpt_cuda_skip_stats(struct FptCudaSkipStats *stats) {
    if (!stats) return 1;
    std::lock_guard<std::mutex> lock(ctx().mutex);
    const unsigned long long *v = ctx().last_skip;
    stats->rows = v[SK_ROWS];
    stats->forwards = v[SK_FORWARDS];
    stats->exact_evals = v[SK_EXACT];
    stats->accepted = v[SK_ACCEPT];
    stats->rejected = v[SK_REJECT];
    stats->escaped = v[SK_ESCAPE];
    stats->handed_over = v[SK_HANDOVER];
    stats->reserved = 0;
    return 0;
}

}  // extern "C"

// mlp.cu -- training and inference of the learned distance surrogate on sm_103a.
//
// Training data: points labelled by the scene's exact distance estimator
// (mapSdf), a share uniform in the model's box and the rest within
// `near_band` of the surface (rejection sampling on the GPU).  Loss:
// asymmetric squared error, overestimates weighted by `overestimate_weight`.
// Optimiser: Adam on an FP32 master copy; BF16 weights and activations in the
// tensor-core passes (mma.sync m16n8k16, FP32 accumulate):
//   train_fwd_bwd_kernel   per warp 32 samples: forward through the 4 hidden
//                          layers, loss, backward deltas (W products through
//                          transposed ldmatrix); writes features,
//                          activations, pre-activations and deltas (bf16)
//   wgrad_kernel           dW_l = dZ_{l+1}^T H_l, split-K over the batch
//   bias_grad_kernel, adam_kernel
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
    float *grad;               // kParams gradients (W4 and b4 accumulated here)
    float *loss;               // sum of the batch loss
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
    if (lane == 0) atomicAdd(A.loss, loss);
    // output layer: dW4[j] = sum_b dout_b H4[b][j], db4 = sum_b dout_b
    for (int j = 0; j < kHid; ++j) {
        float v = dout * __bfloat162float(h4[j]);
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) atomicAdd(A.grad + kW4 + j, v);
    }
    {
        float v = dout;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) atomicAdd(A.grad + kB4, v);
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

// dW[n][k] += sum_b dZ[b][n] H[b][k] over one chunk of the batch.  Block:
// 4 warps, warp w owns columns col0 + 32 w .. + 31 of all 64 rows of dW
// (4 m-tiles x 4 n-tiles); grid.x = batch chunks, grid.y = column blocks.
constexpr int kChunk = 512;
constexpr int kStrideWg = 128 + 8;
__global__ void __launch_bounds__(128) wgrad_kernel(const __nv_bfloat16 *dz, const __nv_bfloat16 *h, int kcols, uint32_t batch,
                                                    float *dw) {
    __shared__ __align__(16) __nv_bfloat16 sdz[16 * kStrideH];
    __shared__ __align__(16) __nv_bfloat16 sh[16 * kStrideWg];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int col0 = blockIdx.y * 128;
    const int my_col = col0 + warp * 32;
    float acc[4][4][4];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int n = 0; n < 4; ++n)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[m][n][q] = 0.0f;
    const uint32_t b0 = blockIdx.x * kChunk, b1 = min(batch, b0 + kChunk);
    for (uint32_t kb = b0; kb < b1; kb += 16) {
        __syncthreads();
        for (int i = threadIdx.x; i < 16 * 32; i += 128) {   // 16 rows x 64 columns as bf16 pairs
            int r = i >> 5, c = (i & 31) * 2;
            __nv_bfloat162 v = __floats2bfloat162_rn(0.0f, 0.0f);
            if (kb + r < b1) v = *reinterpret_cast<const __nv_bfloat162 *>(dz + size_t(kb + r) * kHid + c);
            *reinterpret_cast<__nv_bfloat162 *>(sdz + r * kStrideH + c) = v;
        }
        for (int i = threadIdx.x; i < 16 * 64; i += 128) {
            int r = i >> 6, c = (i & 63) * 2;
            __nv_bfloat162 v = __floats2bfloat162_rn(0.0f, 0.0f);
            if (kb + r < b1 && col0 + c < kcols) v = *reinterpret_cast<const __nv_bfloat162 *>(h + size_t(kb + r) * kcols + col0 + c);
            *reinterpret_cast<__nv_bfloat162 *>(sh + r * kStrideWg + c) = v;
        }
        __syncthreads();
        if (my_col < kcols) {
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                uint32_t a[4];
                load_a_trans(a, sdz, kStrideH, m * 16, 0, lane);   // A(n, b) = dZ[b][n]
#pragma unroll
                for (int n = 0; n < 4; ++n) {
                    uint32_t b[2];
                    load_b_kn(b, sh, kStrideWg, warp * 32 + n * 8, 0, lane);   // B(b, k) = H[b][k]
                    mma16816(acc[m][n], a, b);
                }
            }
        }
    }
    if (my_col >= kcols) return;
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int n = 0; n < 4; ++n)
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                int r = m * 16 + g + hh * 8, c = my_col + n * 8 + t * 2;
                if (c < kcols) atomicAdd(dw + size_t(r) * kcols + c, acc[m][n][hh * 2]);
                if (c + 1 < kcols) atomicAdd(dw + size_t(r) * kcols + c + 1, acc[m][n][hh * 2 + 1]);
            }
}

__global__ void __launch_bounds__(256) bias_grad_kernel(const __nv_bfloat16 *dz, uint32_t batch, float *db) {
    __shared__ float part[256];
    const int col = threadIdx.x & 63, sub = threadIdx.x >> 6;
    float s = 0.0f;
    for (uint32_t b = blockIdx.x * 4u + sub; b < batch; b += gridDim.x * 4u) s += __bfloat162float(dz[size_t(b) * kHid + col]);
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < 64) atomicAdd(db + col, part[col] + part[col + 64] + part[col + 128] + part[col + 192]);
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
__global__ void __launch_bounds__(kTcRows) predict_tc_kernel(Model M, const float4 *pts, float *out, uint32_t n, uint32_t *fail_word) {
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
    cudaFree(hm->data); cudaFree(hm->act);
    delete hm;
}

static bool ensure_rows(HostModel &hm, uint32_t batch, char *error, size_t error_len) {
    const uint32_t rows = (batch + kRowsPerBlock - 1) / kRowsPerBlock * kRowsPerBlock;
    if (hm.rows_cap >= rows) return true;
    cudaFree(hm.act);
    hm.act = nullptr;
    hm.rows_cap = 0;
    const size_t elems = size_t(rows) * (kInPad + 11 * kHid);
    if (!check(cudaMalloc(&hm.act, elems * sizeof(__nv_bfloat16)), "activation buffers", error, error_len)) return false;
    hm.rows_cap = rows;
    return true;
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
}

static void set_attributes() {
    static bool done = false;
    if (done) return;
    cudaFuncSetAttribute(train_fwd_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(train_smem_bytes()));
    cudaFuncSetAttribute(predict_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(forward_smem_bytes()));
    cudaFuncSetAttribute(predict_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tc_smem_bytes()));
    done = true;
}

// Forward + backward of one batch: accumulates into A.grad and A.loss.
static void launch_gradients(const TrainArgs &A, cudaStream_t st) {
    set_attributes();
    const uint32_t blocks = (A.batch + kRowsPerBlock - 1) / kRowsPerBlock;
    train_fwd_bwd_kernel<<<blocks, 32 * kWarpsTrain, train_smem_bytes(), st>>>(A);
    const uint32_t chunks = (A.batch + kChunk - 1) / kChunk;
    wgrad_kernel<<<dim3(chunks, 1), 128, 0, st>>>(A.gdz[0], A.gx, kInPad, A.batch, A.grad + kW0);
    for (int l = 1; l < kHidden; ++l) wgrad_kernel<<<dim3(chunks, 1), 128, 0, st>>>(A.gdz[l], A.gh[l - 1], kHid, A.batch, A.grad + w_offset(l));
    for (int l = 0; l < kHidden; ++l) bias_grad_kernel<<<64, 256, 0, st>>>(A.gdz[l], A.batch, A.grad + b_offset(l));
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
         check(cudaStreamSynchronize(c.stream), "gradient pass", error, error_len);
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

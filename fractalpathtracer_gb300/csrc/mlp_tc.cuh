// mlp_tc.cuh -- the surrogate's forward pass on the 5th-generation tensor
// cores (tcgen05): 128 rows per CTA, one row per thread.
//
// The activations live in tensor memory next to the accumulator: thread t
// writes its row's BF16 features into TMEM lane t (two per 32-bit column),
// and per layer one thread issues the K/16 MMAs of a 128 x 64 x K product
// with A read from tensor memory and B (the layer's weights) from shared
// memory, into a 128 x 64 FP32 accumulator in tensor memory, and commits
// them to an mbarrier.  Every thread then reads its own accumulator row, adds
// the bias, applies SiLU and writes the BF16 row back into its A lane for the
// next layer.  Only the weights take shared memory (40 KB), so four CTAs fit
// on an SM, each with 128 tensor-memory columns.  The arithmetic is
// that of mlp::forward32 (BF16 features, weights and activations, FP32
// accumulation, the f16x2-tanh SiLU of inference, FP32 output layer); only
// the order of the FP32 sums differs.
#pragma once

#include "mlp.cuh"
#include "umma.cuh"

namespace fpt {
namespace mlp {

constexpr int kTcRows = 128;           // M of every MMA; the CTA has one thread per row
constexpr uint32_t kTcCols = 64;       // tensor-memory columns: one 128 x 64 FP32 accumulator
constexpr uint32_t kFwdCols = 128;     // a forward CTA's columns: the accumulator (0-63) and the A operand
constexpr uint32_t kFwdA = 64;         // first column of the A operand (K / 2 columns: 56 for the features)
constexpr uint32_t kCore = 128;        // bytes of one 8 x 8 BF16 core matrix
// Activation tile [k chunk][row group][8 rows][8 bf16]: K-adjacent core
// matrices lie 16 row groups apart, M-adjacent ones 128 bytes apart.
constexpr uint32_t kActK = (kTcRows / 8) * kCore;   // 2048
// Weight tile W[n][k] [k chunk][n group][8 rows][8 bf16].
constexpr uint32_t kWK = (kHid / 8) * kCore;        // 1024
constexpr uint32_t kTcIdesc = umma::idesc_bf16_f32(kTcRows, kHid);
constexpr unsigned long long kMmaWaitNs = 1000000000ull;   // 1 s; a layer takes about a microsecond

struct TcSmem {
    alignas(128) unsigned char w0[kHid * kInPad * 2];
    alignas(128) unsigned char w[kHidden - 1][kHid * kHid * 2];
    float b[kHidden][kHid];                                 // half biases, b / 2 (silu2_bf16_half)
    float w4[kHid];
    float b4;
    uint32_t tmem;                                          // tensor-memory base: accumulator, then the A operand
    alignas(8) uint64_t bar;                                // MMA completion
    // Slack after the tiles: the tensor core reads each tile through a
    // descriptor, and this keeps those reads inside the CTA's shared memory
    // whatever the descriptor strides.
    unsigned char slack[512];
};
inline size_t tc_smem_bytes() { return sizeof(TcSmem); }

// Resident CTAs per SM of a kernel built on tc_forward, from its registers,
// its shared memory, the thread and block limits and the 512 tensor-memory
// columns (kFwdCols per CTA).  (cudaOccupancyMaxActiveBlocksPerMultiprocessor
// answers 1 for these kernels on GB300, where registers, shared memory and
// tensor memory allow 4.)
inline int tc_blocks_per_sm(const void *kernel) {
    cudaFuncAttributes fa{};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return 1;
    int regs_sm = 0, smem_sm = 0, smem_res = 0, threads_sm = 0, blocks_sm = 0;
    cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&smem_res, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
    cudaDeviceGetAttribute(&blocks_sm, cudaDevAttrMaxBlocksPerMultiprocessor, dev);
    const int regs_block = ((fa.numRegs * 32 + 255) / 256) * 256 * (kTcRows / 32);   // allocated per warp in units of 256
    const int smem_block = int(tc_smem_bytes()) + int(fa.sharedSizeBytes) + smem_res;
    int n = int(512u / kFwdCols);
    n = regs_block > 0 ? (regs_sm / regs_block < n ? regs_sm / regs_block : n) : n;
    n = smem_sm / smem_block < n ? smem_sm / smem_block : n;
    n = threads_sm / kTcRows < n ? threads_sm / kTcRows : n;
    n = blocks_sm < n ? blocks_sm : n;
    return n > 0 ? n : 1;
}

__device__ __forceinline__ uint32_t act_offset(int row, int kc) { return (uint32_t(kc) * (kTcRows / 8) + uint32_t(row >> 3)) * kCore + uint32_t(row & 7) * 16u; }
__device__ __forceinline__ uint32_t w_core_offset(int n, int k) {
    return (uint32_t(k >> 3) * (kHid / 8) + uint32_t(n >> 3)) * kCore + uint32_t(n & 7) * 16u + uint32_t(k & 7) * 2u;
}

// Weights into the core-matrix tiles, tensor memory (kFwdCols columns) and
// the mbarrier.  All threads of the 128-thread CTA call it; it ends with a
// barrier.
__device__ __forceinline__ void tc_setup(TcSmem &sm, const Model &M) {
    for (int i = threadIdx.x; i < kHid * kInPad; i += blockDim.x) {
        const int n = i / kInPad, k = i - n * kInPad;
        *reinterpret_cast<__nv_bfloat16 *>(sm.w0 + w_core_offset(n, k)) = M.wbf[kW0 + i];
    }
    for (int l = 1; l < kHidden; ++l)
        for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x) {
            const int n = i / kHid, k = i - n * kHid;
            *reinterpret_cast<__nv_bfloat16 *>(sm.w[l - 1] + w_core_offset(n, k)) = M.wbf[w_offset(l) + i];
        }
    for (int i = threadIdx.x; i < kHidden * kHid; i += blockDim.x) sm.b[i / kHid][i % kHid] = 0.5f * M.params[b_offset(i / kHid) + i % kHid];
    for (int i = threadIdx.x; i < kHid; i += blockDim.x) sm.w4[i] = __bfloat162float(M.wbf[kW4 + i]);
    if (threadIdx.x == 0) {
        sm.b4 = M.params[kB4];
        umma::mbar_init(&sm.bar, 1u);
    }
    if (threadIdx.x < 32) {
        __syncwarp();
        umma::tmem_alloc(&sm.tmem, kFwdCols);
        umma::tmem_relinquish();
    }
    umma::fence_smem_to_async();   // the weight tiles are read by the tensor core
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
}

// Frees the tensor memory; all threads call it (after their last forward).
__device__ __forceinline__ void tc_teardown(TcSmem &sm) {
    umma::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) {
        __syncwarp();
        umma::fence_after_sync();
        umma::tmem_dealloc(sm.tmem, kFwdCols);
    }
}

// The features of mlp::features, as 56 packed BF16 pairs (element 2p in the
// low half of pair p).
__device__ __forceinline__ void feature_pairs(const float u[3], uint32_t f[kInPad / 2]) {
    float v[kInPad];   // the features in input order (the compiler keeps only the pending ones live)
#pragma unroll
    for (int e = kIn; e < kInPad; ++e) v[e] = 0.0f;
    v[0] = u[0];
    v[1] = u[1];
    v[2] = u[2];
#pragma unroll
    for (int r = 0; r < 5; ++r) {
        const float fr = 3.14159265358979f * exp2f(0.4f * float(r));
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            float s, c;
            __sincosf(fr * u[i], &s, &c);
#pragma unroll
            for (int k = r; k < kFreq; k += 5) {
                v[3 + (k * 3 + i) * 2] = s;
                v[3 + (k * 3 + i) * 2 + 1] = c;
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
    for (int p = 0; p < kInPad / 2; ++p) f[p] = pack_bf16(v[2 * p], v[2 * p + 1]);   // one conversion per pair
}

// Forward pass of the CTA's 128 rows: every thread passes its row's
// normalised point and gets the row's output (label units).  `phase` is the
// parity of the next mbarrier phase (the same in every thread).  If an MMA
// does not complete within kMmaWaitNs, every thread gets fail = true and 0.
__device__ __forceinline__ float tc_forward(TcSmem &sm, uint32_t &phase, const float u[3], bool &fail) {
    const int t = threadIdx.x;
    const uint32_t lanes = uint32_t(t & ~31) << 16;   // this warp's 32 tensor-memory lanes
    const uint32_t a_row = sm.tmem + lanes + kFwdA, d_row = sm.tmem + lanes;
    {
        uint32_t f[kInPad / 2];
        feature_pairs(u, f);
#pragma unroll
        for (int q = 0; q < kInPad / 16; ++q) umma::tmem_st8(a_row + 8u * uint32_t(q), f + 8 * q);
        umma::tmem_wait_st();
    }
    float out = 0.0f;
#pragma unroll 1
    for (int L = 0; L < kHidden; ++L) {
        umma::fence_before_sync();
        __syncthreads();
        if (t == 0) {
            umma::fence_after_sync();
            const int ksteps = (L == 0 ? kInPad : kHid) / 16;
            const uint32_t b = umma::smem_u32(L == 0 ? sm.w0 : sm.w[L - 1]);
            for (int j = 0; j < ksteps; ++j)
                umma::mma_bf16_ts(sm.tmem, sm.tmem + kFwdA + 8u * uint32_t(j), umma::smem_desc(b + uint32_t(j) * 2u * kWK, kWK, kCore),
                                  kTcIdesc, uint32_t(j));
            umma::mma_commit(&sm.bar);
        }
        const int late = t == 0 ? int(!umma::mbar_wait(&sm.bar, phase, kMmaWaitNs)) : 0;
        phase ^= 1u;
        if (__syncthreads_or(late)) {
            fail = true;
            return 0.0f;
        }
        umma::fence_after_sync();
        __syncwarp();
        const float *bias = sm.b[L];
#pragma unroll
        for (int h = 0; h < 2; ++h) {   // the accumulator row in two halves of 32 columns
            uint32_t r[32];
            umma::tmem_ld32(d_row + 32u * uint32_t(h), r);
            if (L + 1 < kHidden) {
                uint32_t a[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int c = h * 32 + q * 2;
                    a[q] = silu2_bf16_half(fmaf(__uint_as_float(r[2 * q]), 0.5f, bias[c]), fmaf(__uint_as_float(r[2 * q + 1]), 0.5f, bias[c + 1]));
                }
                umma::tmem_st8(a_row + 16u * uint32_t(h), a);
                umma::tmem_st8(a_row + 16u * uint32_t(h) + 8u, a + 8);
            } else {
                // Output layer: dot product of the (bf16-rounded) last activations with W4.
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int c = h * 32 + q * 2;
                    const uint32_t hh =
                        silu2_bf16_half(fmaf(__uint_as_float(r[2 * q]), 0.5f, bias[c]), fmaf(__uint_as_float(r[2 * q + 1]), 0.5f, bias[c + 1]));
                    out += __uint_as_float(hh << 16) * sm.w4[c] + __uint_as_float(hh & 0xffff0000u) * sm.w4[c + 1];
                }
            }
        }
        if (L + 1 < kHidden) umma::tmem_wait_st();
        else out += sm.b4;
    }
    return out;
}

}  // namespace mlp
}  // namespace fpt

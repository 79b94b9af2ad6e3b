// voxel.cu -- sparse-brick voxelization and exact grid DDA on sm_103a.
//
// Built with -fmad=false: the distance estimator at cell centres, the
// occupancy test, the camera rays and the DDA all round every operation in
// source order, so brick tables and cell sequences are bit-identical to the
// CPU restatement for estimators made of IEEE operations (+ - * / sqrt).
//
// Build pipeline of occupancy bricks (one resident grid per process):
//   brick_stage_kernel     one CTA per 8^3 brick, one thread per cell: distance
//                          at the cell centre and occupancy (classifyAccelerationCell,
//                          shaders/Shaders.metal:4196-4244, legacy coverage),
//                          each evaluated once; the brick is assembled in shared
//                          memory (512 occupancy bytes, 512 fp16 distances, the
//                          64-byte bit mask) and an occupied brick leaves as 100
//                          16-byte vector stores into a staging slot of its own
//   scan kernels           exclusive scan of "brick occupied" in raster order
//                          (brick x fastest): the compaction order of the
//                          reference's host finalize_voxel_storage
//                          (src/metal_bridge.mm:1738-1812), deterministic
//   brick_commit_kernel    one warp per brick: the brick table entry, and for an
//                          occupied brick a 16-byte-vector copy of its staged
//                          payload into its compact slot
// Reference cells (4^3 bricks) keep two passes: brick_classify_kernel counts,
// brick_fill_kernel evaluates the occupied bricks' cells and materials.
// Formats: reference (4^3 bricks of 12-byte VoxelCell, shaders/Shaders.metal:
// 3973-4044) and occupancy bricks (8^3 bricks, uint8 occupancy + fp16
// distance per cell, plus a 64-byte occupancy bitmask per brick for the DDA).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bridge_internal.h"
#include "fpt_de.cuh"
#include "fpt_kernels.h"
#include "image_io.h"
#include "voxel_dda.cuh"

namespace fpt {

enum VoxFormat : uint32_t { VF_REFERENCE = 1, VF_OCCUPANCY = 4 };

struct VoxBuild {
    float bmin[3], cs[3], half_radius, band;
    uint32_t res, brick_grid, fill_interior;
};

// Cell-centre distance and occupancy of the legacy coverage rule.
template <int KIND>
__device__ __forceinline__ bool classify_cell(const DeviceScene &S, const VoxBuild &B, uint32_t x, uint32_t y, uint32_t z,
                                              float &d, float3 &p) {
    p = make_float3(B.bmin[0] + (float(x) + 0.5f) * B.cs[0], B.bmin[1] + (float(y) + 0.5f) * B.cs[1],
                    B.bmin[2] + (float(z) + 0.5f) * B.cs[2]);
    d = scene_eval<KIND>(S, p, EV_RAW).d;
    bool occ = isfinite(d) && fabsf(d) <= B.half_radius * fmaxf(B.band, 0.25f);
    if (B.fill_interior != 0u && isfinite(d) && d < 0.0f) occ = true;
    return occ;
}

template <int KIND, int BS>
__global__ void __launch_bounds__(BS *BS *BS) brick_classify_kernel(const DeviceScene *scene, VoxBuild B, uint32_t *brick_count,
                                                                    unsigned long long *active_cells) {
    const DeviceScene &S = *scene;
    uint32_t b = blockIdx.x;
    uint32_t bx = b % B.brick_grid, by = (b / B.brick_grid) % B.brick_grid, bz = b / (B.brick_grid * B.brick_grid);
    uint32_t l = threadIdx.x;
    uint32_t x = bx * BS + l % BS, y = by * BS + (l / BS) % BS, z = bz * BS + l / (BS * BS);
    bool occ = false;
    if (x < B.res && y < B.res && z < B.res) {
        float d;
        float3 p;
        occ = classify_cell<KIND>(S, B, x, y, z, d, p);
    }
    int count = __syncthreads_count(occ);
    if (threadIdx.x == 0) {
        brick_count[b] = uint32_t(count);
        if (count) atomicAdd(active_cells, (unsigned long long)count);
    }
}

// Exclusive scan of (count > 0) over n bricks: block pass, block-sum pass, add pass.
constexpr int kScanThreads = 1024, kScanPer = 4, kScanBlock = kScanThreads * kScanPer;
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *smem, uint32_t &total) {
    uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= uint32_t(o)) x += y;
    }
    if (lane == 31) smem[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (blockDim.x >> 5) ? smem[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= uint32_t(o)) w += y;
        }
        smem[lane] = w;
    }
    __syncthreads();
    uint32_t warp_prefix = warp ? smem[warp - 1] : 0u;
    total = smem[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + x - v;
}
__global__ void __launch_bounds__(kScanThreads) scan_blocks_kernel(const uint32_t *count, uint32_t n, uint32_t *offset,
                                                                   uint32_t *block_sums) {
    __shared__ uint32_t smem[32];
    uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * kScanPer;
    uint32_t f[kScanPer], s = 0;
    for (int k = 0; k < kScanPer; ++k) {
        f[k] = (base + k < n && count[base + k] > 0u) ? 1u : 0u;
        s += f[k];
    }
    uint32_t total;
    uint32_t pre = block_exclusive_scan(s, smem, total);
    for (int k = 0; k < kScanPer; ++k) {
        if (base + k < n) offset[base + k] = pre;
        pre += f[k];
    }
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}
__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(uint32_t *block_sums, uint32_t nblocks, uint32_t *grand_total) {
    __shared__ uint32_t smem[32];
    uint32_t carry = 0;
    for (uint32_t start = 0; start < nblocks; start += kScanThreads) {
        uint32_t i = start + threadIdx.x;
        uint32_t v = i < nblocks ? block_sums[i] : 0u;
        uint32_t total;
        uint32_t pre = block_exclusive_scan(v, smem, total);
        if (i < nblocks) block_sums[i] = carry + pre;
        carry += total;
    }
    if (threadIdx.x == 0) *grand_total = carry;
}
__global__ void __launch_bounds__(256) scan_add_kernel(uint32_t *offset, uint32_t n, const uint32_t *block_sums) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) offset[i] += block_sums[i / kScanBlock];
}

// Occupancy bricks, classified once: a brick's 100 16-byte vectors (32 of
// occupancy bytes, 64 of fp16 distances, 4 of bit mask) in its staging slot.
constexpr uint32_t kBrickVectors = 100;
constexpr size_t kBrickStageBytes = size_t(kBrickVectors) * 16;
template <int KIND>
__global__ void __launch_bounds__(512) brick_stage_kernel(const DeviceScene *scene, VoxBuild B, uint32_t *brick_count,
                                                          unsigned long long *active_cells, uint4 *stage) {
    __shared__ __align__(16) uint8_t s_occ[512];
    __shared__ __align__(16) __half s_dist[512];
    __shared__ __align__(16) uint32_t s_mask[16];
    const DeviceScene &S = *scene;
    const uint32_t b = blockIdx.x;
    const uint32_t bx = b % B.brick_grid, by = (b / B.brick_grid) % B.brick_grid, bz = b / (B.brick_grid * B.brick_grid);
    const uint32_t l = threadIdx.x;
    const uint32_t x = bx * 8u + (l & 7u), y = by * 8u + ((l >> 3) & 7u), z = bz * 8u + (l >> 6);
    bool occ = false;
    float d = 0.0f;
    const bool inside = x < B.res && y < B.res && z < B.res;
    if (inside) {
        float3 p;
        occ = classify_cell<KIND>(S, B, x, y, z, d, p);
    }
    s_occ[l] = occ ? 1u : 0u;
    s_dist[l] = __float2half_rn(inside ? d : 0.0f);
    const unsigned bal = __ballot_sync(0xffffffffu, occ);
    if ((l & 31u) == 0u) s_mask[l >> 5] = bal;
    const int count = __syncthreads_count(occ);   // also orders the shared-memory writes before the copy-out
    if (count > 0) {
        uint4 *dst = stage + size_t(b) * kBrickVectors;
        if (l < 32u) dst[l] = reinterpret_cast<const uint4 *>(s_occ)[l];
        else if (l < 96u) dst[l] = reinterpret_cast<const uint4 *>(s_dist)[l - 32u];
        else if (l < kBrickVectors) dst[l] = reinterpret_cast<const uint4 *>(s_mask)[l - 96u];
    }
    if (l == 0u) {
        brick_count[b] = uint32_t(count);
        if (count) atomicAdd(active_cells, (unsigned long long)count);
    }
}
__global__ void __launch_bounds__(256) brick_commit_kernel(const uint32_t *brick_count, const uint32_t *brick_offset, uint32_t nb,
                                                           const uint4 *stage, uint32_t *table, uint4 *occ_out, uint4 *dist_out,
                                                           uint4 *mask_out) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < nb; b += warps) {
        if (brick_count[b] == 0u) {
            if (lane == 0u) table[b] = 0u;
            continue;
        }
        const uint32_t id = brick_offset[b];
        if (lane == 0u) table[b] = id + 1u;
        const uint4 *src = stage + size_t(b) * kBrickVectors;
        for (uint32_t k = lane; k < kBrickVectors; k += 32u) {
            const uint4 v = src[k];
            if (k < 32u) occ_out[size_t(id) * 32u + k] = v;
            else if (k < 96u) dist_out[size_t(id) * 64u + (k - 32u)] = v;
            else mask_out[size_t(id) * 4u + (k - 96u)] = v;
        }
    }
}

// Packs a unorm4 the way packVoxelUnorm4 does (shaders/Shaders.metal:4018-4021).
__device__ __forceinline__ uint32_t pack_unorm4(float a, float b, float c, float d) {
    uint32_t q0 = uint32_t(rintf(fminf(fmaxf(a, 0.f), 1.f) * 255.0f)), q1 = uint32_t(rintf(fminf(fmaxf(b, 0.f), 1.f) * 255.0f));
    uint32_t q2 = uint32_t(rintf(fminf(fmaxf(c, 0.f), 1.f) * 255.0f)), q3 = uint32_t(rintf(fminf(fmaxf(d, 0.f), 1.f) * 255.0f));
    return q0 | (q1 << 8) | (q2 << 16) | (q3 << 24);
}

// Reference cells: occupied bricks only, each cell re-evaluated with its
// material (buildVoxelCell, shaders/Shaders.metal:5388-5414) into the brick's
// compact slot.
template <int KIND, int BS>
__global__ void __launch_bounds__(BS *BS *BS) brick_fill_kernel(const DeviceScene *scene, VoxBuild B, const uint32_t *brick_count,
                                                                const uint32_t *brick_offset, uint32_t *table, uint32_t *cells_out) {
    const DeviceScene &S = *scene;
    uint32_t b = blockIdx.x;
    if (brick_count[b] == 0u) {
        if (threadIdx.x == 0) table[b] = 0u;
        return;
    }
    uint32_t id = brick_offset[b];
    if (threadIdx.x == 0) table[b] = id + 1u;
    uint32_t bx = b % B.brick_grid, by = (b / B.brick_grid) % B.brick_grid, bz = b / (B.brick_grid * B.brick_grid);
    uint32_t l = threadIdx.x;
    uint32_t x = bx * BS + l % BS, y = by * BS + (l / BS) % BS, z = bz * BS + l / (BS * BS);
    bool occ = false;
    float d = 0.0f;
    float3 p = make_float3(0.f, 0.f, 0.f);
    bool inside = x < B.res && y < B.res && z < B.res;
    if (inside) occ = classify_cell<KIND>(S, B, x, y, z, d, p);
    size_t slot = size_t(id) * (BS * BS * BS) + l;
    uint32_t c0 = 0u, c1 = 0u, c2 = 0u;
    if (occ) {
        Material m = material_of(S, scene_eval<KIND>(S, p, EV_MATERIAL));
        c0 = pack_unorm4(m.rgb.x, m.rgb.y, m.rgb.z, 0.0f) | 0x80000000u;
        c1 = pack_unorm4(m.roughness, m.specular, m.translucency, (m.ior - 1.0f) / 1.5f);
        c2 = __float_as_uint(m.emission);
    }
    cells_out[slot * 3 + 0] = c0;
    cells_out[slot * 3 + 1] = c1;
    cells_out[slot * 3 + 2] = c2;
}

// Dense reference storage: every cell (voxel_build_kernel, shaders/Shaders.metal:5416-5424).
template <int KIND>
__global__ void __launch_bounds__(256) dense_fill_kernel(const DeviceScene *scene, VoxBuild B, uint32_t *cells_out,
                                                         unsigned long long *active_cells) {
    const DeviceScene &S = *scene;
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    size_t n = size_t(B.res) * B.res * B.res;
    bool occ = false;
    if (i < n) {
        uint32_t x = uint32_t(i % B.res), y = uint32_t((i / B.res) % B.res), z = uint32_t(i / (size_t(B.res) * B.res));
        float d;
        float3 p;
        occ = classify_cell<KIND>(S, B, x, y, z, d, p);
        uint32_t c0 = 0u, c1 = 0u, c2 = 0u;
        if (occ) {
            Material m = material_of(S, scene_eval<KIND>(S, p, EV_MATERIAL));
            c0 = pack_unorm4(m.rgb.x, m.rgb.y, m.rgb.z, 0.0f) | 0x80000000u;
            c1 = pack_unorm4(m.roughness, m.specular, m.translucency, (m.ior - 1.0f) / 1.5f);
            c2 = __float_as_uint(m.emission);
        }
        cells_out[i * 3] = c0; cells_out[i * 3 + 1] = c1; cells_out[i * 3 + 2] = c2;
    }
    unsigned bal = __ballot_sync(0xffffffffu, occ);
    if ((threadIdx.x & 31u) == 0 && bal) atomicAdd(active_cells, (unsigned long long)__popc(bal));
}

// ---------------------------------------------------------------- rays
// Camera ray of a pixel centre with the rotation's sines and cosines taken
// from the host, in separately rounded operations (bit-exact with the CPU).
struct CamExact {
    float pos[3];
    float focal;
    float sr, cr, sp, cp, sy, cy;   // roll, pitch, yaw
};
__device__ __forceinline__ float3 exact_camera_dir(const CamExact &C, float u, float v) {
    float len = sqrtf(u * u + v * v + C.focal * C.focal);
    float x = u / len, y = v / len, z = C.focal / len;
    // rot2(v.xy, roll) then rotateCamera(v, yaw, pitch) (shaders/Shaders.metal:419-436)
    float rx = C.cr * x - C.sr * y, ry = C.sr * x + C.cr * y;
    x = rx; y = ry;
    float y1 = z * C.sp + y * C.cp, z1 = z * C.cp - y * C.sp;
    y = y1; z = z1;
    return make_float3(x * C.cy + z * C.sy, y, -x * C.sy + z * C.cy);
}
__device__ __forceinline__ float2 exact_uv(uint32_t gx, uint32_t gy, uint32_t W, uint32_t H) {
    float u = (float(gx) + 0.5f) / float(W) - 0.5f;
    float v = (float(gy) + 0.5f) / float(H) - 0.5f;
    u = u * (float(W) / float(H));
    return make_float2(u, v);
}
// offsetVoxelRayOrigin, legacy mode (shaders/Shaders.metal:4068-4089).
__device__ __forceinline__ float3 offset_origin(float3 pos, float3 n, float3 dir, float eps) {
    float side = (dir.x * n.x + dir.y * n.y + dir.z * n.z) >= 0.0f ? 1.0f : -1.0f;
    return make_float3(pos.x + n.x * side * eps, pos.y + n.y * side * eps, pos.z + n.z * side * eps);
}
// offsetVoxelRayOrigin in either mode: legacy (a hundredth of the smallest
// cell edge along the directed normal) or precision (precisionOffsetRayOrigin,
// shaders/Shaders.metal:4057-4072: 256 representable floats along the normal,
// an absolute 2^-16 step within 1/32 of zero).
__device__ __forceinline__ float3 offset_origin_mode(float3 pos, float3 n, float3 dir, float eps, uint32_t mode) {
    if (mode != FPT_VOXEL_OFFSET_PRECISION) return offset_origin(pos, n, dir, eps);
    const float side = (dir.x * n.x + dir.y * n.y + dir.z * n.z) >= 0.0f ? 1.0f : -1.0f;
    const float dn[3] = {n.x * side, n.y * side, n.z * side}, p[3] = {pos.x, pos.y, pos.z};
    float r[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int off = int(256.0f * dn[a]);
        int bits = __float_as_int(p[a]);
        bits += p[a] < 0.0f ? -off : off;
        r[a] = fabsf(p[a]) < 1.0f / 32.0f ? p[a] + (1.0f / 65536.0f) * dn[a] : __int_as_float(bits);
    }
    return make_float3(r[0], r[1], r[2]);
}

// Primary + one shadow ray per pixel through the occupancy-brick grid.
__global__ void __launch_bounds__(128) voxel_primary_kernel(vox::Grid g, CamExact C, uint32_t W, uint32_t H, float3 sun,
                                                            float eps, FptCudaVoxelHit *hits, uchar4 *rgba) {
    uint32_t gx = blockIdx.x * 16u + (threadIdx.x & 15u), gy = blockIdx.y * 8u + (threadIdx.x >> 4);
    if (gx >= W || gy >= H) return;
    float2 uv = exact_uv(gx, gy, W, H);
    float3 d = exact_camera_dir(C, uv.x, uv.y);
    float3 o = make_float3(C.pos[0], C.pos[1], C.pos[2]);
    vox::Hit h = vox::trace_bricks(g, o, d);
    FptCudaVoxelHit out;
    out.t = h.hit ? h.t : -1.0f;
    out.cell = h.hit ? uint32_t(h.cell.x) + uint32_t(h.cell.y) * g.res + uint32_t(h.cell.z) * g.res * g.res : 0xffffffffu;
    out.normal_axis = h.hit ? (h.normal.x != 0.f ? (h.normal.x > 0.f ? 1u : 2u) : h.normal.y != 0.f ? (h.normal.y > 0.f ? 3u : 4u)
                                                                              : (h.normal.z > 0.f ? 5u : 6u))
                            : 0u;
    out.steps = h.steps;
    out.shadow_steps = 0;
    out.lit = 0;
    float shade = 0.0f;
    if (h.hit) {
        float3 pos = make_float3(o.x + d.x * h.t, o.y + d.y * h.t, o.z + d.z * h.t);
        float3 n = h.normal;
        if (n.x * d.x + n.y * d.y + n.z * d.z > 0.0f) n = make_float3(-n.x, -n.y, -n.z);
        float3 so = offset_origin(pos, n, sun, eps);
        vox::Hit s = vox::trace_bricks(g, so, sun);
        out.shadow_steps = s.steps ? s.steps : 0u;
        out.lit = s.hit ? 0u : 1u;
        float ndl = fmaxf(n.x * sun.x + n.y * sun.y + n.z * sun.z, 0.0f);
        shade = 0.15f + (out.lit ? 0.85f * ndl : 0.0f);
    }
    hits[size_t(gy) * W + gx] = out;
    if (rgba) {
        unsigned char v = (unsigned char)(fminf(fmaxf(shade, 0.f), 1.f) * 255.0f);
        rgba[size_t(H - 1 - gy) * W + gx] = make_uchar4(v, v, v, 255);
    }
}

__global__ void __launch_bounds__(128) dda_sequence_kernel(vox::Grid g, const float *rays, uint32_t n, uint32_t cap, uint32_t *seq,
                                                           uint32_t *seq_len, FptCudaVoxelHit *hits) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *r = rays + size_t(i) * 6;
    uint32_t len = 0;
    vox::Hit h = vox::trace(g, make_float3(r[0], r[1], r[2]), make_float3(r[3], r[4], r[5]), seq ? seq + size_t(i) * cap : nullptr,
                            cap, &len, nullptr);
    if (seq_len) seq_len[i] = len;
    FptCudaVoxelHit out;
    out.t = h.hit ? h.t : -1.0f;
    out.cell = h.hit ? uint32_t(h.cell.x) + uint32_t(h.cell.y) * g.res + uint32_t(h.cell.z) * g.res * g.res : 0xffffffffu;
    out.normal_axis = 0; out.steps = h.steps; out.shadow_steps = 0; out.lit = h.hit ? 1u : 0u;
    hits[i] = out;
}

// ---------------------------------------------------------------- reference voxel path
// renderVoxelPath (shaders/Shaders.metal:6526-6621) over reference-format
// cells, all samples of a pixel in one thread (voxel_accumulate_all_kernel,
// 7977-7992).  Face normals, stored materials, legacy origin offsets.
__device__ float3 voxel_env(const DeviceScene &S, float3 d) { return environment(d, S); }

__global__ void __launch_bounds__(128) voxel_path_kernel(const DeviceScene *scene, vox::Grid g, float4 *accum, uint32_t sample_begin,
                                                         uint32_t sample_end, uint32_t offset_mode) {
    const DeviceScene &S = *scene;
    uint32_t gx = blockIdx.x * 16u + (threadIdx.x & 15u), gy = blockIdx.y * 8u + (threadIdx.x >> 4);
    if (gx >= S.width || gy >= S.height) return;
    float u = (float(gx) + 0.5f) / float(S.width) - 0.5f, v = (float(gy) + 0.5f) / float(S.height) - 0.5f;
    u = u * (float(S.width) / float(S.height));
    uint32_t pixel = gy * S.width + gx;
    float3 mean = make_float3(0.f, 0.f, 0.f);
    if (sample_begin > 0u) { float4 a = accum[pixel]; mean = make_float3(a.x, a.y, a.z); }
    float cell = fminf(g.cs[0], fminf(g.cs[1], g.cs[2]));
    float eps = cell * 0.01f;
    for (uint32_t sample = sample_begin; sample < sample_end; ++sample) {
        PathRng rng;
        rng.init(S.rng == FPT_CUDA_RNG_PCG, S.seed, pixel, sample, u, v);
        float h1 = rng.uniform(SLOT_LENS0, 0), h2 = rng.uniform(SLOT_LENS1, 0);
        float sr, cr;
        sincosf(2.0f * h1 * kPi, &sr, &cr);
        float s = sqrtf(2.0f * h2 * kPi);
        float3 dir = normalize3(mk3(u + cr * s * S.aa_strength, v + sr * s * S.aa_strength, S.focal));
        dir = rotate_camera(dir, S.yaw, S.pitch, S.roll);
        float3 pos = mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]);
        float3 fp = pos + dir * S.focus_distance;
        float3 lens = mk3(cr * s * S.camera_dof, sr * s * S.camera_dof, 0.0f);
        pos = pos + rotate_camera(lens, S.yaw, S.pitch, S.roll);
        dir = normalize3(fp - pos);
        float3 light = mk3(0.0f), color = mk3(1.0f);
        float sky_mask = 0.0f;
        float3 gradc = background_gradient(dir, S);
        for (int bounce = 0; bounce < int(S.bounces); ++bounce) {
            uint32_t payload = 0;
            vox::Hit hit = vox::trace(g, pos, dir, nullptr, 0, nullptr, &payload);
            if (!hit.hit) {
                if (bounce == 0) sky_mask = 1.0f;
                light = light + environment(dir, S);
                break;
            }
            // unpackVoxelMaterial (shaders/Shaders.metal:4023-4035)
            uint32_t pc = g.cells[size_t(payload) * 3], pp = g.cells[size_t(payload) * 3 + 1];
            Material mt;
            mt.rgb = mk3(float(pc & 255u) / 255.0f, float((pc >> 8) & 255u) / 255.0f, float((pc >> 16) & 255u) / 255.0f);
            mt.roughness = float(pp & 255u) / 255.0f;
            mt.specular = float((pp >> 8) & 255u) / 255.0f;
            mt.translucency = float((pp >> 16) & 255u) / 255.0f;
            mt.ior = mixf(1.0f, 2.5f, float((pp >> 24) & 255u) / 255.0f);
            mt.emission = __uint_as_float(g.cells[size_t(payload) * 3 + 2]);
            mt.surface = 0;
            float3 hp = pos + dir * hit.t;
            if (mt.emission > 0.001f) light = light + mt.rgb * mt.emission;
            float3 nrm = hit.normal;
            if (dot(nrm, dir) > 0.0f) nrm = -nrm;
            if (S.sun[0] == 1.0f) {
                float3 ld = mk3(S.sun_dir[0], S.sun_dir[1], S.sun_dir[2]);
                float a1 = rng.uniform(SLOT_SUN0, bounce), a2 = rng.uniform(SLOT_SUN1, bounce);
                float sa, ca;
                sincosf(a1 * 2.0f * kPi, &sa, &ca);
                float ss = sqrtf(a2) * S.sun[4];
                ld = rotate_camera(ld, ca * ss, sa * ss);
                float3 so = offset_origin_mode(hp, nrm, ld, eps, offset_mode);
                vox::Hit sh = vox::trace(g, so, ld, nullptr, 0, nullptr, nullptr);
                if (!sh.hit)
                    light = light + mk3(S.sun_color[0], S.sun_color[1], S.sun_color[2]) *
                                        (S.sun[3] * fmaxf(dot(nrm, ld), 0.0f) * mt.roughness * (1.0f - mt.translucency));
            }
            float rs = rng.uniform(SLOT_SCATTER, bounce), rf = rng.uniform(SLOT_FRESNEL, bounce);
            bool transmitted = false;
            float f0 = (mt.ior - 1.0f) / (mt.ior + 1.0f);
            f0 = f0 * f0;
            float ct = clampf(dot(nrm, -dir), 0.0f, 1.0f);
            float fres = f0 + (1.0f - f0) * pow5f(1.0f - ct);
            if (rs > mt.translucency) {
                float3 refl = reflect3(dir, nrm);
                float d1 = rng.uniform(SLOT_DIR0, bounce), d2 = rng.uniform(SLOT_DIR1, bounce);
                float3 uu = normalize3(cross3(nrm, mk3(0.0f, 1.0f, 1.0f)));
                float3 vv = cross3(uu, nrm);
                float ra = sqrtf(d2), sn, cs;
                sincosf(kPi * 2.0f * d1, &sn, &cs);
                float3 diffuse = normalize3(uu * (ra * cs) + vv * (ra * sn) + nrm * sqrtf(fmaxf(1.0f - d2, 0.0f)));
                dir = normalize3(mix3(refl, diffuse, mt.roughness));
                if (rf < fres * mt.specular) dir = refl;
                else color = color * mt.rgb;
            } else {
                float3 refr = refract3(dir, nrm, 1.0f / mt.ior);
                float3 refl = reflect3(dir, nrm);
                if (dot(refr, refr) < 0.000001f || !isfinite(refr.x) || rf < fres) dir = normalize3(refl);
                else {
                    dir = normalize3(refr);
                    color = color * (mix3(mk3(1.0f), mt.rgb, 0.35f) * (1.0f - fres * 0.5f));
                    transmitted = true;
                }
            }
            pos = transmitted ? hp + dir * (cell * 1.05f) : offset_origin_mode(hp, nrm, dir, eps, offset_mode);
            if (S.russian_roulette != 0u && bounce + 1 < int(S.bounces) && float(bounce + 1) >= S.rr_start) {
                float surv = clampf(maxc3(color), clampf(S.rr_min_prob, 0.01f, 1.0f), 1.0f);
                if (rng.uniform(SLOT_RR, bounce) > surv) break;
                color = color / surv;
            }
        }
        float3 col = light * color;
        if (S.world[6] == 1.0f) col = mix3(col, gradc, sky_mask);
        col = min3(col, mk3(8.0f));
        mean = mix3(mean, col, 1.0f / float(sample + 1u));
    }
    accum[pixel] = make_float4(mean.x, mean.y, mean.z, 1.0f);
}

// voxel_dda_contract_test (shaders/Shaders.metal:5156-5211): cell
// ownership, tie advance, next-float advance and AABB cases; bit k set
// when case k fails.
__global__ void dda_contract_kernel(uint32_t *failure_mask) {
    if (threadIdx.x != 0) return;
    uint32_t f = 0u;
    vox::Grid g;
    for (int k = 0; k < 3; ++k) { g.bmin[k] = 0.0f; g.bmax[k] = 4.0f; g.cs[k] = 1.0f; }
    g.res = 4u;
    int3 c = make_int3(0, 0, 0);
    auto eq = [](int3 a, int x, int y, int z) { return a.x == x && a.y == y && a.z == z; };
    if (!vox::cell_coordinate(make_float3(1.f, 2.f, 3.f), make_float3(1.f, 1.f, 1.f), g, c) || !eq(c, 1, 2, 3)) f |= 1u << 0;
    if (!vox::cell_coordinate(make_float3(1.f, 2.f, 3.f), make_float3(-1.f, -1.f, -1.f), g, c) || !eq(c, 0, 1, 2)) f |= 1u << 1;
    if (!vox::cell_coordinate(make_float3(4.f, 4.f, 4.f), make_float3(-1.f, -1.f, -1.f), g, c) || !eq(c, 3, 3, 3)) f |= 1u << 2;
    if (vox::cell_coordinate(make_float3(4.f, 4.f, 4.f), make_float3(1.f, 1.f, 1.f), g, c)) f |= 1u << 3;
    if (!vox::cell_coordinate(make_float3(4.f, 4.f, 4.f), make_float3(0.f, 0.f, 0.f), g, c) || !eq(c, 3, 3, 3)) f |= 1u << 4;
    c = make_int3(0, 0, 0);
    int3 st = make_int3(1, 1, 1);
    float3 nt = make_float3(1.f, 1.f, 2.f), dt = make_float3(1.f, 1.f, 1.f), en = make_float3(0.f, 0.f, 0.f);
    float et = 0.0f;
    if (!vox::advance(c, st, nt, dt, et, en) || !eq(c, 1, 1, 0) || nt.x != 2.f || nt.y != 2.f || nt.z != 2.f || et != 1.0f ||
        en.x != -1.f || en.y != 0.f || en.z != 0.f)
        f |= 1u << 5;
    if (!vox::advance(c, st, nt, dt, et, en) || !eq(c, 2, 2, 1) || nt.x != 3.f || nt.y != 3.f || nt.z != 3.f || et != 2.0f)
        f |= 1u << 6;
    c = make_int3(0, 0, 0);
    nt = make_float3(1.f, 2.f, 3.f);
    et = 1.0f;
    if (!vox::advance(c, st, nt, dt, et, en) || __float_as_uint(et) != __float_as_uint(1.0f) + 1u || !eq(c, 1, 0, 0)) f |= 1u << 7;
    float nr, fr;
    if (!vox::ray_aabb(make_float3(-1.f, 2.f, 2.f), make_float3(1.0e-9f, 0.f, 0.f), g.bmin, g.bmax, nr, fr, en) || !(nr > 0.0f) ||
        !(fr > nr))
        f |= 1u << 8;
    if (vox::ray_aabb(make_float3(-1.f, 5.f, 2.f), make_float3(1.f, 0.f, 0.f), g.bmin, g.bmax, nr, fr, en)) f |= 1u << 9;
    *failure_mask = f;
}

// estimate_voxel_focus_distance_kernel (shaders/Shaders.metal:7630-7636).
__global__ void voxel_focus_kernel(vox::Grid g, DeviceScene *scene) {
    if (threadIdx.x != 0) return;
    DeviceScene &S = *scene;
    float3 d = rotate_camera(normalize3(mk3(0.0f, 0.0f, S.focal)), S.yaw, S.pitch, S.roll);
    vox::Hit h = vox::trace(g, mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]), d, nullptr, 0, nullptr, nullptr);
    S.focus_distance = h.hit && h.t > 0.001f ? h.t : 5.0f;
}

// ---------------------------------------------------------------- resident grid
struct VoxelState {
    bool built = false;
    uint32_t format = 0, brick_size = 0, res = 0, brick_grid = 0, active_bricks = 0;
    uint64_t active_cells = 0, memory_bytes = 0;
    float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0}, cs[3] = {0, 0, 0};
    uint32_t *table = nullptr; size_t cap_table = 0;
    uint32_t *count = nullptr; size_t cap_count = 0;
    uint32_t *offset = nullptr; size_t cap_offset = 0;
    uint32_t *sums = nullptr; size_t cap_sums = 0;
    unsigned long long *stats = nullptr; size_t cap_stats = 0;
    uint8_t *occ = nullptr; size_t cap_occ = 0;
    __half *dist = nullptr; size_t cap_dist = 0;
    uint32_t *mask = nullptr; size_t cap_mask = 0;
    uint4 *stage = nullptr; size_t cap_stage = 0;   // occupancy bricks: one staging slot per brick
    uint32_t *cells = nullptr; size_t cap_cells = 0;
    float *rays = nullptr; size_t cap_rays = 0;
    uint32_t *seq = nullptr; size_t cap_seq = 0;
    uint32_t *seq_len = nullptr; size_t cap_seq_len = 0;
    FptCudaVoxelHit *hits = nullptr; size_t cap_hits = 0;
};
static VoxelState &vstate() {
    static VoxelState v;
    return v;
}

static vox::Grid grid_view() {
    VoxelState &V = vstate();
    vox::Grid g;
    for (int k = 0; k < 3; ++k) { g.bmin[k] = V.bmin[k]; g.bmax[k] = V.bmax[k]; g.cs[k] = V.cs[k]; }
    g.res = V.res;
    g.brick_shift = V.brick_size == 8 ? 3u : 2u;
    g.brick_grid = V.brick_grid;
    g.storage = V.format == VF_OCCUPANCY ? 4u : (V.brick_size == 0 ? 0u : 1u);
    g.table = V.table;
    g.occ = V.occ;
    g.mask = reinterpret_cast<const uint64_t *>(V.mask);
    g.cells = V.cells;
    return g;
}

template <int KIND>
static bool launch_build(const DeviceScene *scene, const VoxBuild &B, uint32_t bs, uint32_t format, cudaStream_t st, char *error,
                         size_t error_len) {
    VoxelState &V = vstate();
    const uint32_t nb = B.brick_grid * B.brick_grid * B.brick_grid;
    if (format == VF_OCCUPANCY) {
        if (!ensure_buffer((void **)&V.stage, &V.cap_stage, size_t(nb) * kBrickStageBytes, error, error_len)) return false;
        brick_stage_kernel<KIND><<<nb, 512, 0, st>>>(scene, B, V.count, V.stats, V.stage);
    } else if (bs == 8) {
        brick_classify_kernel<KIND, 8><<<nb, 512, 0, st>>>(scene, B, V.count, V.stats);
    } else {
        brick_classify_kernel<KIND, 4><<<nb, 64, 0, st>>>(scene, B, V.count, V.stats);
    }
    uint32_t nblocks = (nb + kScanBlock - 1) / kScanBlock;
    scan_blocks_kernel<<<nblocks, kScanThreads, 0, st>>>(V.count, nb, V.offset, V.sums);
    scan_sums_kernel<<<1, kScanThreads, 0, st>>>(V.sums, nblocks, reinterpret_cast<uint32_t *>(V.stats + 1));
    scan_add_kernel<<<(nb + 255) / 256, 256, 0, st>>>(V.offset, nb, V.sums);
    if (!check(cudaGetLastError(), "voxel classify/scan launch", error, error_len)) return false;
    // Size the payload from the active-brick total.
    unsigned long long host_stats[2] = {0, 0};
    if (!check(cudaMemcpyAsync(host_stats, V.stats, sizeof(host_stats), cudaMemcpyDeviceToHost, st), "voxel count readback", error,
               error_len))
        return false;
    if (!check(cudaStreamSynchronize(st), "voxel classification", error, error_len)) return false;
    V.active_cells = host_stats[0];
    V.active_bricks = uint32_t(host_stats[1] & 0xffffffffull);
    const size_t cells = std::max<size_t>(1, size_t(V.active_bricks) * bs * bs * bs);
    if (format == VF_OCCUPANCY) {
        if (!ensure_buffer((void **)&V.occ, &V.cap_occ, cells, error, error_len)) return false;
        if (!ensure_buffer((void **)&V.dist, &V.cap_dist, cells * sizeof(__half), error, error_len)) return false;
        if (!ensure_buffer((void **)&V.mask, &V.cap_mask, (cells + 31) / 32 * 4, error, error_len)) return false;
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx().device);
        const uint32_t blocks = std::min<uint32_t>((nb + 7u) / 8u, uint32_t(std::max(sms, 1)) * 32u);
        brick_commit_kernel<<<blocks, 256, 0, st>>>(V.count, V.offset, nb, V.stage, V.table, reinterpret_cast<uint4 *>(V.occ),
                                                     reinterpret_cast<uint4 *>(V.dist), reinterpret_cast<uint4 *>(V.mask));
        V.memory_bytes = size_t(nb) * 4 + cells * (1 + 2) + (cells + 31) / 32 * 4;
    } else {
        if (!ensure_buffer((void **)&V.cells, &V.cap_cells, cells * 12, error, error_len)) return false;
        brick_fill_kernel<KIND, 4><<<nb, 64, 0, st>>>(scene, B, V.count, V.offset, V.table, V.cells);
        V.memory_bytes = size_t(nb) * 4 + cells * 12;
    }
    return check(cudaGetLastError(), "voxel fill launch", error, error_len);
}

// Builds the resident grid for (config, ext).  brick_size 8 -> occupancy
// bricks, 4 -> reference cells, 0 -> reference dense storage.
static bool build_grid(const FptRenderConfig &config, const FptCudaSceneExt *ext, DeviceScene &S, uint32_t brick_size,
                       double *build_ms, char *error, size_t error_len) {
    Context &c = ctx();
    VoxelState &V = vstate();
    uint32_t res = config.voxel_resolution;
    if (res == 0 || res > 4096) { set_error(error, error_len, "voxel resolution %u out of range (1..4096)", res); return false; }
    if (config.voxel_coverage_mode != FPT_VOXEL_COVERAGE_LEGACY) {
        set_error(error, error_len, "voxel coverage mode %u (certified program bounds) is not supported by the CUDA path",
                  config.voxel_coverage_mode);
        return false;
    }
    if (brick_size != 0 && brick_size != 4 && brick_size != 8) { set_error(error, error_len, "brick size must be 4 or 8"); return false; }
    for (int k = 0; k < 3; ++k) {
        if (!(config.voxel_bounds_max[k] > config.voxel_bounds_min[k])) {
            set_error(error, error_len, "voxel bounds must be increasing on every axis");
            return false;
        }
    }
    if (!upload_scene(S, ext, error, error_len)) return false;
    VoxBuild B;
    for (int k = 0; k < 3; ++k) {
        B.bmin[k] = config.voxel_bounds_min[k];
        B.cs[k] = (config.voxel_bounds_max[k] - config.voxel_bounds_min[k]) / float(res);
        V.bmin[k] = config.voxel_bounds_min[k];
        V.bmax[k] = config.voxel_bounds_max[k];
        V.cs[k] = B.cs[k];
    }
    float hx = B.cs[0] * 0.5f, hy = B.cs[1] * 0.5f, hz = B.cs[2] * 0.5f;
    B.half_radius = sqrtf(hx * hx + hy * hy + hz * hz);
    B.band = config.voxel_surface_band;
    B.res = res;
    B.fill_interior = config.voxel_fill_interior;
    V.res = res;
    V.brick_size = brick_size;
    V.format = brick_size == 8 ? VF_OCCUPANCY : VF_REFERENCE;
    V.built = false;
    cudaEventRecord(c.ev0, c.stream);
    if (!ensure_buffer((void **)&V.stats, &V.cap_stats, 64, error, error_len)) return false;
    if (!check(cudaMemsetAsync(V.stats, 0, 64, c.stream), "voxel stats reset", error, error_len)) return false;
    if (brick_size == 0) {
        size_t n = size_t(res) * res * res;
        V.brick_grid = 0;
        if (!ensure_buffer((void **)&V.cells, &V.cap_cells, n * 12, error, error_len)) return false;
        if (S.kind == KIND_BOX) dense_fill_kernel<KIND_BOX><<<unsigned((n + 255) / 256), 256, 0, c.stream>>>(c.scene, B, V.cells, V.stats);
        else dense_fill_kernel<KIND_GENERIC><<<unsigned((n + 255) / 256), 256, 0, c.stream>>>(c.scene, B, V.cells, V.stats);
        unsigned long long cells = 0;
        if (!check(cudaMemcpyAsync(&cells, V.stats, 8, cudaMemcpyDeviceToHost, c.stream), "voxel readback", error, error_len)) return false;
        if (!check(cudaStreamSynchronize(c.stream), "dense voxel build", error, error_len)) return false;
        V.active_cells = cells;
        V.active_bricks = 0;
        V.memory_bytes = n * 12;
    } else {
        uint32_t bg = (res + brick_size - 1) / brick_size;
        B.brick_grid = bg;
        V.brick_grid = bg;
        const size_t nb = size_t(bg) * bg * bg;
        if (!ensure_buffer((void **)&V.table, &V.cap_table, nb * 4, error, error_len)) return false;
        if (!ensure_buffer((void **)&V.count, &V.cap_count, nb * 4, error, error_len)) return false;
        if (!ensure_buffer((void **)&V.offset, &V.cap_offset, nb * 4, error, error_len)) return false;
        if (!ensure_buffer((void **)&V.sums, &V.cap_sums, ((nb + kScanBlock - 1) / kScanBlock + 1) * 4, error, error_len)) return false;
        bool ok = S.kind == KIND_BOX ? launch_build<KIND_BOX>(c.scene, B, brick_size, V.format, c.stream, error, error_len)
                                     : launch_build<KIND_GENERIC>(c.scene, B, brick_size, V.format, c.stream, error, error_len);
        if (!ok) return false;
    }
    cudaEventRecord(c.ev1, c.stream);
    if (!check(cudaStreamSynchronize(c.stream), "voxel build", error, error_len)) return false;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    if (build_ms) *build_ms = ms;
    V.built = true;
    return true;
}

static CamExact exact_camera(const FptRenderConfig &c) {
    CamExact C;
    for (int k = 0; k < 3; ++k) C.pos[k] = c.camera_position[k];
    C.focal = 1.0f / std::tan(c.camera_fov / 2.0f * 3.14159265359f / 180.0f);
    C.sr = std::sin(c.camera_roll); C.cr = std::cos(c.camera_roll);
    C.sp = std::sin(c.camera_yaw_pitch[1]); C.cp = std::cos(c.camera_yaw_pitch[1]);
    C.sy = std::sin(c.camera_yaw_pitch[0]); C.cy = std::cos(c.camera_yaw_pitch[0]);
    return C;
}

int voxel_render_core(const FptRenderConfig &config, const FptCudaSceneExt *ext, DeviceScene &S, const char *output_path,
                      float *linear_output, uint8_t *rgba_output, double *elapsed_ms, uint64_t *voxel_memory_bytes,
                      uint32_t *voxel_active_bricks, uint64_t *voxel_active_cells, double *build_ms, char *error,
                      size_t error_len) {
    Context &c = ctx();
    if (config.voxel_storage == FPT_VOXEL_STORAGE_TEMPLATE_BRICKS) {
        set_error(error, error_len, "template-brick voxel storage is not supported by the CUDA path");
        return 1;
    }
    // renderVoxelPath modes the CUDA path does not restate fail loudly instead
    // of rendering with the defaults.
    if (config.voxel_normal_mode != FPT_VOXEL_NORMAL_FACE) {
        set_error(error, error_len, "voxel normal mode %u (smooth / exact field normals) is not supported by the CUDA path",
                  config.voxel_normal_mode);
        return 1;
    }
    if (config.voxel_material_mode != FPT_VOXEL_MATERIAL_STORED) {
        set_error(error, error_len, "voxel material mode %u (exact materials) is not supported by the CUDA path",
                  config.voxel_material_mode);
        return 1;
    }
    if (config.voxel_leaf_refinement != FPT_VOXEL_LEAF_REFINEMENT_NONE) {
        set_error(error, error_len, "voxel leaf refinement %u is not supported by the CUDA path", config.voxel_leaf_refinement);
        return 1;
    }
    if (config.voxel_offset_mode != FPT_VOXEL_OFFSET_LEGACY && config.voxel_offset_mode != FPT_VOXEL_OFFSET_PRECISION) {
        set_error(error, error_len, "unknown voxel offset mode %u", config.voxel_offset_mode);
        return 1;
    }
    uint32_t bs = config.voxel_storage == FPT_VOXEL_STORAGE_DENSE ? 0u : 4u;
    if (!build_grid(config, ext, S, bs, build_ms, error, error_len)) return 1;
    VoxelState &V = vstate();
    if (voxel_memory_bytes) *voxel_memory_bytes = V.memory_bytes;
    if (voxel_active_bricks) *voxel_active_bricks = V.active_bricks;
    if (voxel_active_cells) *voxel_active_cells = V.active_cells;
    const size_t pixels = size_t(S.width) * S.height;
    if (!ensure_buffer((void **)&c.accum, &c.cap_accum, pixels * sizeof(float4), error, error_len)) return 1;
    if (!ensure_buffer((void **)&c.rgba, &c.cap_rgba, pixels * sizeof(uchar4), error, error_len)) return 1;
    cudaEventRecord(c.ev0, c.stream);
    if (S.focus_distance <= 0.0f) voxel_focus_kernel<<<1, 32, 0, c.stream>>>(grid_view(), c.scene);
    dim3 grid((S.width + 15u) / 16u, (S.height + 7u) / 8u);
    const uint32_t spp = S.samples;
    const uint32_t step = (config.sdf_accumulation_mode == FPT_SDF_ACCUMULATION_CHUNKED)
                              ? std::min(std::max(config.sdf_chunk_samples, 1u), 64u)
                              : (config.sdf_accumulation_mode == FPT_SDF_ACCUMULATION_PER_SAMPLE ? 1u : spp);
    for (uint32_t s0 = 0; s0 < spp; s0 += step)
        voxel_path_kernel<<<grid, 128, 0, c.stream>>>(c.scene, grid_view(), c.accum, s0, std::min(spp, s0 + step),
                                                       config.voxel_offset_mode);
    if (!check(launch_present(c.scene, S.width, S.height, c.accum, c.rgba, c.stream), "present launch", error, error_len)) return 1;
    cudaEventRecord(c.ev1, c.stream);
    if (!check(cudaStreamSynchronize(c.stream), "voxel render", error, error_len)) return 1;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    if (elapsed_ms) *elapsed_ms = ms;
    std::vector<uint8_t> host(pixels * 4);
    uint8_t *rgba = rgba_output ? rgba_output : host.data();
    if (!check(cudaMemcpy(rgba, c.rgba, pixels * 4, cudaMemcpyDeviceToHost), "image readback", error, error_len)) return 1;
    if (linear_output &&
        !check(cudaMemcpy(linear_output, c.accum, pixels * sizeof(float4), cudaMemcpyDeviceToHost), "linear readback", error, error_len))
        return 1;
    if (output_path) {
        if (unique_colour_sample(rgba, pixels) < 2) { set_error(error, error_len, "render output is blank or single-colour"); return 1; }
        std::string err;
        if (!write_png(output_path, S.width, S.height, rgba, err)) { set_error(error, error_len, "%s", err.c_str()); return 1; }
    }
    return 0;
}

}  // namespace fpt

using namespace fpt;

extern "C" {

int fpt_cuda_voxel_build(const struct FptRenderConfig *config, const struct FptCudaSceneExt *ext, uint32_t brick_size,
                         struct FptCudaVoxelInfo *info, char *error, size_t error_len) {
    if (info) std::memset(info, 0, sizeof(*info));
    if (!config) { set_error(error, error_len, "missing voxel config"); return 1; }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    DeviceScene S;
    if (!compile_scene(*config, ext, S, error, error_len)) return 1;
    double ms = 0.0;
    if (!build_grid(*config, ext, S, brick_size, &ms, error, error_len)) return 1;
    VoxelState &V = vstate();
    if (info) {
        info->resolution = V.res; info->brick_size = V.brick_size; info->brick_grid = V.brick_grid;
        info->active_bricks = V.active_bricks; info->active_cells = V.active_cells; info->memory_bytes = V.memory_bytes;
        info->build_ms = ms;
    }
    return 0;
}

int fpt_cuda_voxel_read(uint32_t *brick_table, size_t table_len, uint8_t *occupancy, uint16_t *distance, uint32_t *cells,
                        size_t cell_len, char *error, size_t error_len) {
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    VoxelState &V = vstate();
    if (!V.built) { set_error(error, error_len, "no voxel grid has been built"); return 1; }
    size_t nb = size_t(V.brick_grid) * V.brick_grid * V.brick_grid;
    size_t bsz = size_t(V.brick_size) * V.brick_size * V.brick_size;
    size_t ncell = V.brick_size ? size_t(V.active_bricks) * bsz : size_t(V.res) * V.res * V.res;
    if (brick_table) {
        if (table_len < nb) { set_error(error, error_len, "brick table buffer too small (%zu < %zu)", table_len, nb); return 1; }
        if (!check(cudaMemcpy(brick_table, V.table, nb * 4, cudaMemcpyDeviceToHost), "table readback", error, error_len)) return 1;
    }
    if ((occupancy || distance || cells) && cell_len < ncell) {
        set_error(error, error_len, "cell buffer too small (%zu < %zu)", cell_len, ncell);
        return 1;
    }
    if (occupancy && V.format == VF_OCCUPANCY && ncell &&
        !check(cudaMemcpy(occupancy, V.occ, ncell, cudaMemcpyDeviceToHost), "occupancy readback", error, error_len))
        return 1;
    if (distance && V.format == VF_OCCUPANCY && ncell &&
        !check(cudaMemcpy(distance, V.dist, ncell * 2, cudaMemcpyDeviceToHost), "distance readback", error, error_len))
        return 1;
    if (cells && V.format == VF_REFERENCE && ncell &&
        !check(cudaMemcpy(cells, V.cells, ncell * 12, cudaMemcpyDeviceToHost), "cell readback", error, error_len))
        return 1;
    return 0;
}

int fpt_cuda_dda_sequence(const float *rays, size_t ray_count, uint32_t capacity, uint32_t *sequence, uint32_t *sequence_len,
                          struct FptCudaVoxelHit *hits, char *error, size_t error_len) {
    if (!rays || !hits || ray_count == 0) { set_error(error, error_len, "missing DDA input"); return 1; }
    if (ray_count > 0xffffffffull) { set_error(error, error_len, "too many rays"); return 1; }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    VoxelState &V = vstate();
    if (!V.built) { set_error(error, error_len, "no voxel grid has been built"); return 1; }
    uint32_t n = uint32_t(ray_count);
    if (!ensure_buffer((void **)&V.rays, &V.cap_rays, size_t(n) * 24, error, error_len)) return 1;
    if (!ensure_buffer((void **)&V.hits, &V.cap_hits, size_t(n) * sizeof(FptCudaVoxelHit), error, error_len)) return 1;
    if (!ensure_buffer((void **)&V.seq_len, &V.cap_seq_len, size_t(n) * 4, error, error_len)) return 1;
    bool want_seq = sequence && sequence_len && capacity > 0;
    if (want_seq && !ensure_buffer((void **)&V.seq, &V.cap_seq, size_t(n) * capacity * 4, error, error_len)) return 1;
    if (!check(cudaMemcpyAsync(V.rays, rays, size_t(n) * 24, cudaMemcpyHostToDevice, c.stream), "ray upload", error, error_len)) return 1;
    dda_sequence_kernel<<<(n + 127) / 128, 128, 0, c.stream>>>(grid_view(), V.rays, n, want_seq ? capacity : 0,
                                                              want_seq ? V.seq : nullptr, V.seq_len, V.hits);
    if (!check(cudaStreamSynchronize(c.stream), "DDA sequence", error, error_len)) return 1;
    if (!check(cudaMemcpy(hits, V.hits, size_t(n) * sizeof(FptCudaVoxelHit), cudaMemcpyDeviceToHost), "hit readback", error, error_len))
        return 1;
    if (want_seq) {
        if (!check(cudaMemcpy(sequence_len, V.seq_len, size_t(n) * 4, cudaMemcpyDeviceToHost), "length readback", error, error_len))
            return 1;
        if (!check(cudaMemcpy(sequence, V.seq, size_t(n) * capacity * 4, cudaMemcpyDeviceToHost), "sequence readback", error, error_len))
            return 1;
    }
    return 0;
}

int fpt_test_voxel_dda(const char *metallib_path, char *error, size_t error_len) {
    (void)metallib_path;
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    uint32_t *mask = nullptr;
    if (!check(cudaMalloc(&mask, 4), "contract buffer", error, error_len)) return 1;
    dda_contract_kernel<<<1, 32, 0, c.stream>>>(mask);
    uint32_t f = 0xffffffffu;
    bool ok = check(cudaStreamSynchronize(c.stream), "DDA contract kernel", error, error_len) &&
              check(cudaMemcpy(&f, mask, 4, cudaMemcpyDeviceToHost), "contract readback", error, error_len);
    cudaFree(mask);
    if (!ok) return 1;
    if (f != 0u) { set_error(error, error_len, "DDA contract failure mask: 0x%08x", f); return 1; }
    // 32^3 sphere program, dense cells versus 4^3 bricks (src/metal_bridge.mm:3836-3923).
    FptRenderConfig cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    cfg.sdf_id = FPT_SDF_PROGRAM;
    cfg.voxel_surface_band = 0.5f;
    cfg.sdf_program_count = 1;
    cfg.sdf_program[0].opcode = FPT_SDF_OP_SPHERE;
    cfg.sdf_program[0].data[0] = 1.0f;
    cfg.program_material[0] = cfg.program_material[1] = cfg.program_material[2] = 1.0f;
    cfg.program_material[3] = 1.0f;
    cfg.program_material[6] = 1.5f;
    cfg.voxel_resolution = 32u;
    for (int k = 0; k < 3; ++k) { cfg.voxel_bounds_min[k] = -2.0f; cfg.voxel_bounds_max[k] = 2.0f; }
    cfg.width = cfg.height = 1;
    DeviceScene S;
    if (!compile_scene(cfg, nullptr, S, error, error_len)) return 1;
    std::vector<uint32_t> dense(32u * 32u * 32u * 3u), table(8u * 8u * 8u), bricks;
    if (!build_grid(cfg, nullptr, S, 0u, nullptr, error, error_len)) return 1;
    VoxelState &V = vstate();
    uint64_t dense_cells = V.active_cells;
    if (!check(cudaMemcpy(dense.data(), V.cells, dense.size() * 4, cudaMemcpyDeviceToHost), "dense readback", error, error_len)) return 1;
    if (!build_grid(cfg, nullptr, S, 4u, nullptr, error, error_len)) return 1;
    if (V.active_cells != dense_cells) { set_error(error, error_len, "brick build occupancy totals differ from dense build"); return 1; }
    bricks.resize(size_t(std::max(V.active_bricks, 1u)) * 64u * 3u);
    if (!check(cudaMemcpy(table.data(), V.table, table.size() * 4, cudaMemcpyDeviceToHost), "table readback", error, error_len) ||
        !check(cudaMemcpy(bricks.data(), V.cells, size_t(V.active_bricks) * 64u * 12u, cudaMemcpyDeviceToHost), "brick readback", error,
               error_len))
        return 1;
    for (uint32_t z = 0; z < 32; ++z)
        for (uint32_t y = 0; y < 32; ++y)
            for (uint32_t x = 0; x < 32; ++x) {
                uint32_t page = table[x / 4 + (y / 4) * 8 + (z / 4) * 64];
                const uint32_t *a = &dense[(x + y * 32 + z * 1024) * 3];
                uint32_t zero[3] = {0, 0, 0};
                const uint32_t *b = page ? &bricks[((page - 1) * 64 + x % 4 + (y % 4) * 4 + (z % 4) * 16) * 3] : zero;
                if (a[0] != b[0] || a[1] != b[1] || a[2] != b[2]) {
                    set_error(error, error_len, "brick-build cell mismatch at (%u,%u,%u)", x, y, z);
                    return 1;
                }
            }
    return 0;
}

int fpt_cuda_voxel_render(const struct FptRenderConfig *config, const struct FptCudaSceneExt *ext, struct FptCudaVoxelHit *hits,
                          size_t hit_count, uint8_t *rgba, size_t rgba_len, double *elapsed_ms, char *error, size_t error_len) {
    (void)ext;
    if (elapsed_ms) *elapsed_ms = 0.0;
    if (!config || !hits) { set_error(error, error_len, "missing voxel render input"); return 1; }
    size_t pixels = size_t(config->width) * config->height;
    if (pixels == 0) { set_error(error, error_len, "invalid render size %ux%u", config->width, config->height); return 1; }
    if (hit_count < pixels) { set_error(error, error_len, "hit buffer too small (%zu < %zu)", hit_count, pixels); return 1; }
    if (rgba && rgba_len < pixels * 4) { set_error(error, error_len, "rgba buffer too small"); return 1; }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    VoxelState &V = vstate();
    if (!V.built || V.format != VF_OCCUPANCY) { set_error(error, error_len, "build an occupancy-brick grid first"); return 1; }
    if (!ensure_buffer((void **)&V.hits, &V.cap_hits, pixels * sizeof(FptCudaVoxelHit), error, error_len)) return 1;
    if (!ensure_buffer((void **)&c.rgba, &c.cap_rgba, pixels * 4, error, error_len)) return 1;
    // Sun direction: the extension direction when given, else rotateCamera of the config sun angles.
    float sun[3];
    if (ext && ext->sun_intensity > 0.0f) {
        float n = std::sqrt(ext->sun_direction[0] * ext->sun_direction[0] + ext->sun_direction[1] * ext->sun_direction[1] +
                            ext->sun_direction[2] * ext->sun_direction[2]);
        for (int k = 0; k < 3; ++k) sun[k] = ext->sun_direction[k] / n;
    } else {
        float yaw = config->sun[1] * 3.14159265359f / 180.0f, pitch = config->sun[2] * 3.14159265359f / 180.0f;
        float y = std::sin(pitch), z = std::cos(pitch);
        sun[0] = z * std::sin(yaw); sun[1] = y; sun[2] = z * std::cos(yaw);
    }
    float eps = std::min(V.cs[0], std::min(V.cs[1], V.cs[2])) * 0.01f;
    dim3 grid((config->width + 15u) / 16u, (config->height + 7u) / 8u);
    cudaEventRecord(c.ev0, c.stream);
    voxel_primary_kernel<<<grid, 128, 0, c.stream>>>(grid_view(), exact_camera(*config), config->width, config->height,
                                                    make_float3(sun[0], sun[1], sun[2]), eps, V.hits, c.rgba);
    cudaEventRecord(c.ev1, c.stream);
    if (!check(cudaStreamSynchronize(c.stream), "voxel primary render", error, error_len)) return 1;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    if (elapsed_ms) *elapsed_ms = ms;
    if (!check(cudaMemcpy(hits, V.hits, pixels * sizeof(FptCudaVoxelHit), cudaMemcpyDeviceToHost), "hit readback", error, error_len))
        return 1;
    if (rgba && !check(cudaMemcpy(rgba, c.rgba, pixels * 4, cudaMemcpyDeviceToHost), "image readback", error, error_len)) return 1;
    return 0;
}

}  // extern "C"

// ====================================================================== build without allocation
// fpt_cuda_voxel_build_static: the occupancy-brick build for callers that
// cannot allocate device memory.  Its scratch (scene block, per-brick
// counts and offsets, scan partials, counters) is one file-scope device
// array of fixed size, so the entry point calls no cudaMalloc, cudaFree or
// allocating library routine; the caller passes the outputs.
namespace fpt {

constexpr uint32_t kStaticMaxResolution = 512;                    // 8^3 bricks: at most 64^3 of them
constexpr uint32_t kStaticMaxBricks = 64u * 64u * 64u;
constexpr uint32_t kStaticScanBlocks = (kStaticMaxBricks + kScanBlock - 1) / kScanBlock;

struct StaticVoxelScratch {
    unsigned long long stats[8];            // [0] active cells, [1] low word: active bricks
    uint32_t sums[kStaticScanBlocks + 32];
    uint32_t count[kStaticMaxBricks];
    uint32_t offset[kStaticMaxBricks];
    DeviceScene scene;
};

// About 2.1 MB, held by every GPU that loads the library until the process exits.
static __device__ __align__(256) StaticVoxelScratch g_voxel_static_scratch;

// Device address of g_voxel_static_scratch per device ordinal (the host-side
// name is only a stand-in and must never be passed to a kernel).
constexpr int kStaticMaxDevices = 64;
static StaticVoxelScratch *g_static_scratch_addr[kStaticMaxDevices] = {nullptr};

template <int KIND>
__global__ void __launch_bounds__(512) static_fill_kernel(const DeviceScene *scene, VoxBuild B, const uint32_t *brick_count,
                                                          const uint32_t *brick_offset, uint32_t *table, uint8_t *occ_out,
                                                          uint16_t *dist_out, size_t cell_capacity) {
    const DeviceScene &S = *scene;
    uint32_t b = blockIdx.x;
    if (brick_count[b] == 0u) {
        if (threadIdx.x == 0) table[b] = 0u;
        return;
    }
    uint32_t id = brick_offset[b];
    if (threadIdx.x == 0) table[b] = id + 1u;
    uint32_t bx = b % B.brick_grid, by = (b / B.brick_grid) % B.brick_grid, bz = b / (B.brick_grid * B.brick_grid);
    uint32_t l = threadIdx.x;
    uint32_t x = bx * 8u + l % 8u, y = by * 8u + (l / 8u) % 8u, z = bz * 8u + l / 64u;
    bool inside = x < B.res && y < B.res && z < B.res;
    bool occ = false;
    float d = 0.0f;
    float3 p;
    if (inside) occ = classify_cell<KIND>(S, B, x, y, z, d, p);
    size_t slot = size_t(id) * 512u + l;
    if (slot < cell_capacity) {
        occ_out[slot] = occ ? 1u : 0u;
        dist_out[slot] = __half_as_ushort(__float2half_rn(inside ? d : 0.0f));
    }
}

}  // namespace fpt

extern "C" int fpt_cuda_voxel_build_static(const struct FptRenderConfig *config, const struct FptCudaSceneExt *ext, void *stream,
                                           uint32_t *device_brick_table, size_t table_len, uint8_t *device_occupancy,
                                           uint16_t *device_distance, size_t cell_capacity, struct FptCudaVoxelInfo *info,
                                           char *error, size_t error_len) {
    using namespace fpt;
    if (info) std::memset(info, 0, sizeof(*info));
    if (!config || !device_brick_table || !device_occupancy || !device_distance) {
        set_error(error, error_len, "missing voxel build input or output buffer");
        return 1;
    }
    const uint32_t res = config->voxel_resolution;
    if (res == 0 || res > kStaticMaxResolution) {
        set_error(error, error_len, "voxel resolution %u out of range for the allocation-free build (1..%u)", res,
                  kStaticMaxResolution);
        return 1;
    }
    for (int k = 0; k < 3; ++k) {
        if (!(config->voxel_bounds_max[k] > config->voxel_bounds_min[k])) {
            set_error(error, error_len, "voxel bounds must be increasing on every axis");
            return 1;
        }
    }
    const uint32_t bg = (res + 7u) / 8u;
    const uint32_t nb = bg * bg * bg;
    if (table_len < nb) {
        set_error(error, error_len, "brick table buffer too small (%zu < %u)", table_len, nb);
        return 1;
    }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    DeviceScene S;
    if (!compile_scene(*config, ext, S, error, error_len)) return 1;
    if (S.sky_width || S.surrogate) {
        set_error(error, error_len, "sky textures and surrogate models are not used by the voxel build; clear them");
        return 1;
    }
    int dev = 0;
    if (!check(cudaGetDevice(&dev), "cudaGetDevice", error, error_len)) return 1;
    if (dev < 0 || dev >= kStaticMaxDevices) { set_error(error, error_len, "device ordinal %d out of range", dev); return 1; }
    // Set-up, once per device, with that device current: the device address of the scratch array.
    if (!g_static_scratch_addr[dev]) {
        void *addr = nullptr;
        if (!check(cudaGetSymbolAddress(&addr, g_voxel_static_scratch), "cudaGetSymbolAddress", error, error_len)) return 1;
        g_static_scratch_addr[dev] = static_cast<StaticVoxelScratch *>(addr);
    }
    StaticVoxelScratch *sc = g_static_scratch_addr[dev];
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // The build synchronises its stream twice, which a stream capture cannot record: refuse instead of breaking
    // the caller's graph.
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (!check(cudaStreamIsCapturing(st, &capture), "cudaStreamIsCapturing", error, error_len)) return 1;
    if (capture != cudaStreamCaptureStatusNone) {
        set_error(error, error_len, "the allocation-free voxel build synchronises its stream and cannot run inside a stream capture");
        return 1;
    }
    VoxBuild B;
    for (int k = 0; k < 3; ++k) {
        B.bmin[k] = config->voxel_bounds_min[k];
        B.cs[k] = (config->voxel_bounds_max[k] - config->voxel_bounds_min[k]) / float(res);
    }
    float hx = B.cs[0] * 0.5f, hy = B.cs[1] * 0.5f, hz = B.cs[2] * 0.5f;
    B.half_radius = sqrtf(hx * hx + hy * hy + hz * hz);
    B.band = config->voxel_surface_band;
    B.res = res;
    B.brick_grid = bg;
    B.fill_interior = config->voxel_fill_interior;
    auto t0 = std::chrono::steady_clock::now();
    // The array keeps the previous call's contents: reset the counters.
    if (!check(cudaMemcpyAsync(&sc->scene, &S, sizeof(DeviceScene), cudaMemcpyHostToDevice, st), "scene upload", error, error_len) ||
        !check(cudaMemsetAsync(sc->stats, 0, sizeof(sc->stats), st), "counter reset", error, error_len))
        return 1;
    if (S.kind == KIND_BOX) brick_classify_kernel<KIND_BOX, 8><<<nb, 512, 0, st>>>(&sc->scene, B, sc->count, sc->stats);
    else brick_classify_kernel<KIND_GENERIC, 8><<<nb, 512, 0, st>>>(&sc->scene, B, sc->count, sc->stats);
    const uint32_t nblocks = (nb + kScanBlock - 1) / kScanBlock;
    scan_blocks_kernel<<<nblocks, kScanThreads, 0, st>>>(sc->count, nb, sc->offset, sc->sums);
    scan_sums_kernel<<<1, kScanThreads, 0, st>>>(sc->sums, nblocks, reinterpret_cast<uint32_t *>(sc->stats + 1));
    scan_add_kernel<<<(nb + 255) / 256, 256, 0, st>>>(sc->offset, nb, sc->sums);
    if (!check(cudaGetLastError(), "classification launch", error, error_len)) return 1;
    unsigned long long counts[2] = {0, 0};
    if (!check(cudaMemcpyAsync(counts, sc->stats, sizeof(counts), cudaMemcpyDeviceToHost, st), "count readback", error, error_len) ||
        !check(cudaStreamSynchronize(st), "voxel classification", error, error_len))
        return 1;
    const uint32_t active = uint32_t(counts[1] & 0xffffffffull);
    const size_t need = size_t(active) * 512u;
    if (need > cell_capacity) {
        set_error(error, error_len, "cell buffers too small: %u active bricks need %zu cells (capacity %zu)", active, need,
                  cell_capacity);
        return 1;
    }
    if (S.kind == KIND_BOX)
        static_fill_kernel<KIND_BOX><<<nb, 512, 0, st>>>(&sc->scene, B, sc->count, sc->offset, device_brick_table, device_occupancy,
                                                         device_distance, cell_capacity);
    else
        static_fill_kernel<KIND_GENERIC><<<nb, 512, 0, st>>>(&sc->scene, B, sc->count, sc->offset, device_brick_table,
                                                             device_occupancy, device_distance, cell_capacity);
    if (!check(cudaGetLastError(), "fill launch", error, error_len) || !check(cudaStreamSynchronize(st), "voxel fill", error, error_len))
        return 1;
    if (info) {
        info->resolution = res;
        info->brick_size = 8;
        info->brick_grid = bg;
        info->active_bricks = active;
        info->active_cells = counts[0];
        info->memory_bytes = size_t(nb) * 4 + need * 3;
        info->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return 0;
}

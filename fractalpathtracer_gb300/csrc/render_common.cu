// render_common.cu -- present kernel and the per-kind dispatch of the launchers.
#include "render_impl.cuh"
#include "fpt_post.cuh"

namespace fpt {

// ---------------------------------------------------------------- present
// present_kernel (shaders/Shaders.metal:8012-8025) with highlightAt
// (7466-7481), sampleAccumBilinear (7483-7496), chromaticAt (7498-7507),
// postProcess/toneMap (6778-6825) and the vertical flip of outputIndex.
__global__ void __launch_bounds__(256) present_kernel(const DeviceScene *scene, const float4 *accum, uchar4 *out) {
    const DeviceScene &S = *scene;
    uint32_t x = blockIdx.x * 32u + (threadIdx.x & 31u), y = blockIdx.y * 8u + (threadIdx.x >> 5);
    const uint32_t W = S.width, H = S.height;
    if (x >= W || y >= H) return;
    auto A = [&](uint32_t X, uint32_t Y) { float4 a = accum[size_t(Y) * W + X]; return mk3(a.x, a.y, a.z); };
    auto bil = [&](float u, float v) {
        float px = clampf(u, 0.0f, 1.0f) * float(W) - 0.5f, py = clampf(v, 0.0f, 1.0f) * float(H) - 0.5f;
        int bx = int(floorf(px)), by = int(floorf(py));
        float fx = fractf(px), fy = fractf(py);
        uint32_t x0 = uint32_t(min(max(bx, 0), int(W - 1))), y0 = uint32_t(min(max(by, 0), int(H - 1)));
        uint32_t x1 = min(x0 + 1u, W - 1u), y1 = min(y0 + 1u, H - 1u);
        return mix3(mix3(A(x0, y0), A(x1, y0), fx), mix3(A(x0, y1), A(x1, y1), fx), fy);
    };
    float u = (float(x) + 0.5f) / float(W), v = (float(y) + 0.5f) / float(H);
    float dx = u - 0.5f, dy = v - 0.5f;
    float len = sqrtf(dx * dx + dy * dy);
    float ox = dx * S.post[5] * len / 8.0f, oy = dy * S.post[5] * len / 8.0f;
    float3 center = bil(u, v), col = center;
    if (fabsf(S.post[5]) > 0.00001f) {
        float3 g = bil(u - ox, v - oy), b = bil(u - 2.0f * ox, v - 2.0f * oy);
        col = mk3(center.x, g.y, b.z);
    }
    float3 hl = mk3(0.0f);
    if (S.post[6] > 0.00001f) {
        uint32_t x0 = x > 0 ? x - 1 : x, x1 = min(x + 1, W - 1), y0 = y > 0 ? y - 1 : y, y1 = min(y + 1, H - 1);
        float3 br = max3(A(x, y) - mk3(0.5f), mk3(0.0f));
        br = br + A(x1, y) * 0.25f + A(x0, y) * 0.25f + A(x, y1) * 0.25f + A(x, y0) * 0.25f;
        hl = br * S.post[6];
    }
    float3 o = post_process(col + hl, S);
    out[size_t(H - 1 - y) * W + x] = make_uchar4((unsigned char)(clampf(o.x, 0.f, 1.f) * 255.0f),
                                                 (unsigned char)(clampf(o.y, 0.f, 1.f) * 255.0f),
                                                 (unsigned char)(clampf(o.z, 0.f, 1.f) * 255.0f), 255);
}


// typed_soa_validation_kernel (shaders/Shaders.metal:5106-5154): hash-seeded
// points in the voxel bounds (plus the origin, both corners and the centre);
// the lowered program's distance and gradient against the interpreter's.
// counts: distance failures, gradient failures, max distance error bits, max
// gradient error bits.
__device__ __forceinline__ uint32_t validation_hash(uint32_t v) {   // lowbias32 (C. Wellons), as :4992-4999
    v ^= v >> 16; v *= 0x7feb352du;
    v ^= v >> 15; v *= 0x846ca68bu;
    v ^= v >> 16;
    return v;
}
static __global__ void __launch_bounds__(256) typed_soa_validation_kernel(const DeviceScene *scene, float3 bmin, float3 bmax,
                                                                          uint32_t n, unsigned int *counts) {
    const DeviceScene &S = *scene;
    uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= n) return;
    float3 u = mk3(float(validation_hash(gid * 3u + 0x9e3779b9u)), float(validation_hash(gid * 3u + 0x243f6a88u)),
                   float(validation_hash(gid * 3u + 0xb7e15162u))) * (1.0f / 4294967295.0f);
    float3 p = mk3(mixf(bmin.x, bmax.x, u.x), mixf(bmin.y, bmax.y, u.y), mixf(bmin.z, bmax.z, u.z));
    if (gid == 0u) p = mk3(0.0f);
    if (gid == 1u) p = bmin;
    if (gid == 2u) p = bmax;
    if (gid == 3u) p = (bmin + bmax) * 0.5f;
    const float ref = program_distance(p, S, false).d, direct = soa_distance(p, S);
    const float derr = fabsf(ref - direct);
    if (!isfinite(ref) || !isfinite(direct) || derr > 2.0e-5f * (1.0f + fabsf(ref))) atomicAdd(counts + 0, 1u);
    atomicMax(counts + 2, __float_as_uint(isfinite(derr) ? derr : 3.0e38f));
    float3 rg = program_gradient(p, S, nullptr), dg;
    soa_surface(p, S, dg);
    const float gerr = fmaxf(fabsf(rg.x - dg.x), fmaxf(fabsf(rg.y - dg.y), fabsf(rg.z - dg.z)));
    if (!finite3(rg) || !finite3(dg) || !(gerr <= 1.0e-4f)) atomicAdd(counts + 1, 1u);
    atomicMax(counts + 3, __float_as_uint(isfinite(gerr) ? gerr : 3.0e38f));
}
cudaError_t launch_typed_soa_validation(const DeviceScene *scene, const float bmin[3], const float bmax[3], uint32_t n,
                                        unsigned int *counts, cudaStream_t st) {
    typed_soa_validation_kernel<<<(n + 255u) / 256u, 256, 0, st>>>(scene, make_float3(bmin[0], bmin[1], bmin[2]),
                                                                    make_float3(bmax[0], bmax[1], bmax[2]), n, counts);
    return cudaGetLastError();
}

cudaError_t launch_present(const DeviceScene *scene, uint32_t W, uint32_t H, const float4 *accum, uchar4 *out, cudaStream_t st) {
    dim3 grid((W + 31u) / 32u, (H + 7u) / 8u);
    present_kernel<<<grid, 256, 0, st>>>(scene, accum, out);
    return cudaGetLastError();
}

#define FPT_DECLARE_KIND(n)                                                                                                 \
    cudaError_t launch_pathtrace_k##n(const PathLaunch &, cudaStream_t);                                                    \
    cudaError_t launch_trace_primary_k##n(const DeviceScene *, uint32_t, uint32_t, FptCudaPrimaryHit *, cudaStream_t);        \
    cudaError_t launch_focus_k##n(DeviceScene *, cudaStream_t);                                                              \
    cudaError_t launch_sample_distance_k##n(const DeviceScene *, const float4 *, float4 *, float *, size_t, cudaStream_t);       \
    cudaError_t launch_label_k##n(const DeviceScene *, float4 *, size_t, cudaStream_t);                                      \
    cudaError_t launch_diagnostic_k##n(const DeviceScene *, uint32_t, uint32_t, uint32_t, float, uchar4 *, cudaStream_t);     \
    cudaError_t launch_skip_primary_k##n(const DeviceScene *, uint32_t, uint32_t, const SkipArgs &, FptCudaPrimaryHit *,     \
                                         cudaStream_t);                                                                     \
    cudaError_t launch_certified_steps_k##n(const DeviceScene *, uint32_t, uint32_t, float, float3, uint32_t *, cudaStream_t);
FPT_DECLARE_KIND(0)
FPT_DECLARE_KIND(1)
FPT_DECLARE_KIND(2)
FPT_DECLARE_KIND(3)
FPT_DECLARE_KIND(4)
FPT_DECLARE_KIND(5)

#define FPT_DISPATCH(kind, fn, ...)                            \
    switch (kind) {                                            \
        case KIND_BULB8: return fn##1(__VA_ARGS__);            \
        case KIND_BULB: return fn##2(__VA_ARGS__);             \
        case KIND_BOX: return fn##3(__VA_ARGS__);              \
        case KIND_MENGER: return fn##4(__VA_ARGS__);           \
        case KIND_HYBRID: return fn##5(__VA_ARGS__);           \
        default: return fn##0(__VA_ARGS__);                    \
    }

cudaError_t launch_pathtrace(const PathLaunch &pl, cudaStream_t stream) { FPT_DISPATCH(pl.kind, launch_pathtrace_k, pl, stream) }
cudaError_t launch_trace_primary(uint32_t kind, const DeviceScene *scene, uint32_t W, uint32_t H, FptCudaPrimaryHit *hits,
                                 cudaStream_t st) {
    FPT_DISPATCH(kind, launch_trace_primary_k, scene, W, H, hits, st)
}
cudaError_t launch_focus(uint32_t kind, DeviceScene *scene, cudaStream_t st) { FPT_DISPATCH(kind, launch_focus_k, scene, st) }
cudaError_t launch_sample_distance(uint32_t kind, const DeviceScene *scene, const float4 *pts, float4 *out, float *grads, size_t n,
                                   cudaStream_t st) {
    FPT_DISPATCH(kind, launch_sample_distance_k, scene, pts, out, grads, n, st)
}
cudaError_t launch_diagnostic(uint32_t kind, const DeviceScene *scene, uint32_t W, uint32_t H, uint32_t mode, float max_distance,
                              uchar4 *out, cudaStream_t st) {
    FPT_DISPATCH(kind, launch_diagnostic_k, scene, W, H, mode, max_distance, out, st)
}
cudaError_t launch_diag_final(const DeviceScene *scene, uint32_t W, uint32_t H, const float4 *accum, uchar4 *out, cudaStream_t st) {
    diag_final_kernel<<<(W * H + 255u) / 256u, 256, 0, st>>>(scene, accum, out);
    return cudaGetLastError();
}
cudaError_t launch_label(uint32_t kind, const DeviceScene *scene, float4 *pts, size_t n, cudaStream_t st) {
    FPT_DISPATCH(kind, launch_label_k, scene, pts, n, st)
}
cudaError_t launch_certified_steps(uint32_t kind, const DeviceScene *scene, uint32_t samples, uint32_t stride, float margin, float3 sun,
                                   uint32_t *counts, cudaStream_t st) {
    FPT_DISPATCH(kind, launch_certified_steps_k, scene, samples, stride, margin, sun, counts, st)
}
cudaError_t launch_skip_primary(uint32_t kind, const DeviceScene *scene, uint32_t W, uint32_t H, const SkipArgs &args,
                                FptCudaPrimaryHit *hits, cudaStream_t st) {
    FPT_DISPATCH(kind, launch_skip_primary_k, scene, W, H, args, hits, st)
}

}  // namespace fpt

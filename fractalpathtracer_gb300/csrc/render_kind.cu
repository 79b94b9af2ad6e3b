// render_kind.cu -- instantiates the kernels of one scene kind.
//
// Compiled once per SceneKind with -DFPT_KIND=<n> so the six
// specialisations build in parallel.
#include "render_impl.cuh"

#ifndef FPT_KIND
#error "FPT_KIND must be defined"
#endif

namespace fpt {

cudaError_t launch_pathtrace_kind(const PathLaunch &pl, cudaStream_t stream, int kind_tag);

template <int KIND>
static cudaError_t launch_path_impl(const PathLaunch &pl, cudaStream_t stream) {
    PathParams P;
    P.scene = pl.scene; P.accum = pl.accum; P.work_counter = pl.work_counter;
    P.tiles_x = (pl.width + 7u) / 8u;
    uint32_t tiles_y = (pl.height + 3u) / 4u;
    P.total_work = P.tiles_x * tiles_y * 32u;
    P.sample_begin = pl.sample_begin; P.sample_end = pl.sample_end;
    P.grad_batch = pl.grad_batch ? pl.grad_batch : 8u;
    P.profile = pl.profile;
    int blocks = pl.blocks;
    if (blocks <= 0) {
        int per_sm = 0, sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pathtrace_persistent<KIND>, 128, 0);
        blocks = sms * (per_sm > 0 ? per_sm : 1);
    }
    cudaError_t e = cudaMemsetAsync(pl.work_counter, 0, sizeof(unsigned int), stream);
    if (e != cudaSuccess) return e;
    pathtrace_persistent<KIND><<<blocks, 128, 0, stream>>>(P);
    return cudaGetLastError();
}

#define FPT_CAT2(a, b) a##b
#define FPT_CAT(a, b) FPT_CAT2(a, b)

cudaError_t FPT_CAT(launch_pathtrace_k, FPT_KIND)(const PathLaunch &pl, cudaStream_t stream) {
    return launch_path_impl<FPT_KIND>(pl, stream);
}
cudaError_t FPT_CAT(launch_trace_primary_k, FPT_KIND)(const DeviceScene *scene, uint32_t W, uint32_t H, FptCudaPrimaryHit *hits,
                                                      cudaStream_t st) {
    dim3 grid((W + 15u) / 16u, (H + 7u) / 8u);
    trace_primary_kernel<FPT_KIND><<<grid, 128, 0, st>>>(scene, hits);
    return cudaGetLastError();
}
cudaError_t FPT_CAT(launch_focus_k, FPT_KIND)(DeviceScene *scene, cudaStream_t st) {
    focus_kernel<FPT_KIND><<<1, 32, 0, st>>>(scene);
    return cudaGetLastError();
}
cudaError_t FPT_CAT(launch_sample_distance_k, FPT_KIND)(const DeviceScene *scene, const float4 *pts, float4 *out, float *grads,
                                                        size_t n, cudaStream_t st) {
    unsigned blocks = unsigned((n + 255) / 256);
    sample_distance_kernel<FPT_KIND><<<blocks, 256, 0, st>>>(scene, pts, out, grads, n);
    return cudaGetLastError();
}
#if FPT_KIND == 0
cudaError_t launch_field_sample(const DeviceScene *scene, const float4 *pts, float4 *out, size_t n, cudaStream_t st) {
    unsigned blocks = unsigned((n + 255) / 256);
    field_sample_kernel<KIND_GENERIC><<<blocks, 256, 0, st>>>(scene, pts, out, n);
    return cudaGetLastError();
}
#endif

}  // namespace fpt

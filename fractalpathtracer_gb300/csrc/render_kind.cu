// render_kind.cu -- instantiates the kernels of one scene kind.
//
// Compiled once per SceneKind with -DFPT_KIND=<n> so the six
// specialisations build in parallel.
#include <algorithm>

#include "render_impl.cuh"

#ifndef FPT_KIND
#error "FPT_KIND must be defined"
#endif
// FPT_PART splits a kind's kernels over three objects that build in parallel:
// 0 the path tracer, 1 primary rays / samples / diagnostics, 2 the surrogate
// kernels (skip passes, labels).
#ifndef FPT_PART
#error "FPT_PART must be defined"
#endif

#define FPT_CAT2(a, b) a##b
#define FPT_CAT(a, b) FPT_CAT2(a, b)

namespace fpt {

// The skip pass of the path tracer (part 2): persistent blocks for the engine,
// and the launch.
int FPT_CAT(skip_pass_blocks_k, FPT_KIND)(bool tc, int sms);
void FPT_CAT(launch_skip_pass_k, FPT_KIND)(const WaveParams &W, const SkipArgs &A, bool tc, int blocks, cudaStream_t stream);

#if FPT_PART == 0

template <int KIND>
static cudaError_t launch_path_impl(const PathLaunch &pl, cudaStream_t stream) {
    WaveParams W{};
    W.scene = pl.scene;
    W.tiles_x = (pl.width + 7u) / 8u;
    const uint32_t tiles_y = (pl.height + 3u) / 4u;
    W.pixel_work = W.tiles_x * tiles_y * 32u;
    W.sample_begin = pl.sample_begin;
    W.sample_count = pl.sample_end - pl.sample_begin;
    W.sample_rgb = pl.sample_rgb;
    W.counters = pl.counters;
    W.profile = pl.profile;
    W.path_steps = pl.profile ? pl.path_steps : nullptr;
    W.box_on = pl.skip ? 1u : 0u;
    for (int k = 0; k < 3; ++k) {
        W.box_lo[k] = pl.skip ? pl.skip->lo[k] : 0.0f;
        W.box_hi[k] = pl.skip ? pl.skip->hi[k] : 0.0f;
    }
    const bool skip_pass = pl.skip && pl.skip->use_network;
    W.skip_queue = skip_pass ? 1u : 0u;
    W.refill_batch = pl.refill_batch;
    W.loop_limit_ns = pl.loop_limit_ns ? pl.loop_limit_ns : kLoopLimitNs;
    const uint32_t cap = pl.wave_paths;
    char *base = static_cast<char *>(pl.wave_scratch);
    W.paths = reinterpret_cast<PathRec *>(base);
    W.q_shadow[0] = reinterpret_cast<ShadowJob *>(base + size_t(cap) * 96);
    W.q_shadow[1] = W.q_shadow[0] + cap;
    W.q_march[0] = reinterpret_cast<uint32_t *>(base + size_t(cap) * (96 + 128));
    W.q_march[1] = W.q_march[0] + cap;
    W.q_shade = W.q_march[1] + cap;
    W.q_skip = reinterpret_cast<SkipJob *>(base + wave_skip_offset(cap));
    int sms = 0, dev = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int march_blocks = pl.march_blocks;
    if (march_blocks <= 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_kernel<KIND>, 128, 0);
        march_blocks = sms * (per_sm > 0 ? per_sm : 1);
    }
    // Deep zoom: the camera-ray pass runs the march variant with the FP64 continuation (extension formulas).
    constexpr bool kExt = KIND == KIND_BULB8 || KIND == KIND_BULB || KIND == KIND_BOX || KIND == KIND_MENGER || KIND == KIND_HYBRID;
    const bool fp64 = kExt && pl.fp64 && !pl.skip;
    int fp64_blocks = march_blocks;
    if (fp64 && pl.march_blocks <= 0) {
        int per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, march_kernel<KIND, false, 128, 7, kExt>, 128, 0);
        fp64_blocks = sms * (per > 0 ? per : 1);
    }
    const bool skip_tc = skip_pass && pl.skip->engine == kNetTcgen05;
    const int skip_blocks = skip_pass ? FPT_CAT(skip_pass_blocks_k, FPT_KIND)(skip_tc, sms) : 0;
    if (pl.grids) {
        pl.grids[0] = uint32_t(march_blocks);
        pl.grids[1] = uint32_t(skip_blocks);
    }
    int shade_per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&shade_per_sm, shade_kernel<KIND>, 128, 0);
    const int shade_blocks = sms * (shade_per_sm > 0 ? shade_per_sm : 1);
    const uint64_t total = uint64_t(W.pixel_work) * W.sample_count;
    uint64_t launches = 0;
    auto timed = [&](int category, auto &&launch) {
        const bool t = pl.timer && pl.timer->begin(category, stream);
        launch();
        if (t) pl.timer->end(stream);
        ++launches;
    };
    cudaError_t e = scene_to_constant(pl.scene, stream);
    if (e != cudaSuccess) return e;
    for (uint64_t wb = 0; wb < total; wb += cap) {
        W.wave_base = uint32_t(wb);
        W.n_paths = uint32_t(std::min<uint64_t>(cap, total - wb));
        if ((e = cudaMemsetAsync(W.counters, 0, C_COUNT * sizeof(uint32_t), stream)) != cudaSuccess) return e;
        if (W.path_steps && (e = cudaMemsetAsync(W.path_steps, 0, size_t(W.n_paths) * sizeof(uint32_t), stream)) != cudaSuccess)
            return e;
        if (W.box_on && wb == 0) {
            first_step_kernel<KIND><<<1, 32, 0, stream>>>(pl.scene, W.counters + C_CAMSTEP);
            ++launches;
        }
        camera_kernel<false><<<std::min<uint32_t>((W.n_paths + 255u) / 256u, uint32_t(sms) * 16u), 256, 0, stream>>>(W);
        ++launches;
        for (uint32_t b = 0; b <= pl.bounces; ++b) {
            const int cur = int(b & 1u);
            reset_counters_kernel<<<1, 32, 0, stream>>>(W.counters, cur ^ 1);
            ++launches;
            // Rays of later passes leave a surface (distance under the hand-over
            // margin), so the skip pass would hand them straight back: it runs on
            // the camera rays only, the box clip applies in every pass.
            if (skip_pass && b == 0u)
                timed(KC_SKIP, [&] { FPT_CAT(launch_skip_pass_k, FPT_KIND)(W, *pl.skip, skip_tc, skip_blocks, stream); });
            timed(KC_MARCH, [&] {
                if (fp64 && b == 0u) march_kernel<KIND, false, 128, 7, kExt><<<fp64_blocks, 128, 0, stream>>>(W, cur);
                else march_kernel<KIND><<<march_blocks, 128, 0, stream>>>(W, cur);
            });
            if (b < pl.bounces) timed(KC_SHADE, [&] { shade_kernel<KIND><<<shade_blocks, 128, 0, stream>>>(W, cur); });
        }
        finalize_kernel<false><<<(W.n_paths + 255u) / 256u, 256, 0, stream>>>(W);
        ++launches;
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    const uint32_t pixels = pl.width * pl.height;
    reduce_samples_kernel<<<(pixels + 255u) / 256u, 256, 0, stream>>>(pl.sample_rgb, pl.accum, pixels, pl.sample_begin,
                                                                       W.sample_count);
    ++launches;
    if (pl.launches) *pl.launches += launches;
    return cudaGetLastError();
}

cudaError_t FPT_CAT(launch_pathtrace_k, FPT_KIND)(const PathLaunch &pl, cudaStream_t stream) {
    return launch_path_impl<FPT_KIND>(pl, stream);
}
cudaError_t FPT_CAT(launch_focus_k, FPT_KIND)(DeviceScene *scene, cudaStream_t st) {
    focus_kernel<FPT_KIND><<<1, 32, 0, st>>>(scene);
    return cudaGetLastError();
}
#endif  // FPT_PART == 0

#if FPT_PART == 1
cudaError_t FPT_CAT(launch_trace_primary_k, FPT_KIND)(const DeviceScene *scene, uint32_t W, uint32_t H, FptCudaPrimaryHit *hits,
                                                      cudaStream_t st) {
    dim3 grid((W + 15u) / 16u, (H + 7u) / 8u);
    trace_primary_kernel<FPT_KIND><<<grid, 128, 0, st>>>(scene, hits);
    return cudaGetLastError();
}
cudaError_t FPT_CAT(launch_sample_distance_k, FPT_KIND)(const DeviceScene *scene, const float4 *pts, float4 *out, float *grads,
                                                        size_t n, cudaStream_t st) {
    unsigned blocks = unsigned((n + 255) / 256);
    sample_distance_kernel<FPT_KIND><<<blocks, 256, 0, st>>>(scene, pts, out, grads, n);
    return cudaGetLastError();
}
cudaError_t FPT_CAT(launch_diagnostic_k, FPT_KIND)(const DeviceScene *scene, uint32_t W, uint32_t H, uint32_t mode, float max_distance,
                                                    uchar4 *out, cudaStream_t st) {
    dim3 grid((W + 15u) / 16u, (H + 7u) / 8u);
    diagnostic_kernel<FPT_KIND><<<grid, 128, 0, st>>>(scene, mode, max_distance, 0u, 0u, out);
    return cudaGetLastError();
}
cudaError_t FPT_CAT(launch_certified_steps_k, FPT_KIND)(const DeviceScene *scene, uint32_t samples, uint32_t stride, float margin,
                                                        float3 sun, uint32_t *counts, cudaStream_t st) {
    certified_steps_kernel<FPT_KIND><<<(samples + 127u) / 128u, 128, 0, st>>>(scene, stride, margin, sun, counts);
    return cudaGetLastError();
}
#if FPT_KIND == 0
cudaError_t launch_field_sample(const DeviceScene *scene, const float4 *pts, float4 *out, size_t n, cudaStream_t st) {
    unsigned blocks = unsigned((n + 255) / 256);
    field_sample_kernel<KIND_GENERIC><<<blocks, 256, 0, st>>>(scene, pts, out, n);
    return cudaGetLastError();
}
#endif
#endif  // FPT_PART == 1

#if FPT_PART == 2
int FPT_CAT(skip_pass_blocks_k, FPT_KIND)(bool tc, int sms) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(skip_march_kernel<FPT_KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(skip_smem_bytes()));
        cudaFuncSetAttribute(skip_march_tc_kernel<FPT_KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(mlp::tc_smem_bytes()));
        attr = true;
    }
    int per_sm = 0;
    if (tc)
        per_sm = mlp::tc_blocks_per_sm(reinterpret_cast<const void *>(skip_march_tc_kernel<FPT_KIND>));
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, skip_march_kernel<FPT_KIND>, 32 * kSkipWarps, skip_smem_bytes());
    return sms * (per_sm > 0 ? per_sm : 1);
}
void FPT_CAT(launch_skip_pass_k, FPT_KIND)(const WaveParams &W, const SkipArgs &A, bool tc, int blocks, cudaStream_t stream) {
    scene_to_constant(W.scene, stream);   // a failed copy surfaces at the launch check after the pass
    if (tc)
        skip_march_tc_kernel<FPT_KIND><<<blocks, mlp::kTcRows, mlp::tc_smem_bytes(), stream>>>(W, A);
    else
        skip_march_kernel<FPT_KIND><<<blocks, 32 * kSkipWarps, skip_smem_bytes(), stream>>>(W, A);
}
cudaError_t FPT_CAT(launch_label_k, FPT_KIND)(const DeviceScene *scene, float4 *pts, size_t n, cudaStream_t st) {
    label_kernel<FPT_KIND><<<unsigned((n + 255) / 256), 256, 0, st>>>(scene, pts, n);
    return cudaGetLastError();
}
cudaError_t FPT_CAT(launch_skip_primary_k, FPT_KIND)(const DeviceScene *scene, uint32_t W, uint32_t H, const SkipArgs &args,
                                                     FptCudaPrimaryHit *hits, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(skip_primary_kernel<FPT_KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(skip_smem_bytes()));
        cudaFuncSetAttribute(skip_primary_tc_kernel<FPT_KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(mlp::tc_smem_bytes()));
        attr = true;
    }
    if (args.cam_step) first_step_kernel<FPT_KIND><<<1, 32, 0, st>>>(scene, const_cast<uint32_t *>(args.cam_step));
    if (args.engine == kNetTcgen05) {
        const uint32_t blocks = (W * H + uint32_t(mlp::kTcRows) - 1u) / uint32_t(mlp::kTcRows);
        skip_primary_tc_kernel<FPT_KIND><<<blocks, mlp::kTcRows, mlp::tc_smem_bytes(), st>>>(scene, args, hits);
        return cudaGetLastError();
    }
    const uint32_t warps = (W * H + 31u) / 32u;
    const uint32_t blocks = (warps + kSkipWarps - 1u) / kSkipWarps;
    skip_primary_kernel<FPT_KIND><<<blocks, 32 * kSkipWarps, skip_smem_bytes(), st>>>(scene, args, hits);
    return cudaGetLastError();
}
#endif  // FPT_PART == 2

}  // namespace fpt

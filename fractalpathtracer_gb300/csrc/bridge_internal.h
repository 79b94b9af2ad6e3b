// bridge_internal.h -- state and helpers shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>

#include "fpt_scene.h"

namespace fpt {

// Process-wide CUDA state.  Device buffers are grown on demand and reused
// across calls; calls are serialised by `mutex`.
struct Context {
    std::mutex mutex;
    bool ready = false;
    int device = -1;           // ordinal bound by every entry point (ensure_device)
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    DeviceScene *scene = nullptr; size_t cap_scene = 0;
    float4 *accum = nullptr; size_t cap_accum = 0;
    float4 *sample_rgb = nullptr; size_t cap_sample_rgb = 0;
    void *wave = nullptr; size_t cap_wave = 0;
    uchar4 *rgba = nullptr; size_t cap_rgba = 0;
    unsigned int *counter = nullptr; size_t cap_counter = 0;
    unsigned long long *profile = nullptr; size_t cap_profile = 0;
    uint32_t *path_steps = nullptr; size_t cap_path_steps = 0;   // profile renders: march steps per path of a wave
    float *sky = nullptr; size_t cap_sky = 0;
    FptCudaPrimaryHit *hits = nullptr; size_t cap_hits = 0;
    float4 *points = nullptr; size_t cap_points = 0;
    float4 *samples = nullptr; size_t cap_samples = 0;
    float *grads = nullptr; size_t cap_grads = 0;
    unsigned long long *skip_stats = nullptr; size_t cap_skip_stats = 0;
    unsigned long long last_skip[8] = {0, 0, 0, 0, 0, 0, 0, 0};   // counters of the last skip-march call
    cudaEvent_t *timer_events = nullptr; int timer_capacity = 0;   // per-kernel timing pool (profile renders)
    FptCudaRenderStats last_render = {};
    // launch tuning (set by the autotuner entry point; 0 = defaults)
    uint32_t wave_paths = 0;   // paths per wave; 0 = min(all paths, 16M)
    int march_blocks = 0;
    uint32_t refill_batch = 0;
    unsigned long long loop_limit_ns = 0;   // persistent-loop time limit of later renders (0: 10 s)
    uint32_t network_engine = 0;   // FPT_CUDA_NET_*: surrogate network on tcgen05 (0) or mma.sync (1)
    uint32_t kernel_timing = 0;    // per-kernel event spans in renders without profile statistics too
};

Context &ctx();
void set_error(char *error, size_t error_len, const char *fmt, ...);
bool ensure_device(char *error, size_t error_len);
bool ensure_buffer(void **ptr, size_t *cap, size_t need, char *error, size_t error_len);
bool check(cudaError_t e, const char *what, char *error, size_t error_len);
bool compile_scene(const FptRenderConfig &c, const FptCudaSceneExt *ext, DeviceScene &S, char *error, size_t error_len);
bool hydrate_hdri(FptRenderConfig &config, char *error, size_t error_len);
bool upload_scene(DeviceScene &S, const FptCudaSceneExt *ext, char *error, size_t error_len);
uint32_t scene_kind(const FptCudaSceneExt &e);

// voxel.cu
int voxel_render_core(const FptRenderConfig &config, const FptCudaSceneExt *ext, DeviceScene &S, const char *output_path,
                      float *linear_output, uint8_t *rgba_output, double *elapsed_ms, uint64_t *voxel_memory_bytes,
                      uint32_t *voxel_active_bricks, uint64_t *voxel_active_cells, double *build_ms, char *error,
                      size_t error_len);
// mlp.cu
struct SkipArgs;
bool surrogate_bind(uint64_t model, DeviceScene &S, char *error, size_t error_len);
bool surrogate_args(uint64_t model, const DeviceScene &S, unsigned long long *stats, SkipArgs &A, char *error, size_t error_len);

}  // namespace fpt

// fpt_kernels.h -- host-side launchers of the CUDA kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include "fpt_scene.h"

namespace fpt {

struct SkipArgs;   // skip.cuh

// CUDA-event spans around kernel launches (per-kernel device time of a
// render).  Events come from a pool created by the caller; spans past the
// pool's capacity are not timed.
enum KernelCategory : int { KC_MARCH = 0, KC_SHADE = 1, KC_SKIP = 2, KC_COUNT = 3 };
struct KernelTimer {
    cudaEvent_t *events = nullptr;
    int capacity = 0;   // events in the pool
    int used = 0;
    int cat[512];
    int n = 0;          // completed spans
    bool begin(int c, cudaStream_t st) {
        if (!events || used + 2 > capacity || n >= 512) return false;
        cat[n] = c;
        cudaEventRecord(events[used++], st);
        return true;
    }
    void end(cudaStream_t st) {
        cudaEventRecord(events[used++], st);
        ++n;
    }
};

// Bytes of wave scratch per path: path record (96), two march queues (8),
// two shadow queues (128), shade queue (4), surrogate-skip queue (32, at a
// 16-byte aligned offset after the rest).
constexpr size_t kWaveBytesPerPath = 96 + 8 + 128 + 4 + 32;
inline size_t wave_scratch_bytes(size_t wave_paths) { return wave_paths * kWaveBytesPerPath + 16; }
inline size_t wave_skip_offset(size_t wave_paths) { return (wave_paths * (96 + 8 + 128 + 4) + 15) & ~size_t(15); }

struct PathLaunch {
    const DeviceScene *scene;   // device pointer
    uint32_t kind;              // SceneKind
    uint32_t width, height;
    uint32_t bounces;
    float4 *accum;              // width*height, running mean
    float4 *sample_rgb;         // (sample_end-sample_begin)*width*height scratch: one colour per path, sample-major
    void *wave_scratch;         // wave_scratch_bytes(wave_paths) bytes
    uint32_t wave_paths;        // paths per wave ("wavefront length")
    unsigned int *counters;     // 8 device words
    uint32_t sample_begin, sample_end;
    int march_blocks;           // persistent march grid, <= 0 = one wave of resident blocks
    unsigned long long *profile;  // kProfileSlots device counters or null
    uint32_t *path_steps;       // profile renders: wave_paths words (march steps per path), or null
    const SkipArgs *skip;       // surrogate-skip pass before each march pass, or null
    KernelTimer *timer;         // per-kernel event spans, or null
    uint64_t *launches;         // host counter of kernel launches, or null
    uint32_t *grids;            // out: blocks of the persistent march and skip grids (2 entries), or null
    unsigned long long loop_limit_ns;   // time limit of the persistent loops (0: 10 s)
    uint32_t refill_batch;      // lockstep: finished lanes finish and refill together in groups of this many
    uint32_t fp64;              // camera-ray pass continues stalled FP32 marches in FP64 (deep zoom, pinhole camera)
};

cudaError_t launch_pathtrace(const PathLaunch &pl, cudaStream_t stream);
cudaError_t launch_trace_primary(uint32_t kind, const DeviceScene *scene, uint32_t W, uint32_t H, FptCudaPrimaryHit *hits,
                                 cudaStream_t stream);
cudaError_t launch_focus(uint32_t kind, DeviceScene *scene, cudaStream_t stream);
cudaError_t launch_field_sample(const DeviceScene *scene, const float4 *pts, float4 *out, size_t n, cudaStream_t stream);
cudaError_t launch_sample_distance(uint32_t kind, const DeviceScene *scene, const float4 *pts, float4 *out, float *grads, size_t n,
                                   cudaStream_t stream);
// Labels xyz points with the scene's mapSdf distance (written to w).
cudaError_t launch_label(uint32_t kind, const DeviceScene *scene, float4 *pts, size_t n, cudaStream_t stream);
cudaError_t launch_skip_primary(uint32_t kind, const DeviceScene *scene, uint32_t W, uint32_t H, const SkipArgs &args,
                                FptCudaPrimaryHit *hits, cudaStream_t stream);
// Diagnostic image (modes of FptDiagnosticConfig except 7 and 15) and the mode-7 present.
cudaError_t launch_diagnostic(uint32_t kind, const DeviceScene *scene, uint32_t W, uint32_t H, uint32_t mode, float max_distance,
                              uchar4 *out, cudaStream_t stream);
cudaError_t launch_diag_final(const DeviceScene *scene, uint32_t W, uint32_t H, const float4 *accum, uchar4 *out, cudaStream_t stream);
// Typed SoA vs interpreter over n hash-seeded points; counts[4] as in the kernel.
cudaError_t launch_typed_soa_validation(const DeviceScene *scene, const float bmin[3], const float bmax[3], uint32_t n,
                                        unsigned int *counts, cudaStream_t stream);
// Plain-march and perfect-proposal certified evaluations of camera, shadow and bounce rays of sampled pixels (6 per pixel).
cudaError_t launch_certified_steps(uint32_t kind, const DeviceScene *scene, uint32_t samples, uint32_t stride, float margin, float3 sun,
                                   uint32_t *counts, cudaStream_t stream);
cudaError_t launch_present(const DeviceScene *scene, uint32_t W, uint32_t H, const float4 *accum, uchar4 *out,
                           cudaStream_t stream);

}  // namespace fpt

// render_impl.cuh -- sphere-tracing kernels for sm_103a (templated on the scene kind).
//
// The path tracer is the wavefront pipeline of wavefront.cuh; this file adds
// the in-order sample reduction, primary rays, the focus prepass and the
// batch distance-evaluation kernels.
#pragma once

#include "fpt_march.cuh"
#include "fpt_kernels.h"
#include "diag.cuh"
#include "skip.cuh"
#include "wavefront.cuh"

namespace fpt {

// In-order running mean of a pixel's samples (accumulate kernels,
// shaders/Shaders.metal:7706-7773): accum = mix(prev, s_i, 1/(i+1)).
static __global__ void __launch_bounds__(256) reduce_samples_kernel(const float4 *sample_rgb, float4 *accum, uint32_t pixels,
                                                             uint32_t sample_begin, uint32_t sample_count) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= pixels) return;
    float3 mean = mk3(0.0f);
    if (sample_begin > 0u) { float4 a = accum[p]; mean = mk3(a.x, a.y, a.z); }
    const float4 *src = sample_rgb + size_t(p) * sample_count;
    for (uint32_t i = 0; i < sample_count; ++i) {
        float4 c = src[i];
        mean = mix3(mean, mk3(c.x, c.y, c.z), 1.0f / float(sample_begin + i + 1u));
    }
    accum[p] = make_float4(mean.x, mean.y, mean.z, 1.0f);
}

// ---------------------------------------------------------------- primary rays
template <int KIND>
__global__ void __launch_bounds__(128) trace_primary_kernel(const DeviceScene *scene, FptCudaPrimaryHit *hits) {
    const DeviceScene &S = *scene;
    uint32_t gx = blockIdx.x * 16u + (threadIdx.x & 15u), gy = blockIdx.y * 8u + (threadIdx.x >> 4);
    if (gx >= S.width || gy >= S.height) return;
    float2 uv = screen_uv(gx, gy, S);
    PathRng rng;
    rng.init(false, 0u, 0u, 0u, uv.x, uv.y);
    float3 rp, dr;
    FptCudaPrimaryHit h;
    h.distance = 0.0f; h.normal[0] = h.normal[1] = h.normal[2] = 0.0f; h.steps = 0; h.hit = 0;
    if (camera_ray(S, uv, rng, false, rp, dr)) {
        March m = march_loop<KIND>(S, rp, dr, int(S.render[1]), S.render[3], 0.0002f);
        float travel = len3(m.pos - rp);
        bool hit = m.found && isfinite(travel) && travel < S.render[4] * 0.99f;
        int steps = m.steps;
        float3 hit_pos = m.pos;
        if (S.fp64_bisection && m.stalled && S.sdf_id == FPT_SDF_MANDELBULBER && S.formula != 0) {
            // restart a little before the FP32 stop: a few FP32 ulps of the position
            const float back = 8.0f * 1.1920929e-7f * fmaxf(fmaxf(fabsf(m.pos.x), fabsf(m.pos.y)), fmaxf(fabsf(m.pos.z), 1.0f));
            double t64 = 0.0;
            if (march_fp64<KIND>(S, rp, dr, fmax(double(travel) - double(back), 0.0), int(S.render[1]), t64, steps)) {
                travel = float(t64);
                hit = travel < S.render[4] * 0.99f;
                hit_pos = rp + normalize3(dr) * travel;
            } else {
                hit = false;
            }
        }
        h.distance = travel;
        h.steps = uint32_t(steps);
        h.hit = hit ? 1u : 0u;
        if (hit) {
            float3 n = normal_direct<KIND>(hit_pos, S);
            h.normal[0] = n.x; h.normal[1] = n.y; h.normal[2] = n.z;
        }
    }
    hits[size_t(gy) * S.width + gx] = h;
}

// ---------------------------------------------------------------- focus prepass
// estimate_focus_distance_kernel (shaders/Shaders.metal:5869-5884): one
// thread writes the resolved focus into the scene block in device memory.
template <int KIND>
__global__ void focus_kernel(DeviceScene *scene) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const DeviceScene &S = *scene;
    float3 cam = mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]);
    float3 dr = rotate_camera(normalize3(mk3(0.0f, 0.0f, S.focal)), S.yaw, S.pitch, S.roll);
    March m = march_loop<KIND>(S, cam, dr, 120, 0.001f, 0.001f);
    float d = len3(m.pos - cam);
    if (!isfinite(d) || d <= 0.001f || d > S.render[4] * 0.99f) d = 5.0f;
    scene->focus_distance = d;
}

// ---------------------------------------------------------------- batch evaluation
// mandelbulber_field_sample_kernel (shaders/Shaders.metal:1001-1009).
template <int KIND>
__global__ void field_sample_kernel(const DeviceScene *scene, const float4 *points, float4 *samples, size_t n) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = points[i];
    Field4 f = mandel_field<KIND>(mk3(p.x, p.y, p.z), *scene, 1);
    samples[i] = make_float4(f.d, f.r, f.dr, fabsf(f.state));
}

// mapSdf labels for the surrogate's training points (w <- distance).
template <int KIND>
__global__ void __launch_bounds__(256) label_kernel(const DeviceScene *scene, float4 *pts, size_t n) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pts[i];
    pts[i].w = scene_eval<KIND>(*scene, mk3(p.x, p.y, p.z), EV_MAP).d;
}

// distanceSdf (plus orbit, derivative, iterations where defined) and the
// analytic gradient at a batch of points.
template <int KIND>
__global__ void sample_distance_kernel(const DeviceScene *scene, const float4 *points, float4 *samples, float *grads, size_t n) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DeviceScene &S = *scene;
    float4 p4 = points[i];
    float3 p = mk3(p4.x, p4.y, p4.z);
    Eval e = scene_eval<KIND>(S, p, EV_RAW);
    float dr = 0.0f, it = 0.0f;
    if (S.sdf_id == FPT_SDF_MANDELBULBER) {
        Field4 f = mandel_field<KIND>(p, S, 1);
        dr = f.dr; it = fabsf(f.state);
    }
    samples[i] = make_float4(e.d, S.formula ? e.orbit : 0.0f, dr, it);
    if (grads) {
        float3 g = mk3(0.0f);
        if (S.formula != 0 || S.sdf_id == FPT_SDF_PROGRAM) {
            if (!analytic_gradient<KIND>(S, p, g) && S.sdf_id == FPT_SDF_PROGRAM) g = program_gradient(p, S, nullptr);
        }
        grads[i * 3 + 0] = g.x; grads[i * 3 + 1] = g.y; grads[i * 3 + 2] = g.z;
    }
}

}  // namespace fpt

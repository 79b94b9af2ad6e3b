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
    for (uint32_t i = 0; i < sample_count; ++i) {   // sample-major: sample i of every pixel, then i + 1
        float4 c = sample_rgb[size_t(i) * pixels + p];
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

// ---------------------------------------------------------------- certified-step bound
// What any distance proposal can save under the certificate of the surrogate
// skip (a step s from p is taken when s <= DE(p) + DE(p + s dir): the two
// empty balls overlap).  Per ray: the plain march's evaluations, and the
// evaluations of a march that always takes the longest step the certificate
// allows -- found by a search along the ray whose evaluations are not
// counted (a perfect proposal) -- until the distance falls under the hand-over
// margin, after which the plain march finishes the ray from there.
template <int KIND>
__device__ float longest_certified_step(const DeviceScene &S, float3 p, float3 dir, float d, float limit) {
    auto ok = [&](float s) {
        const float e = scene_eval<KIND>(S, p + dir * s, EV_MAP).d;
        return isfinite(e) && s <= d + e;
    };
    float lo = 0.0f, hi = fminf(d, limit);
    for (int k = 0; k < 24 && hi <= limit && ok(hi); ++k) { lo = hi; hi *= 2.0f; }
    if (lo >= limit) return limit;
    hi = fminf(hi, limit);
    for (int k = 0; k < 12; ++k) {
        const float mid = 0.5f * (lo + hi);
        if (ok(mid)) lo = mid; else hi = mid;
    }
    return lo;
}

// Plain and certified evaluations of one ray (counts[0], counts[1]).
template <int KIND>
__device__ void certified_ray(const DeviceScene &S, float3 o, float3 dir, float margin, uint32_t *counts) {
    const int ni = int(S.render[1]);
    counts[0] = uint32_t(march_loop<KIND>(S, o, dir, ni, S.render[3], 0.0002f).steps);
    float3 p = o;
    float travel = 0.0f, last = 0.0f;
    int steps = 0;
    uint32_t counted = 0;
    const int maxi = march_iteration_limit(ni, S);
    while (steps < maxi) {
        const float d = scene_eval<KIND>(S, p, EV_MAP).d;   // one counted evaluation per position stood on
        ++counted;
        const float th = S.sdf_id == FPT_SDF_MANDELBULBER ? mandel_threshold(p, S) : S.render[3];
        if (!isfinite(d) || d < fmaxf(margin, 4.0f * th)) break;   // the plain march finishes the ray
        const float limit = S.render[4] - travel;
        if (!(limit > 0.0f)) break;
        const float step = longest_certified_step<KIND>(S, p, dir, d, limit);
        if (!(step > 0.0f)) break;
        p = p + dir * step;
        travel += step;
        last = step;
        ++steps;
        if (travel >= S.render[4]) break;
    }
    if (travel < S.render[4] && steps < maxi) {
        // resume the plain march at p (its first evaluation repeats the one just counted)
        const March m = march_loop_from<KIND>(S, o, p, dir, ni, S.render[3], 0.0002f, steps, last);
        counted += uint32_t(m.steps > 0 ? m.steps - 1 : 0);
    }
    counts[1] = counted;
}

// Per sampled pixel (every `stride`-th pixel centre): counts[6] = plain and
// certified evaluations of the camera ray, of its hit's sun shadow ray (when
// the sun is above the surface) and of one cosine-distributed bounce ray, the
// secondary rays starting 0.001 off the surface along the normal as the path
// tracer starts them (zeros where a ray does not exist).
template <int KIND>
__global__ void __launch_bounds__(128) certified_steps_kernel(const DeviceScene *scene, uint32_t stride, float margin, float3 sun,
                                                              uint32_t *counts) {
    const DeviceScene &S = *scene;
    const uint32_t cols = (S.width + stride - 1u) / stride, rows = (S.height + stride - 1u) / stride;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cols * rows) return;
    uint32_t *c = counts + size_t(i) * 6;
    for (int k = 0; k < 6; ++k) c[k] = 0u;
    const uint32_t gx = (i % cols) * stride, gy = (i / cols) * stride;
    const float2 uv = screen_uv(gx, gy, S);
    PathRng rng;
    rng.init(false, 0u, 0u, 0u, uv.x, uv.y);
    float3 rp, dr;
    if (!camera_ray(S, uv, rng, false, rp, dr)) return;
    certified_ray<KIND>(S, rp, dr, margin, c);
    const March m = march_loop<KIND>(S, rp, dr, int(S.render[1]), S.render[3], 0.0002f);
    const float travel = len3(m.pos - rp);
    if (!(m.found && isfinite(travel) && travel < S.render[4] * 0.99f)) return;
    float3 n = normal_direct<KIND>(m.pos, S);
    if (dot(n, dr) > 0.0f) n = -n;
    const float3 o = m.pos + n * 0.001f;
    if (dot(n, sun) > 0.0f) certified_ray<KIND>(S, o, sun, margin, c + 2);
    const uint32_t h1 = pcg_hash(i * 2u + 0x9e3779b9u), h2 = pcg_hash(i * 2u + 1u + 0x7f4a7c15u);
    const float u1 = float(h1 >> 8) * (1.0f / 16777216.0f), u2 = float(h2 >> 8) * (1.0f / 16777216.0f);
    const float3 a = fabsf(n.x) > 0.9f ? mk3(0.0f, 1.0f, 0.0f) : mk3(1.0f, 0.0f, 0.0f);
    const float3 t = normalize3(cross3(n, a)), b = cross3(n, t);
    const float r = sqrtf(u1), ph = 6.28318530718f * u2;
    const float3 bd = normalize3(t * (r * cosf(ph)) + b * (r * sinf(ph)) + n * sqrtf(fmaxf(0.0f, 1.0f - u1)));
    certified_ray<KIND>(S, o, bd, margin, c + 4);
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

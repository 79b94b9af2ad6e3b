// diag.cuh -- diagnostic images (sdf_diagnostic_kernel, shaders/Shaders.metal:7290-7385).
//
// One thread per pixel: the diagnostic march of the reference (marchMandelbulber
// for Mandelbulber scenes, otherwise its own 420-step loop with a 5e-4 floor on
// the hit threshold), then one encoded quantity per mode.  The path-cost modes
// (11-14) replay sdfPathCostDiagnostic (6919-6985): up to 8 samples of the
// reference path with its diagnostic random numbers, counting march steps,
// shadow-march steps, normal evaluations and bounces.  Mode 7 (final colour)
// is produced on the host from a path-traced render.
#pragma once

#include "fpt_march.cuh"
#include "fpt_post.cuh"

namespace fpt {

enum DiagMode : uint32_t {
    DIAG_DEPTH = 0, DIAG_NORMAL = 1, DIAG_MATERIAL = 2, DIAG_HIT_MASK = 3, DIAG_PATH_DIRECT = 4, DIAG_PATH_ENVIRONMENT = 5,
    DIAG_PATH_THROUGHPUT = 6, DIAG_PATH_FINAL = 7, DIAG_DIFFUSE_NORMAL = 8, DIAG_MANDEL_COLOR_INDEX = 9,
    DIAG_MANDEL_PALETTE_POSITION = 10, DIAG_SDF_PRIMARY_STEPS = 11, DIAG_SDF_SHADOW_STEPS = 12, DIAG_SDF_NORMAL_EVALS = 13,
    DIAG_SDF_BOUNCES = 14, DIAG_SDF_BOUNCE_CONTRIBUTION = 15,
};

__device__ __forceinline__ float3 diag_scalar(float v, float scale) {                   // :6842-6845
    float x = clampf(v / fmaxf(scale, 1.0f), 0.0f, 1.0f);
    return mk3(x);
}
__device__ __forceinline__ float3 diag_hdr(float3 c, const DeviceScene &S) {            // :6838-6840
    return post_process(min3(max3(c, mk3(0.0f)), mk3(8.0f)), S);
}
__device__ __forceinline__ float3 diag_random_vector(float3 normal, float2 xy, float seed) {   // randomVector :557-569
    float h1 = hash13(xy.x, xy.y, seed * 2.0f + 0.0f), h2 = hash13(xy.x, xy.y, seed * 2.0f + 1.0f);
    float3 n = normalize3(normal);
    float3 uu = normalize3(cross3(n, mk3(0.0f, 1.0f, 1.0f)));
    float3 vv = cross3(uu, n);
    float ra = sqrtf(h2), s, c;
    sincosf(kPi * 2.0f * h1, &s, &c);
    return normalize3(uu * (ra * c) + vv * (ra * s) + n * sqrtf(fmaxf(1.0f - h2, 0.0f)));
}
__device__ __forceinline__ float2 diag_random_point(float power, float2 xy, float seed) {      // randomPoint :571-577
    float h1 = hash13(xy.x, xy.y, seed * 2.0f + 0.0f), h2 = hash13(xy.x, xy.y, seed * 2.0f + 1.0f);
    float s, c;
    sincosf(2.0f * h1 * kPi, &s, &c);
    float m = sqrtf(2.0f * h2 * kPi) * power;
    return make_float2(c * m, s * m);
}
__device__ __forceinline__ float diag_step(float d, float th, const DeviceScene &S) {          // sdfMarchStep :3643-3681
    return S.sdf_id == FPT_SDF_MANDELBULBER ? mandel_march_step(d, th, S) : fabsf(d) * 0.99f;
}

// marchCounted / marchStepCount (:6857-6910): the generic march loop with a step counter.
template <int KIND>
__device__ float3 diag_march_counted(const DeviceScene &S, float3 dr, float3 rp, int ni, float min_dist, float lod_falloff,
                                     uint32_t &steps) {
    const float3 cam = rp;
    const int max_iter = march_iteration_limit(ni, S);
    for (int i = 0; i < max_iter; ++i) {
        ++steps;
        float d = scene_eval<KIND>(S, rp, EV_MAP).d;
        if (!isfinite(d)) break;
        float th = S.sdf_id == FPT_SDF_MANDELBULBER ? mandel_threshold(rp, S) : min_dist;
        float o = diag_step(d, th, S);
        rp = rp + dr * o;
        float lod = th;
        if (lod_falloff > 0.00001f) {
            float3 r = cam - rp;
            lod = mixf(lod, 0.1f, dot(r, r) * lod_falloff);
            lod = mixf(th, lod, S.render[5]);
        }
        if (S.translucent && material_of(S, scene_eval<KIND>(S, rp, EV_MATERIAL)).translucency > 0.0f) lod = 0.0001f;
        bool converged = S.sdf_id == FPT_SDF_MANDELBULBER ? d < lod : o < lod;
        if (converged || S.render[4] < o) break;
    }
    return rp;
}

// Sun light direction with the diagnostic divergence (:5846-5855, 6909-6916).
__device__ __forceinline__ float3 diag_sun_dir(const DeviceScene &S, float2 xy, float seed) {
    float3 ld = mk3(S.sun_dir[0], S.sun_dir[1], S.sun_dir[2]);
    float h1 = hash13(xy.x, xy.y, seed * 5.0f + 1.0f), h2 = hash13(xy.x, xy.y, seed * 3.0f + 5.0f);
    float s, c;
    sincosf(h1 * 2.0f * kPi, &s, &c);
    float m = sqrtf(h2) * S.sun[4];
    return rotate_camera(ld, c * m, s * m);
}

template <int KIND>
__device__ float3 diag_path_cost(const DeviceScene &S, float2 xy, uint32_t mode) {               // :6919-6985
    const uint32_t samples = min(S.samples, 8u);
    float total_primary = 0.0f, total_shadow = 0.0f, total_normal = 0.0f, total_bounces = 0.0f;
    const float3 cam = mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]);
    for (uint32_t si = 0; si < samples; ++si) {
        const float frame = float(si);
        float3 rp = cam;
        float2 j = diag_random_point(S.aa_strength, xy, frame);
        float3 dr = rotate_camera(normalize3(mk3(xy.x + j.x, xy.y + j.y, S.focal)), S.yaw, S.pitch, S.roll);
        if (S.camera_dof > 0.0f) {
            float3 fp = rp + dr * S.focus_distance;
            float2 lens = diag_random_point(S.camera_dof, xy, frame);
            rp = rp + rotate_camera(mk3(lens.x, lens.y, 0.0f), S.yaw, S.pitch, S.roll);
            dr = normalize3(fp - rp);
        }
        int ni = int(S.render[1]);
        const int bounces = int(S.bounces);   // min(render[0], 8, bounce cap)
        const float far = S.render[4] * 0.99f;
        for (int i = 0; i < bounces; ++i) {
            uint32_t steps = 0;
            rp = diag_march_counted<KIND>(S, dr, rp, ni, S.render[3], 0.0002f, steps);
            total_primary += float(steps);
            ni = int(S.render[1] / (S.render[5] * 2.0f + 1.0f));
            float3 r = rp - cam;
            if (dot(r, r) > far * far) break;
            Material mt = material_of(S, scene_eval<KIND>(S, rp, EV_MATERIAL));
            total_bounces += 1.0f;
            total_normal += 1.0f;
            float3 n = normal_direct<KIND>(rp, S);
            if (S.sun[0] == 1.0f) {
                uint32_t sh = 0;
                diag_march_counted<KIND>(S, diag_sun_dir(S, xy, frame), rp + n * 0.001f, int(S.render[1]), S.render[3], 0.0002f,
                                         sh);
                total_shadow += float(sh);
            }
            float r1 = hash13(xy.x, xy.y, frame * 1.37f + float(i)), r2 = hash13(xy.x, xy.y, frame * 7.91f + float(i));
            float f0 = (mt.ior - 1.0f) / (mt.ior + 1.0f);
            f0 = f0 * f0;
            float ct = clampf(dot(n, -dr), 0.0f, 1.0f);
            float fres = f0 + (1.0f - f0) * pow5f(1.0f - ct);
            if (r1 > mt.translucency) {
                float3 metal = reflect3(dr, n);
                float3 diffuse = diag_random_vector(n, xy, frame * 13.37f + float(i));
                dr = normalize3(mix3(metal, diffuse, mt.roughness));
                if (r2 < fres * mt.specular) dr = metal;
            } else {
                float3 refr = refract3(dr, n, 1.0f / mt.ior), refl = reflect3(dr, n);
                dr = (dot(refr, refr) < 0.000001f || !isfinite(refr.x) || r2 < fres) ? normalize3(refl) : normalize3(refr);
            }
            rp = rp + n * (0.001f * signf(dot(dr, n)));
        }
    }
    const float inv = 1.0f / float(samples);
    const float steps_scale = fmaxf(S.render[1] * fmaxf(S.render[0], 1.0f), 1.0f);
    if (mode == DIAG_SDF_PRIMARY_STEPS) return diag_scalar(total_primary * inv, steps_scale);
    if (mode == DIAG_SDF_SHADOW_STEPS) return diag_scalar(total_shadow * inv, steps_scale);
    if (mode == DIAG_SDF_NORMAL_EVALS) return diag_scalar(total_normal * inv, fmaxf(S.render[0] * 2.0f, 1.0f));
    return diag_scalar(total_bounces * inv, fmaxf(S.render[0], 1.0f));
}

template <int KIND>
__device__ float3 diag_color(const DeviceScene &S, float2 xy, uint32_t mode, float max_distance) {
    if (mode >= DIAG_SDF_PRIMARY_STEPS && mode <= DIAG_SDF_BOUNCES) return diag_path_cost<KIND>(S, xy, mode);
    const float3 ro = mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]);
    float3 rp = ro, rd;
    const bool mb = S.sdf_id == FPT_SDF_MANDELBULBER;
    if (mb) {
        if (!mandel_visible(xy.x, xy.y, S)) return mk3(0.0f);
        rd = mandel_camera_ray(xy.x, xy.y, S);
    } else {
        rd = rotate_camera(normalize3(mk3(xy.x, xy.y, S.focal)), S.yaw, S.pitch, S.roll);
    }
    const int requested = int(fmaxf(S.render[1], 32.0f));
    const int steps = mb ? min(requested, 10000) : min(requested, 420);
    bool hit = false;
    if (mb) {
        March m = march_loop<KIND>(S, rp, rd, steps, S.render[3], 0.0002f);
        rp = m.pos;
        hit = m.found;
    } else {
        const float th = fmaxf(S.render[3], 0.0005f);
        for (int i = 0; i < steps; ++i) {
            float d = scene_eval<KIND>(S, rp, EV_MAP).d;
            if (!isfinite(d)) break;
            if (d < th && len3(rp - ro) > 0.001f) { hit = true; break; }
            rp = rp + rd * diag_step(d, th, S);
            if (len3(rp - ro) > S.render[4]) break;
        }
    }
    if (mode == DIAG_HIT_MASK) return hit ? mk3(1.0f) : mk3(0.0f);
    if (mode == DIAG_DEPTH) {                                                                     // :6827-6832
        if (!hit) return mk3(0.0f);
        float md = max_distance > 0.001f ? max_distance : S.render[4];
        return mk3(1.0f - clampf(len3(rp - ro) / fmaxf(md, 0.001f), 0.0f, 1.0f));
    }
    if (!hit) return mk3(0.0f);
    if (mode == DIAG_DIFFUSE_NORMAL) {
        float3 n = normal_direct<KIND>(rp, S);
        float3 fwd = rotate_camera(mk3(0.0f, 0.0f, 1.0f), S.yaw, S.pitch, S.roll);
        return mk3(0.12f + 0.88f * fmaxf(dot(n, -fwd), 0.0f));
    }
    if (mode == DIAG_MANDEL_COLOR_INDEX || mode == DIAG_MANDEL_PALETTE_POSITION) return mk3(0.0f);   // no generated material
    Material mt = material_of(S, scene_eval<KIND>(S, rp, EV_MATERIAL));
    if (mode == DIAG_MATERIAL) return clamp3(mt.rgb, 0.0f, 1.0f);
    if (mode == DIAG_PATH_DIRECT) {                                                               // sunContribution :5846-5867
        if (S.sun[0] != 1.0f) return diag_hdr(mk3(0.0f), S);
        float3 n = normal_direct<KIND>(rp, S);
        float3 ld = diag_sun_dir(S, xy, 0.0f);
        March sm = march_loop<KIND>(S, rp + n * 0.001f, ld, int(S.render[1]), S.render[3], 0.0002f);
        float3 c = mk3(0.0f);
        if (len3(rp - sm.pos) > S.render[4] * 0.99f)
            c = mk3(S.sun_color[0], S.sun_color[1], S.sun_color[2]) *
                (S.sun[3] * fmaxf(dot(n, ld), 0.0f) * mt.roughness * (1.0f - mt.translucency));
        return diag_hdr(c, S);
    }
    if (mode == DIAG_PATH_ENVIRONMENT) return diag_hdr(environment(rd, S), S);
    float3 n = normal_direct<KIND>(rp, S);
    if (mode == DIAG_PATH_THROUGHPUT) {
        float3 next = normalize3(mix3(reflect3(rd, n), diag_random_vector(n, xy, 0.0f), mt.roughness));
        float a = clampf(dot(next, n) * 0.5f + 0.5f, 0.0f, 1.0f);
        return clamp3(mt.rgb * a, 0.0f, 1.0f);
    }
    return clamp3(n * 0.5f + mk3(0.5f), 0.0f, 1.0f);                                             // normal, :6834-6836
}

template <int KIND>
__global__ void __launch_bounds__(128) diagnostic_kernel(const DeviceScene *scene, uint32_t mode, float max_distance,
                                                         uint32_t ox, uint32_t oy, uchar4 *out) {
    const DeviceScene &S = *scene;
    uint32_t x = blockIdx.x * 16u + (threadIdx.x & 15u) + ox, y = blockIdx.y * 8u + (threadIdx.x >> 4) + oy;
    if (x >= S.width || y >= S.height) return;
    float3 c = diag_color<KIND>(S, screen_uv(x, y, S), mode, max_distance);
    out[size_t(S.height - 1u - y) * S.width + x] = make_uchar4((unsigned char)(clampf(c.x, 0.f, 1.f) * 255.0f),
                                                               (unsigned char)(clampf(c.y, 0.f, 1.f) * 255.0f),
                                                               (unsigned char)(clampf(c.z, 0.f, 1.f) * 255.0f), 255);
}

// Mode 7: the averaged path colour through postProcess, flipped (:7300-7311).
static __global__ void __launch_bounds__(256) diag_final_kernel(const DeviceScene *scene, const float4 *accum, uchar4 *out) {
    const DeviceScene &S = *scene;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.width * S.height) return;
    uint32_t x = i % S.width, y = i / S.width;
    float4 a = accum[i];
    float3 c = post_process(mk3(a.x, a.y, a.z), S);
    out[size_t(S.height - 1u - y) * S.width + x] = make_uchar4((unsigned char)(clampf(c.x, 0.f, 1.f) * 255.0f),
                                                               (unsigned char)(clampf(c.y, 0.f, 1.f) * 255.0f),
                                                               (unsigned char)(clampf(c.z, 0.f, 1.f) * 255.0f), 255);
}

}  // namespace fpt

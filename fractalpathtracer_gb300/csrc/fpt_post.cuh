// fpt_post.cuh -- postProcess / toneMap (shaders/Shaders.metal:6778-6825), shared by the
// present kernel and the diagnostic images.
#pragma once

#include "fpt_math.cuh"
#include "fpt_scene.h"

namespace fpt {

__device__ __forceinline__ float3 gamma_srgb(float3 l) {
    float3 o;
    o.x = l.x <= 0.0031308f ? l.x * 12.92f : 1.055f * powf(fmaxf(l.x, 0.0f), 1.0f / 2.4f) - 0.055f;
    o.y = l.y <= 0.0031308f ? l.y * 12.92f : 1.055f * powf(fmaxf(l.y, 0.0f), 1.0f / 2.4f) - 0.055f;
    o.z = l.z <= 0.0031308f ? l.z * 12.92f : 1.055f * powf(fmaxf(l.z, 0.0f), 1.0f / 2.4f) - 0.055f;
    return o;
}
__device__ __forceinline__ float aces1(float x) { return clampf((x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f), 0.0f, 1.0f); }
__device__ __forceinline__ float3 pbr_neutral(float3 c) {
    float x = fminf(c.x, fminf(c.y, c.z));
    float off = x < 0.08f ? x - 6.25f * x * x : 0.04f;
    c = c - off;
    float peak = maxc3(c);
    if (peak < 0.76f) return c;
    float d = 1.0f - 0.76f;
    float np = 1.0f - d * d / (peak + d - 0.76f);
    c = c * (np / peak);
    float g = 1.0f - 1.0f / (0.15f * (peak - np) + 1.0f);
    return mix3(c, mk3(np), g);
}
__device__ __forceinline__ float3 post_process(float3 c, const DeviceScene &S) {
    float n = S.post[0];
    if (n == 0.0f) c = gamma_srgb(c);
    else if (n == 1.0f) c = mk3(powf(c.x, 1.0f / 2.4f), powf(c.y, 1.0f / 2.4f), powf(c.z, 1.0f / 2.4f));
    else if (n == 2.0f) c = mk3(powf(c.x, 1.0f / 2.6f), powf(c.y, 1.0f / 2.6f), powf(c.z, 1.0f / 2.6f));
    else if (n == 3.0f) c = mk3(aces1(c.x), aces1(c.y), aces1(c.z));
    else if (n == 4.0f) c = pbr_neutral(c);
    c = c * S.post[1] + S.post[2];
    c = (c - mk3(0.5f)) * S.post[4] + mk3(0.5f);
    float l = dot(c, mk3(0.2126f, 0.7152f, 0.0722f));
    c = mix3(mk3(l), c, S.post[3]);
    return clamp3(c, 0.0f, 1.0f);
}
}  // namespace fpt

// bridge.cu -- C ABI of libfpt_cuda.so (include/fpt_cuda.h).
//
// Replaces the Metal device runtime of FPT Metal (src/metal_bridge.mm):
// same entry points, same argument meaning, same error convention
// (0 / 1 plus a message, set_error at src/metal_bridge.mm:41-47).  One
// process-wide CUDA context on the current device, one stream, and device
// buffers kept between calls and grown on demand; no caller pointer is
// retained after a call returns.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <mutex>
#include <string>
#include <vector>

#include "fpt_kernels.h"
#include "fpt_scene.h"
#include "image_io.h"
#include "bridge_internal.h"
#include "skip.cuh"
#include "diag.cuh"

// Layout pins of the reference ABI (src/ffi.rs:494-507, static_asserts of
// src/metal_bridge.mm:32-39): a caller compiled against the reference header
// passes these structs by pointer.
static_assert(sizeof(FptSdfInstruction) == 32, "FptSdfInstruction must be 32 bytes");
static_assert(sizeof(FptRenderConfig) == 30448, "FptRenderConfig must be 30448 bytes");
static_assert(sizeof(FptSdfProfileStats) == 288, "FptSdfProfileStats must be 288 bytes");
static_assert(sizeof(FptDiagnosticConfig) == 24, "FptDiagnosticConfig must be 24 bytes");
static_assert(sizeof(FptMandelbulberFieldSample) == 16, "FptMandelbulberFieldSample must be 16 bytes");

namespace fpt {

// ------------------------------------------------------------------ errors
void set_error(char *error, size_t error_len, const char *fmt, ...) {
    if (!error || error_len == 0) return;
    va_list args;
    va_start(args, fmt);
    vsnprintf(error, error_len, fmt, args);
    va_end(args);
}

// ------------------------------------------------------------------ context
Context &ctx() {
    static Context c;
    return c;
}

// Device ordinal of the process-wide context: FPT_CUDA_DEVICE when set, else
// LOCAL_RANK (one replica per GPU under torchrun), else 0, unless
// fpt_cuda_set_device chose one before the context was created.  The library
// links its own CUDA runtime, so the caller's runtime (torch's included) does
// not select its device: every entry point binds it on the calling thread.
static int default_device_ordinal(int count) {
    for (const char *name : {"FPT_CUDA_DEVICE", "LOCAL_RANK"}) {
        const char *v = std::getenv(name);
        if (v && *v) {
            char *end = nullptr;
            long k = std::strtol(v, &end, 10);
            if (end && *end == 0 && k >= 0) return int(k % count);
        }
    }
    return 0;
}

bool ensure_device(char *error, size_t error_len) {
    Context &c = ctx();
    if (c.ready) return check(cudaSetDevice(c.device), "cudaSetDevice", error, error_len);
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        set_error(error, error_len, "CUDA is unavailable on this machine: %s",
                  e != cudaSuccess ? cudaGetErrorString(e) : "no device");
        return false;
    }
    if (c.device < 0) c.device = default_device_ordinal(count);
    if (c.device >= count) {
        set_error(error, error_len, "CUDA device %d requested but only %d visible", c.device, count);
        return false;
    }
    if (!check(cudaSetDevice(c.device), "cudaSetDevice", error, error_len)) return false;
    e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { set_error(error, error_len, "failed to create CUDA stream: %s", cudaGetErrorString(e)); return false; }
    cudaEventCreate(&c.ev0);
    cudaEventCreate(&c.ev1);
    c.ready = true;
    return true;
}

// A shader source generated from a Mandelbulber formula: the reference compiles
// it into the renderer (src/metal_bridge.mm:4231-4240, 5889-5897; the generator
// defines FPT_MANDEL_GENERATED_FIELD, src/mandelbulber/compiler.rs:1510).  The
// stock shader source (what src/main.rs passes on every other call) is what
// these kernels restate.
static bool generated_formula_source(const char *source, size_t len) {
    if (!source || len == 0) return false;
    static const char marker[] = "#define FPT_MANDEL_GENERATED_FIELD";
    const size_t m = sizeof(marker) - 1;
    if (len < m) return false;
    return std::search(source, source + len, marker, marker + m) != source + len;
}
static bool reject_generated_source(const char *source, size_t len, char *error, size_t error_len) {
    if (!generated_formula_source(source, len)) return false;
    set_error(error, error_len,
              "generated Mandelbulber formulas are not supported by the CUDA path (shader_source defines "
              "FPT_MANDEL_GENERATED_FIELD); use the FptCudaSceneExt formulas with fpt_cuda_render");
    return true;
}

bool ensure_buffer(void **ptr, size_t *cap, size_t need, char *error, size_t error_len) {
    if (*cap >= need && *ptr) return true;
    if (*ptr) cudaFree(*ptr);
    *ptr = nullptr;
    *cap = 0;
    size_t bytes = std::max<size_t>(need, 256);
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
        set_error(error, error_len, "failed to allocate %zu bytes of device memory: %s", bytes, cudaGetErrorString(e));
        *ptr = nullptr;
        return false;
    }
    *cap = bytes;
    return true;
}

bool check(cudaError_t e, const char *what, char *error, size_t error_len) {
    if (e == cudaSuccess) return true;
    set_error(error, error_len, "%s failed: %s", what, cudaGetErrorString(e));
    return false;
}

// ------------------------------------------------------------------ scene compilation
static void host_rotate_camera(const float v_in[3], float yaw, float pitch, float out[3]) {
    // rotateCamera (shaders/Shaders.metal:425-431) in float.
    float x = v_in[0], y = v_in[1], z = v_in[2];
    float sp = std::sin(pitch), cp = std::cos(pitch);
    float y1 = z * sp + y * cp, z1 = z * cp - y * sp;
    y = y1; z = z1;
    float sy = std::sin(yaw), cy = std::cos(yaw);
    out[0] = x * cy + z * sy;
    out[1] = y;
    out[2] = -x * sy + z * cy;
}

uint32_t scene_kind(const FptCudaSceneExt &e) {
    switch (e.formula) {
        case FPT_CUDA_FORMULA_MANDELBULB: return e.power == 8.0f ? KIND_BULB8 : KIND_BULB;
        case FPT_CUDA_FORMULA_MANDELBULB_POWER2: return KIND_BULB;
        case FPT_CUDA_FORMULA_MANDELBOX: return KIND_BOX;
        case FPT_CUDA_FORMULA_MENGER_FOLD: return KIND_MENGER;
        case FPT_CUDA_FORMULA_BULB_MENGER_HYBRID: return KIND_HYBRID;
        default: return KIND_GENERIC;
    }
}

bool compile_scene(const FptRenderConfig &c, const FptCudaSceneExt *ext_in, DeviceScene &S, char *error, size_t error_len) {
    static const FptCudaSceneExt none{};
    const FptCudaSceneExt &e = ext_in ? *ext_in : none;
    std::memset(&S, 0, sizeof(S));
    if (e.formula != 0 && e.formula != FPT_CUDA_FORMULA_MANDELBULB && e.formula != FPT_CUDA_FORMULA_MANDELBULB_POWER2 &&
        e.formula != FPT_CUDA_FORMULA_MANDELBOX &&
        e.formula != FPT_CUDA_FORMULA_MENGER_FOLD && e.formula != FPT_CUDA_FORMULA_BULB_MENGER_HYBRID) {
        set_error(error, error_len, "unsupported extension formula %u", e.formula);
        return false;
    }
    S.sdf_id = c.sdf_id;
    S.formula = e.formula;
    S.kind = scene_kind(e);
    S.width = c.width; S.height = c.height;
    S.samples = std::min(std::max(c.samples, 1u), 512u);
    int bounces = std::min(int(c.render[0]), 8);
    if (c.sdf_bounce_cap > 0u) bounces = std::min(bounces, int(c.sdf_bounce_cap));
    S.bounces = uint32_t(std::max(bounces, 0));
    S.russian_roulette = c.sdf_russian_roulette;
    S.rr_start = c.sdf_rr_start; S.rr_min_prob = c.sdf_rr_min_prob;
    S.normal_mode = c.sdf_normal_mode;
    S.ext_normal = e.normal_mode;
    S.translucent = (e.formula == 0 && (c.sdf_id == FPT_SDF_GLASS_BALL || c.sdf_id == FPT_SDF_README_GLASS ||
                                        (c.sdf_id == FPT_SDF_PROGRAM && c.program_material[5] > 0.0f))) ? 1u : 0u;
    std::memcpy(S.render, c.render, sizeof(S.render));
    std::memcpy(S.cam_pos, c.camera_position, sizeof(S.cam_pos));
    S.yaw = c.camera_yaw_pitch[0]; S.pitch = c.camera_yaw_pitch[1]; S.roll = c.camera_roll;
    S.focal = 1.0f / std::tan(c.camera_fov / 2.0f * 3.14159265359f / 180.0f);
    S.aa_strength = 0.3f / std::max(float(c.width), float(c.height));
    S.camera_fov = c.camera_fov;
    S.camera_dof = c.camera_dof;
    S.focus_distance = c.focus_distance;
    std::memcpy(S.world, c.world, sizeof(S.world));
    std::memcpy(S.world_one_color, c.world_one_color, sizeof(S.world_one_color));
    const float z1[3] = {0.0f, 0.0f, 1.0f};
    host_rotate_camera(z1, c.world[2] * 3.14159265359f / 180.0f, c.world[3] * 3.14159265359f / 180.0f, S.env_light_dir);
    S.world_cos_size = std::cos(std::max(c.world[1], 0.0001f));
    std::memcpy(S.sun, c.sun, sizeof(S.sun));
    std::memcpy(S.sun_color, c.sun_color, sizeof(S.sun_color));
    if (e.sun_intensity > 0.0f) {
        float n = std::sqrt(e.sun_direction[0] * e.sun_direction[0] + e.sun_direction[1] * e.sun_direction[1] +
                            e.sun_direction[2] * e.sun_direction[2]);
        if (!(n > 0.0f)) { set_error(error, error_len, "extension sun direction must be non-zero"); return false; }
        for (int k = 0; k < 3; ++k) S.sun_dir[k] = e.sun_direction[k] / n;
        S.sun_power = e.sun_intensity;
    } else {
        host_rotate_camera(z1, c.sun[1] * 3.14159265359f / 180.0f, c.sun[2] * 3.14159265359f / 180.0f, S.sun_dir);
        S.sun_power = 0.0f;
    }
    std::memcpy(S.background_gradient, c.background_gradient, sizeof(S.background_gradient));
    std::memcpy(S.post, c.post, sizeof(S.post));
    std::memcpy(S.set_values, c.set_values, sizeof(S.set_values));
    std::memcpy(S.vset_values, c.vset_values, sizeof(S.vset_values));
    S.material_mode = c.material_mode;
    S.gradient_count = c.gradient_count;
    S.fractal_style_mode = c.fractal_style_mode;
    std::memcpy(S.fractal_style, c.fractal_style, sizeof(S.fractal_style));
    std::memcpy(S.program_material, c.program_material, sizeof(S.program_material));
    std::memcpy(S.gradient_stops, c.gradient_stops, sizeof(S.gradient_stops));
    // deMandelbox constants (shaders/Shaders.metal:731-737).
    {
        float SC = 2.8f + c.set_values[2], M = 0.25f + c.set_values[3];
        S.box_ref[0] = S.box_ref[1] = S.box_ref[2] = SC / M;
        S.box_ref[3] = std::fabs(SC) / M;
        S.box_ref[4] = std::min(std::max(M, 1.0e-9f), 1.0f);
        S.box_ref[5] = std::fabs(SC - 1.0f);
        S.box_ref[6] = std::pow(std::fabs(SC), -9.0f);
    }
    // deIFS rotation (shaders/Shaders.metal:473-493, 707-709).
    {
        float ax = -51.080209f + c.set_values[2] * 90.0f, ay = c.set_values[3] * 90.0f, az = -29.096322f + c.set_values[4] * 90.0f;
        const float k = 3.14159265359f / 180.0f;
        S.ifs_rot[0] = std::sin(ax * k); S.ifs_rot[1] = std::cos(ax * k);
        S.ifs_rot[2] = std::sin(ay * k); S.ifs_rot[3] = std::cos(ay * k);
        S.ifs_rot[4] = std::sin(az * k); S.ifs_rot[5] = std::cos(az * k);
    }
    {
        const float *v = c.vset_values;
        for (int k = 0; k < 3; ++k) { S.global_rot[2 * k] = std::sin(v[123 + k]); S.global_rot[2 * k + 1] = std::cos(v[123 + k]); }
        bool ident = std::max(c.set_values[0], 1.0f) == 1.0f;
        for (int k = 120; k <= 128; ++k) ident = ident && v[k] == 0.0f;
        S.global_identity = ident ? 1u : 0u;
        float rx = c.set_values[9], ry = c.set_values[10], rz = c.set_values[11];
        S.mb_rot[0] = std::sin(rz); S.mb_rot[1] = std::cos(rz);
        S.mb_rot[2] = std::sin(ry); S.mb_rot[3] = std::cos(ry);
        S.mb_rot[4] = std::sin(rx); S.mb_rot[5] = std::cos(rx);
    }
    // Extension formula.
    S.iterations = e.iterations;
    S.bailout = e.bailout;
    S.power = e.power;
    S.box_scale = e.box_scale;
    S.box_fixed2 = float(double(e.box_fixed_radius) * double(e.box_fixed_radius));
    S.box_min2 = float(double(e.box_min_radius) * double(e.box_min_radius));
    S.box_min_factor = S.box_min2 > 0.0f ? S.box_fixed2 / S.box_min2 : 1.0f;
    S.box_fold_limit = e.box_fold_limit;
    S.box_fold_value = e.box_fold_value;
    S.menger_scale = e.menger_scale;
    S.hybrid_period = e.hybrid_period;
    S.ground_plane = e.ground_plane;
    S.plane_height = e.plane_height;
    S.rng = e.rng; S.seed = e.seed; S.brdf = e.brdf;
    S.albedo = e.albedo; S.ggx_alpha = e.ggx_alpha; S.specular_f0 = e.specular_f0; S.plane_albedo = e.plane_albedo;
    S.fp64_bisection = e.fp64_bisection;
    S.surrogate = e.surrogate;
    S.surrogate_margin = e.surrogate_margin;
    S.surrogate_safety = e.surrogate_safety;
    S.surrogate_max_iters = e.surrogate_max_iters;
    if (e.formula == FPT_CUDA_FORMULA_MANDELBOX && !(S.box_min2 > 0.0f)) {
        set_error(error, error_len, "Mandelbox minimum radius must be positive");
        return false;
    }
    if ((e.formula == FPT_CUDA_FORMULA_MENGER_FOLD || e.formula == FPT_CUDA_FORMULA_BULB_MENGER_HYBRID) && !(e.menger_scale > 1.0f)) {
        set_error(error, error_len, "Menger fold scale must be greater than 1");
        return false;
    }
    S.hdri_enabled = c.hdri_enabled;
    S.hdri_width = c.hdri_width;
    S.hdri_height = c.hdri_height;
    std::memcpy(S.hdri_lut, c.hdri_lut, sizeof(S.hdri_lut));
    S.program_count = std::min<uint32_t>(c.sdf_program_count, FPT_SDF_PROGRAM_MAX_OPS);
    S.shading_count = std::min<uint32_t>(c.sdf_shading_program_count, FPT_SDF_PROGRAM_MAX_OPS);
    std::memcpy(S.program, c.sdf_program, sizeof(S.program));
    std::memcpy(S.shading, c.sdf_shading_program, sizeof(S.shading));
    S.soa = c.sdf_typed_soa;
    S.soa.sphere_count = std::min<uint32_t>(S.soa.sphere_count, FPT_SDF_FLAT_UNION_MAX_PRIMITIVES);
    S.soa.box_count = std::min<uint32_t>(S.soa.box_count, FPT_SDF_FLAT_UNION_MAX_PRIMITIVES);
    S.soa.plane_count = std::min<uint32_t>(S.soa.plane_count, FPT_SDF_FLAT_UNION_MAX_PRIMITIVES);
    S.soa_count = S.program_count > 0u ? S.soa.sphere_count + S.soa.box_count + S.soa.plane_count : 0u;
    return true;
}

// HDRI hydration (src/metal_bridge.mm:2262-2300): 32x16 FP16 box-filtered LUT.
bool hydrate_hdri(FptRenderConfig &config, char *error, size_t error_len) {
    config.hdri_width = 0u;
    config.hdri_height = 0u;
    std::memset(config.hdri_lut, 0, sizeof(config.hdri_lut));
    if (config.hdri_enabled == 0u || config.world[0] != 2.0f) return true;
    const char *path = reinterpret_cast<const char *>(config.hdri_path);
    if (!path[0]) { set_error(error, error_len, "HDRI world mode requires world.hdri"); return false; }
    HdrImage img;
    std::string err;
    try {
        if (!read_radiance_hdr(path, img, err)) { set_error(error, error_len, "%s", err.c_str()); return false; }
    } catch (const std::exception &ex) {
        set_error(error, error_len, "failed to read HDRI %s: %s", path, ex.what());
        return false;
    }
    config.hdri_width = FPT_HDRI_LUT_WIDTH;
    config.hdri_height = FPT_HDRI_LUT_HEIGHT;
    for (uint32_t y = 0; y < FPT_HDRI_LUT_HEIGHT; ++y) {
        uint32_t sy0 = uint32_t((uint64_t(y) * img.height) / FPT_HDRI_LUT_HEIGHT);
        uint32_t sy1 = std::max(sy0 + 1u, uint32_t((uint64_t(y + 1u) * img.height) / FPT_HDRI_LUT_HEIGHT));
        for (uint32_t x = 0; x < FPT_HDRI_LUT_WIDTH; ++x) {
            uint32_t sx0 = uint32_t((uint64_t(x) * img.width) / FPT_HDRI_LUT_WIDTH);
            uint32_t sx1 = std::max(sx0 + 1u, uint32_t((uint64_t(x + 1u) * img.width) / FPT_HDRI_LUT_WIDTH));
            float sum[3] = {0, 0, 0};
            uint32_t n = 0;
            for (uint32_t sy = sy0; sy < std::min(sy1, img.height); ++sy)
                for (uint32_t sx = sx0; sx < std::min(sx1, img.width); ++sx) {
                    size_t s = (size_t(sy) * img.width + sx) * 3;
                    sum[0] += img.rgb[s]; sum[1] += img.rgb[s + 1]; sum[2] += img.rgb[s + 2];
                    ++n;
                }
            size_t d = (size_t(y) * FPT_HDRI_LUT_WIDTH + x) * 3;
            for (int k = 0; k < 3; ++k) config.hdri_lut[d + k] = reference_float_to_half(sum[k] / float(std::max(n, 1u)));
        }
    }
    return true;
}

// Uploads the scene block (and the extension sky texture) to the device.
bool upload_scene(DeviceScene &S, const FptCudaSceneExt *ext, char *error, size_t error_len) {
    Context &c = ctx();
    if (ext && ext->sky_width > 0) {
        if (!ext->sky_rgb || ext->sky_height == 0) { set_error(error, error_len, "extension sky needs sky_rgb and sky_height"); return false; }
        size_t bytes = size_t(ext->sky_width) * ext->sky_height * 3 * sizeof(float);
        if (!ensure_buffer((void **)&c.sky, &c.cap_sky, bytes, error, error_len)) return false;
        if (!check(cudaMemcpyAsync(c.sky, ext->sky_rgb, bytes, cudaMemcpyHostToDevice, c.stream), "sky upload", error, error_len))
            return false;
        S.sky_width = ext->sky_width;
        S.sky_height = ext->sky_height;
        S.sky_rgb = c.sky;
    }
    if (S.surrogate && ext) {
        if (!surrogate_bind(ext->surrogate_model, S, error, error_len)) return false;
    }
    if (!ensure_buffer((void **)&c.scene, &c.cap_scene, sizeof(DeviceScene), error, error_len)) return false;
    return check(cudaMemcpyAsync(c.scene, &S, sizeof(DeviceScene), cudaMemcpyHostToDevice, c.stream), "scene upload", error, error_len);
}

// FP32 fused multiply-add throughput: every thread runs eight independent
// FMA chains (enough independent work to issue one FMA per cycle on every
// scheduler), unrolled so the loop adds about one non-FMA instruction per 256
// FMAs.  Multiplier and addend come from the host, so nothing folds.
__global__ void __launch_bounds__(256) fma_peak_kernel(float *sink, uint32_t trips, float m, float c) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = float(threadIdx.x) * 1.0e-3f + float(k);
    for (uint32_t i = 0; i < trips; ++i) {
#pragma unroll 32
        for (int j = 0; j < 32; ++j) {
#pragma unroll
            for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], m, c);
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == 1.0e30f) sink[0] = s;   // never true: keeps the chains live
}

}  // namespace fpt

using namespace fpt;

namespace {

// Render core shared by fpt_metal_render and fpt_cuda_render.
int render_core(const FptRenderConfig *config, const FptCudaSceneExt *ext, const char *output_path, float *linear_output,
                size_t linear_output_len, uint8_t *rgba_output, size_t rgba_output_len, double *elapsed_ms,
                FptSdfProfileStats *profile_out, uint64_t *voxel_memory_bytes, uint32_t *voxel_active_bricks,
                uint64_t *voxel_active_cells, double *build_ms, char *error, size_t error_len) {
    if (elapsed_ms) *elapsed_ms = 0.0;
    if (profile_out) std::memset(profile_out, 0, sizeof(*profile_out));
    if (!config) { set_error(error, error_len, "missing render config"); return 1; }
    if (config->width == 0 || config->height == 0) {
        set_error(error, error_len, "invalid render size %ux%u", config->width, config->height);
        return 1;
    }
    const size_t pixels = size_t(config->width) * config->height;
    if (linear_output && linear_output_len < pixels * 4) {
        set_error(error, error_len, "linear output buffer is too small (%zu < %zu)", linear_output_len, pixels * 4);
        return 1;
    }
    if (rgba_output && rgba_output_len < pixels * 4) {
        set_error(error, error_len, "rgba output buffer is too small (%zu < %zu)", rgba_output_len, pixels * 4);
        return 1;
    }
    FptRenderConfig hydrated = *config;
    if (!hydrate_hdri(hydrated, error, error_len)) return 1;
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    DeviceScene S;
    if (!compile_scene(hydrated, ext, S, error, error_len)) return 1;
    if (hydrated.renderer_backend == FPT_RENDERER_VOXEL) {
        return voxel_render_core(hydrated, ext, S, output_path, linear_output, rgba_output, elapsed_ms, voxel_memory_bytes,
                                 voxel_active_bricks, voxel_active_cells, build_ms, error, error_len);
    }
    if (hydrated.renderer_backend != FPT_RENDERER_SDF) {
        set_error(error, error_len, "renderer backend %u is not supported by the CUDA path (research backends)",
                  hydrated.renderer_backend);
        return 1;
    }
    if (!upload_scene(S, ext, error, error_len)) return 1;
    if (!ensure_buffer((void **)&c.accum, &c.cap_accum, pixels * sizeof(float4), error, error_len)) return 1;
    if (!ensure_buffer((void **)&c.rgba, &c.cap_rgba, pixels * sizeof(uchar4), error, error_len)) return 1;
    if (!ensure_buffer((void **)&c.counter, &c.cap_counter, 64, error, error_len)) return 1;
    if (!check(cudaMemsetAsync(c.counter, 0, 64, c.stream), "counter reset", error, error_len)) return 1;
    bool want_profile = profile_out != nullptr || hydrated.sdf_profile != 0u;
    if (want_profile) {
        if (!ensure_buffer((void **)&c.profile, &c.cap_profile, kProfileSlots * sizeof(unsigned long long), error, error_len)) return 1;
        if (!check(cudaMemsetAsync(c.profile, 0, kProfileSlots * sizeof(unsigned long long), c.stream), "profile reset", error,
                   error_len))
            return 1;
    }
    cudaEventRecord(c.ev0, c.stream);
    if (hydrated.focus_distance <= 0.0f) {
        if (!check(launch_focus(S.kind, c.scene, c.stream), "focus-distance prepass", error, error_len)) return 1;
    }
    // Accumulation-mode policy (src/metal_bridge.mm:4531-4564).
    const uint32_t spp = S.samples;
    const bool auto_batch = spp <= 16u && hydrated.sdf_id != FPT_SDF_CAGE_FRACTAL;
    const uint32_t mode = hydrated.sdf_accumulation_mode;
    const bool batch = mode == FPT_SDF_ACCUMULATION_BATCH || (mode == FPT_SDF_ACCUMULATION_AUTO && auto_batch) || hydrated.preview;
    const bool chunked = !batch && (mode == FPT_SDF_ACCUMULATION_CHUNKED || mode == FPT_SDF_ACCUMULATION_AUTO);
    uint32_t step = batch ? spp : (chunked ? std::min(std::max(hydrated.sdf_chunk_samples, 1u), 64u) : 1u);
    // Per-path colour scratch: launches of at most `sub` samples keep it
    // under 2 GiB; the in-order reduction makes the split invisible.
    const uint32_t sub_cap = uint32_t(std::max<size_t>(1, (size_t(2) << 30) / (pixels * sizeof(float4))));
    if (!ensure_buffer((void **)&c.sample_rgb, &c.cap_sample_rgb, pixels * sizeof(float4) * std::min(step, sub_cap), error,
                       error_len))
        return 1;
    PathLaunch pl{};
    pl.scene = c.scene; pl.kind = S.kind; pl.width = S.width; pl.height = S.height; pl.bounces = S.bounces;
    pl.accum = c.accum; pl.counters = c.counter; pl.march_blocks = c.march_blocks;
    pl.refill_batch = c.refill_batch;
    pl.fp64 = (S.fp64_bisection && S.sdf_id == FPT_SDF_MANDELBULBER && S.formula != 0 && !(S.camera_dof > 0.0f)) ? 1u : 0u;
    pl.loop_limit_ns = c.loop_limit_ns;
    pl.profile = want_profile ? c.profile : nullptr;
    {
        // Wave scratch: path records and queues for up to wave_paths paths.
        const size_t tiles = size_t((S.width + 7u) / 8u) * ((S.height + 3u) / 4u) * 32u;
        size_t per_launch = tiles * std::min(step, sub_cap);
        size_t cap = c.wave_paths ? c.wave_paths : (size_t(64) << 20);   // one wave per 1080p 16 spp frame
        cap = std::min(cap, per_launch);
        pl.wave_paths = uint32_t(cap);
        if (!ensure_buffer(&c.wave, &c.cap_wave, wave_scratch_bytes(cap), error, error_len)) return 1;
        pl.wave_scratch = c.wave;
        if (want_profile) {
            if (!ensure_buffer((void **)&c.path_steps, &c.cap_path_steps, cap * sizeof(uint32_t), error, error_len)) return 1;
            pl.path_steps = c.path_steps;
        }
    }
    pl.sample_rgb = c.sample_rgb;
    SkipArgs skip;
    if (S.surrogate) {
        if (!ensure_buffer((void **)&c.skip_stats, &c.cap_skip_stats, kSkipStats * sizeof(unsigned long long), error, error_len) ||
            !check(cudaMemsetAsync(c.skip_stats, 0, kSkipStats * sizeof(unsigned long long), c.stream), "skip stats reset", error,
                   error_len) ||
            !surrogate_args(ext->surrogate_model, S, c.skip_stats, skip, error, error_len))
            return 1;
        pl.skip = &skip;
    }
    KernelTimer timer;
    uint64_t launches = 0;
    pl.launches = &launches;
    uint32_t grids[2] = {0, 0};
    pl.grids = grids;
    if (want_profile || c.kernel_timing) {   // per-kernel spans: profile renders, or any render with kernel timing on
        if (!c.timer_events) {
            c.timer_capacity = 1024;
            c.timer_events = new cudaEvent_t[c.timer_capacity];
            for (int i = 0; i < c.timer_capacity; ++i) cudaEventCreate(&c.timer_events[i]);
        }
        timer.events = c.timer_events;
        timer.capacity = c.timer_capacity;
        pl.timer = &timer;
    }
    for (uint32_t start = 0; start < spp; start += step) {
        uint32_t end = std::min(spp, start + step);
        for (uint32_t a = start; a < end; a += sub_cap) {
            pl.sample_begin = a;
            pl.sample_end = std::min(end, a + sub_cap);
            if (!check(launch_pathtrace(pl, c.stream), "path-tracing launch", error, error_len)) return 1;
        }
    }
    if (!check(launch_present(c.scene, S.width, S.height, c.accum, c.rgba, c.stream), "present launch", error, error_len)) return 1;
    ++launches;
    cudaEventRecord(c.ev1, c.stream);
    if (!check(cudaStreamSynchronize(c.stream), "CUDA render", error, error_len)) return 1;
    {
        uint32_t guard = 0;
        if (!check(cudaMemcpy(&guard, c.counter + C_GUARD, sizeof(guard), cudaMemcpyDeviceToHost), "guard readback", error, error_len))
            return 1;
        if (guard) {
            set_error(error, error_len, (guard & 2u) ? "a surrogate network MMA did not complete within 1 s (render aborted)"
                                                     : "a persistent march loop exceeded its time limit and stopped (render aborted)");
            return 1;
        }
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    if (elapsed_ms) *elapsed_ms = double(ms);
    {
        FptCudaRenderStats &rs = c.last_render;
        std::memset(&rs, 0, sizeof(rs));
        rs.kernel_launches = launches + (hydrated.focus_distance <= 0.0f ? 1u : 0u);
        rs.total_ms = ms;
        rs.march_grid = grids[0];
        rs.skip_grid = grids[1];
        double cat_ms[KC_COUNT] = {0.0, 0.0, 0.0};
        uint64_t cat_n[KC_COUNT] = {0, 0, 0};
        for (int i = 0; i < timer.n; ++i) {
            float t = 0.0f;
            cudaEventElapsedTime(&t, timer.events[2 * i], timer.events[2 * i + 1]);
            cat_ms[timer.cat[i]] += t;
            cat_n[timer.cat[i]] += 1;
        }
        rs.march_ms = cat_ms[KC_MARCH]; rs.shade_ms = cat_ms[KC_SHADE]; rs.skip_ms = cat_ms[KC_SKIP];
        rs.march_launches = cat_n[KC_MARCH]; rs.shade_launches = cat_n[KC_SHADE]; rs.skip_launches = cat_n[KC_SKIP];
    }
    std::vector<uint8_t> host_rgba;
    uint8_t *rgba = rgba_output;
    if (!rgba) { host_rgba.resize(pixels * 4); rgba = host_rgba.data(); }
    if (!check(cudaMemcpy(rgba, c.rgba, pixels * 4, cudaMemcpyDeviceToHost), "image readback", error, error_len)) return 1;
    if (linear_output) {
        if (!check(cudaMemcpy(linear_output, c.accum, pixels * sizeof(float4), cudaMemcpyDeviceToHost), "linear readback", error,
                   error_len))
            return 1;
    }
    if (S.surrogate &&
        !check(cudaMemcpy(c.last_skip, c.skip_stats, sizeof(c.last_skip), cudaMemcpyDeviceToHost), "skip stats readback", error,
               error_len))
        return 1;
    if (want_profile && profile_out) {
        unsigned long long v[kProfileSlots];
        if (!check(cudaMemcpy(v, c.profile, sizeof(v), cudaMemcpyDeviceToHost), "profile readback", error, error_len)) return 1;
        profile_out->primary_steps = v[0]; profile_out->secondary_steps = v[1]; profile_out->shadow_steps = v[2];
        profile_out->normal_evals = v[3]; profile_out->bounces = v[4]; profile_out->pixels = v[5];
        profile_out->distance_evals = v[0] + v[1] + v[2]; profile_out->material_evals = v[7];
        c.last_render.march_evals = v[0] + v[1] + v[2];
        c.last_render.shade_evals = v[3] + v[7];
        profile_out->distance_evals_by_phase[0] = v[0];
        profile_out->distance_evals_by_phase[1] = v[1];
        profile_out->distance_evals_by_phase[2] = v[2];
        profile_out->distance_evals_by_phase[3] = v[3];
        profile_out->normal_field_evals = v[3];   // one (dual-number) field evaluation per normal
        for (int k = 0; k < 3; ++k) profile_out->orbit_iterations_by_phase[k] = v[8 + k];
        profile_out->march_orbit_iterations = v[8] + v[9] + v[10];
        profile_out->formula_slot_iterations[0] = profile_out->march_orbit_iterations;   // one formula slot
        profile_out->refinement_steps = v[11];
        profile_out->refinement_distance_evals = v[11];
        profile_out->max_ray_steps = v[12];
        profile_out->max_pixel_steps = v[13];
        profile_out->orbit_iterations_by_phase[3] = v[14];
        profile_out->march_orbit_iterations += v[14];
        profile_out->formula_slot_iterations[0] = profile_out->march_orbit_iterations;
        // Render time apportioned by counted work units (src/metal_bridge.mm:5712-5733).
        const double units[5] = {double(v[0]), double(v[1]), double(v[2]), double(profile_out->normal_field_evals), double(v[4])};
        const double total = units[0] + units[1] + units[2] + units[3] + units[4];
        if (total > 0.0) {
            profile_out->primary_ms_estimate = ms * units[0] / total;
            profile_out->secondary_ms_estimate = ms * units[1] / total;
            profile_out->shadow_ms_estimate = ms * units[2] / total;
            profile_out->normal_ms_estimate = ms * units[3] / total;
            profile_out->bounce_ms_estimate = ms * units[4] / total;
        }
    }
    if (output_path) {
        if (unique_colour_sample(rgba, pixels) < 2) {
            set_error(error, error_len, "render output is blank or single-colour");
            return 1;
        }
        std::string err;
        if (!write_png(output_path, config->width, config->height, rgba, err)) {
            set_error(error, error_len, "%s", err.c_str());
            return 1;
        }
    }
    return 0;
}

}  // namespace

extern "C" {

int fpt_metal_render(const char *metallib_path, const char *stitch_metallib_path, const char *stitch_archive_path,
                     const char *output_path, const char *shader_source, size_t shader_source_len,
                     const struct FptRenderConfig *config, double *build_ms, double *elapsed_ms, uint64_t *voxel_memory_bytes,
                     uint32_t *voxel_active_bricks, uint64_t *voxel_active_cells, uint32_t *voxel_rejected_bricks,
                     struct FptBoundGridStats *bound_grid_stats, uint32_t *stitch_cache_status,
                     struct FptStitchValidationStats *stitch_validation_stats, struct FptStitchPipelineStats *stitch_pipeline_stats,
                     struct FptSdfProfileStats *sdf_profile_stats, float *linear_output, size_t linear_output_len, char *error,
                     size_t error_len) {
    (void)metallib_path; (void)stitch_metallib_path; (void)stitch_archive_path;
    if (build_ms) *build_ms = 0.0;
    if (voxel_memory_bytes) *voxel_memory_bytes = 0;
    if (voxel_active_bricks) *voxel_active_bricks = 0;
    if (voxel_active_cells) *voxel_active_cells = 0;
    if (voxel_rejected_bricks) *voxel_rejected_bricks = 0;
    if (bound_grid_stats) std::memset(bound_grid_stats, 0, sizeof(*bound_grid_stats));
    if (stitch_cache_status) *stitch_cache_status = 0;
    if (stitch_validation_stats) std::memset(stitch_validation_stats, 0, sizeof(*stitch_validation_stats));
    if (stitch_pipeline_stats) std::memset(stitch_pipeline_stats, 0, sizeof(*stitch_pipeline_stats));
    if (elapsed_ms) *elapsed_ms = 0.0;
    if (sdf_profile_stats) std::memset(sdf_profile_stats, 0, sizeof(*sdf_profile_stats));
    if (reject_generated_source(shader_source, shader_source_len, error, error_len)) return 1;
    if (!output_path) { set_error(error, error_len, "missing output path"); return 1; }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    return render_core(config, nullptr, output_path, linear_output, linear_output_len, nullptr, 0, elapsed_ms, sdf_profile_stats,
                       voxel_memory_bytes, voxel_active_bricks, voxel_active_cells, build_ms, error, error_len);
}

int fpt_cuda_render(const struct FptRenderConfig *config, const struct FptCudaSceneExt *ext, const char *output_path,
                    float *linear_output, size_t linear_output_len, uint8_t *rgba_output, size_t rgba_output_len,
                    double *elapsed_ms, struct FptSdfProfileStats *profile, char *error, size_t error_len) {
    std::lock_guard<std::mutex> lock(ctx().mutex);
    return render_core(config, ext, output_path, linear_output, linear_output_len, rgba_output, rgba_output_len, elapsed_ms,
                       profile, nullptr, nullptr, nullptr, nullptr, error, error_len);
}

int fpt_cuda_trace_primary(const struct FptRenderConfig *config, const struct FptCudaSceneExt *ext, struct FptCudaPrimaryHit *hits,
                           size_t hit_count, double *elapsed_ms, char *error, size_t error_len) {
    if (elapsed_ms) *elapsed_ms = 0.0;
    if (!config || !hits) { set_error(error, error_len, "missing primary-ray input"); return 1; }
    if (config->width == 0 || config->height == 0) {
        set_error(error, error_len, "invalid render size %ux%u", config->width, config->height);
        return 1;
    }
    size_t pixels = size_t(config->width) * config->height;
    if (hit_count < pixels) { set_error(error, error_len, "hit buffer is too small (%zu < %zu)", hit_count, pixels); return 1; }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    FptRenderConfig hydrated = *config;
    if (!hydrate_hdri(hydrated, error, error_len)) return 1;
    DeviceScene S;
    if (!compile_scene(hydrated, ext, S, error, error_len)) return 1;
    if (!upload_scene(S, ext, error, error_len)) return 1;
    if (!ensure_buffer((void **)&c.hits, &c.cap_hits, pixels * sizeof(FptCudaPrimaryHit), error, error_len)) return 1;
    SkipArgs skip;
    if (S.surrogate) {
        if (!ensure_buffer((void **)&c.skip_stats, &c.cap_skip_stats, kSkipStats * sizeof(unsigned long long), error, error_len) ||
            !check(cudaMemsetAsync(c.skip_stats, 0, kSkipStats * sizeof(unsigned long long), c.stream), "skip stats reset", error,
                   error_len) ||
            !surrogate_args(ext->surrogate_model, S, c.skip_stats, skip, error, error_len))
            return 1;
    }
    if (S.surrogate) {
        if (!ensure_buffer((void **)&c.counter, &c.cap_counter, 64, error, error_len) ||
            !check(cudaMemsetAsync(c.counter, 0, 64, c.stream), "counter reset", error, error_len))
            return 1;
        skip.guard = c.counter + C_GUARD;
        skip.cam_step = c.counter + C_CAMSTEP;
    }
    cudaEventRecord(c.ev0, c.stream);
    cudaError_t le = S.surrogate ? launch_skip_primary(S.kind, c.scene, S.width, S.height, skip, c.hits, c.stream)
                                 : launch_trace_primary(S.kind, c.scene, S.width, S.height, c.hits, c.stream);
    if (!check(le, "primary-ray launch", error, error_len)) return 1;
    cudaEventRecord(c.ev1, c.stream);
    if (!check(cudaStreamSynchronize(c.stream), "primary-ray trace", error, error_len)) return 1;
    if (S.surrogate) {
        uint32_t guard = 0;
        if (!check(cudaMemcpy(&guard, c.counter + C_GUARD, sizeof(guard), cudaMemcpyDeviceToHost), "guard readback", error, error_len))
            return 1;
        if (guard) {
            set_error(error, error_len, "a surrogate network MMA did not complete within 1 s (trace aborted)");
            return 1;
        }
    }
    if (S.surrogate &&
        !check(cudaMemcpy(c.last_skip, c.skip_stats, sizeof(c.last_skip), cudaMemcpyDeviceToHost), "skip stats readback", error,
               error_len))
        return 1;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    if (elapsed_ms) *elapsed_ms = ms;
    return check(cudaMemcpy(hits, c.hits, pixels * sizeof(FptCudaPrimaryHit), cudaMemcpyDeviceToHost), "hit readback", error,
                 error_len) ? 0 : 1;
}

int fpt_mandelbulber_sample_field(const char *metallib_path, const char *shader_source, size_t shader_source_len,
                                  const struct FptRenderConfig *config, const float *points_xyzw, size_t point_count,
                                  struct FptMandelbulberFieldSample *samples, char *error, size_t error_len) {
    (void)metallib_path;
    if (!config || !points_xyzw || !samples || point_count == 0u) {
        set_error(error, error_len, "missing Mandelbulber field-sampling input");
        return 1;
    }
    if (reject_generated_source(shader_source, shader_source_len, error, error_len)) return 1;
    if (config->sdf_id != FPT_SDF_MANDELBULBER) {
        set_error(error, error_len, "field sampling requires a Mandelbulber scene");
        return 1;
    }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    DeviceScene S;
    if (!compile_scene(*config, nullptr, S, error, error_len)) return 1;
    if (!upload_scene(S, nullptr, error, error_len)) return 1;
    size_t bytes = point_count * sizeof(float4);
    if (!ensure_buffer((void **)&c.points, &c.cap_points, bytes, error, error_len)) return 1;
    if (!ensure_buffer((void **)&c.samples, &c.cap_samples, bytes, error, error_len)) return 1;
    if (!check(cudaMemcpyAsync(c.points, points_xyzw, bytes, cudaMemcpyHostToDevice, c.stream), "point upload", error, error_len))
        return 1;
    if (!check(launch_field_sample(c.scene, c.points, c.samples, point_count, c.stream), "field-sampling launch", error, error_len))
        return 1;
    if (!check(cudaStreamSynchronize(c.stream), "Mandelbulber field-sampling dispatch", error, error_len)) return 1;
    return check(cudaMemcpy(samples, c.samples, bytes, cudaMemcpyDeviceToHost), "sample readback", error, error_len) ? 0 : 1;
}

int fpt_cuda_sample_distance(const struct FptRenderConfig *config, const struct FptCudaSceneExt *ext, const float *points_xyzw,
                             size_t point_count, float *samples, float *gradients, char *error, size_t error_len) {
    if (!config || !points_xyzw || !samples || point_count == 0u) {
        set_error(error, error_len, "missing distance-sampling input");
        return 1;
    }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    DeviceScene S;
    if (!compile_scene(*config, ext, S, error, error_len)) return 1;
    if (!upload_scene(S, ext, error, error_len)) return 1;
    size_t bytes = point_count * sizeof(float4);
    if (!ensure_buffer((void **)&c.points, &c.cap_points, bytes, error, error_len)) return 1;
    if (!ensure_buffer((void **)&c.samples, &c.cap_samples, bytes, error, error_len)) return 1;
    if (gradients && !ensure_buffer((void **)&c.grads, &c.cap_grads, point_count * 3 * sizeof(float), error, error_len)) return 1;
    if (!check(cudaMemcpyAsync(c.points, points_xyzw, bytes, cudaMemcpyHostToDevice, c.stream), "point upload", error, error_len))
        return 1;
    if (!check(launch_sample_distance(S.kind, c.scene, c.points, c.samples, gradients ? c.grads : nullptr, point_count, c.stream),
               "distance-sampling launch", error, error_len))
        return 1;
    if (!check(cudaStreamSynchronize(c.stream), "distance sampling", error, error_len)) return 1;
    if (!check(cudaMemcpy(samples, c.samples, bytes, cudaMemcpyDeviceToHost), "sample readback", error, error_len)) return 1;
    if (gradients &&
        !check(cudaMemcpy(gradients, c.grads, point_count * 3 * sizeof(float), cudaMemcpyDeviceToHost), "gradient readback", error,
               error_len))
        return 1;
    return 0;
}

int fpt_compare_images(const char *baseline_path, const char *candidate_path, const char *report_path, char *error,
                       size_t error_len) {
    if (!baseline_path || !candidate_path || !report_path) { set_error(error, error_len, "missing comparison path"); return 1; }
    Image a, b;
    std::string err;
    try {
        if (!read_png(baseline_path, a, err) || !read_png(candidate_path, b, err)) { set_error(error, error_len, "%s", err.c_str()); return 1; }
    } catch (const std::exception &ex) {
        set_error(error, error_len, "failed to read PNG: %s", ex.what());
        return 1;
    }
    if (a.width != b.width || a.height != b.height) {
        set_error(error, error_len, "dimension mismatch: baseline %ux%u candidate %ux%u", a.width, a.height, b.width, b.height);
        return 1;
    }
    ImageMetrics m = compare_rgba(a.rgba.data(), b.rgba.data(), a.width, a.height);
    FILE *f = std::fopen(report_path, "w");
    if (!f) { set_error(error, error_len, "failed to open report %s", report_path); return 1; }
    std::fprintf(f,
                 "{\n  \"baseline\": \"%s\",\n  \"candidate\": \"%s\",\n  \"width\": %u,\n  \"height\": %u,\n"
                 "  \"mean_absolute_error\": %.17g,\n  \"root_mean_square_error\": %.17g,\n  \"luminance_ssim\": %.17g,\n"
                 "  \"low_frequency_luminance_ssim\": %.17g,\n  \"max_absolute_error\": %.0f,\n  \"changed_pixel_percent\": %.17g,\n"
                 "  \"unique_colours\": {\n    \"baseline\": %zu,\n    \"candidate\": %zu\n  }\n}\n",
                 baseline_path, candidate_path, a.width, a.height, m.mae, m.rmse, m.ssim, m.lf_ssim, m.max_abs, m.changed_pct,
                 m.unique_baseline, m.unique_candidate);
    std::fclose(f);
    return 0;
}

int fpt_metal_device_name(char *name, size_t name_len) {
    if (!name || name_len == 0) return 1;
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(nullptr, 0)) { name[0] = 0; return 1; }
    const int dev = ctx().device;
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) { name[0] = 0; return 1; }
    std::snprintf(name, name_len, "%s", p.name);
    return 0;
}

int fpt_test_async_stitch_context(const char *metallib_path, const char *stitch_metallib_path, const char *stitch_archive_path,
                                  const struct FptRenderConfig *config, struct FptAsyncJitStats *stats, char *error,
                                  size_t error_len) {
    (void)metallib_path; (void)stitch_metallib_path; (void)stitch_archive_path; (void)config;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    set_error(error, error_len, "unsupported: the CUDA path has no runtime shader-stitching JIT");
    return 1;
}

int fpt_metal_preview(const char *metallib_path, const char *stitch_metallib_path, const char *const *stitch_archive_paths,
                      const char *shader_source, size_t shader_source_len, const struct FptRenderConfig *config,
                      const struct FptRenderConfig *scene_configs, uint32_t scene_config_count, uint32_t scene_config_index,
                      char *error, size_t error_len) {
    (void)metallib_path; (void)stitch_metallib_path; (void)stitch_archive_paths; (void)shader_source; (void)shader_source_len;
    (void)config; (void)scene_configs; (void)scene_config_count; (void)scene_config_index;
    set_error(error, error_len, "unsupported: interactive preview needs a window system, which a headless CUDA node lacks");
    return 1;
}

int fpt_cuda_render_stats(struct FptCudaRenderStats *stats) {
    if (!stats) return 1;
    std::lock_guard<std::mutex> lock(ctx().mutex);
    *stats = ctx().last_render;
    return 0;
}

// Diagnostic images (src/metal_bridge.mm:5865-6025; kernel shaders/Shaders.metal:7290-7385): the encoded
// quantity of every pixel written as a PNG at output_path.
int fpt_metal_diagnostic_render(const char *metallib_path, const char *output_path, const char *shader_source,
                                size_t shader_source_len, const struct FptRenderConfig *config,
                                const struct FptDiagnosticConfig *diagnostic, double *elapsed_ms, char *error, size_t error_len) {
    (void)metallib_path;
    if (elapsed_ms) *elapsed_ms = 0.0;
    if (!config || !diagnostic) { set_error(error, error_len, "missing diagnostic render config"); return 1; }
    if (reject_generated_source(shader_source, shader_source_len, error, error_len)) return 1;
    if (!output_path) { set_error(error, error_len, "missing diagnostic output path"); return 1; }
    if (config->width == 0 || config->height == 0) {
        set_error(error, error_len, "invalid render size %ux%u", config->width, config->height);
        return 1;
    }
    const uint32_t mode = diagnostic->mode;
    if (mode > DIAG_SDF_BOUNCE_CONTRIBUTION) { set_error(error, error_len, "unknown diagnostic mode %u", mode); return 1; }
    if (mode == DIAG_SDF_BOUNCE_CONTRIBUTION) {
        set_error(error, error_len, "diagnostic mode %u (bounce contribution) is not supported by the CUDA path", mode);
        return 1;
    }
    if (config->renderer_backend != FPT_RENDERER_SDF) {
        set_error(error, error_len, "diagnostic images of renderer backend %u are not supported by the CUDA path", config->renderer_backend);
        return 1;
    }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    FptRenderConfig hydrated = *config;
    if (!hydrate_hdri(hydrated, error, error_len)) return 1;
    const size_t pixels = size_t(hydrated.width) * hydrated.height;
    float ms = 0.0f;
    if (mode == DIAG_PATH_FINAL) {
        // the path-traced mean of min(max(spp, 16), 64) samples through postProcess
        FptRenderConfig r = hydrated;
        r.samples = std::min(std::max(r.samples, 16u), 64u);
        double rms = 0.0;
        if (render_core(&r, nullptr, nullptr, nullptr, 0, nullptr, 0, &rms, nullptr, nullptr, nullptr, nullptr, nullptr, error,
                        error_len))
            return 1;
        DeviceScene S;
        if (!compile_scene(r, nullptr, S, error, error_len)) return 1;
        if (!check(launch_diag_final(c.scene, S.width, S.height, c.accum, c.rgba, c.stream), "diagnostic present", error, error_len) ||
            !check(cudaStreamSynchronize(c.stream), "diagnostic present", error, error_len))
            return 1;
        ms = float(rms);
    } else {
        DeviceScene S;
        if (!compile_scene(hydrated, nullptr, S, error, error_len)) return 1;
        if (!upload_scene(S, nullptr, error, error_len)) return 1;
        if (!ensure_buffer((void **)&c.rgba, &c.cap_rgba, pixels * sizeof(uchar4), error, error_len)) return 1;
        cudaEventRecord(c.ev0, c.stream);
        if (hydrated.focus_distance <= 0.0f &&
            !check(launch_focus(S.kind, c.scene, c.stream), "focus-distance prepass", error, error_len))
            return 1;
        if (!check(launch_diagnostic(S.kind, c.scene, S.width, S.height, mode, diagnostic->max_distance, c.rgba, c.stream),
                   "diagnostic launch", error, error_len))
            return 1;
        cudaEventRecord(c.ev1, c.stream);
        if (!check(cudaStreamSynchronize(c.stream), "diagnostic render", error, error_len)) return 1;
        cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    }
    if (elapsed_ms) *elapsed_ms = ms;
    std::vector<uint8_t> rgba(pixels * 4);
    if (!check(cudaMemcpy(rgba.data(), c.rgba, pixels * 4, cudaMemcpyDeviceToHost), "diagnostic readback", error, error_len)) return 1;
    std::string err;
    if (!write_png(output_path, hydrated.width, hydrated.height, rgba.data(), err)) {
        set_error(error, error_len, "%s", err.c_str());
        return 1;
    }
    return 0;
}

// Typed SoA validation (src/metal_bridge.mm:4116-4200): the lowered program
// (config->sdf_typed_soa) against the interpreter on 2^20 points.
int fpt_test_typed_soa(const char *metallib_path, const struct FptRenderConfig *config, struct FptStitchValidationStats *stats,
                       char *error, size_t error_len) {
    (void)metallib_path;
    if (!config || !stats) { set_error(error, error_len, "missing typed-SoA validation input"); return 1; }
    std::memset(stats, 0, sizeof(*stats));
    const uint32_t prims = config->sdf_typed_soa.sphere_count + config->sdf_typed_soa.box_count + config->sdf_typed_soa.plane_count;
    if (config->sdf_id != FPT_SDF_PROGRAM || prims == 0u || config->sdf_program_count == 0u) {
        set_error(error, error_len, "typed-SoA validation requires a lowered typed program");
        return 1;
    }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    DeviceScene S;
    if (!compile_scene(*config, nullptr, S, error, error_len) || !upload_scene(S, nullptr, error, error_len)) return 1;
    if (!ensure_buffer((void **)&c.counter, &c.cap_counter, 64, error, error_len) ||
        !check(cudaMemsetAsync(c.counter, 0, 4 * sizeof(unsigned int), c.stream), "counter reset", error, error_len))
        return 1;
    const uint32_t n = 1u << 20;
    unsigned int counts[4] = {0, 0, 0, 0};
    if (!check(launch_typed_soa_validation(c.scene, config->voxel_bounds_min, config->voxel_bounds_max, n, c.counter, c.stream),
               "typed-SoA validation launch", error, error_len) ||
        !check(cudaMemcpyAsync(counts, c.counter, sizeof(counts), cudaMemcpyDeviceToHost, c.stream), "counts readback", error,
               error_len) ||
        !check(cudaStreamSynchronize(c.stream), "typed-SoA validation", error, error_len))
        return 1;
    stats->sample_count = n;
    stats->distance_failures = counts[0];
    stats->gradient_failures = counts[1];
    std::memcpy(&stats->max_distance_error, &counts[2], sizeof(float));
    std::memcpy(&stats->max_gradient_error, &counts[3], sizeof(float));
    if (counts[0] != 0u || counts[1] != 0u) {
        set_error(error, error_len, "typed-SoA validation failed: %u distance, %u gradient", counts[0], counts[1]);
        return 1;
    }
    return 0;
}

int fpt_cuda_certified_steps(const struct FptRenderConfig *config, const struct FptCudaSceneExt *ext, uint32_t stride, float margin,
                             const float *sun_direction, uint32_t *counts, size_t counts_len, char *error, size_t error_len) {
    if (!config || !sun_direction || !counts || stride == 0 || config->width == 0 || config->height == 0) {
        set_error(error, error_len, "missing certified-step input");
        return 1;
    }
    const size_t samples = size_t((config->width + stride - 1) / stride) * ((config->height + stride - 1) / stride);
    if (counts_len < samples * 6) { set_error(error, error_len, "counts buffer too small (%zu < %zu)", counts_len, samples * 6); return 1; }
    const float sl = std::sqrt(sun_direction[0] * sun_direction[0] + sun_direction[1] * sun_direction[1] +
                               sun_direction[2] * sun_direction[2]);
    if (!(sl > 0.0f)) { set_error(error, error_len, "sun direction must be non-zero"); return 1; }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    DeviceScene S;
    if (!compile_scene(*config, ext, S, error, error_len)) return 1;
    S.surrogate = 0;   // the plain march's rules; no model is needed
    if (!upload_scene(S, nullptr, error, error_len)) return 1;
    if (!ensure_buffer((void **)&c.samples, &c.cap_samples, samples * 6 * sizeof(uint32_t), error, error_len)) return 1;
    uint32_t *dev = reinterpret_cast<uint32_t *>(c.samples);
    const float3 sun = make_float3(sun_direction[0] / sl, sun_direction[1] / sl, sun_direction[2] / sl);
    if (!check(launch_certified_steps(S.kind, c.scene, uint32_t(samples), stride, margin, sun, dev, c.stream), "certified-step launch",
               error, error_len) ||
        !check(cudaMemcpyAsync(counts, dev, samples * 6 * sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream), "readback", error,
               error_len) ||
        !check(cudaStreamSynchronize(c.stream), "certified-step bound", error, error_len))
        return 1;
    return 0;
}

int fpt_cuda_measure_fp32_peak(double *tflops, double *launch_ms, char *error, size_t error_len) {
    if (tflops) *tflops = 0.0;
    if (launch_ms) *launch_ms = 0.0;
    if (!tflops) { set_error(error, error_len, "missing output"); return 1; }
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(error, error_len)) return 1;
    Context &c = ctx();
    if (!ensure_buffer((void **)&c.counter, &c.cap_counter, 64, error, error_len)) return 1;
    int sms = 0;
    if (!check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device), "SM count", error, error_len)) return 1;
    const uint32_t blocks = uint32_t(sms) * 8u, threads = 256u, trips = 1024u;   // 2048 threads per SM
    const double flop = double(blocks) * threads * trips * 32.0 * 8.0 * 2.0;
    float best = 1e30f;
    for (int it = 0; it < 8; ++it) {
        cudaEventRecord(c.ev0, c.stream);
        fma_peak_kernel<<<blocks, threads, 0, c.stream>>>(reinterpret_cast<float *>(c.counter), trips, 0.99999f, 1.0e-6f);
        cudaEventRecord(c.ev1, c.stream);
        if (!check(cudaEventSynchronize(c.ev1), "FP32 peak kernel", error, error_len)) return 1;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, c.ev0, c.ev1);
        if (it >= 2) best = std::min(best, ms);   // two warm-up launches
    }
    if (!check(cudaGetLastError(), "FP32 peak launch", error, error_len)) return 1;
    *tflops = flop / (double(best) * 1e-3) / 1e12;
    if (launch_ms) *launch_ms = best;
    return 0;
}

int fpt_cuda_hdri_lut(const char *hdri_path, uint16_t *lut, size_t lut_len, char *error, size_t error_len) {
    const size_t n = size_t(FPT_HDRI_LUT_WIDTH) * FPT_HDRI_LUT_HEIGHT * 3;
    if (!hdri_path || !lut || lut_len < n) { set_error(error, error_len, "missing HDRI path or LUT buffer (%zu halves)", n); return 1; }
    const size_t len = std::strlen(hdri_path);
    FptRenderConfig *cfg = new (std::nothrow) FptRenderConfig();
    if (!cfg) { set_error(error, error_len, "out of host memory"); return 1; }
    if (len >= sizeof(cfg->hdri_path)) {
        delete cfg;
        set_error(error, error_len, "HDRI path longer than %zu bytes", sizeof(cfg->hdri_path) - 1);
        return 1;
    }
    std::memcpy(cfg->hdri_path, hdri_path, len + 1);
    cfg->hdri_enabled = 1u;
    cfg->world[0] = 2.0f;
    const bool ok = hydrate_hdri(*cfg, error, error_len);
    if (ok) std::memcpy(lut, cfg->hdri_lut, n * sizeof(uint16_t));
    delete cfg;
    return ok ? 0 : 1;
}

int fpt_cuda_set_device(int32_t ordinal) {
    if (ordinal < 0) return 1;
    std::lock_guard<std::mutex> lock(ctx().mutex);
    Context &c = ctx();
    if (c.ready) return ordinal == c.device ? 0 : 1;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || ordinal >= count) return 1;
    c.device = ordinal;
    return 0;
}

int fpt_cuda_get_device(int32_t *ordinal) {
    if (!ordinal) return 1;
    std::lock_guard<std::mutex> lock(ctx().mutex);
    if (!ensure_device(nullptr, 0)) { *ordinal = -1; return 1; }
    *ordinal = ctx().device;
    return 0;
}

int fpt_cuda_set_launch_shape(uint32_t wave_paths, int32_t march_blocks) {
    std::lock_guard<std::mutex> lock(ctx().mutex);
    ctx().wave_paths = wave_paths;
    ctx().march_blocks = march_blocks;
    return 0;
}

int fpt_cuda_set_march_schedule(uint32_t schedule, uint32_t batch) {
    if (schedule != 0u || batch > 32u) return 1;
    std::lock_guard<std::mutex> lock(ctx().mutex);
    ctx().refill_batch = batch;
    return 0;
}

int fpt_cuda_set_loop_limit(uint64_t limit_ns) {
    std::lock_guard<std::mutex> lock(ctx().mutex);
    ctx().loop_limit_ns = limit_ns;
    return 0;
}

int fpt_cuda_set_kernel_timing(uint32_t on) {
    if (on > 1u) return 1;
    std::lock_guard<std::mutex> lock(ctx().mutex);
    ctx().kernel_timing = on;
    return 0;
}

int fpt_cuda_set_network_engine(uint32_t engine) {
    if (engine > FPT_CUDA_NET_MMA_SYNC) return 1;
    std::lock_guard<std::mutex> lock(ctx().mutex);
    ctx().network_engine = engine;
    return 0;
}

}  // extern "C"

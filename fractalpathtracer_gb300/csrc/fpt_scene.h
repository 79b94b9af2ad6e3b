// fpt_scene.h -- the device-side scene block.
//
// The host compiles one FptRenderConfig (+ optional FptCudaSceneExt) into a
// DeviceScene: the same parameters, with the per-call constants of the
// reference (camera and light rotations, focal length, Mandelbox factors)
// evaluated once on the host, and the scene kind resolved so kernels can be
// specialised on it.  Kernels read it from global memory (a warp reads the
// same addresses, so the loads broadcast from L1).
#pragma once

#include <stdint.h>
#include "../../include/fpt_cuda.h"

namespace fpt {

enum SceneKind : uint32_t {
    KIND_GENERIC = 0,   // reference scenes, typed programs, anything else: runtime dispatch
    KIND_BULB8 = 1,     // Mandelbulb power 8 (algebraic form)
    KIND_BULB = 2,      // Mandelbulb, any power (trigonometric form)
    KIND_BOX = 3,       // Mandelbox (Mandelbulber full fold)
    KIND_MENGER = 4,    // Menger fold
    KIND_HYBRID = 5,    // Mandelbulb / Menger hybrid schedule
    KIND_COUNT = 6,
    KIND_EXT = 6,       // runtime dispatch over the extension formulas only (batched scenes)
};

// Kinds that pick the formula at run time from DeviceScene::kind.
#ifdef __CUDACC__
__host__ __device__
#endif
constexpr bool runtime_kind(int k) { return k == KIND_GENERIC || k == KIND_EXT; }

struct DeviceScene {
    // --- identity
    uint32_t sdf_id;
    uint32_t formula;          // FPT_CUDA_FORMULA_* (0 = reference scene)
    uint32_t kind;             // SceneKind
    uint32_t width, height, samples;
    uint32_t bounces;          // min(render[0], 8, bounce cap)
    uint32_t russian_roulette;
    float rr_start, rr_min_prob;
    uint32_t normal_mode;      // config sdf_normal_mode
    uint32_t ext_normal;       // FPT_CUDA_NORMAL_*
    uint32_t translucent;      // march checks translucency (glass scenes)

    // --- render / camera
    float render[8];
    float cam_pos[3];
    float yaw, pitch, roll;
    float focal;               // 1 / tan(fov/2)
    float aa_strength;         // 0.3 / max(W, H)
    float camera_fov;          // degrees (Mandelbulber projections)
    float camera_dof;
    float focus_distance;      // resolved (> 0) before the render kernels run
    float inv_wh[2];           // unused by the exact uv path; kept for diagnostics

    // --- world / sun / post
    float world[7];
    float world_one_color[3];
    float env_light_dir[3];    // rotateCamera((0,0,1), world[2..3]) precomputed
    float world_cos_size;      // cos(max(world[1], 1e-4))
    float sun[5];
    float sun_color[3];
    float sun_dir[3];          // rotateCamera((0,0,1), sun[1..2]) or ext direction
    float sun_power;
    float background_gradient[6];
    float post[7];

    // --- fractal parameters
    float set_values[40];
    float vset_values[133];
    uint32_t material_mode, gradient_count, fractal_style_mode;
    float fractal_style[12];
    float program_material[8];
    float gradient_stops[16][4];
    float box_ref[8];          // deMandelbox constants: scale.xyz, scale.w, minRad2, absScalem1, AbsScale, pad
    float ifs_rot[9];          // deIFS rotation sin/cos (sxy cxy syz cyz sxz cxz) + pad
    float global_rot[6];       // Mandelbulber global rotation sin/cos (x, y, z)
    uint32_t global_identity;  // 1 when the Mandelbulber global transform is a pure swizzle
    float mb_rot[6];           // Mandelbulber IFS rotation3 sin/cos

    // --- extension formula
    uint32_t iterations;
    float bailout;
    float power;
    float box_scale, box_fixed2, box_min2, box_min_factor, box_fold_limit, box_fold_value;
    float menger_scale;
    uint32_t hybrid_period;
    uint32_t ground_plane;
    float plane_height;
    uint32_t rng, seed, brdf;
    float albedo, ggx_alpha, specular_f0, plane_albedo;
    uint32_t sky_width, sky_height;
    const float *sky_rgb;      // device pointer
    uint32_t fp64_bisection;
    uint32_t surrogate;
    float surrogate_margin, surrogate_safety;
    uint32_t surrogate_max_iters;
    const void *surrogate_weights;  // device pointer to the packed MLP

    // --- HDRI LUT (reference world mode 2)
    uint32_t hdri_enabled, hdri_width, hdri_height;
    uint16_t hdri_lut[32 * 16 * 3];

    // --- typed programs
    uint32_t program_count, shading_count;
    // Typed program lowered to flat arrays (sdf_typed_soa; the lowering is the
    // host's, src/scene.rs:1211-1531): spheres, boxes and planes in one union.
    uint32_t soa_count;            // 0: not lowered
    FptTypedSoAProgram soa;
    FptSdfInstruction program[FPT_SDF_PROGRAM_MAX_OPS];
    FptSdfInstruction shading[FPT_SDF_PROGRAM_MAX_OPS];
};

}  // namespace fpt

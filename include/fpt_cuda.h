/*
 * fpt_cuda.h -- C ABI of the GB300 (sm_103a) sphere-tracing path.
 *
 * This header is the drop-in seam for FPT Metal's bridge.  The first block
 * declares the structs and entry points of the reference interface with the
 * same names, member order and sizes (reference: src/metal_bridge.h:1-490,
 * mirrored in Rust by src/ffi.rs:89-488, sizes pinned by src/ffi.rs:494-507),
 * so a Rust build that links libfpt_cuda.so instead of fpt_metal_bridge keeps
 * its `extern "C"` declarations unchanged.  The second block declares the
 * side entry points this library adds for per-ray output, voxel bricks, DDA
 * cell sequences, batched scenes and the learned distance surrogate.
 *
 * Conventions shared by every entry point (reference: src/metal_bridge.mm:41-47,
 * 4322-4361):
 *   - return 0 on success, 1 on failure;
 *   - on failure a NUL-terminated message is written into error[0..error_len);
 *   - out-parameters are zeroed on entry;
 *   - every pointer is owned by the caller and is not retained after return;
 *   - calls are synchronous and must be serialised by the caller (one call in
 *     flight per process), as the reference's Rust side does with a mutex.
 */
#ifndef FPT_CUDA_H
#define FPT_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------- */
/* Reference interface (src/metal_bridge.h)                                  */
/* ------------------------------------------------------------------------- */

/* Scene selector values of FptRenderConfig.sdf_id (src/metal_bridge.h:10-24). */
typedef enum FptSdfId {
    FPT_SDF_CORNELL_BOX = 0,
    FPT_SDF_GLASS_BALL = 1,
    FPT_SDF_BALL_FRACTAL = 2,
    FPT_SDF_CAGE_FRACTAL = 3,
    FPT_SDF_IFS_FRACTAL = 4,
    FPT_SDF_MANDELBOX_FRACTAL = 5,
    FPT_SDF_MENGER_SPONGE = 6,
    FPT_SDF_TOWER_FRACTAL = 7,
    FPT_SDF_TREE_FRACTAL = 8,
    FPT_SDF_PROGRAM = 9,
    FPT_SDF_README_CORNELL = 10,
    FPT_SDF_README_GLASS = 11,
    FPT_SDF_MANDELBULBER = 12,
} FptSdfId;

enum {
    FPT_SDF_PROGRAM_MAX_OPS = 64,
    FPT_SDF_FLAT_UNION_MAX_PRIMITIVES = 64,
    FPT_SDF_GRADIENT_MAX_STOPS = 16,
    FPT_HDRI_PATH_CAPACITY = 256,
    FPT_HDRI_LUT_WIDTH = 32,
    FPT_HDRI_LUT_HEIGHT = 16,
};

enum {
    FPT_SDF_STITCH_STATE_FULL = 0,
    FPT_SDF_STITCH_STATE_LEAN = 1,
};

/* Typed SDF program opcodes (src/metal_bridge.h:40-56). */
typedef enum FptSdfOpcode {
    FPT_SDF_OP_ABS = 1,
    FPT_SDF_OP_TRANSLATE = 2,
    FPT_SDF_OP_SCALE = 3,
    FPT_SDF_OP_ROTATE_X = 4,
    FPT_SDF_OP_ROTATE_Y = 5,
    FPT_SDF_OP_ROTATE_Z = 6,
    FPT_SDF_OP_REPEAT = 7,
    FPT_SDF_OP_SORT_DESC = 8,
    FPT_SDF_OP_SPHERE = 16,
    FPT_SDF_OP_BOX = 17,
    FPT_SDF_OP_PLANE = 18,
    FPT_SDF_OP_UNION = 24,
    FPT_SDF_OP_INTERSECTION = 25,
    FPT_SDF_OP_SUBTRACT = 26,
    FPT_SDF_OP_ORBIT_ADD = 32,
} FptSdfOpcode;

/* One typed-program instruction, 32 bytes (src/metal_bridge.h:58-64). */
struct FptSdfInstruction {
    uint32_t opcode;
    uint32_t flags;          /* combine mode: 0 union, 1 intersection, 2 subtract */
    uint32_t material_index;
    uint32_t _pad0;
    float data[4];
};

struct FptPrimitiveInstance {
    float transform[12];
    float data[4];
    uint32_t opcode;
    float distance_scale;
    uint32_t source_instruction;
    uint32_t _pad0;
};

struct FptAffineTransform {
    float transform[12];
    float distance_scale;
    uint32_t _pad0[3];
};

struct FptIndexedPrimitive {
    float data[4];
    uint32_t opcode;
    uint32_t transform_index;
    uint32_t source_instruction;
    uint32_t combine_mode;
};

struct FptTypedSoAProgram {
    uint32_t sphere_count;
    uint32_t box_count;
    uint32_t plane_count;
    uint32_t _pad0;
    float sphere_x[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float sphere_y[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float sphere_z[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float sphere_radius[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    uint32_t sphere_source[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float box_x[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float box_y[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float box_z[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float box_half_x[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float box_half_y[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float box_half_z[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    uint32_t box_source[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float plane_x[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float plane_y[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float plane_z[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float plane_center_x[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float plane_center_y[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float plane_center_z[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    float plane_offset[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    uint32_t plane_source[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
};

typedef enum FptSdfAccumulationMode {
    FPT_SDF_ACCUMULATION_AUTO = 0,
    FPT_SDF_ACCUMULATION_PER_SAMPLE = 1,
    FPT_SDF_ACCUMULATION_BATCH = 2,
    FPT_SDF_ACCUMULATION_CHUNKED = 3,
} FptSdfAccumulationMode;

typedef enum FptRendererBackend {
    FPT_RENDERER_SDF = 0,
    FPT_RENDERER_VOXEL = 1,
    FPT_RENDERER_BOUND_GRID = 2,
    FPT_RENDERER_REGIONAL = 3,
} FptRendererBackend;

typedef enum FptVoxelNormalMode {
    FPT_VOXEL_NORMAL_FACE = 0,
    FPT_VOXEL_NORMAL_SMOOTH = 1,
    FPT_VOXEL_NORMAL_EXACT = 2,
} FptVoxelNormalMode;

typedef enum FptVoxelMaterialMode {
    FPT_VOXEL_MATERIAL_STORED = 0,
    FPT_VOXEL_MATERIAL_EXACT = 1,
} FptVoxelMaterialMode;

typedef enum FptVoxelOffsetMode {
    FPT_VOXEL_OFFSET_LEGACY = 0,
    FPT_VOXEL_OFFSET_PRECISION = 1,
} FptVoxelOffsetMode;

typedef enum FptVoxelStorage {
    FPT_VOXEL_STORAGE_DENSE = 0,
    FPT_VOXEL_STORAGE_SPARSE_BRICKS = 1,
    FPT_VOXEL_STORAGE_TEMPLATE_BRICKS = 3,
} FptVoxelStorage;

typedef enum FptVoxelCoverageMode {
    FPT_VOXEL_COVERAGE_LEGACY = 0,
    FPT_VOXEL_COVERAGE_LIPSCHITZ = 1,
    FPT_VOXEL_COVERAGE_INTERVAL = 2,
} FptVoxelCoverageMode;

typedef enum FptVoxelBuildMode {
    FPT_VOXEL_BUILD_STAGING = 0,
    FPT_VOXEL_BUILD_DIRECT = 1,
} FptVoxelBuildMode;

typedef enum FptVoxelLeafRefinement {
    FPT_VOXEL_LEAF_REFINEMENT_NONE = 0,
    FPT_VOXEL_LEAF_REFINEMENT_SECANT_BISECTION = 1,
    FPT_VOXEL_LEAF_REFINEMENT_RESTRICTED_TRACE = 2,
    FPT_VOXEL_LEAF_REFINEMENT_FIXED_DE = 3,
} FptVoxelLeafRefinement;

/* Whole-render parameter block, 30448 bytes (src/metal_bridge.h:170-267;
 * size asserted at src/metal_bridge.mm:36).  Member meaning follows the
 * reference: render[0] bounces, render[1] march steps, render[2] normal
 * epsilon, render[3] minimum distance, render[4] maximum distance,
 * render[5] fog-LOD mix, render[6] distance halving, render[7] slow-shading
 * stencil; world/sun/post as in src/scene.rs:743-778. */
struct FptRenderConfig {
    uint32_t width;
    uint32_t height;
    uint32_t samples;
    uint32_t preview;
    uint32_t sdf_id;
    uint32_t glass_mode;
    uint32_t sdf_accumulation_mode;
    uint32_t sdf_profile;
    uint32_t sdf_bounce_cap;
    uint32_t sdf_russian_roulette;
    uint32_t sdf_normal_mode;
    uint32_t sdf_chunk_samples;
    float sdf_rr_start;
    float sdf_rr_min_prob;
    float mandel_iteration_scale;

    float camera_position[3];
    float camera_yaw_pitch[2];
    float camera_roll;
    float camera_fov;
    float camera_dof;
    float focus_distance;

    float render[8];
    float world[7];
    float world_one_color[3];
    float sun[5];
    float sun_color[3];
    float background_gradient[6];
    float post[7];
    float set_values[40];
    float vset_values[133];

    uint32_t sdf_program_count;
    uint32_t gradient_count;
    uint32_t material_mode;
    uint32_t hdri_enabled;
    uint32_t hdri_width;
    uint32_t hdri_height;
    uint32_t _pad_hdri[2];
    uint32_t fractal_style_mode;
    uint32_t _pad_style[3];
    float fractal_style[12];
    float program_material[8];
    struct FptSdfInstruction sdf_program[FPT_SDF_PROGRAM_MAX_OPS];
    float gradient_stops[FPT_SDF_GRADIENT_MAX_STOPS][4];
    uint8_t hdri_path[FPT_HDRI_PATH_CAPACITY];
    uint16_t hdri_lut[FPT_HDRI_LUT_WIDTH * FPT_HDRI_LUT_HEIGHT * 3];
    uint32_t renderer_backend;
    uint32_t voxel_resolution;
    uint32_t voxel_normal_mode;
    uint32_t voxel_storage;
    float voxel_bounds_min[3];
    float voxel_surface_band;
    float voxel_bounds_max[3];
    uint32_t voxel_fill_interior;
    uint32_t voxel_coverage_mode;
    uint32_t voxel_build_mode;
    uint32_t voxel_brick_rejection;
    uint32_t voxel_leaf_refinement;
    uint32_t voxel_material_mode;
    uint32_t voxel_offset_mode;
    uint32_t bound_grid_resolution;
    uint32_t bound_grid_profile;
    uint32_t bound_grid_profile_stride;
    uint32_t bound_grid_cage_bounds;
    uint32_t bound_grid_directional;
    uint32_t sdf_program_source_count;
    uint32_t sdf_program_optimization;
    uint32_t regional_program_resolution;
    uint32_t bound_grid_fp16;
    uint32_t sdf_flat_union_count;
    struct FptPrimitiveInstance sdf_flat_union_instances[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    uint32_t sdf_shading_program_count;
    uint32_t sdf_geometry_split;
    struct FptSdfInstruction sdf_shading_program[FPT_SDF_PROGRAM_MAX_OPS];
    uint32_t sdf_topology_specialization;
    uint32_t sdf_runtime_source_bytecode;
    uint32_t sdf_function_stitching;
    uint32_t sdf_stitched_surface;
    uint32_t sdf_stitch_validation;
    uint32_t sdf_stitch_distance_only;
    uint32_t sdf_stitch_split_graph;
    uint32_t sdf_stitch_fusion;
    uint32_t sdf_canonical_count;
    uint32_t sdf_canonical_source_count;
    struct FptPrimitiveInstance sdf_canonical_primitives[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    uint32_t sdf_canonical_transform_count;
    uint32_t _pad_canonical_indexed[3];
    struct FptAffineTransform sdf_canonical_transforms[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    struct FptIndexedPrimitive sdf_indexed_primitives[FPT_SDF_FLAT_UNION_MAX_PRIMITIVES];
    struct FptTypedSoAProgram sdf_typed_soa;
};

struct FptBoundGridStats {
    uint64_t macro_cells[3];
    uint64_t certified_skips[3];
    uint64_t candidate_intervals[3];
    uint64_t candidate_misses[3];
    uint64_t candidate_hits[3];
    uint64_t unknown_intervals[3];
    uint64_t field_evaluations[3];
    uint64_t directional_steps[3];
    uint64_t cell_exit_clamps[3];
    uint64_t unknown_derivative_intervals[3];
    uint64_t profiled_paths;
    uint64_t certified_cells;
    uint64_t unknown_cells;
    uint64_t sampled_bound_failures;
    uint64_t sampled_false_skips;
    uint64_t certified_derivative_cells;
    uint64_t unknown_derivative_cells;
    uint64_t sampled_derivative_failures;
    uint64_t regional_cells;
    uint64_t regional_fallback_cells;
    uint64_t regional_unique_programs;
    uint64_t regional_retained_instructions;
    uint64_t regional_sampled_distance_failures;
    uint64_t regional_profiled_paths;
    uint64_t regional_distance_evaluations[3];
    uint64_t regional_atlas_evaluations[3];
    uint64_t regional_full_program_evaluations[3];
    uint64_t regional_cell_entries[3];
    uint64_t regional_same_cell_reuses[3];
    uint64_t regional_same_program_reuses[3];
    uint64_t regional_program_id_loads[3];
    uint64_t regional_header_loads[3];
    uint64_t regional_dynamic_instructions[3];
    uint64_t regional_pruned_cells;
    uint64_t regional_pruned_primitives;
    uint64_t regional_repeat_seam_fallback_cells;
    uint64_t regional_unsupported_fallback_cells;
    uint64_t regional_no_dominance_cells;
};

struct FptStitchValidationStats {
    uint64_t sample_count;
    uint64_t distance_failures;
    uint64_t gradient_failures;
    float max_distance_error;
    float max_gradient_error;
};

struct FptStitchPipelineStats {
    uint32_t instruction_count;
    uint32_t transform_instruction_count;
    uint32_t primitive_instruction_count;
    uint32_t primitive_type_runs;
    uint32_t union_count;
    uint32_t intersection_count;
    uint32_t subtraction_count;
    uint32_t thread_execution_width;
    uint32_t max_total_threads_per_threadgroup;
    uint32_t graph_node_count;
    uint64_t static_threadgroup_memory_bytes;
    uint64_t runtime_source_bytes;
    double runtime_library_compile_ms;
    double runtime_pipeline_link_ms;
};

struct FptSdfProfileStats {
    uint64_t primary_steps;
    uint64_t secondary_steps;
    uint64_t shadow_steps;
    uint64_t normal_evals;
    uint64_t bounces;
    uint64_t pixels;
    uint64_t distance_evals;
    uint64_t march_orbit_iterations;
    uint64_t refinement_steps;
    uint64_t normal_field_evals;
    uint64_t material_evals;
    uint64_t max_ray_steps;
    uint64_t max_pixel_steps;
    uint64_t distance_evals_by_phase[4];
    uint64_t orbit_iterations_by_phase[4];
    uint64_t formula_slot_iterations[9];
    uint64_t refinement_distance_evals;
    double primary_ms_estimate;
    double secondary_ms_estimate;
    double shadow_ms_estimate;
    double normal_ms_estimate;
    double bounce_ms_estimate;
};

struct FptAsyncJitStats {
    double fallback_render_ms;
    double jit_build_ms;
    double stitched_render_ms;
    uint32_t cache_status;
    uint32_t fallback_completed_before_jit;
    float max_absolute_error;
    uint32_t _pad0;
};

typedef enum FptDiagnosticMode {
    FPT_DIAGNOSTIC_DEPTH = 0,
    FPT_DIAGNOSTIC_NORMAL = 1,
    FPT_DIAGNOSTIC_MATERIAL = 2,
    FPT_DIAGNOSTIC_HIT_MASK = 3,
    FPT_DIAGNOSTIC_PATH_DIRECT = 4,
    FPT_DIAGNOSTIC_PATH_ENVIRONMENT = 5,
    FPT_DIAGNOSTIC_PATH_THROUGHPUT = 6,
    FPT_DIAGNOSTIC_PATH_FINAL = 7,
    FPT_DIAGNOSTIC_DIFFUSE_NORMAL = 8,
    FPT_DIAGNOSTIC_MANDEL_COLOR_INDEX = 9,
    FPT_DIAGNOSTIC_MANDEL_PALETTE_POSITION = 10,
    FPT_DIAGNOSTIC_SDF_PRIMARY_STEPS = 11,
    FPT_DIAGNOSTIC_SDF_SHADOW_STEPS = 12,
    FPT_DIAGNOSTIC_SDF_NORMAL_EVALS = 13,
    FPT_DIAGNOSTIC_SDF_BOUNCES = 14,
    FPT_DIAGNOSTIC_SDF_BOUNCE_CONTRIBUTION = 15,
} FptDiagnosticMode;

struct FptDiagnosticConfig {
    uint32_t mode;
    uint32_t _pad0;
    float max_distance;
    float normal_mix;
    uint32_t dispatch_origin[2];
};

struct FptMandelbulberFieldSample {
    float distance;
    float radius;
    float derivative;
    float iterations;
};

/* Replaces fpt_metal_render (src/metal_bridge.h:404-425; implementation
 * src/metal_bridge.mm:4298-5863).  metallib_path, stitch_metallib_path,
 * stitch_archive_path and shader_source are accepted and ignored (there is
 * no Metal library to load); research statistics the CUDA path does not
 * produce (bound-grid, stitch) are zero-filled.  Writes the presented 8-bit
 * image as PNG to output_path (when non-NULL) and, when linear_output is
 * non-NULL, the width*height*4 float accumulation buffer. */
int fpt_metal_render(const char *metallib_path,
                     const char *stitch_metallib_path,
                     const char *stitch_archive_path,
                     const char *output_path,
                     const char *shader_source,
                     size_t shader_source_len,
                     const struct FptRenderConfig *config,
                     double *build_ms,
                     double *elapsed_ms,
                     uint64_t *voxel_memory_bytes,
                     uint32_t *voxel_active_bricks,
                     uint64_t *voxel_active_cells,
                     uint32_t *voxel_rejected_bricks,
                     struct FptBoundGridStats *bound_grid_stats,
                     uint32_t *stitch_cache_status,
                     struct FptStitchValidationStats *stitch_validation_stats,
                     struct FptStitchPipelineStats *stitch_pipeline_stats,
                     struct FptSdfProfileStats *sdf_profile_stats,
                     float *linear_output,
                     size_t linear_output_len,
                     char *error,
                     size_t error_len);

/* Replaces fpt_metal_diagnostic_render (src/metal_bridge.h:427-435;
 * src/metal_bridge.mm:5865-6025).  Supported modes: depth, normal,
 * hit mask, primary steps. */
int fpt_metal_diagnostic_render(const char *metallib_path,
                                const char *output_path,
                                const char *shader_source,
                                size_t shader_source_len,
                                const struct FptRenderConfig *config,
                                const struct FptDiagnosticConfig *diagnostic,
                                double *elapsed_ms,
                                char *error,
                                size_t error_len);

/* Replaces fpt_mandelbulber_sample_field (src/metal_bridge.h:437-446;
 * src/metal_bridge.mm:4205-4296; kernel shaders/Shaders.metal:1001-1009):
 * point_count xyzw points in, one {distance, radius, derivative, |iterations|}
 * per point out. */
int fpt_mandelbulber_sample_field(const char *metallib_path,
                                  const char *shader_source,
                                  size_t shader_source_len,
                                  const struct FptRenderConfig *config,
                                  const float *points_xyzw,
                                  size_t point_count,
                                  struct FptMandelbulberFieldSample *samples,
                                  char *error,
                                  size_t error_len);

/* Host-only PNG comparison (src/metal_bridge.h:448-452;
 * src/metal_bridge.mm:6062-6145): MAE, RMSE, 8x8 luminance SSIM,
 * 64x64 low-frequency SSIM, written as JSON to report_path. */
int fpt_compare_images(const char *baseline_path,
                       const char *candidate_path,
                       const char *report_path,
                       char *error,
                       size_t error_len);

/* src/metal_bridge.h:454: device name, or returns 1 without a device. */
int fpt_metal_device_name(char *name, size_t name_len);

/* src/metal_bridge.h:456-458 (src/metal_bridge.mm:3715-3926): runs the
 * voxel DDA / AABB / cell-ownership contract cases on the GPU and a 32^3
 * sphere build both ways; 0 when every case holds. */
int fpt_test_voxel_dda(const char *metallib_path, char *error, size_t error_len);

/* src/metal_bridge.h:460-467: research JIT path; always returns 1 with
 * "unsupported" (there is no runtime shader compiler here). */
int fpt_test_async_stitch_context(const char *metallib_path,
                                  const char *stitch_metallib_path,
                                  const char *stitch_archive_path,
                                  const struct FptRenderConfig *config,
                                  struct FptAsyncJitStats *stats,
                                  char *error,
                                  size_t error_len);

/* src/metal_bridge.h:469-474: field + gradient parity of the typed-program
 * evaluator over 2^20 hash-seeded points (tolerances 2e-5*(1+|d|) and 1e-4,
 * shaders/Shaders.metal:5106-5154). */
int fpt_test_typed_soa(const char *metallib_path,
                       const struct FptRenderConfig *config,
                       struct FptStitchValidationStats *stats,
                       char *error,
                       size_t error_len);

/* src/metal_bridge.h:476-486: interactive window; always returns 1 with
 * "unsupported" (no window system on a headless GPU node). */
int fpt_metal_preview(const char *metallib_path,
                      const char *stitch_metallib_path,
                      const char *const *stitch_archive_paths,
                      const char *shader_source,
                      size_t shader_source_len,
                      const struct FptRenderConfig *config,
                      const struct FptRenderConfig *scene_configs,
                      uint32_t scene_config_count,
                      uint32_t scene_config_index,
                      char *error,
                      size_t error_len);

/* ------------------------------------------------------------------------- */
/* Side entry points added by this library                                   */
/* ------------------------------------------------------------------------- */

/* Formula selected by FptCudaSceneExt.formula.  0 keeps the reference
 * scene of FptRenderConfig.sdf_id.  2, 3 and 8 follow Mandelbulber's formula
 * numbering (src/mandelbulber.rs:1414-1425) and the FP64 orbit code of
 * src/mandelbulber/orbit.rs (mandelbulb 766-778, quadratic triplex
 * "mandelbulb power 2" 752-764, mandelbox 1636-1693, finalizers 638-683). */
enum {
    FPT_CUDA_FORMULA_REFERENCE = 0,
    FPT_CUDA_FORMULA_MANDELBULB = 2,
    FPT_CUDA_FORMULA_MANDELBULB_POWER2 = 3,
    FPT_CUDA_FORMULA_MANDELBOX = 8,
    FPT_CUDA_FORMULA_MENGER_FOLD = 100,
    FPT_CUDA_FORMULA_BULB_MENGER_HYBRID = 101,
};

enum { FPT_CUDA_RNG_HASH13 = 0, FPT_CUDA_RNG_PCG = 1 };
enum { FPT_CUDA_BRDF_REFERENCE = 0, FPT_CUDA_BRDF_LAMBERT_GGX = 1 };
enum { FPT_CUDA_NORMAL_CONFIG = 0, FPT_CUDA_NORMAL_ANALYTIC = 1 };
/* SKIP: learned step proposals certified by the exact DE, plus the model's
 * box (rays are clipped to it; leaving it is a miss).  BOX: the box alone,
 * no network (the same march without the learned part). */
enum { FPT_CUDA_SURROGATE_OFF = 0, FPT_CUDA_SURROGATE_SKIP = 1, FPT_CUDA_SURROGATE_BOX = 2 };

/* Scene features beyond FptRenderConfig.  A zero-initialised struct (or a
 * NULL pointer) means the reference's semantics exactly. */
struct FptCudaSceneExt {
    uint32_t formula;            /* FPT_CUDA_FORMULA_* */
    uint32_t iterations;         /* formula iterations (0: set_values[1] for Mandelbulber scenes) */
    float bailout;               /* escape radius (0: set_values[2]) */
    float power;                 /* Mandelbulb power */
    float box_scale;             /* Mandelbox scale */
    float box_min_radius;        /* Mandelbox minimum radius */
    float box_fixed_radius;      /* Mandelbox fixed radius */
    float box_fold_limit;        /* Mandelbox folding limit */
    float box_fold_value;        /* Mandelbox folding value */
    float menger_scale;          /* Menger fold scale */
    uint32_t menger_iterations;  /* Menger fold iterations (hybrid: Menger slot every (period) steps) */
    uint32_t hybrid_period;      /* hybrid schedule: bulb iterations per Menger iteration + 1 */
    uint32_t ground_plane;       /* 1: union with the plane y = plane_height */
    float plane_height;
    uint32_t rng;                /* FPT_CUDA_RNG_* */
    uint32_t seed;
    uint32_t brdf;               /* FPT_CUDA_BRDF_* */
    float albedo;                /* Lambert albedo of the fractal */
    float ggx_alpha;             /* GGX roughness (alpha) of the fractal's specular lobe */
    float specular_f0;           /* Schlick F0 of that lobe */
    float plane_albedo;          /* Lambert albedo of the ground plane */
    uint32_t normal_mode;        /* FPT_CUDA_NORMAL_* */
    uint32_t sky_width;          /* equirect sky (RGB float, row 0 = +y pole); 0 = none */
    uint32_t sky_height;
    const float *sky_rgb;        /* host pointer, sky_width*sky_height*3 floats */
    float sun_direction[3];      /* used with the equirect sky for sun NEE */
    float sun_intensity;
    uint32_t fp64_bisection;     /* 1: FP64 bisection at representable-position stops */
    uint32_t surrogate;          /* FPT_CUDA_SURROGATE_* (needs a trained model) */
    uint64_t surrogate_model;    /* handle from fpt_cuda_mlp_create */
    float surrogate_margin;      /* exact-DE hand-over distance for surrogate skips (0: 0.1) */
    float surrogate_safety;      /* step = safety * surrogate distance */
    uint32_t surrogate_max_iters;/* skip iterations per ray before the exact march takes over (0: 64) */
    uint32_t _reserved[7];
};

/* Per-primary-ray output of fpt_cuda_trace_primary. */
struct FptCudaPrimaryHit {
    float distance;     /* travel from the camera to the hit (or to the stop point) */
    float normal[3];    /* unit surface normal at the hit (0 on a miss) */
    uint32_t steps;     /* distance-estimator evaluations of the march */
    uint32_t hit;       /* 1 when the march converged on the surface */
};

/* Primary-ray march of every pixel (pixel-centre rays, no jitter, no DOF):
 * the camera ray of shaders/Shaders.metal:5926-5956 marched with
 * march / marchMandelbulber (3700-3783) and normalAt (3871-3971) or the
 * analytic-derivative normal.  hits has width*height entries, row-major,
 * row 0 at the bottom of the image (the accumulation layout). */
int fpt_cuda_trace_primary(const struct FptRenderConfig *config,
                           const struct FptCudaSceneExt *ext,
                           struct FptCudaPrimaryHit *hits,
                           size_t hit_count,
                           double *elapsed_ms,
                           char *error,
                           size_t error_len);

/* fpt_metal_render with a scene extension.  Same outputs; output_path may be
 * NULL (no PNG).  Russian roulette, accumulation mode and chunking follow
 * FptRenderConfig exactly. */
int fpt_cuda_render(const struct FptRenderConfig *config,
                    const struct FptCudaSceneExt *ext,
                    const char *output_path,
                    float *linear_output,
                    size_t linear_output_len,
                    uint8_t *rgba_output,
                    size_t rgba_output_len,
                    double *elapsed_ms,
                    struct FptSdfProfileStats *profile,
                    char *error,
                    size_t error_len);

/* Distance-estimator samples: xyz points (stride 4 floats) in, one
 * {distance, orbit, derivative, iterations} per point out, evaluated by the
 * scene's distance function (distanceSdf, shaders/Shaders.metal:3564-3610,
 * or the extension formula).  gradients (optional, 3 floats per point) gets
 * the analytic gradient when the scene has one. */
int fpt_cuda_sample_distance(const struct FptRenderConfig *config,
                             const struct FptCudaSceneExt *ext,
                             const float *points_xyzw,
                             size_t point_count,
                             float *samples,
                             float *gradients,
                             char *error,
                             size_t error_len);

/* Resident voxel grid built by fpt_cuda_voxel_build. */
struct FptCudaVoxelInfo {
    uint32_t resolution;
    uint32_t brick_size;      /* 8: occupancy bricks, 4: reference cells, 0: dense reference cells */
    uint32_t brick_grid;      /* bricks per axis */
    uint32_t active_bricks;
    uint64_t active_cells;
    uint64_t memory_bytes;    /* brick table + payload */
    double build_ms;
};

/* One traced voxel ray. */
struct FptCudaVoxelHit {
    float t;                  /* entry distance of the first occupied cell, -1 on a miss */
    uint32_t cell;            /* x + y*res + z*res^2 of that cell, 0xffffffff on a miss */
    uint32_t normal_axis;     /* face entered: 1 +x, 2 -x, 3 +y, 4 -y, 5 +z, 6 -z (0 = none) */
    uint32_t steps;           /* cells visited by the primary ray */
    uint32_t shadow_steps;    /* cells visited by the shadow ray */
    uint32_t lit;             /* 1 when the shadow ray escaped (sequence call: 1 on hit) */
};

/* Voxelizes the scene's distance estimator over FptRenderConfig's voxel
 * bounds and resolution and keeps the grid resident for the calls below
 * (classifier shaders/Shaders.metal:4196-4244, legacy coverage;
 * buildVoxelCell 5388-5414; brick ids in raster order as the host
 * compaction of src/metal_bridge.mm:1738-1812).  brick_size 8 builds
 * occupancy bricks (uint8 occupancy + fp16 distance per cell, uint32
 * brick table, 0 = empty else index + 1); 4 builds the reference's 4^3
 * bricks of 12-byte cells; 0 the reference's dense cells. */
int fpt_cuda_voxel_build(const struct FptRenderConfig *config,
                         const struct FptCudaSceneExt *ext,
                         uint32_t brick_size,
                         struct FptCudaVoxelInfo *info,
                         char *error,
                         size_t error_len);

/* Copies the resident grid to the host: brick table (brick_grid^3 words),
 * and per compact cell the occupancy bytes and fp16 distances (occupancy
 * bricks) or the 3-word reference cells. NULL skips an output. */
int fpt_cuda_voxel_read(uint32_t *brick_table,
                        size_t table_len,
                        uint8_t *occupancy,
                        uint16_t *distance,
                        uint32_t *cells,
                        size_t cell_len,
                        char *error,
                        size_t error_len);

/* Traces ray_count rays (origin xyz, direction xyz per ray) through the
 * resident grid with the exact DDA of traceVoxel (shaders/Shaders.metal:
 * 4492-4612) and records every visited cell (x + y*res + z*res^2), up to
 * `capacity` per ray; sequence_len gets the full visit count. */
int fpt_cuda_dda_sequence(const float *rays,
                          size_t ray_count,
                          uint32_t capacity,
                          uint32_t *sequence,
                          uint32_t *sequence_len,
                          struct FptCudaVoxelHit *hits,
                          char *error,
                          size_t error_len);

/* Primary ray per pixel centre plus one sun shadow ray per hit through the
 * resident occupancy-brick grid (legacy origin offset, shaders/Shaders.metal:
 * 4068-4089).  hits: width*height, row 0 at the bottom; rgba (optional):
 * shaded image, row 0 at the top. */
int fpt_cuda_voxel_render(const struct FptRenderConfig *config,
                          const struct FptCudaSceneExt *ext,
                          struct FptCudaVoxelHit *hits,
                          size_t hit_count,
                          uint8_t *rgba,
                          size_t rgba_len,
                          double *elapsed_ms,
                          char *error,
                          size_t error_len);

/* Occupancy-brick voxel build that allocates nothing.  No counterpart in
 * the reference: it serves callers that cannot allocate device memory --
 * an engine that owns all GPU memory through its own pool, or a frame loop
 * that cannot afford the implicit device synchronisation of cudaMalloc and
 * cudaFree.  The caller passes device buffers for the outputs (brick table,
 * occupancy bytes, fp16 distance bits) and a stream (NULL: the legacy
 * default stream); the results equal fpt_cuda_voxel_build with
 * brick_size 8.  Scratch lives in one fixed device array of about 2.1 MB
 * that every GPU loading the library holds until the process exits, so the
 * resolution is limited to 512.  The first call on a device looks up that
 * array's device address; make it before any stream capture.  The call is
 * synchronous and cannot be captured: it synchronises `stream` to read the
 * brick count back before the fill, and again at the end, and it returns 1
 * with an error when `stream` is capturing.  Every call shares the array:
 * calls that overlap on the GPU race. */
int fpt_cuda_voxel_build_static(const struct FptRenderConfig *config,
                                const struct FptCudaSceneExt *ext,
                                void *stream,
                                uint32_t *device_brick_table,
                                size_t table_len,
                                uint8_t *device_occupancy,
                                uint16_t *device_distance,
                                size_t cell_capacity,
                                struct FptCudaVoxelInfo *info,
                                char *error,
                                size_t error_len);

/* ---- Learned distance surrogate (no counterpart in the reference) ----
 * Network: 3-D point -> 99 Fourier features (the point normalised to the
 * box, sin/cos of pi 2^(6k/15) u for k < 16) -> 4 x 64 SiLU -> 1 distance;
 * BF16 weights and activations, FP32 accumulation, FP32 master copy.
 * Parameter layout (floats): W0[64][112] (columns 99..111 zero), b0[64],
 * W1[64][64], b1, W2, b2, W3, b3, W4[64], b4 -- 19777 values. */
struct FptCudaMlpConfig {
    float bounds_min[3];         /* box of the training points; all geometry must lie inside */
    float bounds_max[3];
    uint32_t points;             /* training points, labelled by the scene's exact DE */
    float near_fraction;         /* share drawn within near_band of the surface */
    float near_band;             /* world units (0: 0.05) */
    uint32_t batch;              /* rows per optimisation step */
    uint32_t steps;              /* Adam steps (0: initialise only) */
    float lr;                    /* peak learning rate, cosine decay to 2% (0: 2e-3) */
    float overestimate_weight;   /* loss weight of overestimates (0: 10) */
    uint32_t seed;
    uint32_t _reserved[4];
};

struct FptCudaMlpStats {
    float loss_first;            /* mean loss of the first batch */
    float loss_last;             /* mean loss of the last batch */
    double data_ms;              /* training-data generation */
    double train_ms;             /* optimisation */
    uint32_t params;
    uint32_t steps;
    float label_scale;           /* network output x label_scale = distance */
    uint32_t near_points;
};

/* Counters of the last render or primary trace that used the surrogate
 * skip (FPT_CUDA_SURROGATE_SKIP). */
struct FptCudaSkipStats {
    uint64_t rows;               /* network rows used for proposals */
    uint64_t forwards;           /* warp-wide network passes (32 rows each) */
    uint64_t exact_evals;        /* exact DE evaluations inside the skip pass */
    uint64_t accepted;           /* proposals certified by the exact DE */
    uint64_t rejected;           /* proposals refused (plain step taken) */
    uint64_t escaped;            /* rays found leaving the box (misses) */
    uint64_t handed_over;        /* rays handed to the exact march */
    uint64_t reserved;
};

/* Generates the training data on the GPU, trains the network with the
 * library's own BF16 tensor-core forward/backward kernels and Adam, and
 * returns a handle.  The scene (config + ext) supplies the exact DE. */
int fpt_cuda_mlp_create(const struct FptRenderConfig *config,
                        const struct FptCudaSceneExt *ext,
                        const struct FptCudaMlpConfig *mlp,
                        uint64_t *model,
                        struct FptCudaMlpStats *stats,
                        char *error,
                        size_t error_len);
int fpt_cuda_mlp_destroy(uint64_t model);
/* Network distance at n xyzw points (w ignored). */
int fpt_cuda_mlp_predict(uint64_t model, const float *points_xyzw, size_t n, float *distances, char *error, size_t error_len);
int fpt_cuda_mlp_get_params(uint64_t model, float *params, size_t len, char *error, size_t error_len);
int fpt_cuda_mlp_set_params(uint64_t model, const float *params, size_t len, char *error, size_t error_len);
/* Gradients of the mean asymmetric loss over n labelled points (xyz, w =
 * target distance) with the current parameters; no update. */
int fpt_cuda_mlp_gradients(uint64_t model,
                           const float *points_xyzw,
                           size_t n,
                           float overestimate_weight,
                           float *gradients,
                           size_t len,
                           float *loss,
                           char *error,
                           size_t error_len);
int fpt_cuda_skip_stats(struct FptCudaSkipStats *stats);
/* Test hook for the bounded waits of the tensor-core kernels (no fault is
 * made): one CTA holding tensor memory waits 20 ms at most on an mbarrier,
 * once after an arrival and once with none.  result[0] / result[1]: 1 = the
 * wait completed, 2 = it ran out; result[2] / result[3]: ns each wait took.
 * The kernel frees its tensor memory and the context stays usable. */
int fpt_test_bounded_waits(uint32_t *result, size_t result_len, char *error, size_t error_len);

/* Launch and timing record of the last fpt_cuda_render / fpt_metal_render
 * (no counterpart in the reference).  Kernel times are sums of CUDA-event
 * spans on the library's stream around each launch; they are recorded when
 * the call asked for profile statistics or kernel timing is on
 * (fpt_cuda_set_kernel_timing).  Evaluation counts need profile statistics. */
struct FptCudaRenderStats {
    uint64_t kernel_launches;    /* kernels launched by the render */
    uint64_t march_launches;
    uint64_t shade_launches;
    uint64_t skip_launches;
    uint64_t march_evals;        /* DE evaluations in the march kernel (profile renders) */
    uint64_t shade_evals;        /* normal + material evaluations in the shade kernel (profile renders) */
    double march_ms;
    double shade_ms;
    double skip_ms;
    double total_ms;             /* the call's elapsed_ms */
    uint32_t march_grid;         /* blocks of the persistent march kernel */
    uint32_t skip_grid;          /* blocks of the persistent skip kernel (0: no skip pass) */
};
int fpt_cuda_render_stats(struct FptCudaRenderStats *stats);

/* Kernel timing of later renders (no counterpart in the reference): 1 records
 * the per-kernel event spans of FptCudaRenderStats in every render, without
 * the profile counters (whose atomics add work to the kernels); 0 (default)
 * records them only in profile renders.  Returns 1 for other values. */
int fpt_cuda_set_kernel_timing(uint32_t on);

/* Launch shape of later single-scene renders (no counterpart in the
 * reference): paths per wave (0: min(all paths of a launch, 64M)) and the
 * persistent march grid (0: one wave of resident blocks).  Results do not
 * depend on either. */
int fpt_cuda_set_launch_shape(uint32_t wave_paths, int32_t march_blocks);

/* The bound a perfect distance proposal puts on the surrogate skip (no
 * counterpart in the reference).  For every `stride`-th pixel centre of the
 * config's image, counts gets six numbers: the distance evaluations of the
 * plain march and of a "certified" march for the camera ray, for the sun
 * shadow ray of its hit (toward sun_direction, when the sun is above the
 * surface) and for one cosine-distributed bounce ray of that hit (secondary
 * rays start 0.001 off the surface along the normal, as the path tracer starts
 * them; zeros where a ray does not exist).  The certified march stands on each
 * position once and always takes the longest step the skip's certificate
 * allows (s <= DE(p) + DE(p + s dir)) -- found by a search along the ray that
 * is not counted, i.e. a perfect proposal -- until the distance falls under
 * max(margin, 4 x the hit threshold); the plain march finishes the ray from
 * there.  Plain over certified is the most any proposal can save.
 * counts_len >= 6 x ceil(width / stride) x ceil(height / stride). */
int fpt_cuda_certified_steps(const struct FptRenderConfig *config,
                             const struct FptCudaSceneExt *ext,
                             uint32_t stride,
                             float margin,
                             const float *sun_direction,
                             uint32_t *counts,
                             size_t counts_len,
                             char *error,
                             size_t error_len);

/* Measured FP32 throughput of this device: a kernel of independent FMA chains
 * (2048 threads per SM) timed with CUDA events, best of six launches after two
 * warm-ups, about 2 ms each.  tflops = 2 x FMAs / time; launch_ms (optional)
 * the best launch.  No counterpart in the reference; it is the denominator of
 * the FP32 roofline the benchmark reports for the march kernel.  Changes no
 * clock or other device setting. */
int fpt_cuda_measure_fp32_peak(double *tflops, double *launch_ms, char *error, size_t error_len);

/* The 32x16 FP16 environment LUT that a render in world mode 2 samples,
 * built from a Radiance .hdr file exactly as the bridge hydrates
 * FptRenderConfig.hdri_lut before every render (src/metal_bridge.mm:2262-2300).
 * No counterpart in the reference, where hydration is internal; host only.
 * lut gets 32*16*3 halves (lut_len at least that). */
int fpt_cuda_hdri_lut(const char *hdri_path, uint16_t *lut, size_t lut_len, char *error, size_t error_len);

/* CUDA device of this process's context (no counterpart in the reference,
 * which takes the system default Metal device).  The library links its own
 * CUDA runtime, so the caller's runtime does not choose its device.  Default:
 * the ordinal in the environment variable FPT_CUDA_DEVICE, else LOCAL_RANK
 * (one replica per GPU under torchrun), else 0.  fpt_cuda_set_device must come
 * before the first call that uses the GPU; later it succeeds only for the
 * device already bound.  Returns 1 for an ordinal that is not visible. */
int fpt_cuda_set_device(int32_t ordinal);
/* The ordinal bound by the context (created on first use); 1 without a GPU. */
int fpt_cuda_get_device(int32_t *ordinal);

/* March schedule of later single-scene renders.  Schedule 0 (the only one)
 * is lockstep: each distance evaluation runs to completion on every lane, and
 * lanes whose ray finished write it and take the next ray together once
 * `batch` of them wait (0 = 8, 1 = at once, at most 32).  Returns 1 for any
 * other schedule or batch.  Images do not depend on the batch. */
int fpt_cuda_set_march_schedule(uint32_t schedule, uint32_t batch);

/* Engine of the surrogate network in later skip passes and predictions:
 * FPT_CUDA_NET_TCGEN05 (default: 5th-generation tensor cores, 128 rows per
 * CTA, accumulators in tensor memory) or FPT_CUDA_NET_MMA_SYNC (warp-level
 * mma.sync, 32 rows per warp).  Both compute the same network; outputs differ
 * only in the order of the FP32 sums.  Returns 1 for an unknown engine. */
#define FPT_CUDA_NET_TCGEN05 0u
#define FPT_CUDA_NET_MMA_SYNC 1u
int fpt_cuda_set_network_engine(uint32_t engine);

/* Time limit of the persistent loops of later single-scene renders, in ns
 * (0: 10 s).  A loop that reaches it stops, and the render returns 1 with
 * "exceeded its time limit"; the context stays usable. */
int fpt_cuda_set_loop_limit(uint64_t limit_ns);

/* ---- Batched scenes (no counterpart in the reference; its render-batch
 * command only reuses the process, src/main.rs:2269) ----
 * count scenes (extension formulas, the same sample count, no sky image, no
 * surrogate) of any size and iteration count render together: every spp
 * pass covers all scenes with one persistent launch per march pass, and the
 * pass is one CUDA graph replayed spp times.  Each scene's image equals its
 * fpt_cuda_render image at the same seed.  Outputs are concatenated in scene
 * order: linear_output W_k*H_k*4 floats per scene (accumulation buffer, row
 * 0 = bottom), rgba_output W_k*H_k*4 bytes per scene (top row first).  The
 * launch shape comes from fpt_cuda_autotune_batch when it tuned the same
 * workload key, else the default. */
struct FptCudaBatchStats {
    double elapsed_ms;           /* graph replays (all passes), CUDA events */
    double build_ms;             /* graph capture + instantiation */
    uint64_t paths;              /* sum of W*H*spp */
    uint32_t scenes;
    uint32_t passes;
    uint32_t graph_launches;
    uint32_t kernel_launches_per_pass;
    uint32_t block_size;         /* march kernel */
    uint32_t registers;          /* march kernel registers per thread */
    uint32_t wave_paths;         /* paths per wave */
    uint32_t tuned;              /* 1 when the autotuner's choice was used */
    uint64_t workload_key;
    uint32_t refill;             /* march finish/refill group (0: default 8) */
    uint32_t _pad;
};
int fpt_cuda_render_batch(const struct FptRenderConfig *configs,
                          const struct FptCudaSceneExt *exts,
                          size_t count,
                          float *linear_output,
                          size_t linear_output_len,
                          uint8_t *rgba_output,
                          size_t rgba_output_len,
                          struct FptCudaBatchStats *stats,
                          char *error,
                          size_t error_len);

struct FptCudaTuneCandidate {
    uint32_t block_size;
    uint32_t registers;
    uint32_t wave_paths;
    uint32_t refill;             /* march finish/refill group (0: default 8) */
    double median_ms;            /* median render time over the timed rounds */
};
struct FptCudaTuneResult {
    uint32_t candidates;
    uint32_t chosen;             /* index into tried; 0 is the default shape */
    uint32_t rounds;
    uint32_t _pad;
    uint64_t workload_key;
    struct FptCudaTuneCandidate tried[16];
};
/* Times every launch-shape candidate on this batch (one warm-up, then
 * `rounds` interleaved rounds), keeps the fastest when it beats the default
 * by 3%, and remembers the choice for the batch's workload key. */
int fpt_cuda_autotune_batch(const struct FptRenderConfig *configs,
                            const struct FptCudaSceneExt *exts,
                            size_t count,
                            uint32_t rounds,
                            struct FptCudaTuneResult *result,
                            char *error,
                            size_t error_len);

#ifdef __cplusplus
}
#endif

#endif /* FPT_CUDA_H */

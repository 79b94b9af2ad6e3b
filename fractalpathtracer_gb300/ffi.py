"""ctypes mirror of the C ABI in include/fpt_cuda.h.

The structs follow the reference's Rust FFI declarations field for field
(src/ffi.rs:89-394, sizes pinned by src/ffi.rs:494-507), so a config built
here is byte-identical to one the reference's scene loader would pass to
``fpt_metal_render``.
"""
from __future__ import annotations

import ctypes as C

SDF_CORNELL_BOX = 0
SDF_GLASS_BALL = 1
SDF_BALL_FRACTAL = 2
SDF_CAGE_FRACTAL = 3
SDF_IFS_FRACTAL = 4
SDF_MANDELBOX_FRACTAL = 5
SDF_MENGER_SPONGE = 6
SDF_TOWER_FRACTAL = 7
SDF_TREE_FRACTAL = 8
SDF_PROGRAM = 9
SDF_README_CORNELL = 10
SDF_README_GLASS = 11
SDF_MANDELBULBER = 12

OP_ABS, OP_TRANSLATE, OP_SCALE = 1, 2, 3
OP_ROTATE_X, OP_ROTATE_Y, OP_ROTATE_Z = 4, 5, 6
OP_REPEAT, OP_SORT_DESC = 7, 8
OP_SPHERE, OP_BOX, OP_PLANE = 16, 17, 18
OP_UNION, OP_INTERSECTION, OP_SUBTRACT = 24, 25, 26
OP_ORBIT_ADD = 32

ACCUMULATION_AUTO, ACCUMULATION_PER_SAMPLE, ACCUMULATION_BATCH, ACCUMULATION_CHUNKED = 0, 1, 2, 3
RENDERER_SDF, RENDERER_VOXEL = 0, 1
VOXEL_STORAGE_DENSE, VOXEL_STORAGE_SPARSE_BRICKS, VOXEL_STORAGE_TEMPLATE_BRICKS = 0, 1, 3
VOXEL_BUILD_STAGING, VOXEL_BUILD_DIRECT = 0, 1

FORMULA_REFERENCE = 0
FORMULA_MANDELBULB = 2
FORMULA_MANDELBULB_POWER2 = 3
FORMULA_MANDELBOX = 8
FORMULA_MENGER_FOLD = 100
FORMULA_BULB_MENGER_HYBRID = 101
RNG_HASH13, RNG_PCG = 0, 1
BRDF_REFERENCE, BRDF_LAMBERT_GGX = 0, 1
NORMAL_CONFIG, NORMAL_ANALYTIC = 0, 1
SURROGATE_OFF, SURROGATE_SKIP = 0, 1

MAX_OPS = 64
MAX_PRIMS = 64
MAX_STOPS = 16


class FptSdfInstruction(C.Structure):
    _fields_ = [("opcode", C.c_uint32), ("flags", C.c_uint32), ("material_index", C.c_uint32),
                ("_pad0", C.c_uint32), ("data", C.c_float * 4)]


class FptPrimitiveInstance(C.Structure):
    _fields_ = [("transform", C.c_float * 12), ("data", C.c_float * 4), ("opcode", C.c_uint32),
                ("distance_scale", C.c_float), ("source_instruction", C.c_uint32), ("_pad0", C.c_uint32)]


class FptAffineTransform(C.Structure):
    _fields_ = [("transform", C.c_float * 12), ("distance_scale", C.c_float), ("_pad0", C.c_uint32 * 3)]


class FptIndexedPrimitive(C.Structure):
    _fields_ = [("data", C.c_float * 4), ("opcode", C.c_uint32), ("transform_index", C.c_uint32),
                ("source_instruction", C.c_uint32), ("combine_mode", C.c_uint32)]


_F64 = C.c_float * MAX_PRIMS
_U64 = C.c_uint32 * MAX_PRIMS


class FptTypedSoAProgram(C.Structure):
    _fields_ = [("sphere_count", C.c_uint32), ("box_count", C.c_uint32), ("plane_count", C.c_uint32),
                ("_pad0", C.c_uint32),
                ("sphere_x", _F64), ("sphere_y", _F64), ("sphere_z", _F64), ("sphere_radius", _F64),
                ("sphere_source", _U64),
                ("box_x", _F64), ("box_y", _F64), ("box_z", _F64), ("box_half_x", _F64), ("box_half_y", _F64),
                ("box_half_z", _F64), ("box_source", _U64),
                ("plane_x", _F64), ("plane_y", _F64), ("plane_z", _F64), ("plane_center_x", _F64),
                ("plane_center_y", _F64), ("plane_center_z", _F64), ("plane_offset", _F64), ("plane_source", _U64)]


class FptRenderConfig(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("samples", C.c_uint32), ("preview", C.c_uint32),
        ("sdf_id", C.c_uint32), ("glass_mode", C.c_uint32), ("sdf_accumulation_mode", C.c_uint32),
        ("sdf_profile", C.c_uint32), ("sdf_bounce_cap", C.c_uint32), ("sdf_russian_roulette", C.c_uint32),
        ("sdf_normal_mode", C.c_uint32), ("sdf_chunk_samples", C.c_uint32),
        ("sdf_rr_start", C.c_float), ("sdf_rr_min_prob", C.c_float), ("mandel_iteration_scale", C.c_float),
        ("camera_position", C.c_float * 3), ("camera_yaw_pitch", C.c_float * 2), ("camera_roll", C.c_float),
        ("camera_fov", C.c_float), ("camera_dof", C.c_float), ("focus_distance", C.c_float),
        ("render", C.c_float * 8), ("world", C.c_float * 7), ("world_one_color", C.c_float * 3),
        ("sun", C.c_float * 5), ("sun_color", C.c_float * 3), ("background_gradient", C.c_float * 6),
        ("post", C.c_float * 7), ("set_values", C.c_float * 40), ("vset_values", C.c_float * 133),
        ("sdf_program_count", C.c_uint32), ("gradient_count", C.c_uint32), ("material_mode", C.c_uint32),
        ("hdri_enabled", C.c_uint32), ("hdri_width", C.c_uint32), ("hdri_height", C.c_uint32),
        ("_pad_hdri", C.c_uint32 * 2), ("fractal_style_mode", C.c_uint32), ("_pad_style", C.c_uint32 * 3),
        ("fractal_style", C.c_float * 12), ("program_material", C.c_float * 8),
        ("sdf_program", FptSdfInstruction * MAX_OPS), ("gradient_stops", (C.c_float * 4) * MAX_STOPS),
        ("hdri_path", C.c_uint8 * 256), ("hdri_lut", C.c_uint16 * (32 * 16 * 3)),
        ("renderer_backend", C.c_uint32), ("voxel_resolution", C.c_uint32), ("voxel_normal_mode", C.c_uint32),
        ("voxel_storage", C.c_uint32), ("voxel_bounds_min", C.c_float * 3), ("voxel_surface_band", C.c_float),
        ("voxel_bounds_max", C.c_float * 3), ("voxel_fill_interior", C.c_uint32),
        ("voxel_coverage_mode", C.c_uint32), ("voxel_build_mode", C.c_uint32),
        ("voxel_brick_rejection", C.c_uint32), ("voxel_leaf_refinement", C.c_uint32),
        ("voxel_material_mode", C.c_uint32), ("voxel_offset_mode", C.c_uint32),
        ("bound_grid_resolution", C.c_uint32), ("bound_grid_profile", C.c_uint32),
        ("bound_grid_profile_stride", C.c_uint32), ("bound_grid_cage_bounds", C.c_uint32),
        ("bound_grid_directional", C.c_uint32), ("sdf_program_source_count", C.c_uint32),
        ("sdf_program_optimization", C.c_uint32), ("regional_program_resolution", C.c_uint32),
        ("bound_grid_fp16", C.c_uint32), ("sdf_flat_union_count", C.c_uint32),
        ("sdf_flat_union_instances", FptPrimitiveInstance * MAX_PRIMS),
        ("sdf_shading_program_count", C.c_uint32), ("sdf_geometry_split", C.c_uint32),
        ("sdf_shading_program", FptSdfInstruction * MAX_OPS),
        ("sdf_topology_specialization", C.c_uint32), ("sdf_runtime_source_bytecode", C.c_uint32),
        ("sdf_function_stitching", C.c_uint32), ("sdf_stitched_surface", C.c_uint32),
        ("sdf_stitch_validation", C.c_uint32), ("sdf_stitch_distance_only", C.c_uint32),
        ("sdf_stitch_split_graph", C.c_uint32), ("sdf_stitch_fusion", C.c_uint32),
        ("sdf_canonical_count", C.c_uint32), ("sdf_canonical_source_count", C.c_uint32),
        ("sdf_canonical_primitives", FptPrimitiveInstance * MAX_PRIMS),
        ("sdf_canonical_transform_count", C.c_uint32), ("_pad_canonical_indexed", C.c_uint32 * 3),
        ("sdf_canonical_transforms", FptAffineTransform * MAX_PRIMS),
        ("sdf_indexed_primitives", FptIndexedPrimitive * MAX_PRIMS),
        ("sdf_typed_soa", FptTypedSoAProgram),
    ]


class FptSdfProfileStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "primary_steps", "secondary_steps", "shadow_steps", "normal_evals", "bounces", "pixels",
        "distance_evals", "march_orbit_iterations", "refinement_steps", "normal_field_evals",
        "material_evals", "max_ray_steps", "max_pixel_steps")] + [
        ("distance_evals_by_phase", C.c_uint64 * 4), ("orbit_iterations_by_phase", C.c_uint64 * 4),
        ("formula_slot_iterations", C.c_uint64 * 9), ("refinement_distance_evals", C.c_uint64),
        ("primary_ms_estimate", C.c_double), ("secondary_ms_estimate", C.c_double),
        ("shadow_ms_estimate", C.c_double), ("normal_ms_estimate", C.c_double),
        ("bounce_ms_estimate", C.c_double)]


class FptStitchPipelineStats(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in (
        "instruction_count", "transform_instruction_count", "primitive_instruction_count",
        "primitive_type_runs", "union_count", "intersection_count", "subtraction_count",
        "thread_execution_width", "max_total_threads_per_threadgroup", "graph_node_count")] + [
        ("static_threadgroup_memory_bytes", C.c_uint64), ("runtime_source_bytes", C.c_uint64),
        ("runtime_library_compile_ms", C.c_double), ("runtime_pipeline_link_ms", C.c_double)]


class FptStitchValidationStats(C.Structure):
    _fields_ = [("sample_count", C.c_uint64), ("distance_failures", C.c_uint64),
                ("gradient_failures", C.c_uint64), ("max_distance_error", C.c_float),
                ("max_gradient_error", C.c_float)]


class FptBoundGridStats(C.Structure):
    _fields_ = [(n, C.c_uint64 * 3) for n in (
        "macro_cells", "certified_skips", "candidate_intervals", "candidate_misses", "candidate_hits",
        "unknown_intervals", "field_evaluations", "directional_steps", "cell_exit_clamps",
        "unknown_derivative_intervals")] + [(n, C.c_uint64) for n in (
        "profiled_paths", "certified_cells", "unknown_cells", "sampled_bound_failures", "sampled_false_skips",
        "certified_derivative_cells", "unknown_derivative_cells", "sampled_derivative_failures",
        "regional_cells", "regional_fallback_cells", "regional_unique_programs",
        "regional_retained_instructions", "regional_sampled_distance_failures", "regional_profiled_paths")] + [
        (n, C.c_uint64 * 3) for n in (
            "regional_distance_evaluations", "regional_atlas_evaluations", "regional_full_program_evaluations",
            "regional_cell_entries", "regional_same_cell_reuses", "regional_same_program_reuses",
            "regional_program_id_loads", "regional_header_loads", "regional_dynamic_instructions")] + [
        (n, C.c_uint64) for n in (
            "regional_pruned_cells", "regional_pruned_primitives", "regional_repeat_seam_fallback_cells",
            "regional_unsupported_fallback_cells", "regional_no_dominance_cells")]


class FptAsyncJitStats(C.Structure):
    _fields_ = [("fallback_render_ms", C.c_double), ("jit_build_ms", C.c_double),
                ("stitched_render_ms", C.c_double), ("cache_status", C.c_uint32),
                ("fallback_completed_before_jit", C.c_uint32), ("max_absolute_error", C.c_float),
                ("_pad0", C.c_uint32)]


class FptDiagnosticConfig(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("_pad0", C.c_uint32), ("max_distance", C.c_float),
                ("normal_mix", C.c_float), ("dispatch_origin", C.c_uint32 * 2)]


class FptMandelbulberFieldSample(C.Structure):
    _fields_ = [("distance", C.c_float), ("radius", C.c_float), ("derivative", C.c_float),
                ("iterations", C.c_float)]


class FptCudaSceneExt(C.Structure):
    _fields_ = [
        ("formula", C.c_uint32), ("iterations", C.c_uint32), ("bailout", C.c_float), ("power", C.c_float),
        ("box_scale", C.c_float), ("box_min_radius", C.c_float), ("box_fixed_radius", C.c_float),
        ("box_fold_limit", C.c_float), ("box_fold_value", C.c_float), ("menger_scale", C.c_float),
        ("menger_iterations", C.c_uint32), ("hybrid_period", C.c_uint32), ("ground_plane", C.c_uint32),
        ("plane_height", C.c_float), ("rng", C.c_uint32), ("seed", C.c_uint32), ("brdf", C.c_uint32),
        ("albedo", C.c_float), ("ggx_alpha", C.c_float), ("specular_f0", C.c_float),
        ("plane_albedo", C.c_float), ("normal_mode", C.c_uint32), ("sky_width", C.c_uint32),
        ("sky_height", C.c_uint32), ("sky_rgb", C.POINTER(C.c_float)), ("sun_direction", C.c_float * 3),
        ("sun_intensity", C.c_float), ("fp64_bisection", C.c_uint32), ("surrogate", C.c_uint32),
        ("surrogate_model", C.c_uint64), ("surrogate_margin", C.c_float), ("surrogate_safety", C.c_float),
        ("surrogate_max_iters", C.c_uint32), ("_reserved", C.c_uint32 * 7),
    ]


class FptCudaPrimaryHit(C.Structure):
    _fields_ = [("distance", C.c_float), ("normal", C.c_float * 3), ("steps", C.c_uint32), ("hit", C.c_uint32)]


# Sizes pinned by the reference (src/ffi.rs:494-507).
REFERENCE_SIZES = {
    "FptSdfInstruction": 32, "FptPrimitiveInstance": 80, "FptAffineTransform": 64,
    "FptIndexedPrimitive": 32, "FptTypedSoAProgram": 5136, "FptStitchPipelineStats": 72,
    "FptRenderConfig": 30448, "FptSdfProfileStats": 288, "FptDiagnosticConfig": 24,
    "FptMandelbulberFieldSample": 16, "FptAsyncJitStats": 40,
}


def default_config() -> FptRenderConfig:
    """Field values of ``default_config`` (src/scene.rs:743-778)."""
    c = FptRenderConfig()
    c.width, c.height, c.samples = 768, 768, 64
    c.sdf_id = SDF_CORNELL_BOX
    c.sdf_rr_start, c.sdf_rr_min_prob, c.mandel_iteration_scale = 3.0, 0.2, 1.0
    c.sdf_chunk_samples = 8
    c.camera_position[:] = [0.1, 0.1, -5.0]
    c.camera_yaw_pitch[:] = [0.0, 0.0]
    c.camera_roll, c.camera_fov, c.camera_dof = 0.0, 90.0, 0.01
    c.render[:] = [5.0, 312.0, 0.0005, 0.0005, 1000.0, 0.25, 0.0, 0.0]
    c.world[:] = [0.0, 1.0, 120.0, 30.0, 1.0, 1.0, 0.0]
    c.world_one_color[:] = [1.0, 1.0, 1.0]
    c.sun[:] = [0.0, 120.0, 30.0, 1.0, 0.0]
    c.sun_color[:] = [1.0, 1.0, 1.0]
    c.background_gradient[:] = [1.0] * 6
    c.post[:] = [0.0, 1.0, 0.0, 1.0, 1.0, 0.0, 0.0]
    c.program_material[:] = [1.0, 1.0, 1.0, 1.0, 0.0, 0.0, 1.5, 0.0]
    c.fractal_style[:] = [0.0, 1.0, 0.5, 1.0, 1.0, 0.0, 0.0, 0.0, 1.0, 1.0, 1.0, 0.0]
    c.voxel_resolution = 128
    c.voxel_storage = VOXEL_STORAGE_SPARSE_BRICKS
    c.voxel_bounds_min[:] = [-4.0, -4.0, -4.0]
    c.voxel_surface_band = 1.0
    c.voxel_bounds_max[:] = [4.0, 4.0, 4.0]
    c.bound_grid_resolution = 32
    c.bound_grid_profile_stride = 4
    c.focus_distance = 0.0
    return c


def layout_sizes() -> dict:
    return {name: C.sizeof(globals()[name]) for name in REFERENCE_SIZES}

"""ctypes binding of libdfpt.so (declarations in include/dfpt.h).

The library is the only compute path: there is no CPU fallback. Loading fails loudly when the
shared object has not been built (``python dayflower-path-tracer_gb300/build.py``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libdfpt.so"

DFPT_OK = 0
ERRORS = {
    -1: "DFPT_ERR_INVALID_ARGUMENT",
    -2: "DFPT_ERR_CUDA",
    -3: "DFPT_ERR_OUT_OF_MEMORY",
    -4: "DFPT_ERR_INVALID_SCENE",
    -5: "DFPT_ERR_TIMEOUT",
    -6: "DFPT_ERR_NOT_SUPPORTED",
}

f32p = C.POINTER(C.c_float)
i32p = C.POINTER(C.c_int32)
u8p = C.POINTER(C.c_uint8)
u64p = C.POINTER(C.c_uint64)
f64p = C.POINTER(C.c_double)


class SceneDesc(C.Structure):
    _fields_ = [
        ("point2fs", f32p), ("point2fs_count", C.c_int64),
        ("point3fs", f32p), ("point3fs_count", C.c_int64),
        ("vector3fs", f32p), ("vector3fs_count", C.c_int64),
        ("planes", i32p), ("planes_count", C.c_int64),
        ("spheres", f32p), ("spheres_count", C.c_int64),
        ("terrains", f32p), ("terrains_count", C.c_int64),
        ("triangles", i32p), ("triangles_count", C.c_int64),
        ("bounding_volume_hierarchies", i32p), ("bounding_volume_hierarchies_count", C.c_int64),
        ("textures", f32p), ("textures_count", C.c_int64),
        ("surfaces", f32p), ("surfaces_count", C.c_int64),
        ("primitives", i32p), ("primitives_count", C.c_int64),
        ("primitives_object_to_world", f32p), ("primitives_object_to_world_count", C.c_int64),
        ("primitives_world_to_object", f32p), ("primitives_world_to_object_count", C.c_int64),
        ("camera", f32p), ("camera_count", C.c_int64),
        ("primitive_extensions", f32p), ("primitive_extensions_count", C.c_int64),
    ]


class Sky(C.Structure):
    _fields_ = [
        ("perez_relative_luminance", C.c_double * 5),
        ("perez_x", C.c_double * 5),
        ("perez_y", C.c_double * 5),
        ("zenith_relative_luminance", C.c_double),
        ("zenith_x", C.c_double),
        ("zenith_y", C.c_double),
        ("theta", C.c_float),
        ("orthonormal_basis_u", C.c_float * 3),
        ("orthonormal_basis_v", C.c_float * 3),
        ("orthonormal_basis_w", C.c_float * 3),
        ("sun_direction", C.c_float * 3),
        ("sun_direction_world", C.c_float * 3),
        ("sun_origin", C.c_float * 3),
        ("is_sky_active", C.c_int32),
        ("is_sun_active", C.c_int32),
    ]


class Params(C.Structure):
    _fields_ = [
        ("renderer_type", C.c_int32),
        ("tone_mapper_type", C.c_int32),
        ("shader_type", C.c_int32),
        ("normal_mapping", C.c_int32),
        ("wireframes", C.c_int32),
        ("pt_ray_depth_maximum", C.c_int32),
        ("pt_ray_depth_russian_roulette", C.c_int32),
        ("tone_mapper_exposure", C.c_float),
        ("ao_maximum_distance", C.c_float),
        ("global_amplitude", C.c_float),
        ("global_frequency", C.c_float),
        ("global_gain", C.c_float),
        ("global_lacunarity", C.c_float),
        ("global_octaves", C.c_int32),
        ("selected_primitive_offset", C.c_int32),
        ("rng_kind", C.c_int32),
        ("seed", C.c_uint64),
    ]


class DiffParams(C.Structure):
    _fields_ = [
        ("albedo", f32p),
        ("emission", f32p),
        ("phong_exponent", f32p),
        ("turbidity", C.c_float),
        ("sun_direction", C.c_float * 3),
    ]


# Symbol -> (restype, argtypes). Every entry point of include/dfpt.h is listed here.
SIGNATURES = {
    "dfpt_params_default": (None, [C.POINTER(Params)]),
    "dfpt_create": (C.c_int, [C.POINTER(SceneDesc), C.POINTER(Sky), C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "dfpt_destroy": (C.c_int, [C.c_void_p]),
    "dfpt_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "dfpt_set_camera": (C.c_int, [C.c_void_p, f32p]),
    "dfpt_set_transforms": (C.c_int, [C.c_void_p, f32p, f32p, C.c_int32]),
    "dfpt_set_surfaces": (C.c_int, [C.c_void_p, f32p, C.c_int64]),
    "dfpt_set_sky": (C.c_int, [C.c_void_p, C.POINTER(Sky)]),
    "dfpt_set_params": (C.c_int, [C.c_void_p, C.POINTER(Params)]),
    "dfpt_clear": (C.c_int, [C.c_void_p]),
    "dfpt_render": (C.c_int, [C.c_void_p, C.c_int32]),
    "dfpt_synchronize": (C.c_int, [C.c_void_p]),
    "dfpt_read_bgra8": (C.c_int, [C.c_void_p, u8p]),
    "dfpt_read_film": (C.c_int, [C.c_void_p, f32p, i32p]),
    "dfpt_read_film_mean": (C.c_int, [C.c_void_p, f64p]),
    "dfpt_film_mean_noalloc": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "dfpt_read_primitive_offsets": (C.c_int, [C.c_void_p, i32p]),
    "dfpt_read_hits": (C.c_int, [C.c_void_p, i32p, i32p, i32p, f32p, f32p]),
    "dfpt_read_counters": (C.c_int, [C.c_void_p, u64p]),
    "dfpt_set_counting": (C.c_int, [C.c_void_p, C.c_int32]),
    "dfpt_launch_count": (C.c_int, [C.c_void_p, u64p]),
    "dfpt_set_profiling": (C.c_int, [C.c_void_p, C.c_int32]),
    "dfpt_set_tuning": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int32]),
    "dfpt_get_tuning": (C.c_int, [C.c_void_p, C.c_char_p, i32p]),
    "dfpt_tune_frame": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float)]),
    "dfpt_l2_reset": (C.c_int, []),
    "dfpt_probe_read_bandwidth": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, f64p]),
    "dfpt_read_profile": (C.c_int, [C.c_void_p, f64p, i32p]),
    "dfpt_last_error": (C.c_char_p, []),
    "dfpt_builder_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "dfpt_builder_destroy": (C.c_int, [C.c_void_p]),
    "dfpt_builder_add_texture": (C.c_int, [C.c_void_p, f32p, C.c_int32]),
    "dfpt_builder_add_surface": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_float]),
    "dfpt_builder_add_shape": (C.c_int, [C.c_void_p, C.c_int32, f32p]),
    "dfpt_builder_add_mesh": (C.c_int, [C.c_void_p, f32p, C.c_int64, i32p, C.c_int64, C.c_int32]),
    "dfpt_builder_add_primitive": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, f32p]),
    "dfpt_builder_set_camera": (C.c_int, [C.c_void_p, f32p, f32p, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int32]),
    "dfpt_builder_compile": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "dfpt_builder_set_exhaustive": (C.c_int, [C.c_void_p, C.c_int32]),
    "dfpt_compiled_destroy": (C.c_int, [C.c_void_p]),
    "dfpt_compiled_describe": (C.c_int, [C.c_void_p, C.POINTER(SceneDesc)]),
    "dfpt_sky_set": (C.c_int, [C.POINTER(Sky), f32p, C.c_float]),
    "dfpt_diff_forward": (C.c_int, [C.c_void_p, C.POINTER(DiffParams), C.c_int32, f32p]),
    "dfpt_diff_backward": (C.c_int, [C.c_void_p, f32p, f64p, f64p, f64p, f64p]),
    "dfpt_diff_end": (C.c_int, [C.c_void_p]),
    "dfpt_batch_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "dfpt_batch_destroy": (C.c_int, [C.c_void_p]),
    "dfpt_batch_add": (C.c_int, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(Sky), C.POINTER(Params), C.c_int32, C.c_int32,
                                 C.c_int32, i32p]),
    "dfpt_batch_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "dfpt_batch_set_tuning": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int64]),
    "dfpt_batch_get_tuning": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int64)]),
    "dfpt_batch_render": (C.c_int, [C.c_void_p]),
    "dfpt_batch_clear": (C.c_int, [C.c_void_p]),
    "dfpt_batch_render_range": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64]),
    "dfpt_batch_resolve": (C.c_int, [C.c_void_p]),
    "dfpt_batch_synchronize": (C.c_int, [C.c_void_p]),
    "dfpt_batch_read_film": (C.c_int, [C.c_void_p, C.c_int32, f32p, i32p]),
    "dfpt_batch_read_bgra8": (C.c_int, [C.c_void_p, C.c_int32, u8p]),
    "dfpt_batch_launch_count": (C.c_int, [C.c_void_p, u64p]),
    # Extensions outside the public header (test and measurement hooks).
    "dfpt_set_strict": (C.c_int, [C.c_void_p, C.c_int32]),
    "dfpt_set_record_hits": (C.c_int, [C.c_void_p, C.c_int32]),
    "dfpt_set_graphs": (C.c_int, [C.c_void_p, C.c_int32]),
}

_lib = None


class DfptError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build the renderer core first (build.py)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int) -> int:
    """Raises DfptError for negative status codes; passes indices and DFPT_OK through."""
    if code < 0:
        msg = load().dfpt_last_error()
        raise DfptError(code, msg.decode() if msg else "")
    return code


def ptr(array, ctype):
    return array.ctypes.data_as(C.POINTER(ctype))

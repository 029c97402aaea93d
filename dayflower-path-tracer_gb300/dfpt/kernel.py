"""RendererKernel: the reference's renderer-kernel interface over libdfpt.so.

Method names follow AbstractRendererKernel / AbstractImageKernel / GPURendererKernel
(src/main/java/org/dayflower/pathtracer/kernel/), in snake_case:
  update(w, h, image_data_byte, local_size)  GPURendererKernel.update        (GPURendererKernel.java:411-449)
  execute()                                  Kernel.execute(range)           (DayflowerApplication.java:853)
  clear_film_flags() / clear()               AbstractImageKernel.java:119-127
  get(image_data_byte)                       Kernel.get(byte[])              (DayflowerApplication.java:855)
  update_camera/update_primitives/update_sun_and_sky                         (GPURendererKernel.java:455-569)
  toggle_sky/toggle_sun/toggle_primitive_material/toggle_primitive_selection  (GPURendererKernel.java:314-397)
  set_renderer_type, set_tone_mapper_type, ... and the matching getters     (AbstractRendererKernel.java:383-580)
  toggle_renderer_type/_normal_mapping/_wireframes, toggle_shader_type       (AbstractRendererKernel.java:591-690)
  is_renderer_type_*, has_changed/set_changed                                (AbstractRendererKernel.java:238-297, 383)
  set_global_*/get_global_* (noise parameters)                               (AbstractKernel.java:205-295)
Errors: a size mismatch in update() raises ValueError, the IllegalArgumentException of
AbstractImageKernel.java:146-148; device failures raise DfptError.
"""
from __future__ import annotations

import ctypes as C
import struct

import numpy as np

from . import _lib
from ._lib import check, ptr
from .scene import CLEAR_COAT, GLASS, LAMBERTIAN, PHONG, REFLECTION, CompiledScene, SkyState

RENDERER_TYPE_AMBIENT_OCCLUSION = 1
RENDERER_TYPE_PATH_TRACER = 2
RENDERER_TYPE_RAY_CASTER = 3
RENDERER_TYPE_RAY_MARCHER = 4
RENDERER_TYPE_RAY_TRACER = 5
RENDERER_TYPE_SURFACE_NORMALS = 6
SHADER_TYPE_FLAT = 1
SHADER_TYPE_GOURAUD = 2
TONE_MAPPER_TYPE_FILMIC_CURVE_ACES_MODIFIED = 1
TONE_MAPPER_TYPE_REINHARD = 2
TONE_MAPPER_TYPE_REINHARD_MODIFIED_1 = 3
TONE_MAPPER_TYPE_REINHARD_MODIFIED_2 = 4
BOOLEAN_FALSE = 0
BOOLEAN_TRUE = 1
RNG_COUNTER = 0
RNG_LCG = 1


def default_params() -> _lib.Params:
    p = _lib.Params()
    _lib.load().dfpt_params_default(C.byref(p))
    return p


class RendererKernel:
    """One compiled scene resident on the GPU plus its film; see the module docstring."""

    def __init__(self, compiled: CompiledScene, sky: SkyState | None = None, params: dict | None = None):
        self._lib = _lib.load()
        self.compiled = compiled
        self.sky = sky if sky is not None else SkyState()
        self.params = default_params()
        for k, v in (params or {}).items():
            setattr(self.params, k, v)
        self._h = None
        self.resolution_x = 0
        self.resolution_y = 0
        self._selected_primitive_offset = -1
        self._selected_primitive_index = -1
        self._has_changed = False

    # -- lifecycle -------------------------------------------------------------------------
    def update(self, resolution_x: int, resolution_y: int, image_data_byte=None, local_size: int = 0) -> None:
        if image_data_byte is not None and resolution_x * resolution_y * 4 != len(image_data_byte):
            raise ValueError("resolutionX * resolutionY * 4 != imageDataByte.length: "
                             f"resolutionX={resolution_x}, resolutionY={resolution_y}, imageDataByte.length={len(image_data_byte)}")
        self.dispose()
        desc = self.compiled.desc()
        h = C.c_void_p()
        check(self._lib.dfpt_create(C.byref(desc), C.byref(self.sky.raw), int(resolution_x), int(resolution_y), C.byref(h)))
        self._h = h
        self.resolution_x, self.resolution_y = int(resolution_x), int(resolution_y)
        self._push_params()

    def dispose(self) -> None:
        if self._h:
            self._lib.dfpt_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.dispose()
        except Exception:
            pass

    def _need(self):
        if not self._h:
            raise RuntimeError("update(...) must be called before rendering")
        return self._h

    def _push_params(self):
        check(self._lib.dfpt_set_params(self._need(), C.byref(self.params)))

    # -- rendering -------------------------------------------------------------------------
    def execute(self, passes: int = 1) -> None:
        check(self._lib.dfpt_render(self._need(), int(passes)))

    def synchronize(self) -> None:
        check(self._lib.dfpt_synchronize(self._need()))

    def clear(self) -> None:
        check(self._lib.dfpt_clear(self._need()))

    def clear_film_flags(self) -> None:
        """The film-clear flag applies to exactly one pass; nothing is left to reset."""

    def get(self, image_data_byte=None) -> np.ndarray:
        out = image_data_byte if image_data_byte is not None else np.empty(self.resolution_x * self.resolution_y * 4, np.uint8)
        arr = np.frombuffer(out, dtype=np.uint8) if not isinstance(out, np.ndarray) else out
        check(self._lib.dfpt_read_bgra8(self._need(), ptr(arr, C.c_uint8)))
        return arr

    def film(self):
        n = self.resolution_x * self.resolution_y
        rgb = np.empty(n * 3, np.float32)
        samples = np.empty(n, np.int32)
        check(self._lib.dfpt_read_film(self._need(), ptr(rgb, C.c_float), ptr(samples, C.c_int32)))
        return rgb.reshape(self.resolution_y, self.resolution_x, 3), samples.reshape(self.resolution_y, self.resolution_x)

    def film_mean(self) -> np.ndarray:
        m = np.empty(3, np.float64)
        check(self._lib.dfpt_read_film_mean(self._need(), ptr(m, C.c_double)))
        return m

    def primitive_offsets(self) -> np.ndarray:
        out = np.empty(self.resolution_x * self.resolution_y, np.int32)
        check(self._lib.dfpt_read_primitive_offsets(self._need(), ptr(out, C.c_int32)))
        return out

    def hits(self):
        n = self.resolution_x * self.resolution_y
        prim, typ, off = (np.empty(n, np.int32) for _ in range(3))
        dist = np.empty(n, np.float32)
        nrm = np.empty(3 * n, np.float32)
        check(self._lib.dfpt_read_hits(self._need(), ptr(prim, C.c_int32), ptr(typ, C.c_int32), ptr(off, C.c_int32),
                                       ptr(dist, C.c_float), ptr(nrm, C.c_float)))
        return prim, typ, off, dist, nrm.reshape(n, 3)

    def set_record_hits(self, enabled: bool) -> None:
        check(self._lib.dfpt_set_record_hits(self._need(), 1 if enabled else 0))

    def set_strict(self, enabled: bool) -> None:
        check(self._lib.dfpt_set_strict(self._need(), 1 if enabled else 0))

    def set_counting(self, enabled: bool) -> None:
        check(self._lib.dfpt_set_counting(self._need(), 1 if enabled else 0))

    def set_graphs(self, enabled: bool) -> None:
        check(self._lib.dfpt_set_graphs(self._need(), 1 if enabled else 0))

    def counters(self) -> np.ndarray:
        c = np.empty(6, np.uint64)
        check(self._lib.dfpt_read_counters(self._need(), ptr(c, C.c_uint64)))
        return c

    PROFILE_KINDS = ("camera", "trace", "shade", "shadow", "final", "simple", "wireframe", "film", "end", "sort")

    def set_profiling(self, enabled: bool) -> None:
        check(self._lib.dfpt_set_profiling(self._need(), 1 if enabled else 0))

    def read_profile(self) -> dict:
        ms = np.zeros(len(self.PROFILE_KINDS), np.float64)
        n = np.zeros(len(self.PROFILE_KINDS), np.int32)
        check(self._lib.dfpt_read_profile(self._need(), ptr(ms, C.c_double), ptr(n, C.c_int32)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.PROFILE_KINDS)}

    def set_tuning(self, key: str, value: int) -> None:
        check(self._lib.dfpt_set_tuning(self._need(), key.encode(), int(value)))

    def get_tuning(self, key: str) -> int:
        v = C.c_int32()
        check(self._lib.dfpt_get_tuning(self._need(), key.encode(), C.byref(v)))
        return int(v.value)

    def tune_frame_native(self, frames: int = 16) -> float:
        """dfpt_tune_frame: the C-ABI's own frame tuner (for hosts without Python); returns the
        chosen structure's device milliseconds per one-pass frame. Leaves the film and the random
        streams as they were."""
        ms = C.c_float()
        check(self._lib.dfpt_tune_frame(self._need(), int(frames), C.byref(ms)))
        return float(ms.value)

    def launch_count(self) -> int:
        c = C.c_uint64()
        check(self._lib.dfpt_launch_count(self._need(), C.byref(c)))
        return int(c.value)

    def set_stream(self, cuda_stream: int) -> None:
        check(self._lib.dfpt_set_stream(self._need(), C.c_void_p(cuda_stream)))

    # -- scene updates ---------------------------------------------------------------------
    def update_camera(self, camera=None) -> None:
        if camera is not None:
            self.compiled.camera[:] = np.asarray(camera, np.float32)
        check(self._lib.dfpt_set_camera(self._need(), ptr(self.compiled.camera, C.c_float)))

    def update_primitives(self) -> None:
        c = self.compiled
        check(self._lib.dfpt_set_transforms(self._need(), ptr(c.primitives_object_to_world, C.c_float),
                                            ptr(c.primitives_world_to_object, C.c_float), c.primitive_count))

    def update_sun_and_sky(self) -> None:
        check(self._lib.dfpt_set_sky(self._need(), C.byref(self.sky.raw)))

    def toggle_sky(self) -> None:
        """GPURendererKernel.toggleSky: flips the sky and marks a change; pushed when a handle exists."""
        self.sky.raw.is_sky_active = 0 if self.sky.raw.is_sky_active == 1 else 1
        self._has_changed = True
        if self._h:
            self.update_sun_and_sky()

    def toggle_sun(self) -> None:
        """GPURendererKernel.toggleSun: flips the sun and marks a change; pushed when a handle exists."""
        self.sky.raw.is_sun_active = 0 if self.sky.raw.is_sun_active == 1 else 1
        self._has_changed = True
        if self._h:
            self.update_sun_and_sky()

    def toggle_primitive_material(self) -> None:
        off = self._selected_primitive_offset
        if off == -1:
            return
        so = int(self.compiled.primitives[off + 2])
        old = int(self.compiled.surfaces[so])
        order = [CLEAR_COAT, GLASS, LAMBERTIAN, PHONG, REFLECTION]
        if 0 <= old - 1 < len(order):
            self.compiled.surfaces[so] = order[(old - 1 + 1) % len(order)]
            self._has_changed = True
            if self._h:
                check(self._lib.dfpt_set_surfaces(self._h, ptr(self.compiled.surfaces, C.c_float), self.compiled.surfaces.size))

    def toggle_primitive_selection(self, x: int, y: int) -> None:
        offs = self.primitive_offsets()
        index = y * self.resolution_x + x
        if 0 <= index < len(offs):
            po = int(offs[index])
            if po == self._selected_primitive_offset:
                self._selected_primitive_index = -1
                self._selected_primitive_offset = -1
            else:
                self._selected_primitive_index = po // 3
                self._selected_primitive_offset = po
            self.params.selected_primitive_offset = self._selected_primitive_offset
            self._push_params()

    def get_selected_primitive_index(self) -> int:
        return self._selected_primitive_index

    # -- settings (AbstractRendererKernel setters) ------------------------------------------
    @staticmethod
    def _differs(old, new) -> bool:
        """!=, with Float.compare's semantics for floats (NaN equals NaN, -0.0 differs from 0.0)."""
        if isinstance(old, float) or isinstance(new, float):
            def bits(v):
                return struct.unpack("<I", struct.pack("<f", float("nan") if v != v else v))[0]
            return bits(float(old)) != bits(float(new))
        return old != new

    def _set(self, name, value, allowed=None, mark=True):
        if allowed is not None and value not in allowed:
            return  # the reference ignores unknown values
        if self._differs(getattr(self.params, name), value):
            setattr(self.params, name, value)
            if mark:
                self._has_changed = True  # the setters and toggles of AbstractRendererKernel mark a change
            if self._h:
                self._push_params()

    def has_changed(self) -> bool:
        """AbstractRendererKernel.hasChanged (AbstractRendererKernel.java:238-240)."""
        return self._has_changed

    def set_changed(self, has_changed: bool) -> None:
        """AbstractRendererKernel.setChanged (AbstractRendererKernel.java:383-385)."""
        self._has_changed = bool(has_changed)

    # Renderer-type predicates (AbstractRendererKernel.java:247-297).
    def is_renderer_type_ambient_occlusion(self) -> bool:
        return self.params.renderer_type == RENDERER_TYPE_AMBIENT_OCCLUSION

    def is_renderer_type_path_tracer(self) -> bool:
        return self.params.renderer_type == RENDERER_TYPE_PATH_TRACER

    def is_renderer_type_ray_caster(self) -> bool:
        return self.params.renderer_type == RENDERER_TYPE_RAY_CASTER

    def is_renderer_type_ray_marcher(self) -> bool:
        return self.params.renderer_type == RENDERER_TYPE_RAY_MARCHER

    def is_renderer_type_ray_tracer(self) -> bool:
        return self.params.renderer_type == RENDERER_TYPE_RAY_TRACER

    def is_renderer_type_surface_normals(self) -> bool:
        return self.params.renderer_type == RENDERER_TYPE_SURFACE_NORMALS

    # Toggles (AbstractRendererKernel.java:591-690): unknown current values stay as they are.
    _RENDERER_TYPE_CYCLE = {RENDERER_TYPE_AMBIENT_OCCLUSION: RENDERER_TYPE_PATH_TRACER,
                            RENDERER_TYPE_PATH_TRACER: RENDERER_TYPE_RAY_CASTER,
                            RENDERER_TYPE_RAY_CASTER: RENDERER_TYPE_RAY_MARCHER,
                            RENDERER_TYPE_RAY_MARCHER: RENDERER_TYPE_RAY_TRACER,
                            RENDERER_TYPE_RAY_TRACER: RENDERER_TYPE_SURFACE_NORMALS,
                            RENDERER_TYPE_SURFACE_NORMALS: RENDERER_TYPE_AMBIENT_OCCLUSION}

    def toggle_renderer_type(self) -> None:
        nxt = self._RENDERER_TYPE_CYCLE.get(self.params.renderer_type)
        if nxt is not None:
            self._set("renderer_type", nxt)

    def toggle_renderer_normal_mapping(self) -> None:
        v = self.params.normal_mapping
        if v in (BOOLEAN_FALSE, BOOLEAN_TRUE):
            self._set("normal_mapping", BOOLEAN_TRUE if v == BOOLEAN_FALSE else BOOLEAN_FALSE)

    def toggle_renderer_wireframes(self) -> None:
        v = self.params.wireframes
        if v in (BOOLEAN_FALSE, BOOLEAN_TRUE):
            self._set("wireframes", BOOLEAN_TRUE if v == BOOLEAN_FALSE else BOOLEAN_FALSE)

    def toggle_shader_type(self) -> None:
        v = self.params.shader_type
        if v in (SHADER_TYPE_FLAT, SHADER_TYPE_GOURAUD):
            self._set("shader_type", SHADER_TYPE_GOURAUD if v == SHADER_TYPE_FLAT else SHADER_TYPE_FLAT)

    # Scene accessors (AbstractRendererKernel getCompiledScene / getSky / getCamera): the compiled
    # scene's arrays, the sky record and the camera's 19 floats.
    def get_compiled_scene(self) -> CompiledScene:
        return self.compiled

    def get_sky(self) -> SkyState:
        return self.sky

    def get_camera(self) -> np.ndarray:
        return self.compiled.camera

    def set_renderer_type(self, v: int) -> None:
        self._set("renderer_type", v, (1, 2, 3, 4, 5, 6))

    def set_tone_mapper_type(self, v: int) -> None:
        self._set("tone_mapper_type", v, (1, 2, 3, 4))

    def set_tone_mapper_exposure(self, v: float) -> None:
        self._set("tone_mapper_exposure", float(v))

    def set_shader_type(self, v: int) -> None:
        self._set("shader_type", v, (1, 2))

    def set_renderer_normal_mapping(self, v: int) -> None:
        self._set("normal_mapping", v, (0, 1))

    def set_renderer_wireframes(self, v: int) -> None:
        self._set("wireframes", v, (0, 1))

    def set_renderer_pt_ray_depth_maximum(self, v: int) -> None:
        self._set("pt_ray_depth_maximum", int(v))

    def set_renderer_pt_ray_depth_russian_roulette(self, v: int) -> None:
        self._set("pt_ray_depth_russian_roulette", int(v))

    def set_renderer_ao_maximum_distance(self, v: float) -> None:
        self._set("ao_maximum_distance", float(v))

    def set_global_amplitude(self, v: float) -> None:
        self._set("global_amplitude", float(v), mark=False)  # AbstractKernel's setters mark nothing

    def set_global_frequency(self, v: float) -> None:
        self._set("global_frequency", float(v), mark=False)  # AbstractKernel's setters mark nothing

    def set_global_gain(self, v: float) -> None:
        self._set("global_gain", float(v), mark=False)  # AbstractKernel's setters mark nothing

    def set_global_lacunarity(self, v: float) -> None:
        self._set("global_lacunarity", float(v), mark=False)  # AbstractKernel's setters mark nothing

    def set_global_octaves(self, v: int) -> None:
        self._set("global_octaves", int(v), mark=False)

    def set_seed(self, seed: int, rng_kind: int = RNG_COUNTER) -> None:
        self.params.seed = int(seed) & ((1 << 64) - 1)
        self.params.rng_kind = int(rng_kind)
        if self._h:
            self._push_params()

    def get_renderer_type(self) -> int:
        return self.params.renderer_type

    def get_tone_mapper_type(self) -> int:
        return self.params.tone_mapper_type

    def get_tone_mapper_exposure(self) -> float:
        return self.params.tone_mapper_exposure

    def get_shader_type(self) -> int:
        return self.params.shader_type

    def get_renderer_pt_ray_depth_maximum(self) -> int:
        return self.params.pt_ray_depth_maximum

    def get_renderer_pt_ray_depth_russian_roulette(self) -> int:
        return self.params.pt_ray_depth_russian_roulette

    def get_renderer_ao_maximum_distance(self) -> float:
        return self.params.ao_maximum_distance

    def get_renderer_normal_mapping(self) -> int:
        return self.params.normal_mapping

    def get_renderer_wireframes(self) -> int:
        return self.params.wireframes

    def get_global_amplitude(self) -> float:
        return self.params.global_amplitude

    def get_global_frequency(self) -> float:
        return self.params.global_frequency

    def get_global_gain(self) -> float:
        return self.params.global_gain

    def get_global_lacunarity(self) -> float:
        return self.params.global_lacunarity

    def get_global_octaves(self) -> int:
        return self.params.global_octaves

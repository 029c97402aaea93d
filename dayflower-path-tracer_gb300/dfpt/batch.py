"""BatchRenderer: many compiled scenes rendered together over libdfpt.so's dfpt_batch_* API.

The reference has no batch form (one GPURendererKernel renders one scene); this is the
multi-scene counterpart of RendererKernel. Every scene keeps its own resolution, samples per
pixel, camera, sky and renderer settings; the path tracer's stages run once per wave over the
samples of all scenes (see include/dfpt.h). Each scene's film equals what a RendererKernel with the
same scene, sky and seed holds after `spp` passes.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, ptr
from .kernel import default_params
from .scene import CompiledScene, SkyState


class BatchRenderer:
    def __init__(self):
        self._lib = _lib.load()
        h = C.c_void_p()
        check(self._lib.dfpt_batch_create(C.byref(h)))
        self._h = h
        self._keep = []  # scenes, skies and params stay alive while the batch exists
        self.sizes = []  # (width, height, spp) per scene

    def add(self, compiled: CompiledScene, width: int, height: int, spp: int, sky: SkyState | None = None,
            params: dict | None = None) -> int:
        sky = sky if sky is not None else SkyState()
        p = default_params()
        for k, v in (params or {}).items():
            setattr(p, k, v)
        desc = compiled.desc()
        idx = C.c_int32()
        check(self._lib.dfpt_batch_add(self._h, C.byref(desc), C.byref(sky.raw), C.byref(p), int(width), int(height), int(spp),
                                       C.byref(idx)))
        self._keep.append((compiled, sky, p))
        self.sizes.append((int(width), int(height), int(spp)))
        return idx.value

    def set_tuning(self, key: str, value: int) -> None:
        check(self._lib.dfpt_batch_set_tuning(self._h, key.encode(), int(value)))

    def get_tuning(self, key: str) -> int:
        v = C.c_int64()
        check(self._lib.dfpt_batch_get_tuning(self._h, key.encode(), C.byref(v)))
        return v.value

    @property
    def total_samples(self) -> int:
        return self.get_tuning("total_samples")

    def render(self) -> None:
        check(self._lib.dfpt_batch_render(self._h))

    def clear(self) -> None:
        check(self._lib.dfpt_batch_clear(self._h))

    def render_range(self, first_sample: int, count: int) -> None:
        check(self._lib.dfpt_batch_render_range(self._h, int(first_sample), int(count)))

    def resolve(self) -> None:
        check(self._lib.dfpt_batch_resolve(self._h))

    def synchronize(self) -> None:
        check(self._lib.dfpt_batch_synchronize(self._h))

    def film(self, index: int):
        w, h, _ = self.sizes[index]
        rgb = np.empty(w * h * 3, np.float32)
        samples = np.empty(w * h, np.int32)
        check(self._lib.dfpt_batch_read_film(self._h, int(index), ptr(rgb, C.c_float), ptr(samples, C.c_int32)))
        return rgb.reshape(h, w, 3), samples.reshape(h, w)

    def get(self, index: int) -> np.ndarray:
        w, h, _ = self.sizes[index]
        out = np.empty(w * h * 4, np.uint8)
        check(self._lib.dfpt_batch_read_bgra8(self._h, int(index), ptr(out, C.c_uint8)))
        return out

    def launch_count(self) -> int:
        v = C.c_uint64()
        check(self._lib.dfpt_batch_launch_count(self._h, C.byref(v)))
        return v.value

    def set_stream(self, stream) -> None:
        check(self._lib.dfpt_batch_set_stream(self._h, C.c_void_p(int(stream) if stream else 0)))

    def dispose(self) -> None:
        if self._h:
            self._lib.dfpt_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.dispose()
        except Exception:
            pass

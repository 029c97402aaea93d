"""Benchmark workloads on disk, readable without loading libdfpt.so.

A workload is a compiled scene (the 14 arrays and the optional primitive extension records), its
sky (the dfpt_sky fields) and the complete renderer parameters (every dfpt_params field), with the
image size. `prepare` generates one with the synthetic generators (libdfpt's scene compiler and
Sky.set) and writes it once; `load` reads it back into the same ctypes records with numpy alone, so
a process that renders a workload on the CPU - bench.py's reference arm, which times the oracle -
never maps the GPU library. The file name carries a hash of the sources that shape a workload
(generators, scene builder, compiler), so a changed generator never reads a stale file.
"""
from __future__ import annotations

import ctypes as C
import hashlib
from pathlib import Path

import numpy as np

from . import _lib
from .scene import FLOAT_ARRAYS, INT_ARRAYS, CompiledScene, SkyState

_PKG = Path(__file__).resolve().parent
CACHE_DIR = _PKG.parent / "_build" / "workloads"
_SOURCES = (_PKG / "synthetic.py", _PKG / "scene.py", _PKG / "noise_tables.py", _PKG.parent / "csrc" / "dfpt_scene.cpp")


def _key() -> str:
    h = hashlib.sha1()
    for p in _SOURCES:
        h.update(p.read_bytes())
    return h.hexdigest()[:12]


def cache_path(name: str, width: int, height: int) -> Path:
    return CACHE_DIR / f"{name}_{int(width)}x{int(height)}_{_key()}.npz"


def params_to_dict(p: _lib.Params) -> dict:
    return {k: getattr(p, k) for k, _ in p._fields_}


def params_from_dict(d: dict) -> _lib.Params:
    p = _lib.Params()
    for k, _ in p._fields_:
        setattr(p, k, type(getattr(p, k))(d[k]))
    return p


def _sky_fields(sky: SkyState) -> dict:
    return {k: np.asarray(v) for k, v in sky.as_dict().items()}


def save(path, scene: CompiledScene, sky: SkyState, params: _lib.Params, size, meta: dict | None = None) -> Path:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    arrays = {f"scene.{k}": v for k, v in scene.arrays().items()}
    arrays["scene.primitive_extensions"] = scene.primitive_extensions
    arrays.update({f"sky.{k}": v for k, v in _sky_fields(sky).items()})
    arrays.update({f"params.{k}": np.asarray(v) for k, v in params_to_dict(params).items()})
    arrays["size"] = np.asarray(size, np.int64)
    arrays["name"] = np.asarray(scene.name)
    for k, v in (meta or {}).items():
        arrays[f"meta.{k}"] = np.asarray(v)
    tmp = path.with_suffix(".tmp.npz")
    np.savez(tmp, **arrays)
    tmp.replace(path)
    return path


def load(path):
    """Returns (scene, sky, params struct, (width, height), meta dict); touches no shared library."""
    z = np.load(path, allow_pickle=False)
    scene = CompiledScene(str(z["name"]), **{k: z[f"scene.{k}"] for k in FLOAT_ARRAYS + INT_ARRAYS},
                          primitive_extensions=z["scene.primitive_extensions"])
    sky = SkyState.from_dict({k[4:]: (z[k].tolist()) for k in z.files if k.startswith("sky.")})
    params = params_from_dict({k[7:]: z[k].item() for k in z.files if k.startswith("params.")})
    meta = {k[5:]: z[k].item() for k in z.files if k.startswith("meta.")}
    w, h = (int(v) for v in z["size"])
    return scene, sky, params, (w, h), meta


def generate(name: str, width: int, height: int):
    """The benchmark workload `name` from its seeded generator: (scene, sky, params dict, size)."""
    from . import synthetic

    if name == "mesh_scene":
        return synthetic.mesh_scene(width=width, height=height)
    if name == "sphere_scene":
        return synthetic.sphere_scene(0, width, height)
    if name == "instances_scene":
        return synthetic.instances_scene(width=width, height=height)
    raise ValueError(f"unknown workload {name!r}")


def full_params(params: dict) -> _lib.Params:
    """dfpt_params_default (loads libdfpt) with the workload's settings applied."""
    p = _lib.Params()
    _lib.load().dfpt_params_default(C.byref(p))
    for k, v in params.items():
        setattr(p, k, v)
    return p


def prepare(name: str = "mesh_scene", width: int = 1920, height: int = 1080) -> Path:
    """Generates the workload and writes it to its cache path (once per generator version)."""
    path = cache_path(name, width, height)
    if path.exists():
        return path
    scene, sky, params, size = generate(name, width, height)
    return save(path, scene, sky, full_params(params), size,
                meta={"triangles": int(scene.triangles.size // 12), "primitives": scene.primitive_count})

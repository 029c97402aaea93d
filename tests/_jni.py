"""Test helper: builds dayflower-path-tracer_gb300/jni/dfpt_jni.c against the jni.h stand-in and the
fake JNIEnv (tests/jni/), linked to the built libdfpt.so, and calls its native methods the way
CudaRendererKernel.java does."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
SHIM = ROOT / "dayflower-path-tracer_gb300" / "jni" / "dfpt_jni.c"
JAVA = ROOT / "dayflower-path-tracer_gb300" / "jni" / "CudaRendererKernel.java"
PREFIX = "Java_org_dayflower_pathtracer_kernel_CudaRendererKernel_"
SCENE_ORDER = ("point2fs", "point3fs", "vector3fs", "planes", "spheres", "terrains", "triangles",
               "bounding_volume_hierarchies", "textures", "surfaces", "primitives",
               "primitives_object_to_world", "primitives_world_to_object", "camera")


def build(out_dir: Path) -> Path:
    """Compiles the shim and the fake environment into one shared library (warnings are errors)."""
    from dfpt import _lib

    libdir = _lib.LIB_PATH.parent
    out = Path(out_dir) / "libdfpt_jni_test.so"
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", "-shared", "-fPIC",
           "-I", str(ROOT / "tests" / "jni"), "-I", str(ROOT / "include"),
           str(SHIM), str(ROOT / "tests" / "jni" / "fake_env.c"),
           "-L", str(libdir), "-ldfpt", f"-Wl,-rpath,{libdir}", "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def java_natives() -> dict:
    """name -> list of Java parameter types of CudaRendererKernel's native methods."""
    src = JAVA.read_text()
    out = {}
    for name, args in re.findall(r"private static native \w+ (\w+)\(([^)]*)\);", src):
        out[name] = [a.strip().split()[0] for a in args.split(",") if a.strip()]
    return out


def c_natives() -> dict:
    """name -> number of parameters of the shim's exported JNI functions."""
    src = SHIM.read_text()
    out = {}
    for name, args in re.findall(PREFIX + r"(\w+)\(\s*([^)]*)\)\s*\{", src):
        out[name] = len([a for a in args.split(",") if a.strip()])
    return out


class Shim:
    """The shim's native methods over the fake JNIEnv; arrays are numpy arrays kept alive here."""

    def __init__(self, path: Path):
        self.so = C.CDLL(str(path))
        so = self.so
        so.fake_env.restype = C.c_void_p
        so.fake_array.restype = C.c_void_p
        so.fake_array.argtypes = [C.c_void_p, C.c_int32, C.c_int]
        so.fake_free.argtypes = [C.c_void_p]
        so.fake_exception_class.restype = C.c_char_p
        so.fake_exception_message.restype = C.c_char_p
        self.env = C.c_void_p(so.fake_env())
        self._arrays = []
        for name, types in java_natives().items():
            f = getattr(so, PREFIX + name)
            conv = {"long": C.c_int64, "int": C.c_int32}
            f.argtypes = [C.c_void_p, C.c_void_p] + [conv.get(t, C.c_void_p) for t in types]
            f.restype = C.c_int64 if name == "nativeCreate" else None
            setattr(self, name, self._caller(f))

    def _caller(self, f):
        def call(*args):
            self.so.fake_reset()
            r = f(self.env, None, *args)
            return r
        return call

    def array(self, a):
        """A fake Java array over numpy array `a` (None: a null reference)."""
        if a is None:
            return None
        a = np.ascontiguousarray(a)
        self._arrays.append(a)
        return C.c_void_p(self.so.fake_array(a.ctypes.data, a.size, a.itemsize))

    def exception(self):
        cls = self.so.fake_exception_class().decode()
        return (cls, self.so.fake_exception_message().decode()) if cls else None

    def violations(self) -> int:
        return self.so.fake_violations()


def sky_arrays(sky):
    """CudaRendererKernel.skyDoubles / skyFloats / flags of a dfpt_sky."""
    r = sky.raw
    d = np.asarray(list(r.perez_relative_luminance) + list(r.perez_x) + list(r.perez_y) +
                   [r.zenith_relative_luminance, r.zenith_x, r.zenith_y], np.float64)
    f = np.asarray([r.theta] + list(r.orthonormal_basis_u) + list(r.orthonormal_basis_v) + list(r.orthonormal_basis_w) +
                   list(r.sun_direction) + list(r.sun_direction_world) + list(r.sun_origin), np.float32)
    flags = (1 if r.is_sky_active else 0) | (2 if r.is_sun_active else 0)
    return d, f, flags


def param_arrays(p):
    """CudaRendererKernel.paramInts / paramFloats of a dfpt_params."""
    ints = np.asarray([p.renderer_type, p.tone_mapper_type, p.shader_type, p.normal_mapping, p.wireframes,
                       p.pt_ray_depth_maximum, p.pt_ray_depth_russian_roulette, p.global_octaves,
                       p.selected_primitive_offset], np.int32)
    floats = np.asarray([p.tone_mapper_exposure, p.ao_maximum_distance, p.global_amplitude, p.global_frequency,
                         p.global_gain, p.global_lacunarity], np.float32)
    return ints, floats


def create(shim: Shim, scene, sky, width, height, seed, drop=None):
    """nativeCreate with the scene's 14 arrays (`drop`: the name of one to pass as null)."""
    arrays = [shim.array(None if k == drop else getattr(scene, k)) for k in SCENE_ORDER]
    d, f, flags = sky_arrays(sky)
    return shim.nativeCreate(*arrays, shim.array(d), shim.array(f), flags, width, height, seed)

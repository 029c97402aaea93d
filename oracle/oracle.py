"""ctypes loader of the CPU oracle (oracle.cpp). TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use this module, as the
checker of the GPU core; the product never imports it. See oracle.cpp's header for what it
restates and its parity status.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        if not LIB.exists() or LIB.stat().st_mtime < (HERE / "oracle.cpp").stat().st_mtime:
            build()
        _lib = C.CDLL(str(LIB))
        vp = C.c_void_p
        _lib.oracle_render.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        _lib.oracle_render.restype = C.c_int
        _lib.oracle_intersect.argtypes = [vp, vp, vp, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp]
        _lib.oracle_sky.argtypes = [vp, vp, C.c_int, vp]
        _lib.oracle_simplex3.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int]
        _lib.oracle_simplex3.restype = C.c_double
        _lib.oracle_fbm3.argtypes = [C.c_double] * 4 + [C.c_int] + [C.c_double] * 3 + [C.c_int]
        _lib.oracle_fbm3.restype = C.c_double
        _lib.oracle_random.argtypes = [C.c_int, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint64, C.c_int, vp]
        _lib.oracle_tonemap.argtypes = [vp, vp, C.c_int, vp]
        _lib.oracle_philox.argtypes = [vp, vp, vp]
        _lib.oracle_diff.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp, C.c_double, vp, vp, vp, vp]
        _lib.oracle_diff.restype = C.c_int
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def render(scene, sky, params, width, height, passes=1, precision=64, threads=0, pass_begin=0, rows=None,
           stats=False, hits=False, rng_state=None, want_bgra=False):
    """Renders with the oracle. Returns a dict of numpy arrays (film, sum, sumsq, offsets, ...)."""
    lib = load()
    n = width * height
    r0, r1 = rows if rows is not None else (0, height)
    out = {
        "film": np.zeros(n * 3, np.float64),
        "sum": np.zeros(n * 3, np.float64),
        "sumsq": np.zeros(n * 3, np.float64),
        "primitive_offsets": np.full(n, -1, np.int32),
        "counters": np.zeros(6, np.uint64),
    }
    if want_bgra:
        out["bgra"] = np.zeros(n * 4, np.uint8)
    if hits:
        out["hit_prim"] = np.full(n, -1, np.int32)
        out["hit_type"] = np.full(n, -1, np.int32)
        out["hit_off"] = np.full(n, -1, np.int32)
        out["hit_dist"] = np.zeros(n, np.float64)
        out["hit_normal"] = np.zeros(n * 3, np.float64)
    desc = scene.desc()
    rc = lib.oracle_render(C.addressof(desc), C.addressof(sky.raw), C.addressof(params), width, height, pass_begin, passes,
                           precision, threads, r0, r1, _p(out["film"]), _p(out["sum"]), _p(out["sumsq"]),
                           _p(out["primitive_offsets"]), _p(out.get("bgra")), _p(out.get("hit_prim")), _p(out.get("hit_type")),
                           _p(out.get("hit_off")), _p(out.get("hit_dist")), _p(out.get("hit_normal")), _p(rng_state),
                           _p(out["counters"]))
    if rc != 0:
        raise RuntimeError(f"oracle_render failed: {rc}")
    return out


def intersect(scene, params, ray6, testing=False, precision=32):
    lib = load()
    desc = scene.desc()
    r = np.asarray(ray6, np.float64)
    dist = np.zeros(1, np.float64)
    ints = np.full(3, -1, np.int32)
    point = np.zeros(3, np.float64)
    normal = np.zeros(3, np.float64)
    lib.oracle_intersect(C.addressof(desc), C.addressof(params), _p(r), 1 if testing else 0, precision, _p(dist),
                         _p(ints[0:1]), ints[1:2].ctypes.data_as(C.c_void_p), ints[2:3].ctypes.data_as(C.c_void_p),
                         _p(point), _p(normal))
    return float(dist[0]), int(ints[0]), int(ints[1]), int(ints[2]), point, normal


def sky(sky_state, direction, precision=64):
    lib = load()
    d = np.asarray(direction, np.float64)
    out = np.zeros(3, np.float64)
    lib.oracle_sky(C.addressof(sky_state.raw), _p(d), precision, _p(out))
    return out


def simplex3(x, y, z, precision=32):
    return load().oracle_simplex3(x, y, z, precision)


def fbm3(frequency, gain, minimum, maximum, octaves, x, y, z, precision=32):
    return load().oracle_fbm3(frequency, gain, minimum, maximum, octaves, x, y, z, precision)


def random(kind, state, pixel, pass_index, seed, count):
    out = np.zeros(count, np.float32)
    load().oracle_random(kind, state, pixel, pass_index, seed, count, _p(out))
    return out


def tonemap(params, rgb, precision=32):
    out = np.zeros(4, np.uint8)
    v = np.asarray(rgb, np.float64)
    load().oracle_tonemap(C.addressof(params), _p(v), precision, _p(out))
    return out


def philox(counter, key):
    c = np.asarray(counter, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    load().oracle_philox(_p(c), _p(k), _p(out))
    return [int(x) for x in out]


def diff(scene, sky, params, width, height, albedo, emission, exponent, turbidity, sun_direction, dldi, pass_begin=0,
         passes=1, threads=0):
    """FP64 host adjoint. `sky` must be Sky.set(sun_direction, turbidity). Returns (image (H, W, 3),
    grads dict) with grads of sum(dldi * image) per primitive (albedo, emission, phong_exponent)
    and for turbidity and the sun direction."""
    lib = load()
    n_prim = scene.primitives.size // 3
    a = np.ascontiguousarray(np.asarray(albedo, np.float64).reshape(-1))
    e = np.ascontiguousarray(np.asarray(emission, np.float64).reshape(-1))
    x = np.ascontiguousarray(np.asarray(exponent, np.float64).reshape(-1))
    s = np.ascontiguousarray(np.asarray(sun_direction, np.float64))
    w = np.ascontiguousarray(np.asarray(dldi, np.float64).reshape(-1))
    assert a.size == 3 * n_prim and e.size == 3 * n_prim and x.size == n_prim and w.size == 3 * width * height
    img = np.zeros(3 * width * height, np.float64)
    g = np.zeros(7 * n_prim + 4, np.float64)
    desc = scene.desc()
    rc = lib.oracle_diff(C.addressof(desc), C.addressof(sky.raw), C.addressof(params), width, height, pass_begin, passes, threads,
                         _p(a), _p(e), _p(x), float(turbidity), _p(s), _p(w), _p(img), _p(g))
    if rc != 0:
        raise RuntimeError(f"oracle_diff failed: {rc}")
    gp = g[:7 * n_prim].reshape(n_prim, 7)
    return img.reshape(height, width, 3), {"albedo": gp[:, 0:3].copy(), "emission": gp[:, 3:6].copy(),
                                           "phong_exponent": gp[:, 6].copy(), "turbidity": float(g[7 * n_prim]),
                                           "sun_direction": g[7 * n_prim + 1:].copy()}

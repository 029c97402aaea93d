"""The C-ABI library on a host without a GPU: symbols, defaults, validation paths (CPU only).

No compute call is made here: every case below fails validation (or reads host-side defaults)
before the library touches a device.
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

HEADER = Path(__file__).resolve().parents[1] / "include" / "dfpt.h"


def test_every_declared_symbol_is_exported(lib):
    names = set(re.findall(r"^\s*(?:const char\*|void|int)\s+(dfpt_\w+)\s*\(", HEADER.read_text(), re.M))
    assert len(names) >= 30
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from dfpt import _lib

    names = set(re.findall(r"^\s*(?:const char\*|void|int)\s+(dfpt_\w+)\s*\(", HEADER.read_text(), re.M))
    assert names <= set(_lib.SIGNATURES), names - set(_lib.SIGNATURES)


def test_param_defaults_match_reference():
    from dfpt.kernel import default_params

    p = default_params()
    # AbstractRendererKernel.java:171-184 and AbstractKernel.java:160-168
    assert (p.renderer_type, p.tone_mapper_type, p.shader_type, p.normal_mapping, p.wireframes) == (2, 1, 2, 1, 0)
    assert (p.pt_ray_depth_maximum, p.pt_ray_depth_russian_roulette) == (5, 5)
    assert p.tone_mapper_exposure == 1.0 and p.ao_maximum_distance == 200.0
    assert (p.global_amplitude, p.global_frequency, p.global_gain, p.global_lacunarity, p.global_octaves) == \
        (np.float32(0.5), np.float32(0.2), 0.5, 2.0, 2)
    assert p.selected_primitive_offset == -1


def _scene():
    from dfpt import synthetic

    return synthetic.sphere_scene(0, 16, 16)


def _create(lib, scene, sky, w=16, h=16):
    h_ = C.c_void_p()
    desc = scene.desc()
    return lib.dfpt_create(C.byref(desc), C.byref(sky.raw), w, h, C.byref(h_))


@pytest.mark.parametrize("mutate, code", [
    (lambda s: s.primitives.__setitem__(1, 999), -4),           # sphere offset past spheres[]
    (lambda s: s.primitives.__setitem__(2, 600), -4),           # surface offset past surfaces[]
    (lambda s: s.surfaces.__setitem__(1, 1e6), -4),             # albedo texture offset past textures[]
    (lambda s: s.planes.__setitem__(0, -3), -4),                # negative point offset
    (lambda s: s.spheres.__setitem__(0, 1e9), -4),              # sphere position offset
])
def test_invalid_scenes_rejected_before_device_work(lib, mutate, code):
    scene, sky, _, _ = _scene()
    scene = scene.copy()
    mutate(scene)
    assert _create(lib, scene, sky) == code
    assert lib.dfpt_last_error()


def test_bad_bvh_rejected(lib):
    from dfpt import synthetic

    scene, sky, _, _ = synthetic.small_mesh_scene(width=8, height=8, frequency=2, grid=4)
    s = scene.copy()
    s.bounding_volume_hierarchies[1] = 0  # a skip pointer that points backwards would loop forever
    assert _create(lib, s, sky) == -4
    s = scene.copy()
    s.bounding_volume_hierarchies[0] = 7  # unknown node type
    assert _create(lib, s, sky) == -4
    s = scene.copy()
    s.bounding_volume_hierarchies[4] = 10_000_000  # left child not the next node / out of range
    assert _create(lib, s, sky) in (-4, -6)


def test_bad_sizes(lib):
    scene, sky, _, _ = _scene()
    assert _create(lib, scene, sky, 0, 16) == -1
    assert _create(lib, scene, sky, 16, -1) == -1
    from dfpt.kernel import RendererKernel

    k = RendererKernel(scene, sky)
    with pytest.raises(ValueError, match="resolutionX \\* resolutionY \\* 4"):
        k.update(16, 16, bytearray(16 * 16 * 3))


def test_noalloc_rejects_bad_sizes_without_device(lib):
    out = (C.c_double * 3)()
    rgb = (C.c_float * 3)()
    assert lib.dfpt_film_mean_noalloc(C.cast(rgb, C.c_void_p), 0, C.cast(out, C.c_void_p), None) == -1
    assert lib.dfpt_film_mean_noalloc(C.cast(rgb, C.c_void_p), (1 << 28) + 1, C.cast(out, C.c_void_p), None) == -1
    assert lib.dfpt_film_mean_noalloc(None, 10, C.cast(out, C.c_void_p), None) == -1


@pytest.mark.parametrize("ext", [
    np.zeros(5, np.float32),                                                 # not 4 per primitive
    np.tile(np.asarray([-1.0, 1, 1, 1], np.float32), 4),                     # negative exponent
    np.tile(np.asarray([50.0, np.nan, 1, 1], np.float32), 4),                # NaN emission scale
    np.tile(np.asarray([50.0, 1, -2, 1], np.float32), 4),                    # negative emission scale
])
def test_bad_primitive_extensions_rejected(lib, ext):
    scene, sky, _, _ = _scene()
    s = scene.copy()
    assert s.primitive_count == 4
    s.primitive_extensions = ext
    assert _create(lib, s, sky) == -4
    assert b"extension" in lib.dfpt_last_error()


def test_read_probe_rejects_bad_arguments_without_device(lib):
    g = C.c_double()
    buf = (C.c_uint8 * 64)()
    base = C.cast(buf, C.c_void_p).value
    aligned = (base + 15) // 16 * 16
    assert lib.dfpt_probe_read_bandwidth(None, 1 << 20, 1, None, C.byref(g)) == -1
    assert lib.dfpt_probe_read_bandwidth(C.c_void_p(aligned + 4), 1 << 20, 1, None, C.byref(g)) == -1  # not 16-byte aligned
    assert lib.dfpt_probe_read_bandwidth(C.c_void_p(aligned), 4096, 1, None, C.byref(g)) == -1  # under 1 MiB
    assert lib.dfpt_probe_read_bandwidth(C.c_void_p(aligned), (1 << 20) + 8, 1, None, C.byref(g)) == -1  # not a multiple of 16
    assert lib.dfpt_probe_read_bandwidth(C.c_void_p(aligned), 1 << 20, 0, None, C.byref(g)) == -1


def test_handle_entry_points_reject_a_null_handle_without_device(lib):
    """The tuning entry points check their arguments before any device work."""
    ms = C.c_float(-1.0)
    v = C.c_int32()
    assert lib.dfpt_tune_frame(None, 4, C.byref(ms)) == -1
    assert lib.dfpt_set_tuning(None, b"tail_bounce", 0) == -1
    assert lib.dfpt_get_tuning(None, b"tail_bounce", C.byref(v)) == -1
    assert b"NULL" in lib.dfpt_last_error() or b"handle" in lib.dfpt_last_error()

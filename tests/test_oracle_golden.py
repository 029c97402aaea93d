"""The CPU oracle against the golden known-answer vectors (CPU only).

The vectors in tests/golden/ come from tests/golden/make_golden.py: published Philox4x32-10
known answers and pure-Python restatements of the reference's LCG, simplex noise, Perez sky and
image pipeline, written independently of oracle/oracle.cpp.
"""
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _load(name):
    return json.loads((GOLDEN / name).read_text())


def test_philox_known_answers(oracle_mod):
    for case in _load("philox.json")["cases"]:
        assert oracle_mod.philox(case["counter"], case["key"]) == case["out"]


def test_lcg_stream(oracle_mod):
    for case in _load("lcg.json")["cases"]:
        got = oracle_mod.random(1, case["state"], 0, 0, 0, len(case["floats"]))
        assert [float(x) for x in got] == case["floats"]


def test_counter_stream_is_philox(oracle_mod):
    # Draw i of pixel p, pass q = top 24 bits of word (i % 4) of Philox((q, i/4, seed_hi, 'DFPT'), (p, seed_lo)).
    seed = 0x0123456789ABCDEF
    got = oracle_mod.random(0, 0, 17, 5, seed, 8)
    for i in range(8):
        words = oracle_mod.philox([5, i // 4, seed >> 32, 0x44465054], [17, seed & 0xFFFFFFFF])
        assert got[i] == np.float32((words[i % 4] >> 8) * (1.0 / 16777216.0))


def test_simplex_and_fbm(oracle_mod):
    g = _load("noise.json")
    for x, y, z, v in g["simplex3"]:
        assert oracle_mod.simplex3(x, y, z, 32) == v
    for x, y, z, v in g["fbm3"]:
        assert oracle_mod.fbm3(0.5, 0.5, -0.26, 0.26, 16, x, y, z, 32) == v


def test_synthetic_noise_matches_oracle(oracle_mod):
    from dfpt import synthetic

    rng = np.random.default_rng(3)
    p = rng.uniform(-30, 30, (64, 3)).astype(np.float32)
    vec = synthetic.simplex3(p[:, 0], p[:, 1], p[:, 2])
    for i in range(len(p)):
        assert vec[i] == np.float32(oracle_mod.simplex3(*p[i], 32))


def test_sky_fp64(oracle_mod):
    from dfpt.scene import SkyState

    g = _load("sky.json")
    sky = SkyState(g["sun_direction_world"], g["turbidity"])
    for case in g["cases"]:
        got = oracle_mod.sky(sky, case["direction"], 64)
        np.testing.assert_allclose(got, case["rgb"], rtol=1e-6, atol=1e-9)


def test_tonemap_pipeline(oracle_mod):
    from dfpt.kernel import default_params

    for case in _load("tonemap.json")["cases"]:
        p = default_params()
        p.tone_mapper_type = case["kind"]
        p.tone_mapper_exposure = case["exposure"]
        got = oracle_mod.tonemap(p, case["rgb"], 32)
        assert list(got) == case["bgra"], case


def _single_shape_scene(shape):
    from dfpt.scene import CompiledScene, pack_argb

    eye = np.eye(4, dtype=np.float32).reshape(-1)
    tex = [4, 3, pack_argb(0.5, 0.5, 0.5)]
    base = dict(textures=tex, surfaces=[3, 0, 0, 0, 0, 0], primitives_object_to_world=eye, primitives_world_to_object=eye,
                camera=np.zeros(19, np.float32))
    if shape == "sphere":
        return CompiledScene(point3fs=[0, 0, 0], spheres=[0, 2], primitives=[2, 0, 0], **base)
    if shape == "plane":
        return CompiledScene(point3fs=[0, 0, 0, 0, 0, 1, 1, 0, 0], vector3fs=[0, 1, 0], planes=[0, 3, 6, 0], primitives=[1, 0, 0], **base)
    return CompiledScene(point3fs=[0, 0, 0, 1, 0, 0, 0, 1, 0], vector3fs=[0, 0, 1, 1, 0, 0], point2fs=[0, 0],
                         triangles=[0, 3, 6, 0, 0, 0, 0, 0, 0, 3, 3, 3], primitives=[4, 0, 0], **base)


@pytest.mark.parametrize("precision", [32, 64])
def test_intersection_known_answers(oracle_mod, precision):
    from dfpt.kernel import default_params

    p = default_params()
    p.shader_type = 1  # flat: the triangle normal from its edges
    for case in _load("intersect.json")["cases"]:
        scene = _single_shape_scene(case["shape"])
        t, prim, typ, off, point, normal = oracle_mod.intersect(scene, p, case["ray"], False, precision)
        if case["t"] is None:
            assert prim == -1 and t == 100000.0
        else:
            assert prim == 0 and t == pytest.approx(case["t"], rel=1e-6)
            np.testing.assert_allclose(normal, case["normal"], atol=1e-6)
        # isTesting returns the same distance.
        t2 = oracle_mod.intersect(scene, p, case["ray"], True, precision)[0]
        assert t2 == t


@pytest.mark.parametrize("name", ["spheres", "meshes"])
def test_oracle_reproduces_golden_renders(oracle_mod, name):
    from dfpt.kernel import default_params
    from dfpt.scene import FLOAT_ARRAYS, INT_ARRAYS, CompiledScene, SkyState

    z = np.load(GOLDEN / f"render_{name}.npz")
    scene = CompiledScene(name, **{k: z["scene_" + k] for k in FLOAT_ARRAYS + INT_ARRAYS})
    sky = SkyState.from_dict(json.loads(str(z["sky"])))
    p = default_params()
    for k, v in json.loads(str(z["params"])).items():
        setattr(p, k, v)
    w, h = int(z["width"]), int(z["height"])
    pt = oracle_mod.render(scene, sky, p, w, h, passes=int(z["pt_passes"]), precision=64)
    np.testing.assert_allclose(pt["film"], z["pt_film"], rtol=1e-9, atol=1e-12)
    p.renderer_type = 3
    rc = oracle_mod.render(scene, sky, p, w, h, passes=1, precision=32, hits=True, want_bgra=True)
    assert np.array_equal(rc["hit_prim"], z["rc_hit_prim"])
    assert np.array_equal(rc["hit_off"], z["rc_hit_off"])
    assert np.array_equal(rc["hit_dist"], z["rc_hit_dist"])
    assert np.abs(rc["bgra"].astype(int) - z["rc_bgra"].astype(int)).max() <= 1

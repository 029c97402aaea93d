"""CPU: per-primitive extension records (Phong exponent, emission scale) in the scene builder and
the oracle. The reference drops PhongMaterial's exponent (SceneCompiler.java:760-768; the kernel
uses 50) and clamps emission to 8 bits (ConstantTexture.java:150-155); the records carry both.

Checked with the strict-FP32 oracle on the same random stream:
  - records that restate the defaults (exponent 50, scale 1) leave the film bit for bit unchanged;
  - an emitter's emission scale multiplies what the camera sees of it: with a black albedo and the
    sun off, the film of a pixel on the emitter is the emission texture colour times the scale;
  - a Phong region's exponent changes its film (and only where Phong surfaces are seen).
The builder places a record per primitive, in primitive order.
"""
import numpy as np
import pytest


def _params(d):
    from dfpt.kernel import default_params

    p = default_params()
    for k, v in d.items():
        setattr(p, k, v)
    return p


def _emitter_scene(scale):
    from dfpt import scene as sc

    b = sc.SceneBuilder()
    black = b.constant(0, 0, 0)
    b.primitive(b.plane((0, 0, 0), (0, 0, 1), (1, 0, 0)), b.surface(sc.LAMBERTIAN, black, b.constant(0.2, 0.4, 0.6), black),
                emission_scale=scale)
    b.camera((0, 3, 0.01), (0, 0, 0), 60.0, (16, 12))
    sky = sc.SkyState((0.3, 0.9, 0.3), 2.0)
    sky.raw.is_sun_active = 0
    sky.raw.is_sky_active = 0
    return b.compile("emitter"), sky


def test_builder_places_records_in_primitive_order():
    from dfpt import synthetic

    cs, *_ = synthetic.mesh_scene(width=64, height=36, frequency=4, grid=8)
    ext = cs.primitive_extensions.reshape(-1, 4)
    assert ext.shape == (cs.primitive_count, 4)
    # Regions 1 and 3 are Phong with exponents U(10, 200); the Lambertian regions and the ground keep 50.
    assert ext[0, 0] == 50 and ext[2, 0] == 50 and ext[4, 0] == 50
    assert 10 <= ext[1, 0] <= 200 and 10 <= ext[3, 0] <= 200 and ext[1, 0] != ext[3, 0]
    assert (ext[:, 1:] == 1).all()
    plain, *_ = synthetic.small_mesh_scene(width=16, height=12)
    assert plain.primitive_extensions.size == 0


def test_instances_lights_are_hdr_triangle_primitives():
    from dfpt import synthetic
    from dfpt.scene import TRIANGLE

    cs, *_ = synthetic.instances_scene(width=32, height=18, frequency=2, count=4, lights=30)
    prims = cs.primitives.reshape(-1, 3)
    ext = cs.primitive_extensions.reshape(-1, 4)
    assert len(prims) == 34 and (prims[4:, 0] == TRIANGLE).all()
    assert (ext[:4] == [50, 1, 1, 1]).all()
    assert (ext[4:, 1] >= 1).all() and (ext[4:, 1] <= 20).all() and (ext[4:, 1] == ext[4:, 3]).all()
    assert ext[4:, 1].std() > 1


def test_default_records_change_nothing(oracle_mod):
    from dfpt import synthetic

    scene, sky, params, (w, h) = synthetic.small_mesh_scene(width=32, height=24)
    with_ext = scene.copy()
    with_ext.primitive_extensions = np.tile(np.asarray([50, 1, 1, 1], np.float32), scene.primitive_count)
    a = oracle_mod.render(scene, sky, _params(params), w, h, passes=2, precision=32)["film"]
    b = oracle_mod.render(with_ext, sky, _params(params), w, h, passes=2, precision=32)["film"]
    assert np.array_equal(a, b)


@pytest.mark.parametrize("scale", [1.0, 7.5, 20.0])
def test_emission_scale_multiplies_emission(oracle_mod, scale):
    cs, sky = _emitter_scene(scale)
    out = oracle_mod.render(cs, sky, _params(dict(renderer_type=2, pt_ray_depth_maximum=3)), 16, 12, passes=1, precision=64)
    film = out["film"].reshape(-1, 3)
    lit = film.sum(1) > 0
    assert lit.mean() > 0.5
    q = lambda v: np.float32(np.float32(int(np.float32(v) * np.float32(255) + np.float32(0.5))) / np.float32(255))
    expect = np.array([q(0.2), q(0.4), q(0.6)], np.float64) * scale
    np.testing.assert_allclose(film[lit], np.broadcast_to(expect, film[lit].shape), rtol=1e-6)


def test_phong_exponent_changes_phong_regions(oracle_mod):
    from dfpt import synthetic

    scene, sky, params, (w, h) = synthetic.mesh_scene(width=48, height=27, frequency=6, grid=16)
    ext = scene.primitive_extensions.reshape(-1, 4)
    flat = scene.copy()
    flat.primitive_extensions = np.tile(np.asarray([50, 1, 1, 1], np.float32), scene.primitive_count)
    p = _params(params)
    a = oracle_mod.render(scene, sky, p, w, h, passes=2, precision=32, hits=True)
    b = oracle_mod.render(flat, sky, p, w, h, passes=2, precision=32)
    prim = a["hit_prim"] // 3
    phong = np.isin(prim, np.nonzero(ext[:, 0] != 50)[0])
    assert phong.sum() > 20
    diff = np.abs(a["film"] - b["film"]).reshape(-1, 3).sum(1) > 0
    assert diff[phong].mean() > 0.5

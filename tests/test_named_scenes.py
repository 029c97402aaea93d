"""CPU: the reference's named scenes (dfpt.scenes, Scenes.java:81-480) built from the reference's
resource directory (skipped when it is absent): dispatch, missing resources, the material
showcase's layout and camera, the House_2 rectangles, and the oracle's ray cast of the compiled
scenes (the primitives the camera should see are hit)."""
from pathlib import Path

import numpy as np
import pytest

from dfpt import scene as sc
from dfpt import scenes
from conftest import reference_resources

RES = reference_resources() or Path("missing-reference-resources")
pytestmark = pytest.mark.skipif(not (RES / "model").exists(),
                                reason="reference resources not available (set DFPT_REFERENCE_RESOURCES)")

BUILT = ("Girl_Scene", "House_2_Scene", "Image_Scene", "Material_Showcase_Scene", "Monkey_Scene", "Terrain_Scene",
         "Wine_Glass_Scene")


def test_dispatch_and_missing_resources():
    for name in ("House_Scene", "Zealot_Scene"):  # their files are not among the resources
        with pytest.raises(FileNotFoundError):
            scenes.scene_by_name(RES, name)
    a, _ = scenes.scene_by_name(RES, "No_Such_Scene")
    b, _ = scenes.scene_by_name(RES, "Material_Showcase_Scene")
    for k, v in a.arrays().items():
        assert np.array_equal(v, getattr(b, k)), k


def test_material_showcase_layout():
    cs, sky = scenes.scene_by_name(RES, "Material_Showcase_Scene")
    prims = cs.primitives.reshape(-1, 3)
    assert len(prims) == 16
    assert prims[0, 0] == sc.PLANE and (prims[1:, 0] == sc.SPHERE).all()
    o2w = cs.primitives_object_to_world.reshape(-1, 16)
    xs = [40, 80, 120, 160, 200, 280, 320, 360, 400, 440, 480, 520, 560, 640, 680]
    assert np.array_equal(o2w[1:, 3], np.array(xs, np.float32))
    assert (o2w[1:, 7] == np.float32(16.5)).all() and (o2w[1:, 11] == np.float32(20.0)).all()
    materials = cs.surfaces[prims[:, 2]].astype(int)
    assert materials.tolist() == [sc.LAMBERTIAN, sc.CLEAR_COAT, sc.GLASS, sc.LAMBERTIAN, sc.REFLECTION, sc.PHONG] + \
        [sc.LAMBERTIAN] * 8 + [sc.REFLECTION, sc.GLASS]
    # The last sphere's surface carries noise amount 1 and scale 16.
    assert cs.surfaces[prims[15, 2] + 4] == 1.0 and cs.surfaces[prims[15, 2] + 5] == 16.0
    cam = cs.camera
    assert np.array_equal(cam[1:4], np.array([295.0, 42.0, 332.6], np.float32))
    assert cam[4] == 90.0 and cam[6] == 30.0 and cam[18] == 1.0 and tuple(cam[16:18]) == (800.0, 800.0)
    u, v, w = cam[7:10], cam[10:13], cam[13:16]
    assert u.tolist() == [-1.0, 0.0, 0.0] and v.tolist() == [0.0, 1.0, 0.0] and w.tolist() == [0.0, 0.0, -1.0]
    assert np.signbit(w).tolist() == [True, True, True] and np.signbit(v).tolist() == [False, False, True]
    assert tuple(sky.sun_direction_world_input) == (1.0, 1.0, 1.0) and sky.turbidity == 2.0
    # Texture types the showcase uses: image (Texture_2.png 512 x 512 and the normal map), blend,
    # bullseye, UV, surface normal, fBm, checkerboard, constant.
    types = set()
    t = 0
    while t < cs.textures.size:
        types.add(int(cs.textures[t]))
        t += int(cs.textures[t + 1])
    assert types == {sc.TEX_BLEND, sc.TEX_BULLSEYE, sc.TEX_CHECKERBOARD, sc.TEX_CONSTANT, sc.TEX_FBM, sc.TEX_IMAGE,
                     sc.TEX_SURFACE_NORMAL, sc.TEX_UV}


def test_resolution_follows_the_application():
    cs, _ = scenes.scene_by_name(RES, "Monkey_Scene", resolution=(1920, 1080))
    assert tuple(cs.camera[16:18]) == (1920.0, 1080.0)
    b = sc.SceneBuilder()
    b.primitive(b.sphere((0, 0, 0), 1), b.surface(sc.LAMBERTIAN, b.constant(1, 1, 1), b.constant(0, 0, 0), b.constant(0, 0, 0)))
    b.camera((0, 0, 5), (0, 0, 0), 90.0, (1920, 1080))
    assert b.compile().camera[5] == cs.camera[5]  # the compiler's field of view Y at that size


def test_house2_rectangles():
    cs, _ = scenes.scene_by_name(RES, "House_2_Scene")
    prims = cs.primitives.reshape(-1, 3)
    assert prims[:, 0].tolist() == [sc.TRIANGLE_MESH, sc.PLANE, sc.TRIANGLE_MESH, sc.TRIANGLE_MESH]
    tri = cs.triangles.reshape(-1, 12)
    assert len(tri) == 2 + 2 + 32
    # Triangle records (Triangle.java:44-99): normal offsets at 3..5, tangent offsets at 9..11,
    # element offsets into vector3fs. Each rectangle triangle has its flat, axis-aligned unit
    # normal at every corner and a unit tangent orthogonal to it.
    v3 = cs.vector3fs
    for corner in range(3):
        n = np.stack([v3[tri[:, 3 + corner] + k] for k in range(3)], -1)
        t = np.stack([v3[tri[:, 9 + corner] + k] for k in range(3)], -1)
        assert ((np.abs(n) == 1.0).sum(axis=1) == 1).all() and ((n == 0) | (np.abs(n) == 1)).all()
        assert np.allclose(np.linalg.norm(t, axis=1), 1.0, atol=1e-6)
        assert np.allclose((n * t).sum(axis=1), 0.0, atol=1e-6)


@pytest.mark.parametrize("name", BUILT)
def test_named_scene_file_round_trip(tmp_path, name):
    cs, _ = scenes.scene_by_name(RES, name)
    p = tmp_path / f"{name}.scene"
    cs.write(p)
    back = sc.CompiledScene.read(p)
    assert back.name == name
    for k, v in cs.arrays().items():  # bit for bit (degenerate texture coordinates give NaN tangents)
        assert v.tobytes() == getattr(back, k).tobytes(), k


def test_named_scenes_raycast(oracle_mod):
    from dfpt.kernel import default_params

    p = default_params()
    p.renderer_type = 3
    w, h = 96, 64
    expect = {"Material_Showcase_Scene": 12, "Monkey_Scene": 1, "Girl_Scene": 2, "House_2_Scene": 3}
    for name, at_least in expect.items():
        cs, sky = scenes.scene_by_name(RES, name, resolution=(w, h))
        hit = oracle_mod.render(cs, sky, p, w, h, passes=1, precision=32, hits=True)["hit_prim"]
        seen = set(int(x) // 3 for x in np.unique(hit) if x >= 0)
        assert len(seen - {0} if name != "House_2_Scene" else seen - {1}) >= at_least, (name, seen)

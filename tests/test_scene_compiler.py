"""The C++ scene compiler and BVH builder against the pure-Python restatement (CPU only).

Both restate SceneCompiler.compile and BoundingVolumeHierarchy.createBoundingVolumeHierarchy;
the arrays they produce for the same scene must agree bit for bit (the data contract the GPU
core consumes). Also: .scene file round trip, BVH structural invariants on a larger mesh, and
the sky set-up against the reference's formulas.
"""
import math
import struct

import numpy as np
import pytest


def _mesh_desc(freq, seed):
    from dfpt import synthetic

    pos, idx, region, nrm, uv = synthetic.displaced_icosphere(freq, 0.1, seed)
    tng = synthetic.tangents_for(nrm)
    v11 = np.concatenate([pos, nrm, uv, tng], 1).astype(np.float32)
    return v11, idx


def _scene(freq=2, seed=5):
    """One description fed to both compilers: plane, two spheres sharing a shape, a mesh (with a
    transform), a single triangle, blend and checkerboard textures."""
    from dfpt import scene as sc
    from oracle import scene_ref

    v11, idx = _mesh_desc(freq, seed)
    tri_v = np.array([[0, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0], [1, 0, 0, 0, 1, 0, 1, 0, 1, 0, 0], [0, 1, 0, 0, 1, 0, 0, 1, 1, 0, 0]], np.float32)
    textures = [
        [4, 3, sc.pack_argb(0, 0, 0)],
        [4, 3, sc.pack_argb(0.7, 0.2, 0.1)],
        [3, 8, sc.pack_argb(0.5, 0.5, 0.5), sc.pack_argb(0.5, 0.5, 0.5), 1.0, 0.0, 5.0, 5.0],
        [1, 5, 1, 2, 0.25],  # blend of textures 1 and 2
        [4, 3, sc.pack_argb(0, 0, 0)],  # equal to texture 0
    ]
    surfaces = [(3, 2, 0, 0, 0.0, 0.0), (2, 1, 4, 0, 0.0, 0.0), (4, 3, 0, 0, 0.5, 2.0), (3, 1, 0, 4, 0.0, 0.0)]
    shapes = [("plane", (0, 0, 0), (0, 0, 1), (1, 0, 0)), ("sphere", (0, 0, 0), 1.0), ("mesh", v11, idx),
              ("triangle", tri_v)]
    xf = [((0, 0, 0), (0, 0, 0, 1), (1, 1, 1)), ((2, 1, 0), (0, 0, 0, 1), (1, 1, 1)), ((-2, 1, 0.5), (0, 0, 0, 1), (1, 1, 1)),
          ((0, 2, 0), (0, 0.38268343, 0, 0.9238795), (1, 1.2, 1)), ((0, 0, 3), (0, 0, 0, 1), (1, 1, 1))]
    prims = [(0, 0, 0), (1, 1, 1), (1, 3, 2), (2, 2, 3), (3, 3, 4)]
    b = sc.SceneBuilder()
    for t in textures:
        b.texture(t)
    for s in surfaces:
        b.surface(*s)
    sid = [b.plane(*shapes[0][1:]), b.sphere(shapes[1][1], shapes[1][2]),
           b.mesh(v11[:, 0:3], idx, v11[:, 3:6], v11[:, 6:8], v11[:, 8:11]),
           b.mesh(tri_v[:, 0:3], [[0, 1, 2]], tri_v[:, 3:6], tri_v[:, 6:8], tri_v[:, 8:11], as_mesh=False)]
    for shape, surf, x in prims:
        b.primitive(sid[shape], surf, *xf[x])
    b.camera((0, 2, 10), (0, 0, 0), 90.0, (64, 48))
    cs = b.compile("t")
    desc = {"textures": textures, "surfaces": surfaces, "shapes": shapes, "camera": list(cs.camera),
            "primitives": [(shape, surf, *scene_ref.transform_matrices(*xf[x])) for shape, surf, x in prims]}
    return cs, scene_ref.compile_scene(desc)


def _bits(a, dtype):
    a = np.asarray(a, dtype)
    return a.view(np.uint32 if dtype == np.float32 else np.int32)


def test_compiler_matches_python_restatement():
    cs, ref = _scene()
    for key in ("point2fs", "point3fs", "vector3fs", "spheres", "textures", "surfaces", "primitives_object_to_world",
                "primitives_world_to_object"):
        got, exp = getattr(cs, key), np.asarray(ref[key], np.float32)
        assert got.shape == exp.shape, key
        assert np.array_equal(_bits(got, np.float32), _bits(exp, np.float32)), key
    for key in ("planes", "triangles", "bounding_volume_hierarchies", "primitives"):
        assert np.array_equal(getattr(cs, key), np.asarray(ref[key], np.int32)), key


def test_bvh_structure_invariants():
    """Every triangle in exactly one leaf; children inside parents; skip pointers forward."""
    from dfpt import scene as sc

    v11, idx = _mesh_desc(12, 7)  # 2,880 triangles
    b = sc.SceneBuilder()
    t = b.constant(0.5, 0.5, 0.5)
    b.primitive(b.mesh(v11[:, 0:3], idx, v11[:, 3:6], v11[:, 6:8], v11[:, 8:11]), b.surface(3, t, t, t))
    b.camera((0, 0, 5), (0, 0, 0))
    cs = b.compile()
    bvh, p3 = cs.bounding_volume_hierarchies, cs.point3fs
    seen = []
    off, stack = 0, []
    nodes = 0
    while off < len(bvh):
        typ, nxt, mn, mx = bvh[off:off + 4]
        assert typ in (1, 2)
        assert nxt == -1 or nxt > off
        lo, hi = p3[mn:mn + 3], p3[mx:mx + 3]
        assert (lo <= hi).all()
        nodes += 1
        if typ == 2:
            n = bvh[off + 4]
            assert 1 <= n
            seen += list(bvh[off + 5:off + 5 + n])
            off += 5 + n
        else:
            assert bvh[off + 4] == off + 5
            off += 5
    assert sorted(seen) == list(range(0, 12 * len(idx), 12))


def test_scene_file_round_trip(tmp_path):
    from dfpt.scene import CompiledScene

    cs, _ = _scene()
    p = tmp_path / "t.scene"
    cs.write(p)
    back = CompiledScene.read(p)
    for k, v in cs.arrays().items():
        assert np.array_equal(v, getattr(back, k)), k
    # Big-endian DataOutputStream layout: UTF name then int length + elements.
    raw = p.read_bytes()
    assert struct.unpack(">H", raw[:2])[0] == 1 and raw[2:3] == b"t"
    assert struct.unpack(">i", raw[3:7])[0] == cs.point2fs.size
    with pytest.raises(ValueError):
        bad = tmp_path / "bad.scene"
        bad.write_bytes(raw[:40])
        CompiledScene.read(bad)


def test_sky_set_matches_formulas():
    """Sky.set (Sky.java:295-333) restated in Python float64 against the C++ set-up."""
    from dfpt.scene import SkyState

    d, t = (0.5, 0.70710677, 0.5), 2.0
    s = SkyState(d, t).raw
    v = np.asarray(d, np.float32)
    ln = np.float32(np.sqrt(np.float32(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])))
    dw = v / ln
    sz = float(dw[1])
    theta = float(np.float32(math.acos(min(max(sz, -1.0), 1.0))))
    assert s.theta == pytest.approx(theta, abs=0)
    chi = (4.0 / 9.0 - t / 120.0) * (float(np.float32(math.pi)) - 2.0 * theta)
    assert s.zenith_relative_luminance == pytest.approx(((4.0453 * t - 4.9710) * math.tan(chi) - 0.2155 * t + 2.4192) * 1000.0, rel=1e-15)
    assert list(s.perez_relative_luminance) == pytest.approx([0.17872 * t - 1.46303, -0.35540 * t + 0.42749, -0.02266 * t + 5.32505,
                                                               0.12064 * t - 2.57705, -0.06696 * t + 0.37027], rel=1e-15)
    assert list(s.sun_origin) == pytest.approx([float(x) * 10000.0 for x in dw], rel=1e-7)
    assert list(s.sun_direction) == pytest.approx([float(dw[0]), float(dw[2]), float(dw[1])], rel=1e-7)


@pytest.mark.parametrize("kind", ["icosphere", "heightfield"])
def test_sorted_sweep_matches_exhaustive_split_search(kind):
    """The builder's sorted-list split search (prefix bounds over centroid order) picks the same
    splits as the reference's loop over every item per candidate: identical arrays. The grid
    heightfield has many equal centroids (ties at split positions)."""
    from dfpt import scene as sc, synthetic

    def compile_(exhaustive):
        b = sc.SceneBuilder()
        t = b.constant(0.5, 0.5, 0.5)
        if kind == "icosphere":
            pos, idx, _, nrm, uv = synthetic.displaced_icosphere(20, 0.1, 3)
            b.primitive(b.mesh(pos, idx, nrm, uv), b.surface(3, t, t, t))
        else:
            pos, idx = synthetic.heightfield(64, 6.0, 1.0, 3)[:2]
            b.primitive(b.mesh(pos, idx), b.surface(3, t, t, t))
        b.camera((0, 0, 5), (0, 0, 0))
        return b.compile(exhaustive_bvh=exhaustive)

    fast, slow = compile_(False), compile_(True)
    for k, v in fast.arrays().items():
        assert np.array_equal(v, getattr(slow, k)), k

"""CPU: the OBJ loader (ObjectLoader.load restated) on small models written here, and - when the
reference's model files are mounted - on its icosphere.obj, the model BoundingVolumeHierarchyTest
builds (src/main/java/org/dayflower/pathtracer/test/BoundingVolumeHierarchyTest.java)."""
from pathlib import Path

import numpy as np
import pytest
from conftest import reference_resources

F = np.float32

QUAD_MODEL = """# two groups, a quad (fan triangulated) and a triangle
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 0 0 1
vt 0 0
vt 1 0
vt 1 1
vt 0 1
g top
usemtl red
f 1/1 2/2 3/3 4/4
g side
usemtl blue
f 1/4 2/3 5/1
"""


def _builder():
    from dfpt import scene as sc

    return sc.SceneBuilder()


def test_fan_triangulation_groups_and_surfaces():
    from dfpt import obj

    b = _builder()
    seen = []

    def mapper(group, material):
        seen.append((group, material))
        t = b.constant(0.5, 0.5, 0.5)
        return b.surface(3, t, t, t)

    prims = obj.load(b, QUAD_MODEL, surface_mapper=mapper)
    assert len(prims) == 2
    assert seen == [("top", "red"), ("side", "blue")]
    model = obj.ObjModel(QUAD_MODEL)
    assert len(model.faces) == 9  # quad -> 2 triangles (1,2,3), (1,3,4); + 1 triangle
    assert [f[0] for f in model.faces[:6]] == [0, 1, 2, 0, 2, 3]
    b.camera((0, 0, 5), (0, 0, 0))
    cs = b.compile("quad")
    assert cs.triangles.size // 12 == 3


def test_triangle_group_is_its_first_vertex_group():
    """A model vertex keeps the group of its first occurrence, and a triangle goes with the group
    of its first vertex (ObjectLoader.java:141-142): a face of group `side` that starts with a
    vertex first seen in `top` (material `red`) stays in `top` with `red`."""
    from dfpt import obj

    text = QUAD_MODEL.replace("f 1/4 2/3 5/1", "f 1/1 2/2 5/4")
    b = _builder()
    seen = []
    obj.load(b, text, surface_mapper=lambda g, m: seen.append((g, m)) or b.surface(3, b.constant(1, 1, 1), b.constant(0, 0, 0), b.constant(0, 0, 0)))
    assert seen == [("top", "red")]  # one primitive; material also of the first vertex's first occurrence


def test_normals_tangents_and_uv_flip_follow_the_reference_formulas():
    from dfpt import obj

    model = obj.ObjModel(QUAD_MODEL)
    uv, pos, nrm, tng, groups, mats, tris = model.indexed()
    # No vn: per-position normals = normalised sums of normalised face normals (float math).
    p = np.asarray(model.positions, F)
    acc = np.zeros((5, 3), F)
    for a, bb, c in ((0, 1, 2), (0, 2, 3), (0, 1, 4)):
        e0, e1 = p[bb] - p[a], p[c] - p[a]
        n = np.array([e0[1] * e1[2] - e0[2] * e1[1], e0[2] * e1[0] - e0[0] * e1[2], e0[0] * e1[1] - e0[1] * e1[0]], F)
        n = (n / F(np.sqrt(np.float64(n[0] * n[0] + n[1] * n[1] + n[2] * n[2])))).astype(F)
        for k in (a, bb, c):
            acc[k] = (acc[k] + n).astype(F)
    exp = acc / np.sqrt((acc[:, 0] * acc[:, 0] + acc[:, 1] * acc[:, 1] + acc[:, 2] * acc[:, 2]).astype(np.float64)).astype(F)[:, None]
    key = {tuple(v): i for i, v in enumerate(model.positions)}
    for i in range(len(pos)):
        assert np.array_equal(nrm[i], exp[key[tuple(pos[i])]])
    # Tangent z repeats the y expression (the reference's formula).
    assert np.all((tng[:, 2] == tng[:, 1]) | np.isnan(tng[:, 2]))
    # Texture coordinates are flipped to (u, 1 - v) when the triangles are made.
    b = _builder()
    obj.load(b, QUAD_MODEL)
    b.camera((0, 0, 5), (0, 0, 0))
    cs = b.compile("quad")
    v = set(np.round(cs.point2fs.reshape(-1, 2)[:, 1], 6))
    assert v <= {0.0, 1.0}


def test_mixed_tokens_share_index_zero_and_vn_is_used():
    from dfpt import obj

    text = "v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nvn 0 0 -1\nf 1//2 2//2 3\n"
    model = obj.ObjModel(text)
    assert model.has_normal and not model.has_uv
    uv, pos, nrm, tng, groups, mats, tris = model.indexed()
    # "3" has no vn: it takes normal index 0 (the reference's default), the others normal 2.
    assert nrm[0].tolist() == [0.0, 0.0, -1.0] and nrm[2].tolist() == [0.0, 0.0, 1.0]
    assert np.isnan(tng).all()  # no texture coordinates: zero tangents normalised


def test_java_float_parsing():
    from dfpt.obj import _java_float

    assert _java_float("1.5f") == F(1.5)
    assert np.isnan(_java_float("NaN"))
    assert _java_float("-Infinity") == -np.inf
    assert _java_float("0.1") == F(0.1)


ICO = (reference_resources() or Path("missing-reference-resources")) / "model" / "icosphere.obj"


@pytest.mark.skipif(not ICO.exists(), reason="the reference's model files are not mounted")
def test_reference_icosphere_compiles_with_a_valid_bvh():
    from dfpt import obj

    b = _builder()
    prims = obj.load(b, ICO)
    assert len(prims) >= 1
    b.camera((0, 0, 5), (0, 0, 0))
    cs = b.compile("icosphere")
    bvh = cs.bounding_volume_hierarchies
    off, tris = 0, []
    while off < len(bvh):
        typ, nxt = bvh[off], bvh[off + 1]
        assert typ in (1, 2) and (nxt == -1 or nxt > off)
        if typ == 2:
            n = bvh[off + 4]
            tris += list(bvh[off + 5:off + 5 + n])
            off += 5 + n
        else:
            off += 5
    assert sorted(tris) == list(range(0, cs.triangles.size, 12))

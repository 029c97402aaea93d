"""GPU: primitive culling leaves every result of the reference's primitive loop unchanged.

Scenes with 16 or more bounded primitives trace through a BVH over padded world bounds and test
the reachable primitives in primitive order (trace_culled). The checks: strict ray-cast hits
(ids bit-exact, distances and normals bit-exact) equal with culling on and off and equal to the
strict-FP32 oracle's linear loop; path-traced films with the same stream equal (rtol 1e-5, the
float atomics of the shadow contributions); after dfpt_set_transforms moves primitives the
rebuilt structure still agrees.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _params(d):
    from dfpt.kernel import default_params

    p = default_params()
    for k, v in d.items():
        setattr(p, k, v)
    return p


def _copy(cs):
    from dfpt.scene import CompiledScene

    return CompiledScene(cs.name, **{k: v.copy() for k, v in cs.arrays().items()})


def _kernel(cs, sky, params, w, h, culling, strict=False, hits=False):
    """culling: 0 the full loop, 1 a world-box test per primitive, 2 BVH candidates."""
    from dfpt.kernel import RendererKernel

    k = RendererKernel(_copy(cs), sky, params)
    k.update(w, h)
    k.set_strict(strict)
    k.set_record_hits(hits)
    k.set_tuning("primitive_culling", int(culling))
    return k


@pytest.fixture(scope="module")
def many():
    from dfpt import synthetic
    from dfpt.scene import SkyState

    cs, params, (w, h), truth, start = synthetic.inverse_scene(seed=21, width=64, height=48, count=64, phong_every=4)
    return cs, SkyState(truth["sun_direction"], 2.5), params, w, h


def test_culling_modes_selectable(many):
    cs, sky, params, w, h = many
    k = _kernel(cs, sky, params, w, h, 1)
    for mode in (2, 0, 1):
        k.set_tuning("primitive_culling", mode)
        assert k.get_tuning("primitive_culling") == mode
    k.dispose()


@pytest.mark.parametrize("mode", [1, 2])
def test_culled_raycast_bit_exact(many, oracle_mod, mode):
    cs, sky, params, w, h = many
    p = dict(params, renderer_type=3)
    got = []
    for culling in (mode, 0):
        k = _kernel(cs, sky, p, w, h, culling, strict=True, hits=True)
        k.execute(1)
        got.append([a.copy() for a in k.hits()])
        k.dispose()
    for a, b in zip(got[0], got[1]):
        assert np.array_equal(a, b)
    ref = oracle_mod.render(cs, sky, _params(p), w, h, passes=1, precision=32, hits=True)
    prim, typ, off, dist, nrm = got[0]
    assert np.array_equal(prim, ref["hit_prim"])
    assert np.array_equal(off, ref["hit_off"])
    hit = prim >= 0
    assert hit.sum() > 0
    assert np.array_equal(dist[hit].astype(np.float32), ref["hit_dist"][hit].astype(np.float32))


@pytest.mark.parametrize("mode", [1, 2])
def test_culled_path_tracing_equal(many, mode):
    cs, sky, params, w, h = many
    films = []
    for culling in (mode, 0):
        k = _kernel(cs, sky, params, w, h, culling)
        k.set_counting(True)
        k.execute(4)
        f, n = k.film()
        films.append((f.copy(), n.copy()))
        k.dispose()
    assert np.array_equal(films[0][1], films[1][1])
    np.testing.assert_allclose(films[0][0], films[1][0], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("mode", [1, 2])
def test_culling_follows_transform_updates(many, mode):
    cs, sky, params, w, h = many
    p = dict(params, renderer_type=3)
    o2w = cs.primitives_object_to_world.reshape(-1, 16).copy()
    w2o = cs.primitives_world_to_object.reshape(-1, 16).copy()
    # Shift every sphere (primitives 1..) by +0.7 in x: object-to-world adds, world-to-object subtracts.
    o2w[1:, 3] += 0.7
    w2o[1:, 3] -= 0.7 * w2o[1:, 0]
    w2o[1:, 7] -= 0.7 * w2o[1:, 4]
    w2o[1:, 11] -= 0.7 * w2o[1:, 8]
    res = []
    for culling in (mode, 0):
        k = _kernel(cs, sky, p, w, h, culling, strict=True, hits=True)
        k.execute(1)
        before = k.hits()[0].copy()
        k.compiled.primitives_object_to_world = o2w.reshape(-1).astype(np.float32)
        k.compiled.primitives_world_to_object = w2o.reshape(-1).astype(np.float32)
        k.update_primitives()
        k.execute(1)
        res.append((before, k.hits()[0].copy()))
        k.dispose()
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1])
    assert not np.array_equal(res[0][0], res[0][1])  # the move changed what the camera sees

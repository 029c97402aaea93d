"""GPU: the reference's named scenes (dfpt.scenes) through the whole chain - image decoding, OBJ
loading, scene compiler, C-ABI, kernels - against the oracle on the same compiled scenes.

The resource directory is synthetic (tests/_imaging.write_resources: the reference's file names,
generated textures and sphere models), so the scenes' own construction code runs with every
texture type, image textures, normal mapping, glass and reflection. Tolerances:
  ray caster, strict kernels - primitive ids and shape offsets bit-exact, distances rtol 1e-5
      (Terrain_Scene included: the strict kernels evaluate the march's sin in double and round
      once to float, as the reference's Java path and the oracle do);
  path tracer, same RNG stream on both sides, 4 passes - film mean absolute difference < 1% of
      the mean radiance (FP32 transcendentals may part a few paths).
"""
import numpy as np
import pytest

from _imaging import write_resources

pytestmark = pytest.mark.gpu

NAMES = ("Material_Showcase_Scene", "Monkey_Scene", "Girl_Scene", "Wine_Glass_Scene", "House_2_Scene", "Image_Scene",
         "Terrain_Scene")
W, H = 64, 48


@pytest.fixture(scope="module")
def resources(tmp_path_factory):
    return write_resources(str(tmp_path_factory.mktemp("resources")))


def _params(d):
    from dfpt.kernel import default_params

    p = default_params()
    for k, v in d.items():
        setattr(p, k, v)
    return p


@pytest.mark.parametrize("name", NAMES)
def test_named_scene_raycast_and_pathtrace(resources, oracle_mod, name):
    from dfpt import scenes
    from dfpt.kernel import RendererKernel

    cs, sky = scenes.scene_by_name(resources, name, resolution=(W, H))
    rc = dict(renderer_type=3)
    k = RendererKernel(cs, sky, rc)
    k.update(W, H)
    k.set_strict(True)
    k.set_record_hits(True)
    k.execute(1)
    prim, _typ, off, dist, _nrm = (a.copy() for a in k.hits())
    k.dispose()
    ref = oracle_mod.render(cs, sky, _params(rc), W, H, passes=1, precision=32, hits=True)
    assert np.array_equal(prim, ref["hit_prim"])
    assert np.array_equal(off, ref["hit_off"])
    hit = prim >= 0
    assert hit.sum() > 0
    np.testing.assert_allclose(dist[hit], ref["hit_dist"][hit], rtol=1e-5, atol=0)

    pt = dict(renderer_type=2, pt_ray_depth_maximum=5, pt_ray_depth_russian_roulette=3)
    k = RendererKernel(cs, sky, pt)
    k.update(W, H)
    k.set_strict(True)
    k.execute(4)
    film, samples = k.film()
    k.dispose()
    assert (samples == 4).all()
    ref = oracle_mod.render(cs, sky, _params(pt), W, H, passes=4, precision=32)
    a, b = film.reshape(-1).astype(np.float64), ref["film"]
    assert np.isfinite(a).all()
    assert np.abs(a - b).mean() < 0.01 * b.mean(), (np.abs(a - b).mean(), b.mean())

"""GPU: batched rendering against one-scene rendering of the same scenes.

A scene's film from a batch must equal the film of a RendererKernel that rendered the same scene,
sky and seed for `spp` passes: the same paths (the RNG is keyed by pixel and sample) and the same
Kahan sequence per pixel (samples enter the film in sample order). The only freedom is the order
of the float atomics that add sun contributions of one path (a few ulps): rtol 1e-5. The one-scene
path itself is checked against the CPU oracle in test_gpu_parity.py.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (seed, triangles, width, height, spp): uneven sizes; 24x16x5 = 1920 samples spans two 1024-slot
# waves, so waves cut scenes mid-pixel and hold pieces of several scenes.
CASES = [(11, 300, 24, 16, 5), (12, 2000, 40, 30, 3), (13, 800, 32, 32, 7), (14, 5000, 16, 48, 2)]


@pytest.fixture(scope="module")
def batch_scenes():
    from dfpt import synthetic

    out = []
    for seed, tris, w, h, spp in CASES:
        cs, sky, params = synthetic.batch_scene(seed, tris, w, h)
        out.append((cs, sky, params, w, h, spp))
    return out


@pytest.fixture(scope="module")
def single_renders(batch_scenes):
    from dfpt.kernel import RendererKernel

    res = []
    for cs, sky, params, w, h, spp in batch_scenes:
        k = RendererKernel(cs, sky, params)
        k.update(w, h)
        k.execute(spp)
        film, n = k.film()
        res.append((film.copy(), n.copy(), k.get().copy()))
        k.dispose()
    return res


@pytest.mark.parametrize("capacity, defer", [(1024, 0), (4096, 0), (1 << 20, 0), (4096, 1), (1 << 20, 1)])
def test_batch_films_equal_single_scene_films(batch_scenes, single_renders, capacity, defer):
    """Every scene's film equals its single-scene render with waves of any capacity, with the sun
    shadow rays traced per bounce or all bounces' deferred to one launch (float atomics of the
    sun contributions: a few ulps)."""
    from dfpt.batch import BatchRenderer

    b = BatchRenderer()
    for cs, sky, params, w, h, spp in batch_scenes:
        b.add(cs, w, h, spp, sky, params)
    b.set_tuning("wave_capacity", capacity)
    b.set_tuning("shadow_defer", defer)
    assert b.get_tuning("shadow_defer") == defer
    assert b.total_samples == sum(w * h * spp for *_, w, h, spp in batch_scenes)
    b.render()
    b.synchronize()
    assert b.launch_count() > 0
    for i, (film_s, n_s, bgra_s) in enumerate(single_renders):
        film_b, n_b = b.film(i)
        assert np.array_equal(n_b, n_s), i
        assert (n_b == CASES[i][4]).all()
        np.testing.assert_allclose(film_b, film_s, rtol=1e-5, atol=1e-6, err_msg=f"scene {i}")
        assert np.abs(b.get(i).astype(int) - bgra_s.astype(int)).max() <= 1
    b.dispose()


def test_batch_render_range_pieces_equal_whole(batch_scenes):
    """Rendering the global sample sequence in uneven pieces gives the films of one render."""
    from dfpt.batch import BatchRenderer

    def make():
        b = BatchRenderer()
        for cs, sky, params, w, h, spp in batch_scenes:
            b.add(cs, w, h, spp, sky, params)
        b.set_tuning("wave_capacity", 2048)
        return b

    whole = make()
    whole.render()
    pieces = make()
    pieces.clear()
    total = pieces.total_samples
    cut = [0, 1000, 2048, 5000, total]
    for a, c in zip(cut[:-1], cut[1:]):
        pieces.render_range(a, c - a)
    pieces.resolve()
    pieces.synchronize()
    for i in range(len(batch_scenes)):
        fa, na = whole.film(i)
        fb, nb = pieces.film(i)
        assert np.array_equal(na, nb)
        np.testing.assert_allclose(fa, fb, rtol=1e-5, atol=1e-6)


def test_batch_autotuner_picks_a_candidate(batch_scenes):
    from dfpt.autotune import tune_batch
    from dfpt.batch import BatchRenderer

    b = BatchRenderer()
    for cs, sky, params, w, h, spp in batch_scenes:
        b.add(cs, w, h, spp, sky, params)
    r = tune_batch(b, capacities=(1024, 4096), configs=(0, 2))
    assert r["best"]["trace_config"] in (0, 2)
    assert b.get_tuning("wave_capacity") == r["best"]["wave_capacity"]
    b.render()
    b.synchronize()
    _, n = b.film(0)
    assert (n == CASES[0][4]).all()


def test_batch_rejects_unsupported_scenes(batch_scenes):
    from dfpt._lib import DfptError
    from dfpt.batch import BatchRenderer

    cs, sky, params, w, h, spp = batch_scenes[0]
    b = BatchRenderer()
    b.add(cs, w, h, spp, sky, params)
    with pytest.raises(DfptError):
        b.add(cs, w, h, spp, sky, dict(params, pt_ray_depth_maximum=params["pt_ray_depth_maximum"] + 1))
    with pytest.raises(DfptError):
        b.add(cs, w, h, spp, sky, dict(params, rng_kind=1))
    with pytest.raises(DfptError):
        b.add(cs, w, h, spp, sky, dict(params, renderer_type=3))
    with pytest.raises(DfptError):
        b.add(cs, w, h, 0, sky, params)
    with pytest.raises(DfptError):
        b.set_tuning("wave_capacity", 10)
    assert b.get_tuning("scenes") == 1

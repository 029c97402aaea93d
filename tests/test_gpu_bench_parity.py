"""GPU: the configuration bench.py measures, checked against the FP64 oracle.

Bench mode = the fast (FMA) kernel set, passes run in waves of up to 64 through the wave kernels
with pixel-major slots, traversal configuration 16 (the compact pair walk), rays binned between
bounces, every bounce's sun shadow rays deferred to one launch per wave, and the primitive culling
the autotuner picks on the large scenes. The scenes are the benchmark generators: the sphere scene
at its full 512x512 (with a two-colour checkerboard), and the mesh and instances scenes scaled down
so the oracle finishes in seconds (same generators; fewer triangles, fewer pixels). The batch case
renders four scenes of uneven size in one BatchRenderer.

Per case, two checks (tests/_parity.py; its statistics are pinned on the CPU by
tests/test_parity_statistic.py):
  same stream   - GPU and oracle draw the same random numbers (same seed and passes): relative RMSE
                  <= 1% and image means within 0.1% (only FP32/FMA arithmetic separates the two);
  converged     - the GPU film at N spp against an independent oracle render at M = 4N spp:
                  converged relative RMSE <= 1% (squared difference minus the noise term, within
                  3 standard errors of that estimate), fewer
                  than 1% of the pixel channels with |z| > 4, |mean z| < 0.2 (or 4 standard
                  errors); over 8 x 8 pixel blocks for the scene with HDR emitters.
Thin-lens depth of field and the fisheye lens (GPURendererKernel.java:643-704) are checked in the
strict ray caster (hit ids bit-exact) and in bench mode. The interactive frame loop's mode (one
pass per call through the tail launch) is checked on the scaled mesh scene the same way.
"""
import numpy as np
import pytest

from _parity import assert_converged, film_stats, oracle_pair, same_stream_mean_ratio, same_stream_rel_rmse

pytestmark = pytest.mark.gpu

BENCH_TUNING = {"wide_samples": 64, "ray_sort": 1, "shadow_defer": 1, "trace_config": 16}
SEED_SAME, SEED_ORACLE = 0x5EED0001, 0x0AC1E002


def _bench_kernel(scene, sky, params, w, h, seed, culling=0, tuning=BENCH_TUNING):
    from dfpt.kernel import RendererKernel

    k = RendererKernel(scene, sky, params)
    k.update(w, h)
    k.set_strict(False)
    for key, v in tuning.items():
        k.set_tuning(key, v)
    k.set_tuning("primitive_culling", culling)
    k.set_seed(seed)
    return k


def _render(scene, sky, params, w, h, n, seed, culling=0, tuning=BENCH_TUNING):
    k = _bench_kernel(scene, sky, params, w, h, seed, culling, tuning)
    assert all(k.get_tuning(key) == v for key, v in tuning.items())
    k.execute(n)
    film, samples = k.film()
    film, samples = film.copy(), samples.copy()
    k.dispose()
    # Every pixel holds n samples, except where the fisheye lens rejected a pass's ray: that pass
    # set the pixel black with a count of 1 (filmSetColor), and later passes add to it.
    assert (samples <= n).all() and (samples >= 1).all()
    assert (samples == n).mean() > 0.5
    assert np.isfinite(film).all()
    return film


def _check(oracle_mod, scene, sky, params, w, h, n, cullings=(0,), mask=None, block=None, z_tail=0.01, tuning=BENCH_TUNING):
    """`mask`: the pixels compared (all by default); the fisheye case leaves out the pixels whose
    jittered rays fall on both sides of the lens circle (their film restarts at each rejection,
    so their mean is not the plain mean of their samples). `block`: the converged statistics over
    k x k pixel blocks instead of pixels (scenes with HDR emitters)."""
    same, full = oracle_pair(oracle_mod, scene, sky, params, w, h, n, 4 * n, SEED_ORACLE)
    keep = np.ones(w * h, bool) if mask is None else mask

    def px(a):
        return np.asarray(a, np.float64).reshape(-1, 3)[keep].reshape(-1)

    ref = {k: px(full[k]) for k in ("sum", "sumsq", "sum1", "sumsq1")}
    ref["half"] = full["half"]
    out = {}
    for c in cullings:
        a_same = _render(scene, sky, params, w, h, n, SEED_ORACLE, c, tuning)
        rel = same_stream_rel_rmse(px(a_same), px(same["film"]))
        ratio = same_stream_mean_ratio(px(a_same), px(same["film"]))
        assert rel <= 0.01 and abs(ratio) <= 1e-3, (c, rel, ratio)
        a = _render(scene, sky, params, w, h, n, SEED_SAME, c, tuning)
        s = film_stats(px(a), n, ref, 4 * n, block=None if block is None else (h, w, block))
        assert_converged(s, z_tail=z_tail)
        out[c] = (rel, s)
    return out


def test_sphere_scene_512_bench_mode(oracle_mod):
    from dfpt import synthetic

    scene, sky, params, (w, h) = synthetic.sphere_scene(0, 512, 512, checker_colors=((0.8, 0.8, 0.8), (0.1, 0.1, 0.1)))
    _check(oracle_mod, scene, sky, params, w, h, 64)


def test_mesh_scene_scaled_bench_mode(oracle_mod):
    """mesh_scene's generator at frequency 30 (18,000 icosphere triangles in Lambertian and Phong
    regions) over a 128x128 heightfield, 192x108, depth 8, ACES."""
    from dfpt import synthetic

    scene, sky, params, (w, h) = synthetic.mesh_scene(width=192, height=108, frequency=30, grid=128)
    _check(oracle_mod, scene, sky, params, w, h, 128)


# The interactive frame loop's mode: one pass per call (plain passes) in pixel-tile order, the tail
# launch from bounce t compiled for b resident blocks, the deferred shadow rays binned by origin cell.
FRAME_TUNING = {"wide_samples": 1, "trace_config": 16, "pixel_tiles": 1, "pass_shadow_sort": 1}


@pytest.mark.parametrize("tail_bounce,tail_blocks", [(1, 4), (0, 3)])
def test_mesh_scene_scaled_frame_mode(oracle_mod, tail_bounce, tail_blocks):
    """The scaled mesh scene (as above) rendered pass by pass in the frame loop's configuration."""
    from dfpt import synthetic

    scene, sky, params, (w, h) = synthetic.mesh_scene(width=192, height=108, frequency=30, grid=128)
    tuning = dict(FRAME_TUNING, tail_bounce=tail_bounce, tail_blocks=tail_blocks)
    _check(oracle_mod, scene, sky, params, w, h, 128, tuning=tuning)


def test_instances_scene_scaled_bench_mode(oracle_mod):
    """instances_scene's generator with 2,880-triangle icospheres (40 instances, Glass, Reflection and
    Lambertian) and 100 of its HDR area lights (triangle primitives, emission U(1, 20)), 192x108,
    with primitive culling modes 1 and 2. The lights are found by BSDF sampling alone, so single
    pixels' radiance is heavy-tailed at 512 spp: the converged statistics run over 8 x 8 pixel
    blocks; the same-stream check stays per pixel."""
    from _parity import HDR_Z_TAIL
    from dfpt import synthetic

    scene, sky, params, (w, h) = synthetic.instances_scene(width=192, height=108, frequency=12, lights=100)
    _check(oracle_mod, scene, sky, params, w, h, 512, cullings=(1, 2), block=8, z_tail=HDR_Z_TAIL)


# (seed, triangles, width, height, spp): uneven sizes and sample counts in one batch.
BATCH = [(21, 2000, 64, 64, 64), (22, 20000, 96, 72, 32), (23, 300, 48, 32, 128), (24, 60000, 80, 60, 64)]


def test_batch_scenes_against_oracle(oracle_mod):
    """Each scene of a batch (waves of 2^20 slots over all four scenes, configuration 16, binning)
    against the oracle: its film drew the scene's own seed from sample 0, so it is compared with the
    oracle's same-seed render (same stream) and with an independent 4x-spp render (converged)."""
    from dfpt import synthetic
    from dfpt.batch import BatchRenderer

    scenes = [synthetic.batch_scene(seed, tris, w, h) + (w, h, spp) for seed, tris, w, h, spp in BATCH]
    b = BatchRenderer()
    for cs, sky, params, w, h, spp in scenes:
        b.add(cs, w, h, spp, sky, params)
    b.set_tuning("wave_capacity", 1 << 20)
    b.set_tuning("trace_config", 16)
    b.set_tuning("ray_sort", 1)
    b.render()
    b.synchronize()
    films = [b.film(i) for i in range(len(scenes))]
    b.dispose()
    for (cs, sky, params, w, h, spp), (film, n) in zip(scenes, films):
        assert (n == spp).all()
        same, _ = oracle_pair(oracle_mod, cs, sky, params, w, h, spp, spp + 1, params["seed"])
        assert same_stream_rel_rmse(film, same["film"]) <= 0.01
        assert abs(same_stream_mean_ratio(film, same["film"])) <= 1e-3
        _, full = oracle_pair(oracle_mod, cs, sky, params, w, h, spp, 4 * spp, SEED_ORACLE)
        assert_converged(film_stats(film, spp, full, 4 * spp))


# ---- thin lens and fisheye ---------------------------------------------------------------------

def _lens_scene(kind):
    """small_mesh_scene with a thin lens (aperture 0.25, focal distance 10) or the fisheye lens."""
    from dfpt import synthetic

    scene, sky, params, (w, h) = synthetic.small_mesh_scene(width=96, height=64)
    scene = scene.copy()
    if kind == "thin_lens":
        scene.camera[0] = 0.25
        scene.camera[6] = 10.0
    else:
        scene.camera[18] = 2.0
    return scene, sky, params, (w, h)


def _params(d):
    from dfpt.kernel import default_params

    p = default_params()
    for k, v in d.items():
        setattr(p, k, v)
    return p


@pytest.mark.parametrize("kind", ["thin_lens", "fisheye"])
def test_lens_raycast_bit_exact(oracle_mod, kind):
    from dfpt.kernel import RendererKernel

    scene, sky, params, (w, h) = _lens_scene(kind)
    rc = dict(params, renderer_type=3)
    k = RendererKernel(scene, sky, rc)
    k.update(w, h)
    k.set_strict(True)
    k.set_record_hits(True)
    k.execute(3)
    prim, typ, off, dist, nrm = (a.copy() for a in k.hits())
    film, _ = k.film()
    film = film.copy()
    k.dispose()
    ref = oracle_mod.render(scene, sky, _params(rc), w, h, passes=3, precision=32, hits=True)
    assert np.array_equal(prim, ref["hit_prim"])
    assert np.array_equal(typ, ref["hit_type"])
    assert np.array_equal(off, ref["hit_off"])
    hit = prim >= 0
    assert hit.sum() > 100
    np.testing.assert_allclose(dist[hit], ref["hit_dist"][hit], rtol=1e-5, atol=0)
    np.testing.assert_allclose(nrm[hit], ref["hit_normal"].reshape(-1, 3)[hit], rtol=1e-5, atol=1e-6)
    if kind == "fisheye":
        # Pixels outside the lens circle are rejected (no ray, black film) on both sides.
        ys, xs = np.divmod(np.arange(w * h), w)
        sx = 2.0 * (xs + 0.5) / (w - 1) - 1.0
        sy = 2.0 * (ys + 0.5) / (h - 1) - 1.0
        outside = sx * sx + sy * sy > 1.02
        assert outside.sum() > 0
        assert (prim[outside] == -1).all()
        assert (film.reshape(-1, 3)[outside] == 0).all()
        assert (ref["film"].reshape(-1, 3)[outside] == 0).all()
    else:
        # The lens moves the ray origins: primary hits differ from the pinhole camera's.
        from dfpt import synthetic

        pin, *_ = synthetic.small_mesh_scene(width=96, height=64)
        ref_pin = oracle_mod.render(pin, sky, _params(rc), w, h, passes=3, precision=32, hits=True)
        assert not np.array_equal(ref_pin["hit_dist"], ref["hit_dist"])


def _fisheye_unambiguous(w, h):
    """Pixels whose tent-jittered sample points (offsets in (-1, 1) pixel) all fall inside, or all
    outside, the fisheye lens circle, with a margin."""
    ys, xs = np.divmod(np.arange(w * h), w)
    lo_x, hi_x = 2.0 * (xs - 1.0) / (w - 1) - 1.0, 2.0 * (xs + 1.0) / (w - 1) - 1.0
    lo_y, hi_y = 2.0 * (ys - 1.0) / (h - 1) - 1.0, 2.0 * (ys + 1.0) / (h - 1) - 1.0
    far = np.maximum(lo_x ** 2, hi_x ** 2) + np.maximum(lo_y ** 2, hi_y ** 2)
    near = np.where(lo_x * hi_x <= 0, 0.0, np.minimum(lo_x ** 2, hi_x ** 2)) + \
        np.where(lo_y * hi_y <= 0, 0.0, np.minimum(lo_y ** 2, hi_y ** 2))
    return (far < 0.98) | (near > 1.02)


@pytest.mark.parametrize("kind", ["thin_lens", "fisheye"])
def test_lens_pathtrace_bench_mode(oracle_mod, kind):
    scene, sky, params, (w, h) = _lens_scene(kind)
    mask = _fisheye_unambiguous(w, h) if kind == "fisheye" else None
    if mask is not None:
        assert mask.mean() > 0.8
    _check(oracle_mod, scene, sky, params, w, h, 128, mask=mask)

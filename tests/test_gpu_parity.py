"""GPU parity: the CUDA core through the C-ABI against the CPU oracle on the same inputs.

Tolerances (written per test):
  ray caster, strict kernels  - primitive/shape ids bit-exact, distance and normal rtol 1e-5;
  path tracer, same RNG stream- film mean absolute difference < 1% of the mean radiance (the two
                                sides trace the same paths; FP32 transcendentals may diverge a few);
  path tracer vs FP64 oracle  - relative RMSE <= 1% of the converged radiance and per-pixel
                                z-scores against the oracle's sample variance (tests/_parity.py);
                                the bench configuration is checked in test_gpu_bench_parity.py.
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


def _kernel(scene, sky, params, w, h, strict=False, hits=False):
    from dfpt.kernel import RendererKernel

    k = RendererKernel(scene, sky, params)
    k.update(w, h)
    k.set_strict(strict)
    k.set_record_hits(hits)
    return k


@pytest.fixture(scope="module")
def scenes():
    from dfpt import synthetic

    return {
        "spheres": synthetic.sphere_scene(0, 96, 64),
        "meshes": synthetic.small_mesh_scene(width=96, height=64),
    }


@pytest.mark.parametrize("name", ["spheres", "meshes"])
def test_raycast_hits_bit_exact(scenes, oracle_mod, name):
    scene, sky, params, (w, h) = scenes[name]
    params = dict(params, renderer_type=3)
    k = _kernel(scene, sky, params, w, h, strict=True, hits=True)
    k.execute(1)
    prim, typ, off, dist, nrm = k.hits()
    ref = oracle_mod.render(scene, sky, _params(params), w, h, passes=1, precision=32, hits=True, want_bgra=True)
    assert np.array_equal(prim, ref["hit_prim"])
    assert np.array_equal(typ, ref["hit_type"])
    assert np.array_equal(off, ref["hit_off"])
    hit = prim >= 0
    assert hit.sum() > 0
    np.testing.assert_allclose(dist[hit], ref["hit_dist"][hit], rtol=1e-5, atol=0)
    np.testing.assert_allclose(nrm[hit], ref["hit_normal"].reshape(-1, 3)[hit], rtol=1e-5, atol=1e-6)
    assert np.array_equal(k.primitive_offsets(), ref["primitive_offsets"])
    # The displayed image: Phong shading quantised to 8 bits, then tone map and sRGB.
    bgra = k.get().astype(np.int32)
    assert np.abs(bgra - ref["bgra"].astype(np.int32)).max() <= 1
    k.dispose()


@pytest.mark.parametrize("name", ["spheres", "meshes"])
def test_raycast_fast_kernels_ids(scenes, oracle_mod, name):
    """Ray-casting mode runs the strict kernels even when the fast set is selected: its hit ids are
    bit-exact whatever the kernel-set choice."""
    scene, sky, params, (w, h) = scenes[name]
    params = dict(params, renderer_type=3)
    k = _kernel(scene, sky, params, w, h, strict=False, hits=True)
    k.execute(1)
    prim, typ, off, dist, _ = k.hits()
    ref = oracle_mod.render(scene, sky, _params(params), w, h, passes=1, precision=32, hits=True)
    assert np.array_equal(prim, ref["hit_prim"])
    assert np.array_equal(off, ref["hit_off"])
    hit = prim >= 0
    np.testing.assert_allclose(dist[hit], ref["hit_dist"][hit], rtol=1e-5, atol=0)
    k.dispose()


@pytest.mark.parametrize("name", ["spheres", "meshes"])
def test_pathtrace_same_stream(scenes, oracle_mod, name):
    scene, sky, params, (w, h) = scenes[name]
    k = _kernel(scene, sky, params, w, h, strict=True)
    k.execute(8)
    film, samples = k.film()
    assert (samples == 8).all()
    ref = oracle_mod.render(scene, sky, _params(params), w, h, passes=8, precision=32)
    a, b = film.reshape(-1).astype(np.float64), ref["film"]
    assert np.abs(a - b).mean() < 0.01 * b.mean()
    assert np.mean(np.abs(a - b) < 1e-4 * np.maximum(1.0, np.abs(b))) > 0.9
    k.dispose()


@pytest.mark.parametrize("name", ["spheres", "meshes"])
def test_pathtrace_converged_rmse_and_zscores(scenes, oracle_mod, name):
    """Fast kernels, one pass at a time: the film at 256 spp against an independent FP64 oracle
    render at 1024 spp (converged relative RMSE <= 1% and z-scores, tests/_parity.py), and with
    the oracle's own seed against its first 256 passes (same stream: relative RMSE <= 1%)."""
    from _parity import assert_converged, film_stats, oracle_pair, same_stream_rel_rmse

    scene, sky, params, (w, h) = scenes[name]
    spp = 256
    k = _kernel(scene, sky, params, w, h, strict=False)
    k.set_tuning("wide_samples", 1)
    k.set_seed(12345)
    k.execute(spp)
    film, _ = k.film()
    a = film.reshape(-1).astype(np.float64)
    same, full = oracle_pair(oracle_mod, scene, sky, params, w, h, spp, 4 * spp, seed=777)
    assert_converged(film_stats(a, spp, full, 4 * spp))
    k.dispose()
    k = _kernel(scene, sky, params, w, h, strict=False)
    k.set_tuning("wide_samples", 1)
    k.set_seed(777)
    k.execute(spp)
    film2, _ = k.film()
    assert same_stream_rel_rmse(film2, same["film"]) <= 0.01
    k.dispose()


def test_lcg_stream_matches_oracle(scenes, oracle_mod):
    scene, sky, params, (w, h) = scenes["spheres"]
    from dfpt.kernel import RNG_LCG

    k = _kernel(scene, sky, params, w, h, strict=True)
    seed = 777
    k.set_seed(seed, RNG_LCG)
    k.execute(4)
    film, _ = k.film()
    mask = (1 << 64) - 1

    def splitmix(x):
        x = (x + 0x9E3779B97F4A7C15) & mask
        x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & mask
        x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & mask
        return x ^ (x >> 31)

    state = np.array([splitmix((seed + i) & mask) for i in range(w * h)], dtype=np.uint64)
    p = _params(dict(params, rng_kind=RNG_LCG, seed=seed))
    ref = oracle_mod.render(scene, sky, p, w, h, passes=4, precision=32, rng_state=state)
    a, b = film.reshape(-1).astype(np.float64), ref["film"]
    assert np.abs(a - b).mean() < 0.01 * b.mean()
    k.dispose()


@pytest.mark.parametrize("mode", [1, 4, 5, 6])
def test_other_renderers(scenes, oracle_mod, mode):
    scene, sky, params, (w, h) = scenes["meshes"]
    params = dict(params, renderer_type=mode)
    k = _kernel(scene, sky, params, w, h, strict=True)
    k.execute(2)
    film, _ = k.film()
    ref = oracle_mod.render(scene, sky, _params(params), w, h, passes=2, precision=32)
    a, b = film.reshape(-1).astype(np.float64), ref["film"]
    assert np.abs(a - b).mean() <= 0.01 * max(b.mean(), 1e-3)
    assert np.mean(np.abs(a - b) <= 2.0 / 255.0 + 1e-4) > 0.97
    k.dispose()


def test_wireframes_and_selection(scenes, oracle_mod):
    scene, sky, params, (w, h) = scenes["meshes"]
    params = dict(params, renderer_type=3, wireframes=1)
    k = _kernel(scene, sky, params, w, h, strict=True)
    k.execute(1)
    film, samples = k.film()
    ref = oracle_mod.render(scene, sky, _params(params), w, h, passes=1, precision=32, want_bgra=True)
    black_gpu = (film.reshape(-1, 3).sum(1) == 0)
    black_ref = (ref["film"].reshape(-1, 3).sum(1) == 0)
    assert (black_gpu != black_ref).mean() < 0.002
    # Selection tint: select the primitive under the centre pixel.
    k.toggle_primitive_selection(w // 2, h // 2)
    sel = k.get_selected_primitive_index()
    k.execute(1)
    offs = k.primitive_offsets()
    if sel >= 0:
        img = k.get().reshape(h, w, 4)
        assert img[h // 2, w // 2, 1] >= 200  # green channel tinted
    assert offs[(h // 2) * w + w // 2] == (sel * 3 if sel >= 0 else -1)
    k.dispose()


COMPACT_PAIR_CONFIG = 16  # the compact pair walk, whose stack depth the pair_stack key limits


def test_trace_configs_agree(scenes):
    """Every traversal launch configuration visits the same nodes and finds the same hits (a fresh
    handle per configuration, so every run draws from pass 0 of the same stream). The compact pair
    walk also runs with 1- and 2-entry stacks, which drop stack entries on most walks: its hits
    stay exact, and its node counter may count a right child twice (the threaded continuation
    re-tests one its parent's step rejected), never fewer. The sun shadow rays walked in another
    configuration than the closest hits (shadow_config) change nothing either."""
    scene, sky, params, (w, h) = scenes["meshes"]
    ref = None
    n = None
    cases = None
    cfg = 0
    while cases is None or cfg < len(cases):
        k = _kernel(scene, sky, dict(params, renderer_type=2), w, h, strict=False, hits=True)
        if cases is None:
            n = k.get_tuning("trace_configs")
            assert n > COMPACT_PAIR_CONFIG
            cases = [(c, 8, -1) for c in range(n)] + [(COMPACT_PAIR_CONFIG, 1, -1), (COMPACT_PAIR_CONFIG, 2, -1)]
            cases += [(COMPACT_PAIR_CONFIG, 8, 0), (COMPACT_PAIR_CONFIG, 8, 1), (0, 8, COMPACT_PAIR_CONFIG)]
        k.set_tuning("trace_config", cases[cfg][0])
        k.set_tuning("pair_stack", cases[cfg][1])
        k.set_tuning("shadow_config", cases[cfg][2])
        k.set_counting(True)
        k.execute(1)
        film, _ = k.film()
        got = (k.hits()[0].copy(), film.copy(), k.counters().copy())
        k.dispose()
        if ref is None:
            ref = got
        else:
            assert np.array_equal(got[0], ref[0]), cases[cfg]
            if cases[cfg][1] == 8:
                assert np.array_equal(got[2], ref[2]), (cases[cfg], got[2], ref[2])  # same segments, nodes and triangles
            else:
                same = [0, 1, 3, 5]  # segments and triangles
                assert np.array_equal(got[2][same], ref[2][same]), (cases[cfg], got[2], ref[2])
                assert got[2][2] >= ref[2][2] and got[2][4] >= ref[2][4], (cases[cfg], got[2], ref[2])
            # Shadow contributions of one path are added with float atomics in any order: a few ulps.
            assert np.allclose(got[1], ref[1], rtol=1e-5, atol=1e-6), (cases[cfg], np.abs(got[1] - ref[1]).max())
        cfg += 1


@pytest.mark.parametrize("name", ["spheres", "meshes"])
def test_wide_passes_equal_pass_by_pass(scenes, name):
    """dfpt_render(h, n) with wide passes (k passes per wave through the batch stages) gives the
    film of n single passes: same samples per pixel, same Kahan order; float atomics of the sun
    contributions leave a few ulps (rtol 1e-5). A clear between calls restarts both the same way;
    the selection buffer and the image come from the last (normal) pass in both. The same holds
    with the shadow rays of all bounces deferred to one launch, and with the shadow rays walked in
    another traversal configuration (shadow_config: any hit is the same hit-or-miss)."""
    scene, sky, params, (w, h) = scenes[name]
    out = []
    # (passes per wave, ray binning, deferred shadow rays, shadow rays' traversal configuration)
    for wide, sort, defer, scfg in ((1, 0, 0, -1), (8, 1, 0, -1), (8, 0, 0, -1), (8, 1, 1, -1), (8, 0, 1, -1),
                                    (8, 1, 1, 0), (8, 0, 0, 1), (1, 0, 0, 11)):
        k = _kernel(scene, sky, dict(params, renderer_type=2), w, h)
        k.set_tuning("wide_samples", wide)
        k.set_tuning("ray_sort", sort)
        k.set_tuning("shadow_defer", defer)
        k.set_tuning("shadow_config", scfg)
        k.execute(13)
        k.clear()
        k.execute(11)
        film, n = k.film()
        out.append((film.copy(), n.copy(), k.primitive_offsets().copy(), k.get().copy()))
        k.dispose()
    fa, na, pa, ba = out[0]
    assert (na == 11).sum() > 0.9 * na.size
    for fb, nb, pb, bb in out[1:]:
        assert np.array_equal(na, nb)
        np.testing.assert_allclose(fa, fb, rtol=1e-5, atol=1e-6)
        assert np.array_equal(pa, pb)
        assert np.abs(ba.astype(int) - bb.astype(int)).max() <= 1


def test_obj_model_raycast_bit_exact(oracle_mod):
    """A scene loaded from OBJ text (fan-triangulated quads, two groups, computed normals and
    tangents) through the whole chain: loader -> compiler -> C-ABI -> strict ray caster, hit ids
    bit-exact and distances within rtol 1e-5 of the strict-FP32 oracle."""
    from dfpt import obj, scene as sc
    from dfpt.synthetic import geodesic_sphere

    pos, idx = geodesic_sphere(6)[:2]
    lines = [f"v {x:.6f} {y:.6f} {z:.6f}" for x, y, z in pos]
    lines += ["vt 0 0", "vt 1 0", "vt 0.5 1", "g top"]
    half = len(idx) // 2
    for k, (a, b, c) in enumerate(idx):
        if k == half:
            lines.append("g bottom")
        lines.append(f"f {a + 1}/1 {b + 1}/2 {c + 1}/3")
    lines += ["v -3 -1.2 -3", "v 3 -1.2 -3", "v 3 -1.2 3", "v -3 -1.2 3", "g floor", f"f {len(pos) + 1} {len(pos) + 2} {len(pos) + 3} {len(pos) + 4}"]
    b = sc.SceneBuilder()
    white, black = b.constant(0.8, 0.8, 0.8), b.constant(0, 0, 0)
    mats = {}

    def mapper(group, material):
        if group not in mats:
            mats[group] = b.surface(3, b.constant(*(0.3 + 0.2 * len(mats),) * 3), black, black)
        return mats[group]

    prims = obj.load(b, "\n".join(lines), surface_mapper=mapper, position=(0.2, 0.1, 0.0))
    assert len(prims) >= 2
    b.camera((0, 1.5, 4.5), (0, 0, 0), 60.0, (64, 48))
    cs = b.compile("obj_scene")
    sky = sc.SkyState((0.3, 0.9, 0.3), 2.5)
    params = dict(renderer_type=3, pt_ray_depth_maximum=5, pt_ray_depth_russian_roulette=3)
    k = _kernel(cs, sky, params, 64, 48, strict=True, hits=True)
    k.execute(1)
    prim, typ, off, dist, nrm = k.hits()
    ref = oracle_mod.render(cs, sky, _params(params), 64, 48, passes=1, precision=32, hits=True)
    assert np.array_equal(prim, ref["hit_prim"])
    assert np.array_equal(off, ref["hit_off"])
    hit = prim >= 0
    assert hit.sum() > 100
    np.testing.assert_allclose(dist[hit], ref["hit_dist"][hit], rtol=1e-5, atol=0)


def test_pixel_tile_order_keeps_every_pixel(scenes):
    """Plain passes in 8 x 4 pixel-tile slot order (pixel_tiles) trace each pixel's sample from the
    same counter-based stream as row order: the same films (sun contributions are added with float
    atomics: a few ulps), hit records and selection buffer."""
    scene, sky, params, (w, h) = scenes["meshes"]
    assert w % 8 == 0 and h % 4 == 0
    out = []
    for tiles in (0, 1):
        k = _kernel(scene, sky, dict(params, renderer_type=2), w, h, strict=False, hits=True)
        k.set_tuning("wide_samples", 1)
        k.set_tuning("pixel_tiles", tiles)
        assert k.get_tuning("pixel_tiles") == tiles
        k.execute(3)
        film, samples = k.film()
        out.append((film.copy(), samples.copy(), [x.copy() for x in k.hits()], k.primitive_offsets().copy()))
        k.dispose()
    (f0, s0, h0, p0), (f1, s1, h1, p1) = out
    assert (s0 == 3).all() and (s1 == 3).all()
    assert np.allclose(f0, f1, rtol=1e-5, atol=1e-6), np.abs(f0 - f1).max()
    for a, b in zip(h0, h1):
        assert np.array_equal(a, b)
    assert np.array_equal(p0, p1)


@pytest.mark.parametrize("rng_kind,hits", [(0, False), (1, True)])
def test_native_frame_tuner_leaves_film_and_streams(scenes, rng_kind, hits):
    """dfpt_tune_frame renders one-pass frames with every candidate launch structure, then puts back
    the film, image, selection buffer, per-pixel random states (the LCG's too), primary-hit records
    and pass counter: a handle that tuned between two renders ends with the film, selection buffer
    and hit records of a handle that never tuned (films within the ulps of float atomics), and the
    tunings it leaves are values the C-ABI accepts."""
    scene, sky, params, (w, h) = scenes["meshes"]
    params = dict(params, renderer_type=2, pt_ray_depth_maximum=6, pt_ray_depth_russian_roulette=3, rng_kind=rng_kind)
    out = []
    for tune in (False, True):
        k = _kernel(scene, sky, params, w, h, strict=False, hits=hits)
        cfg0 = k.get_tuning("trace_config")
        k.execute(3)
        if tune:
            ms = k.tune_frame_native(2)
            assert ms > 0
            assert k.get_tuning("trace_config") in (cfg0, 16, 17)
            assert -1 <= k.get_tuning("tail_bounce") <= 4 and k.get_tuning("tail_blocks") in (2, 3, 4)
            assert k.get_tuning("pass_shadow_sort") in (0, 1)
        k.execute(2)
        film, n = k.film()
        out.append((film.copy(), n.copy(), k.primitive_offsets().copy(), [a.copy() for a in k.hits()] if hits else []))
        k.dispose()
    (fa, na, pa, ha), (fb, nb, pb, hb) = out
    assert (na == 5).all() and np.array_equal(na, nb)
    np.testing.assert_allclose(fb, fa, rtol=1e-5, atol=1e-6)
    assert np.array_equal(pa, pb)
    for x, y in zip(ha, hb):
        assert np.array_equal(x, y)


def test_native_frame_tuner_picks_culling_with_the_same_film():
    """On a scene with many bounded primitives (64 spheres on a plane) the C-ABI frame tuner also
    times the primitive culling modes; whichever it keeps, renders after it equal a handle that never
    tuned (every culling mode gives the same hits)."""
    from dfpt import synthetic

    scene, sky, params, (w, h) = synthetic.spheres_on_plane(width=64, height=48, count=64)
    out = []
    for tune in (False, True):
        k = _kernel(scene, sky, dict(params), w, h, strict=False)
        k.execute(2)
        if tune:
            assert k.tune_frame_native(2) > 0
            assert k.get_tuning("primitive_culling") in (0, 1, 2)
        k.execute(2)
        film, n = k.film()
        out.append((film.copy(), n.copy(), k.primitive_offsets().copy()))
        k.dispose()
    (fa, na, pa), (fb, nb, pb) = out
    assert np.array_equal(na, nb) and (na == 4).all()
    np.testing.assert_allclose(fb, fa, rtol=1e-5, atol=1e-6)
    assert np.array_equal(pa, pb)


@pytest.mark.parametrize("name", ["spheres", "meshes"])
def test_tail_launch_equals_per_bounce_launches(scenes, name):
    """The tail kernel (tail_bounce t: bounces t .. depth-1 and the final any-hit of each path in
    one launch, from the camera rays on with t = 0, compiled for 2, 3 or 4 resident blocks) takes
    every path through the same steps as a launch per bounce (t = -1): the same films (sun contributions are added with float atomics: a few ulps),
    the same segments, nodes and triangles, the same selection buffer - with the deferred shadow
    rays binned by origin cell before their launch (pass_shadow_sort) or not, and with bounce 1's
    rays binned by direction and origin cell (pass_ray_sort, the grid's bits) or not."""
    scene, sky, params, (w, h) = scenes[name]
    params = dict(params, renderer_type=2, pt_ray_depth_maximum=6, pt_ray_depth_russian_roulette=3)
    ref = None
    for tb, sort, rays, blocks in ((-1, 0, 0, 2), (1, 0, 0, 2), (2, 0, 0, 2), (5, 0, 0, 2), (-1, 1, 0, 2),
                                   (2, 1, 0, 2), (1, 1, 0, 3), (2, 1, 0, 4), (0, 0, 0, 2), (0, 1, 0, 4),
                                   (-1, 0, 9, 2), (1, 1, 12, 3), (2, 1, 6, 2), (-1, 1, 15, 2)):
        k = _kernel(scene, sky, params, w, h, strict=False)
        k.set_tuning("wide_samples", 1)
        k.set_tuning("tail_blocks", blocks)
        k.set_tuning("tail_bounce", tb)
        k.set_tuning("pass_shadow_sort", sort)
        k.set_tuning("pass_ray_sort", rays)
        k.set_counting(True)
        k.execute(4)
        film, samples = k.film()
        got = (film.copy(), k.counters().copy(), k.primitive_offsets().copy())
        k.dispose()
        assert (samples == 4).all()
        if ref is None:
            ref = got
            continue
        assert np.allclose(got[0], ref[0], rtol=1e-5, atol=1e-6), (tb, sort, rays, blocks, np.abs(got[0] - ref[0]).max())
        assert np.array_equal(got[1], ref[1]), (tb, sort, rays, blocks, got[1], ref[1])
        assert np.array_equal(got[2], ref[2]), (tb, sort, rays, blocks)

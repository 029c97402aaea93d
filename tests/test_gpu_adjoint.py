"""GPU: the path-replay adjoint (dfpt_diff_forward / dfpt_diff_backward) against the FP64 host
adjoint of the oracle and against central finite differences of the GPU's own renders.

Tolerances:
  GPU vs FP64 host adjoint (same RNG streams, same estimator): per parameter group, the relative
      norm of the difference <= 2% (FP32 paths may part from FP64 ones at a few edges);
  GPU vs central differences, h = 1e-3, same seed for both sides (a fresh handle per evaluation, so
      the same pass indices): albedo, emission, turbidity with Russian roulette off: 2% of the
      gradient + a small floor;
  sun direction (a derivative over the rim of the sun's cone, shadows included) vs central
      differences as means over 32 seeds, with and without a ground plane: within 3 standard errors;
  Phong exponent (score-function gradient vs finite differences, two different estimators of the
      same derivative): agreement within 4 combined standard errors over independent seeds.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(plane=True, rr=True, count=9, w=32, h=24, phong_every=3, seed=11):
    from dfpt import synthetic

    cs, params, (ww, hh), truth, start = synthetic.inverse_scene(seed=seed, width=w, height=h, count=count,
                                                                 phong_every=phong_every, plane=plane)
    if not rr:
        params = dict(params, pt_ray_depth_russian_roulette=params["pt_ray_depth_maximum"] + 1)
    params = dict(params, seed=7)
    n = cs.primitives.size // 3
    theta = dict(albedo=start["albedo"].astype(np.float64), emission=np.zeros((n, 3)),
                 phong_exponent=truth["phong_exponent"].astype(np.float64), turbidity=2.5,
                 sun_direction=np.array([0.3, 0.9, 0.25]))
    return cs, params, ww, hh, theta


def _gpu(cs, params, w, h, theta, W, spp, seed=None):
    from dfpt.diff import DiffRenderer
    from dfpt.kernel import RendererKernel
    from dfpt.scene import SkyState

    k = RendererKernel(cs, SkyState(tuple(theta["sun_direction"]), theta["turbidity"]), params)
    k.update(w, h)
    if seed is not None:
        k.set_seed(seed)
    d = DiffRenderer(k)
    img = d.forward(theta["albedo"], theta["emission"], theta["phong_exponent"], theta["turbidity"], theta["sun_direction"], spp)
    g = d.backward(W) if W is not None else None
    k.dispose()
    return img, g


def _shift(theta, key, index, delta):
    t = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in theta.items()}
    if isinstance(t[key], np.ndarray):
        t[key].reshape(-1)[index] += delta
    else:
        t[key] += delta
    return t


def test_gpu_adjoint_matches_fp64_host_adjoint(oracle_mod):
    from dfpt.kernel import default_params
    from dfpt.scene import SkyState

    cs, params, w, h, theta = _scene(plane=True, rr=True)
    W = np.random.default_rng(5).normal(size=(h, w, 3)).astype(np.float32)
    spp = 4
    img, g = _gpu(cs, params, w, h, theta, W, spp)
    p = default_params()
    for k, v in params.items():
        setattr(p, k, v)
    sky = SkyState(tuple(theta["sun_direction"]), theta["turbidity"])
    himg, hg = oracle_mod.diff(cs, sky, p, w, h, theta["albedo"], theta["emission"], theta["phong_exponent"], theta["turbidity"],
                               theta["sun_direction"], W.astype(np.float64), passes=spp)
    assert np.abs(img - himg).mean() < 0.01 * np.abs(himg).mean()
    for key in ("albedo", "emission", "phong_exponent", "sun_direction"):
        a, b = np.asarray(g[key], np.float64).ravel(), np.asarray(hg[key], np.float64).ravel()
        assert np.linalg.norm(b) > 0, key
        assert np.linalg.norm(a - b) <= 0.02 * np.linalg.norm(b), (key, a, b)
    assert abs(g["turbidity"] - hg["turbidity"]) <= 0.02 * abs(hg["turbidity"]) + 1e-6


def test_gpu_adjoint_matches_central_differences():
    cs, params, w, h, theta = _scene(plane=True, rr=False)
    W = np.random.default_rng(6).normal(size=(h, w, 3)).astype(np.float32)
    spp = 4
    _, g = _gpu(cs, params, w, h, theta, W, spp)

    def loss(t):
        img, _ = _gpu(cs, params, w, h, t, None, spp)
        return float(np.sum(W.astype(np.float64) * img))

    hstep = 1e-3
    checks = [("albedo", prim * 3 + c, g["albedo"][prim, c]) for prim in (0, 1, 3) for c in range(3)]
    checks += [("emission", prim * 3 + 2, g["emission"][prim, 2]) for prim in (0, 2)]
    checks.append(("turbidity", None, g["turbidity"]))
    bad = []
    for key, idx, gv in checks:
        fd = (loss(_shift(theta, key, idx, hstep)) - loss(_shift(theta, key, idx, -hstep))) / (2 * hstep)
        if abs(gv - fd) > 0.02 * abs(fd) + 2e-3:
            bad.append((key, idx, gv, fd))
    assert not bad, bad



@pytest.mark.parametrize("plane", [False, True])
def test_gpu_sun_direction_gradient_matches_fd(plane):
    """The sun direction's derivative is taken over the rim of the sun's cone (shadow edges that
    cross it included): compared with central differences (h = 1e-2, common random numbers) as a
    mean over 32 seeds of 8 spp each, the loss being the whole image's radiance; |mean gap| within
    3 standard errors or 2%. With the ground plane the spheres' shadows move with the sun."""
    cs, params, w, h, theta = _scene(plane=plane, rr=False, w=64, h=48)
    W = np.ones((h, w, 3), np.float32)
    spp, seeds, hstep = 8, 32, 1e-2
    gaps, fds = [], []
    for sd in range(seeds):
        _, g = _gpu(cs, params, w, h, theta, W, spp, seed=100 + sd)
        fd = np.zeros(3)
        for j in range(3):
            lp = float(np.sum(_gpu(cs, params, w, h, _shift(theta, "sun_direction", j, hstep), None, spp, seed=100 + sd)[0]))
            lm = float(np.sum(_gpu(cs, params, w, h, _shift(theta, "sun_direction", j, -hstep), None, spp, seed=100 + sd)[0]))
            fd[j] = (lp - lm) / (2 * hstep)
        gaps.append(fd - g["sun_direction"])
        fds.append(fd)
    gaps, fds = np.asarray(gaps), np.asarray(fds)
    se = gaps.std(axis=0, ddof=1) / np.sqrt(seeds)
    gap, fd = gaps.mean(axis=0), fds.mean(axis=0)
    bad = [(j, fd[j] - gap[j], fd[j], se[j]) for j in range(3) if abs(gap[j]) > max(3 * se[j], 0.02 * abs(fd[j]))]
    assert not bad, bad
    j = int(np.argmax(np.abs(fd)))
    assert 3 * se[j] < 0.05 * abs(fd[j]), (se, fd)


def test_gpu_phong_exponent_gradient_is_unbiased():
    """A Phong ground plane reflecting a bright sphere: d(loss)/d(exponent of the plane) from the
    score function and from central differences (h = 1), each averaged over 8 seeds."""
    from dfpt import scene as sc

    b = sc.SceneBuilder()
    black = b.constant(0, 0, 0)
    white = b.constant(1, 1, 1)
    b.primitive(b.plane((0, 0, 0), (0, 0, 1), (1, 0, 0)), b.surface(sc.PHONG, b.constant(0.8, 0.8, 0.8), black, black))
    b.primitive(b.sphere((0, 0, 0), 0.6), b.surface(sc.LAMBERTIAN, black, b.constant(1, 0.9, 0.8), black), position=(0, 1.2, -1))
    b.primitive(b.sphere((0, 0, 0), 0.5), b.surface(sc.LAMBERTIAN, white, black, black), position=(1.5, 0.5, 0.5))
    b.camera((0, 1.5, 5), (0, 0.2, -1), 50.0, (48, 32))
    cs = b.compile("phong_probe")
    params = dict(renderer_type=2, pt_ray_depth_maximum=3, pt_ray_depth_russian_roulette=9, tone_mapper_type=2, tone_mapper_exposure=1.0)
    w, h = 48, 32
    n = cs.primitives.size // 3
    theta = dict(albedo=np.ones((n, 3)), emission=np.zeros((n, 3)), phong_exponent=np.array([20.0, 50.0, 50.0]), turbidity=2.0,
                 sun_direction=np.array([0.2, 0.5, -0.8]))
    yy, xx = np.mgrid[0:h, 0:w]
    W = np.exp(-((xx - w / 2) ** 2 + (yy - h * 0.6) ** 2) / (2 * 6.0 ** 2))[..., None].repeat(3, 2).astype(np.float32)
    adj, fds = [], []
    for s in range(8):
        _, g = _gpu(cs, params, w, h, theta, W, 64, seed=100 + s)
        adj.append(g["phong_exponent"][0])
        lp = float(np.sum(W * _gpu(cs, params, w, h, _shift(theta, "phong_exponent", 0, 1.0), None, 64, seed=100 + s)[0]))
        lm = float(np.sum(W * _gpu(cs, params, w, h, _shift(theta, "phong_exponent", 0, -1.0), None, 64, seed=100 + s)[0]))
        fds.append((lp - lm) / 2.0)
    adj, fds = np.array(adj), np.array(fds)
    se = np.sqrt(adj.var(ddof=1) / len(adj) + fds.var(ddof=1) / len(fds))
    assert abs(adj.mean()) > 3 * np.sqrt(adj.var(ddof=1) / len(adj)), adj  # a measurable gradient
    assert abs(adj.mean() - fds.mean()) <= 4 * se, (adj.mean(), fds.mean(), se)


def test_inverse_rendering_step_reduces_loss():
    """A few gradient steps on the sphere albedos (torch autograd.Function over the C-ABI pair)
    lower the L2 loss against a target rendered at the true albedos; FP64 loss reduction."""
    torch = pytest.importorskip("torch")
    from dfpt.diff import DiffRenderer, render_function
    from dfpt.kernel import RendererKernel
    from dfpt.scene import SkyState
    from dfpt import synthetic

    cs, params, (w, h), truth, start = synthetic.inverse_scene(seed=12, width=48, height=32, count=9, phong_every=3)
    k = RendererKernel(cs, SkyState(truth["sun_direction"], truth["turbidity"]), params)
    k.update(w, h)
    d = DiffRenderer(k)
    target = torch.from_numpy(d.forward(truth["albedo"], None, truth["phong_exponent"], truth["turbidity"], truth["sun_direction"], 64)).double()
    fn = render_function()
    albedo = torch.tensor(start["albedo"], dtype=torch.float32, requires_grad=True)
    emission = torch.zeros_like(albedo)
    exponent = torch.tensor(start["phong_exponent"])
    turb = torch.tensor(float(start["turbidity"]), requires_grad=True)
    sun = torch.tensor(start["sun_direction"])
    losses = []
    for it in range(6):
        img = fn.apply(d, 16, albedo, emission, exponent, turb, sun)
        loss = ((img.double() - target) ** 2).sum()
        losses.append(float(loss))
        loss.backward()
        with torch.no_grad():
            albedo -= 0.5 * albedo.grad / (albedo.grad.abs().max() + 1e-12) * 0.05
            albedo.clamp_(0.01, 1.0)
            turb -= 0.1 * torch.sign(turb.grad)
            albedo.grad = None
            turb.grad = None
    assert losses[-1] < losses[0], losses
    k.dispose()


def test_wave_adjoint_equals_pass_by_pass_adjoint():
    """The forward and the replay in waves of passes (wide_samples 8) give the gradients of the
    pass-by-pass forward and replay (wide_samples 1): same paths, same records; float atomics and
    summation order leave small differences (rtol 1e-4 per group norm)."""
    from dfpt.diff import DiffRenderer
    from dfpt.kernel import RendererKernel
    from dfpt.scene import SkyState

    cs, params, w, h, theta = _scene(plane=True, rr=True)
    W = np.random.default_rng(9).normal(size=(h, w, 3)).astype(np.float32)
    out = []
    for wide in (1, 8):
        k = RendererKernel(cs, SkyState(tuple(theta["sun_direction"]), theta["turbidity"]), params)
        k.update(w, h)
        k.set_tuning("wide_samples", wide)
        d = DiffRenderer(k)
        img = d.forward(theta["albedo"], theta["emission"], theta["phong_exponent"], theta["turbidity"], theta["sun_direction"], 6)
        out.append((img.copy(), d.backward(W)))
        k.dispose()
    (ia, ga), (ib, gb) = out
    np.testing.assert_allclose(ia, ib, rtol=1e-5, atol=1e-6)
    for key in ("albedo", "emission", "phong_exponent", "sun_direction"):
        a, b = np.asarray(ga[key]).ravel(), np.asarray(gb[key]).ravel()
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(a) + 1e-6, key
    assert abs(ga["turbidity"] - gb["turbidity"]) <= 1e-4 * abs(ga["turbidity"]) + 1e-6

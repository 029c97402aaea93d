"""CPU: the FP64 host adjoint of the oracle against central finite differences of the oracle's own
FP64 renders (no GPU).

The loss is linear, L = sum(W * image) with fixed random weights W, and both sides of every
difference use the same RNG streams (same pass indices and seed), so L is a deterministic smooth
function of albedo, emission and turbidity when Russian roulette is off (its decisions depend on the
albedo). Step h = 1e-3 (central). Tolerance: 2% of the gradient, plus a small absolute floor for
near-zero entries. The sun direction's derivative (over the rim of the sun's cone, shadows
included) is compared with finite differences as a mean over blocks of passes, within 3 standard
errors.
"""
import numpy as np
import pytest


def _params(d):
    from dfpt.kernel import default_params

    p = default_params()
    for k, v in d.items():
        setattr(p, k, v)
    return p


def _setup(plane, width=24, height=16):
    from dfpt import synthetic

    cs, params, (w, h), truth, start = synthetic.inverse_scene(seed=11, width=width, height=height, count=9, phong_every=3, plane=plane)
    params = dict(params, pt_ray_depth_russian_roulette=params["pt_ray_depth_maximum"] + 1, seed=7)
    n = cs.primitives.size // 3
    theta = dict(albedo=start["albedo"].astype(np.float64), emission=np.zeros((n, 3)), phong_exponent=start["phong_exponent"].astype(np.float64),
                 turbidity=2.5, sun_direction=np.array([0.3, 0.9, 0.25]))
    return cs, _params(params), w, h, theta


def _loss(oracle_mod, cs, p, w, h, theta, W, passes=2):
    from dfpt.scene import SkyState

    sky = SkyState(tuple(theta["sun_direction"]), theta["turbidity"])
    img, g = oracle_mod.diff(cs, sky, p, w, h, theta["albedo"], theta["emission"], theta["phong_exponent"], theta["turbidity"],
                             theta["sun_direction"], W, passes=passes)
    return float(np.sum(W * img)), g


def _fd(oracle_mod, cs, p, w, h, theta, W, key, index, hstep=1e-3):
    def shifted(sign):
        t = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in theta.items()}
        if isinstance(t[key], np.ndarray):
            t[key].reshape(-1)[index] += sign * hstep
        else:
            t[key] += sign * hstep
        return _loss(oracle_mod, cs, p, w, h, t, W)[0]

    return (shifted(+1) - shifted(-1)) / (2 * hstep)


def _close(g, fd, rel=0.02, floor=1e-4):
    return abs(g - fd) <= rel * abs(fd) + floor


def test_host_adjoint_albedo_emission_turbidity_match_fd(oracle_mod):
    cs, p, w, h, theta = _setup(plane=True)
    W = np.random.default_rng(3).normal(size=(h, w, 3))
    _, g = _loss(oracle_mod, cs, p, w, h, theta, W)
    checks = []
    for prim in (0, 1, 3, 5):
        for c in range(3):
            checks.append(("albedo", prim * 3 + c, g["albedo"][prim, c]))
    for prim in (0, 2, 4):
        checks.append(("emission", prim * 3 + 1, g["emission"][prim, 1]))
    checks.append(("turbidity", None, g["turbidity"]))
    bad = []
    for key, idx, gv in checks:
        fd = _fd(oracle_mod, cs, p, w, h, theta, W, key, idx)
        if not _close(gv, fd):
            bad.append((key, idx, gv, fd))
    assert any(abs(gv) > 1e-3 for _, _, gv in checks)
    assert not bad, bad


@pytest.mark.parametrize("plane", [False, True])
def test_host_adjoint_sun_direction_matches_fd(oracle_mod, plane):
    """The sun direction moves the cone the sun sample is drawn from; its derivative is taken over
    the cone's rim (visibility included), a different estimator from the per-sample derivative a
    finite difference with common random numbers sees, so the two are compared as means: blocks
    of passes, each giving an adjoint and a central difference (h = 1e-2) on its own passes, and
    |mean gap| within 3 standard errors of the mean gap or 2% of the difference. With the ground
    plane the spheres' shadows move with the sun: the case a derivative with the visibility held
    fixed gets wrong."""
    cs, p, w, h, theta = _setup(plane=plane, width=64, height=48)
    W = np.ones((h, w, 3))  # the whole image's radiance: a derivative the blocks agree on in sign
    blocks, per, hstep = 32, 8, 1e-2
    from dfpt.scene import SkyState

    def run(t, b):
        sky = SkyState(tuple(t["sun_direction"]), t["turbidity"])
        img, g = oracle_mod.diff(cs, sky, p, w, h, t["albedo"], t["emission"], t["phong_exponent"], t["turbidity"],
                                 t["sun_direction"], W, pass_begin=b * per, passes=per)
        return float(np.sum(W * img)), g["sun_direction"]

    gaps, fds, adj = [], [], []
    for b in range(blocks):
        g = run(theta, b)[1]
        fd = np.zeros(3)
        for j in range(3):
            tp = dict(theta, sun_direction=theta["sun_direction"].copy())
            tm = dict(theta, sun_direction=theta["sun_direction"].copy())
            tp["sun_direction"][j] += hstep
            tm["sun_direction"][j] -= hstep
            fd[j] = (run(tp, b)[0] - run(tm, b)[0]) / (2 * hstep)
        adj.append(g)
        fds.append(fd)
        gaps.append(fd - g)
    gaps, fds, adj = np.asarray(gaps), np.asarray(fds), np.asarray(adj)
    se = gaps.std(axis=0, ddof=1) / np.sqrt(blocks)
    gap, fd = gaps.mean(axis=0), fds.mean(axis=0)
    assert np.abs(fd).max() > 1e-2
    bad = [(j, adj[:, j].mean(), fd[j], se[j]) for j in range(3) if abs(gap[j]) > max(3 * se[j], 0.02 * abs(fd[j]))]
    assert not bad, bad
    # The comparison can see a bias of 5% of the largest component.
    j = int(np.argmax(np.abs(fd)))
    assert 3 * se[j] < 0.05 * abs(fd[j]), (se, fd)

"""Statistics of a path-traced film against an FP64 oracle render (test helper).

The criterion: within 1% relative RMSE of the converged linear radiance, with per-pixel z-scores
against the oracle's sample variance.

  a : the film under test, N samples per pixel (any stream);
  b : the oracle's FP64 film, M >= N samples per pixel from an independent stream, with its
      per-pixel sums and sums of squares.

Each pixel channel's difference a - b has expected square bias^2 + s2 (1/N + 1/M), s2 the
per-sample variance (estimated from the oracle's M samples). Subtracting the noise term from the
mean squared difference leaves the squared bias of the converged images: `converged_rel_rmse` is its
square root over the mean radiance. The z-scores take the oracle's two halves apart: the difference
a - b2 (b2 = the mean of the second M/2 samples) over the standard deviation from the first half's
sample variance, s1 (1/N + 2/M). The variance estimate is then independent of the difference, so an
unbiased film's z-scores have mean 0 even where the radiance is heavy-tailed (bright emitters hit by
few samples: with b's own variance, a pixel whose b drew no emitter hit gets a small b and a small
variance at once, which skews the mean z upward). tests/test_parity_statistic.py pins these
thresholds on the CPU: two independent oracle renders pass, and the same film scaled by 1% fails.
"""
from __future__ import annotations

import numpy as np


def _var(s, sq, k):
    return np.maximum(sq - s * s / k, 0.0) / (k - 1)


def _blocks(x, shape, k):
    """Per-channel means over k x k pixel blocks of an (h * w * 3) array (edge blocks cropped)."""
    h, w = shape
    hb, wb = h // k, w // k
    x = np.asarray(x, np.float64).reshape(h, w, 3)[:hb * k, :wb * k]
    return x.reshape(hb, k, wb, k, 3).mean(axis=(1, 3)).reshape(-1)


def film_stats(a, n, ref, m, block=None):
    """ref: the oracle's per-channel "sum" and "sumsq" over all m samples, and "sum1"/"sumsq1" over
    the first m/2 of them (oracle_pair returns both). block=(h, w, k): the same statistics over the
    means of k x k pixel blocks (a block mean averages k^2 pixels' samples, so its distribution is
    close to normal where single pixels are heavy-tailed; its variance is the mean of the pixels'
    variances over k^2)."""
    a = np.asarray(a, np.float64).reshape(-1)
    b = ref["sum"] / m
    s2 = _var(ref["sum"], ref["sumsq"], m)
    h = int(ref.get("half", m // 2))
    s1 = _var(ref["sum1"], ref["sumsq1"], h)
    b2 = (ref["sum"] - ref["sum1"]) / (m - h)
    div = 1.0
    if block is not None:
        hh, ww, k = block
        a, b, b2, s2, s1 = (_blocks(x, (hh, ww), k) for x in (a, b, b2, s2, s1))
        div = float(k * k)
    v = s2 / div * (1.0 / n + 1.0 / m)
    d2 = (a - b) ** 2
    mean = float(b.mean())
    bias2 = float((d2 - v).mean())
    ok = s1 > 1e-12
    z = (a - b2)[ok] / np.sqrt(s1[ok] / div * (1.0 / n + 1.0 / (m - h)))
    return {
        "raw_rel_rmse": float(np.sqrt(d2.mean()) / mean),
        "converged_rel_rmse": float(np.sqrt(max(bias2, 0.0)) / mean),
        "bias2_rel": bias2 / mean ** 2,
        "bias2_se_rel": float((d2 - v).std() / np.sqrt(d2.size) / mean ** 2),
        "z_beyond_4": float(np.mean(np.abs(z) > 4.0)),
        "z_mean": float(z.mean()),
        "z_mean_se": float(z.std() / np.sqrt(max(z.size, 1))),
        "values": int(a.size),
    }


# Fraction of block z-scores allowed beyond |z| = 4 on scenes with HDR emitters (emission up to 20,
# found by BSDF sampling alone): their block means keep a heavier tail than a normal's.
HDR_Z_TAIL = 0.03


def assert_converged(stats, rmse=0.01, z_tail=0.01, z_mean=0.2):
    """The 1% converged RMSE and the z-score checks; the message carries every statistic. The
    squared-bias estimate must be consistent with a converged RMSE <= `rmse`: at most rmse^2 plus
    3 of its standard errors (where the noise term dominates - heavy-tailed radiance - the point
    estimate alone swings by more than 1%). The mean z-score must stay within `z_mean` or 4 standard
    errors of its own sample mean, whichever is wider (heavy tails widen the spread of z, not its
    expectation)."""
    bias2 = (stats["converged_rel_rmse"] ** 2 if stats["converged_rel_rmse"] > 0 else stats["bias2_rel"])
    assert bias2 - 3.0 * stats["bias2_se_rel"] <= rmse * rmse, stats
    assert stats["z_beyond_4"] < z_tail, stats
    assert abs(stats["z_mean"]) < max(z_mean, 4.0 * stats["z_mean_se"]), stats


def same_stream_mean_ratio(a, b):
    """mean(a) / mean(b) - 1 for two films on the same stream: the estimators' agreement on the
    whole image, free of sampling noise."""
    return float(np.mean(np.asarray(a, np.float64)) / np.mean(np.asarray(b, np.float64)) - 1.0)


def same_stream_rel_rmse(a, b):
    """Relative RMSE of two films that drew the same random numbers (same seed and passes): only
    arithmetic differences (FP32 vs FP64, FMA, transcendental functions) separate them."""
    a = np.asarray(a, np.float64).reshape(-1)
    b = np.asarray(b, np.float64).reshape(-1)
    return float(np.sqrt(np.mean((a - b) ** 2)) / b.mean())


def oracle_pair(oracle_mod, scene, sky, params, w, h, n, m, seed):
    """FP64 oracle renders with `seed`: the first n passes alone (the same-stream reference) and all
    m passes (the converged reference, with the sums of its first m/2 passes), from one m-pass sweep
    in pieces: passes [0, n), [n, m/2), [m/2, m)."""
    from dfpt.kernel import default_params

    p = default_params()
    for k, v in dict(params, seed=seed).items():
        setattr(p, k, v)
    h2 = max(m // 2, n)
    first = oracle_mod.render(scene, sky, p, w, h, passes=n, precision=64)
    sum1, sumsq1 = first["sum"].copy(), first["sumsq"].copy()
    if h2 > n:
        mid = oracle_mod.render(scene, sky, p, w, h, passes=h2 - n, precision=64, pass_begin=n)
        sum1 += mid["sum"]
        sumsq1 += mid["sumsq"]
    full = {"sum1": sum1, "sumsq1": sumsq1, "sum": sum1.copy(), "sumsq": sumsq1.copy(), "half": h2}
    if m > h2:
        rest = oracle_mod.render(scene, sky, p, w, h, passes=m - h2, precision=64, pass_begin=h2)
        full["sum"] += rest["sum"]
        full["sumsq"] += rest["sumsq"]
    full["film"] = full["sum"] / m
    return first, full

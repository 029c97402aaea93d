"""Statistics of a path-traced film against an FP64 oracle render (test helper).

The criterion: within 1% relative RMSE of the converged linear radiance, with per-pixel z-scores
against the oracle's sample variance.

  a : the film under test, N samples per pixel (any stream);
  b : the oracle's FP64 film, M >= N samples per pixel from an independent stream, with its
      per-pixel sums and sums of squares.

Each pixel channel's difference a - b has expected square bias^2 + s2 (1/N + 1/M), s2 the
per-sample variance (estimated from the oracle's M samples). Subtracting the noise term from the
mean squared difference leaves the squared bias of the converged images: `converged_rel_rmse` is its
square root over the mean radiance. z-scores divide the differences by their standard deviation;
with M = 4N the variance estimate comes mostly from samples independent of b's own, so the z-scores
of an unbiased film are close to standard normal. tests/test_parity_statistic.py pins these
thresholds on the CPU: two independent oracle renders pass, and the same film scaled by 1% fails.
"""
from __future__ import annotations

import numpy as np


def film_stats(a, n, ref, m):
    a = np.asarray(a, np.float64).reshape(-1)
    b = ref["sum"] / m
    s2 = np.maximum(ref["sumsq"] - ref["sum"] ** 2 / m, 0.0) / (m - 1)
    v = s2 * (1.0 / n + 1.0 / m)
    d2 = (a - b) ** 2
    mean = float(b.mean())
    bias2 = float((d2 - v).mean())
    ok = s2 > 1e-12
    z = (a - b)[ok] / np.sqrt(v[ok])
    return {
        "raw_rel_rmse": float(np.sqrt(d2.mean()) / mean),
        "converged_rel_rmse": float(np.sqrt(max(bias2, 0.0)) / mean),
        "bias2_se_rel": float((d2 - v).std() / np.sqrt(d2.size) / mean ** 2),
        "z_beyond_4": float(np.mean(np.abs(z) > 4.0)),
        "z_mean": float(z.mean()),
        "pixels": int(a.size // 3),
    }


def assert_converged(stats, rmse=0.01, z_tail=0.01, z_mean=0.2):
    """The 1% converged RMSE and the z-score checks; the message carries every statistic."""
    assert stats["converged_rel_rmse"] <= rmse, stats
    assert stats["z_beyond_4"] < z_tail, stats
    assert abs(stats["z_mean"]) < z_mean, stats


def same_stream_rel_rmse(a, b):
    """Relative RMSE of two films that drew the same random numbers (same seed and passes): only
    arithmetic differences (FP32 vs FP64, FMA, transcendental functions) separate them."""
    a = np.asarray(a, np.float64).reshape(-1)
    b = np.asarray(b, np.float64).reshape(-1)
    return float(np.sqrt(np.mean((a - b) ** 2)) / b.mean())


def oracle_pair(oracle_mod, scene, sky, params, w, h, n, m, seed):
    """FP64 oracle renders with `seed`: the first n passes alone (the same-stream reference) and all
    m passes (the converged reference), from one m-pass sweep: passes 0..n-1, then n..m-1, sums added."""
    from dfpt.kernel import default_params

    p = default_params()
    for k, v in dict(params, seed=seed).items():
        setattr(p, k, v)
    first = oracle_mod.render(scene, sky, p, w, h, passes=n, precision=64)
    rest = oracle_mod.render(scene, sky, p, w, h, passes=m - n, precision=64, pass_begin=n)
    full = {"sum": first["sum"] + rest["sum"], "sumsq": first["sumsq"] + rest["sumsq"]}
    full["film"] = full["sum"] / m
    return first, full

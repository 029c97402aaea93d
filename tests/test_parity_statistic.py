"""CPU: the converged-RMSE and z-score statistics of tests/_parity.py have the power they claim.

Two independent FP64 oracle renders of the same scene (N = 64 against M = 256 samples per pixel)
pass every check; the same film with a bias planted on the CPU (the oracle's film scaled by 1% or
2%) fails them. The same holds over 8 x 8 pixel blocks on a heavy-tailed scene (instances with HDR
area lights, emission up to 20), the form the GPU test of that scene uses. The GPU parity tests
apply the same statistics to the CUDA core's films.
"""
import numpy as np
import pytest

from _parity import HDR_Z_TAIL, assert_converged, film_stats, oracle_pair, same_stream_rel_rmse


@pytest.fixture(scope="module")
def renders(oracle_mod):
    from dfpt import synthetic

    scene, sky, params, (w, h) = synthetic.small_mesh_scene(width=96, height=64)
    n, m = 64, 256
    a_first, _ = oracle_pair(oracle_mod, scene, sky, params, w, h, n, n + 1, seed=0xA11CE)
    b_first, b_full = oracle_pair(oracle_mod, scene, sky, params, w, h, n, m, seed=0xB0B)
    return a_first["film"], b_first["film"], b_full, n, m


def test_independent_oracle_renders_pass(renders):
    a, _, ref, n, m = renders
    s = film_stats(a, n, ref, m)
    assert_converged(s)
    assert s["raw_rel_rmse"] > s["converged_rel_rmse"]  # the noise is subtracted, not ignored


@pytest.mark.parametrize("scale", [0.99, 1.01])
def test_one_percent_bias_fails_the_z_scores(renders, scale):
    a, _, ref, n, m = renders
    s = film_stats(a * scale, n, ref, m)
    with pytest.raises(AssertionError):
        assert_converged(s, rmse=1.0)  # the z-score checks alone reject it


@pytest.mark.parametrize("scale", [0.98, 1.02])
def test_two_percent_bias_fails_the_converged_rmse(renders, scale):
    a, _, ref, n, m = renders
    s = film_stats(a * scale, n, ref, m)
    assert s["converged_rel_rmse"] > 0.01, s
    with pytest.raises(AssertionError):
        assert_converged(s, z_tail=1.0, z_mean=1e9)  # the RMSE check alone rejects it


def test_same_stream_identity(renders):
    _, b_first, ref, n, m = renders
    assert same_stream_rel_rmse(b_first, b_first) == 0.0
    assert np.allclose(ref["film"] * m, ref["sum"])


@pytest.fixture(scope="module")
def hdr_renders(oracle_mod):
    from dfpt import synthetic

    scene, sky, params, (w, h) = synthetic.instances_scene(width=96, height=56, frequency=6, lights=40)
    n, m = 128, 512
    a_first, _ = oracle_pair(oracle_mod, scene, sky, params, w, h, n, n + 1, seed=0xA11CE)
    _, b_full = oracle_pair(oracle_mod, scene, sky, params, w, h, n, m, seed=0xB0B)
    return a_first["film"], b_full, n, m, (h, w, 8)


def test_hdr_scene_blocks_pass_and_planted_bias_fails(hdr_renders):
    a, ref, n, m, block = hdr_renders
    # Block z-scores of HDR emitters keep a heavier tail than a normal's: 3% beyond |z| = 4.
    assert_converged(film_stats(a, n, ref, m, block=block), z_tail=HDR_Z_TAIL)
    for scale in (0.98, 1.02):
        s = film_stats(a * scale, n, ref, m, block=block)
        assert s["converged_rel_rmse"] > 0.01, s
        with pytest.raises(AssertionError):
            assert_converged(s, rmse=1.0, z_tail=HDR_Z_TAIL)
        with pytest.raises(AssertionError):
            assert_converged(s, z_tail=1.0, z_mean=1e9)

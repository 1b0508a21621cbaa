"""The counter-based thermal-noise stream of the stochastic forms (models A
and B, spinodal decomposition), on the CPU.

The examples draw gaussian(0, std) from rand() with the polar method in the
serial order of the cells (examples/phase_transitions/model_A/model_A.cpp:
13-40), which no parallel code can reproduce.  The library and the oracle
draw deviate k = step * cells + cell of one SplitMix64 stream instead, with
the Box-Muller transform.  Here the oracle's stream is restated in numpy,
its moments checked, and the zero-noise forms checked against the
deterministic ones (those are pinned to the reference by the fixtures).
"""
import numpy as np

from mmsp_gb300 import inputs


def numpy_gaussian(seed, k):
    k = np.asarray(k, dtype=np.uint64)
    z1 = inputs.splitmix64(seed, 1, 0)  # shape check of the helper
    assert z1.shape == (1,)
    out = np.empty(k.shape)
    for n, kk in enumerate(k.ravel()):
        z = inputs.splitmix64(seed, 2, int(2 * kk))
        u1 = float(z[0] >> np.uint64(11)) * 2.0 ** -53
        u2 = float(z[1] >> np.uint64(11)) * 2.0 ** -53
        out.ravel()[n] = np.sqrt(-2.0 * np.log(1.0 - u1)) * np.cos(6.283185307179586 * u2)
    return out


def test_oracle_stream_matches_numpy_restatement(oracle):
    ks = [0, 1, 2, 17, 1000, 123456789, 2 ** 40 + 3]
    for seed in (0, 7, 2 ** 53):
        want = numpy_gaussian(seed, ks)
        got = np.array([oracle.gaussian(seed, k) for k in ks])
        assert np.allclose(got, want, rtol=1e-14, atol=1e-15)


def test_stream_moments(oracle):
    x = np.array([oracle.gaussian(11, k) for k in range(200000)])
    assert abs(x.mean()) < 0.01
    assert abs(x.std() - 1.0) < 0.01
    assert abs((x ** 3).mean()) < 0.03 and abs((x ** 4).mean() - 3.0) < 0.05
    assert np.isfinite(x).all()


def test_zero_noise_is_the_deterministic_form(oracle):
    c = inputs.noisy_composition((12, 14), 0.0, 1.0, 3)
    assert np.array_equal(oracle.ch_shipped_noise(c, 15, noise=0.0, seed=5), oracle.ch_shipped(c, 15))
    assert np.array_equal(oracle.ac_scalar_noise(c, 15, noise=0.0, seed=5), oracle.ac_scalar_shipped(c, 15))
    # and noise moves the result, step0 continues the stream
    a = oracle.ac_scalar_noise(c, 10, noise=1.4, seed=5)
    assert not np.array_equal(a, oracle.ac_scalar_shipped(c, 10))
    b = oracle.ac_scalar_noise(oracle.ac_scalar_noise(c, 4, noise=1.4, seed=5), 6, noise=1.4, seed=5, step0=4)
    assert np.array_equal(a, b)

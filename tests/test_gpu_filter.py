"""Spectral response functions on the GPU (clblm_gpu_filter) against the
oracle's clblm_FLTRFN: several channels in one call (boxcar, Hanning,
Gaussian by its centre, a channel wider than 20 input panels), binary64
with one fixed-order reduction per channel: to 1e-12."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spectrum():
    v1, dv, n = 900.0, 0.001, 200001
    v = v1 + dv * np.arange(n)
    rng = np.random.default_rng(7)
    x = 1.0 + 0.2 * np.sin(v / 3.0)
    for c in rng.uniform(900.0, 1100.0, 400):
        x -= 0.4 * np.exp(-((v - c) / 0.02) ** 2)
    return x, v1, dv


def test_filter_channels_match_oracle(gpu_lib, oracle_mod):
    from clblm_gb300 import synth
    x, v1, dv = _spectrum()
    channels = [(950.13, 0.5, np.ones(21)), (950.37, 0.25, np.hanning(41) + 0.01),
                (1000.0, -0.1, np.exp(-np.linspace(-3, 3, 61) ** 2)), (905.11, 0.07, np.linspace(0.1, 1.0, 2999))]
    want = [oracle_mod.fltrfn(x, v1, dv, *c) for c in channels]
    h = gpu_lib.Handle(synth.line_list(1000, 600.0, 700.0, seed=0))
    try:
        got = h.filter(x, v1, dv, channels)
        again = h.filter(x, v1, dv, channels)
        with pytest.raises(gpu_lib.ClblmError):
            h.filter(x, v1, dv, [(950.0, 0.5, np.ones(21))])  # the reference's STOP (see the oracle test)
    finally:
        h.close()
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=0)
    assert np.array_equal(got, again)

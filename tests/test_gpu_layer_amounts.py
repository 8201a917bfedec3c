"""Layer averages and amounts of a nadir path on the GPU (ALAYER + FPACK in
binary64) against the oracle's restatement."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GCAIR = 1.0e-3 * 8.314472e7 / 6.02214199e23


def _profile(nlev=61, seed=0):
    rng = np.random.default_rng(seed)
    z = np.concatenate([[0.0], np.cumsum(rng.uniform(0.2, 7.0, nlev - 1))])
    t = 288.0 - 6.5 * np.minimum(z, 11.0) + 1.5 * np.maximum(z - 20.0, 0.0) + rng.normal(0, 1.0, nlev)
    p = 1013.0 * np.exp(-z / 7.2)
    rho = p / (GCAIR * t)
    vmr = np.stack([np.maximum(1e-2 * np.exp(-z / 2.0), 4e-6), np.full(nlev, 4e-4), 3e-7 + 0 * z,
                    np.where(z > 30, 0.0, 1e-6)], axis=1)
    vmr[5, 2] = vmr[6, 2]  # equal densities -> linear rule somewhere
    return z, p, t, rho[:, None] * vmr


def test_layer_amounts_match_oracle(gpu_lib):
    z, p, t, den = _profile()
    want = O.layer_amounts(z, p, t, den)
    from clblm_gb300 import synth
    h = gpu_lib.Handle(synth.line_list(1000, 600.0, 700.0, seed=0))
    got = h.layer_amounts(z, p, t, den, earth_radius=6371.23)
    h.close()
    for k in ("pave", "tave", "wtot", "secant"):
        np.testing.assert_allclose(got[k], want[k], rtol=1e-13, err_msg=k)
    np.testing.assert_allclose(got["w"], want["w"], rtol=1e-13, atol=0)

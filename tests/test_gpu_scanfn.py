"""The GPU wavenumber-space scan (clblm_gpu_scanfn) against the oracle's
restatement of clblm_SCANFN: every function, both ways of giving a sinc's
width, spectra finer and coarser than HWHM/12 (INTERP), a shrink (SHRKSC)
of up to 120 points per mean, the box average of the pre-box smoothing, and
device buffers.  binary64 on both sides; the scan adds the same terms in the
same order, except that ZF at a point is formed from its value at JMIN in
one step, not by repeated additions: agreement to 1e-10 of the largest
output, and most points equal."""
import math

import numpy as np
import pytest

from clblm_gb300 import capi_types as T

pytestmark = pytest.mark.gpu


def _spectrum(v1=1000.0, v2=1030.0, dv=0.001, seed=0, nlines=120, width=0.01):
    n = int(round((v2 - v1) / dv)) + 1
    v = v1 + dv * np.arange(n)
    rng = np.random.default_rng(seed)
    x = 1.0 + 0.3 * np.sin(2 * math.pi * (v - v1) / 7.0)
    for c in rng.uniform(v1, v2, nlines):
        x -= 0.5 * np.exp(-((v - c) / width) ** 2)
    return x, v1, dv


def _handle(gpu_lib):
    from clblm_gb300 import synth
    return gpu_lib.Handle(synth.line_list(1000, 600.0, 700.0, seed=0))


def _check(got, want, exact_frac=0.5):
    scale = np.abs(want).max()
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-10 * scale)
    assert np.mean(got == want) >= exact_frac, np.mean(got == want)


CASES = [
    # funct_id, hwhm, v1out, v2out, dvout, input dv
    (1, 0.05, 1005.0, 1025.0, 0.02, 0.001),     # box average (CNVRCT)
    (1, 0.0125, 1005.0, 1025.0, 0.025, 0.005),  # pre-box: the box spacing on a coarse input (INTERP first)
    (2, 0.05, 1005.0, 1025.0, 0.01, 0.001),     # triangle, shrink by 4
    (3, 0.05, 1005.0, 1025.0, 0.01, 0.001),     # Gaussian
    (3, 0.02, 1005.0, 1025.0, 0.0, 0.001),      # Gaussian at its default sampling
    (3, 0.3, 1005.0, 1025.0, 0.05, 0.0002),     # Gaussian, shrink by 120
    (4, 0.03, 1005.0, 1025.0, 0.01, 0.001),     # sinc**2
    (5, 0.03, 1006.0, 1024.0, 0.01, 0.001),     # sinc
    (-4, 0.08, 1005.0, 1025.0, 0.01, 0.001),    # sinc**2 by its first zero
    (-5, 0.06, 1006.0, 1024.0, 0.01, 0.001),    # sinc by its first zero
    (3, 0.05, 1005.0, 1025.0, 0.01, 0.01),      # input coarser than HWHM/12: INTERP, then no shrink
    (2, 0.1, 1005.0, 1025.0, 0.02, 0.02),       # INTERP, triangle
]


@pytest.mark.parametrize("fid,hw,a,b,dvout,dv", CASES)
def test_scanfn_matches_oracle(gpu_lib, oracle_mod, fid, hw, a, b, dvout, dv):
    x, v1, dv = _spectrum(dv=dv)
    want, w1, wdv = oracle_mod.scanfn(x, v1, dv, fid, hw, a, b, dvout)
    h = _handle(gpu_lib)
    try:
        got, g1, gdv = h.scanfn(T.scanfn_struct(fid, hw, a, b, dvout), x, v1, dv)
        assert h.stats()["launches"] >= 1
    finally:
        h.close()
    assert (g1, gdv, len(got)) == (w1, wdv, len(want))
    _check(got, want)


def test_scanfn_long_spectrum(gpu_lib, oracle_mod):
    """200 cm-1 at 2e-4 (1 M points, 417 input panels), Gaussian of
    HWHM 0.25 on 0.05: 3,200 output points from shrunk means of 100."""
    x, v1, dv = _spectrum(v1=900.0, v2=1100.0, dv=2e-4, seed=3, nlines=2000)
    want, w1, wdv = oracle_mod.scanfn(x, v1, dv, 3, 0.25, 920.0, 1080.0, 0.05)
    h = _handle(gpu_lib)
    try:
        got, g1, gdv = h.scanfn(T.scanfn_struct(3, 0.25, 920.0, 1080.0, 0.05), x, v1, dv)
    finally:
        h.close()
    assert (g1, gdv, len(got)) == (w1, wdv, len(want))
    _check(got, want)


def test_scanfn_identity_cases(gpu_lib, oracle_mod):
    """HWHM <= 0 returns the spectrum; a box no wider than two input points
    returns the (interpolated) spectrum."""
    x, v1, dv = _spectrum(v2=1005.0)
    h = _handle(gpu_lib)
    try:
        got, g1, gdv = h.scanfn(T.scanfn_struct(3, 0.0, 1001.0, 1004.0, 0.01), x, v1, dv)
        assert (g1, gdv) == (v1, dv) and np.array_equal(got, x)
        want, w1, wdv = oracle_mod.scanfn(x, v1, dv, 1, 0.024, 1001.0, 1004.0, 0.001)
        got, g1, gdv = h.scanfn(T.scanfn_struct(1, 0.024, 1001.0, 1004.0, 0.001), x, v1, dv)
        assert (g1, gdv, len(got)) == (w1, wdv, len(want))
        np.testing.assert_array_equal(got, want)
    finally:
        h.close()


def test_scanfn_device_buffers(gpu_lib, oracle_mod):
    import torch
    x, v1, dv = _spectrum()
    scan = T.scanfn_struct(3, 0.05, 1005.0, 1025.0, 0.01)
    want, _, _ = oracle_mod.scanfn(x, v1, dv, 3, 0.05, 1005.0, 1025.0, 0.01)
    dx = torch.tensor(x, dtype=torch.float64, device="cuda")
    dout = torch.zeros(len(want) + 3, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    h = _handle(gpu_lib)
    try:
        h.scanfn_device(scan, dx.data_ptr(), len(x), v1, dv, dout.data_ptr(), len(dout))
    finally:
        h.close()
    got = dout.cpu().numpy()
    _check(got[:len(want)], want)
    assert np.all(got[len(want):] == 0)


def test_scanfn_rejects(gpu_lib):
    x, v1, dv = _spectrum(v2=1002.0)
    h = _handle(gpu_lib)
    try:
        for fid, hw, dvout, code in ((6, 0.05, 0.01, 1), (-2, 0.05, 0.01, 1), (5, 0.2, 0.001, 6)):
            with pytest.raises(gpu_lib.ClblmError) as e:
                h.scanfn(T.scanfn_struct(fid, hw, 1000.5, 1001.5, dvout), x, v1, dv)
            assert e.value.code == code
    finally:
        h.close()

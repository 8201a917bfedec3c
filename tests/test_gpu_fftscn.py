"""The GPU FFT scan against the oracle's clblm_FFTSCN restatement."""
import math

import numpy as np
import pytest

from oracle import fftscn as S
from clblm_gb300 import capi_types as T

pytestmark = pytest.mark.gpu


def _spectrum(v1=1000.0, v2=1100.0, dv=0.002, seed=0):
    n = int(round((v2 - v1) / dv)) + 1
    v = v1 + dv * np.arange(n)
    rng = np.random.default_rng(seed)
    x = 1.0 + 0.3 * np.sin(2 * math.pi * (v - v1) / 7.0)
    for c in rng.uniform(v1, v2, 300):  # narrow lines
        x -= 0.5 * np.exp(-((v - c) / 0.01) ** 2)
    return x, v1, dv


@pytest.mark.parametrize("funct_id,prebox,deconv,fill", [
    (2, -1.0, 0, 0.0), (3, -1.0, 0, 0.0), (4, -1.0, 0, 0.0), (5, -1.0, 0, 0.0), (6, -1.0, 0, 1.0),
    (7, -1.0, 0, 1.0), (8, -1.0, 0, 0.0), (3, 0.02, 1, 1.0), (5, 0.02, 0, 0.0), (1, -1.0, 0, 0.0)])
def test_scan_matches_oracle(gpu_lib, funct_id, prebox, deconv, fill):
    x, v1, dv = _spectrum()
    hw = 0.3771 if funct_id != 1 else 0.05
    want, v1s, dvs = S.fftscn(x, v1, dv, funct_id, hw, 1030.0, 1070.0, fill=fill, prebox_hw=prebox,
                              deconv_prebox=bool(deconv))
    h = gpu_lib.Handle(*_lines())
    got, g1, gdv = h.fftscn(T.scan_struct(funct_id, hw, 1030.0, 1070.0, padding=fill, prebox_hw=prebox,
                                          deconv_prebox=deconv), x, v1, dv)
    h.close()
    assert (g1, gdv, len(got)) == (v1s, dvs, len(want))
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-11 * np.abs(want).max())


@pytest.mark.parametrize("funct_id,hw,a,b,prebox,dvout,dv", [
    (9, 0.3, 1030.0, 1070.0, -1.0, 0.0, 0.002),     # Norton-Beer weak
    (10, 0.3, 1030.0, 1070.0, -1.0, 0.0, 0.002),    # Norton-Beer medium
    (11, 0.3, 1030.0, 1070.0, -1.0, 0.0, 0.002),    # Norton-Beer strong
    (2, 4.0, 1040.0, 1060.0, -1.0, 0.0, 0.002),     # triangle from its transform (IVX = -1)
    (3, 12.0, 1040.0, 1060.0, -1.0, 0.0, 0.002),    # Gaussian, IVX = -1
    (14, 0.1, 1030.0, 1070.0, -1.0, 0.0, 0.002),    # Kiruna (asymmetric, IVX = -1)
    (3, 0.3, 1030.0, 1070.0, -1.0, 0.0, 0.1),       # a coarse input, interpolated first
    (5, 0.3771, 1030.0, 1070.0, -1.0, 0.01, 0.002), # onto DVOUT
    (103, 0.3, 1030.0, 1070.0, 0.01, 0.0, 0.002),   # boxed outside: scan + deconvolution
    (-1, 0.3, 1030.0, 1070.0, 0.01, 0.0, 0.002),    # the deconvolution alone
])
def test_scan_options_match_oracle(gpu_lib, funct_id, hw, a, b, prebox, dvout, dv):
    x, v1, dv = _spectrum(dv=dv)
    parms = (0.05, 0.9, 0.1)
    want, v1s, dvs = S.fftscn(x, v1, dv, funct_id, hw, a, b, prebox_hw=prebox, dvout=dvout, parms=parms)
    h = gpu_lib.Handle(*_lines())
    try:
        got, g1, gdv = h.fftscn(T.scan_struct(funct_id, hw, a, b, prebox_hw=prebox, dvout=dvout, parms=parms), x,
                                v1, dv)
    finally:
        h.close()
    assert (g1, gdv, len(got)) == (v1s, dvs, len(want))
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-11 * np.abs(want).max())


def test_scan_large_transform(gpu_lib):
    """4.2 M input points, 3.2 M of them loaded: a 2^24-point transform (256
    records of 65536; the sinc rectangle ends inside a later record)."""
    x, v1, dv = _spectrum(v1=600.0, v2=1020.0, dv=1e-4, seed=1)
    hw = 1.0 / (0.8 * S.C[4])
    want, v1s, dvs = S.fftscn(x, v1, dv, 5, hw, 700.0, 900.0)
    h = gpu_lib.Handle(*_lines())
    got, g1, gdv = h.fftscn(T.scan_struct(5, hw, 700.0, 900.0), x, v1, dv)
    h.close()
    assert len(got) == len(want)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-10 * np.abs(want).max())


def _lines():
    from clblm_gb300 import synth
    return (synth.line_list(1000, 600.0, 700.0, seed=0),)

"""The oracle's FFT scan (clblm_FFTSCN restated) against properties that
hold for the reference: unit-area scanning functions, the Gaussian and sinc
line shapes of the requested half width, boxcar averages."""
import math

import numpy as np
import pytest

from oracle import fftscn as S


def _grid(v1=1000.0, v2=1100.0, dv=0.01):
    n = int(round((v2 - v1) / dv)) + 1
    return v1 + dv * np.arange(n), dv


@pytest.mark.parametrize("funct_id", [2, 3, 4, 5, 6, 7, 8])
def test_constant_spectrum_stays_constant(funct_id):
    v, dv = _grid()
    out, v1s, dvs = S.fftscn(np.ones_like(v), v[0], dv, funct_id, 0.3, 1030.0, 1070.0, fill=1.0)
    assert dvs == dv and v1s <= 1030.0
    # the apodization's value at zero path difference: 1, except Hamming's
    # 0.53835685 * 1.857504 as the reference rounds it
    h0 = 0.53835685 * (1.0 + 0.857504) if funct_id == 7 else 1.0
    np.testing.assert_allclose(out, h0, rtol=0, atol=1e-12)


def test_gaussian_line_shape():
    v, dv = _grid(dv=0.005)
    x = np.zeros_like(v)
    i0 = len(v) // 2
    x[i0] = 1.0
    hw = 0.25
    out, v1s, dvs = S.fftscn(x, v[0], dv, 3, hw, 1040.0, 1060.0)
    vo = v1s + dvs * np.arange(len(out))
    ils = dv * math.sqrt(math.log(2) / math.pi) / hw * np.exp(-math.log(2) * ((vo - v[i0]) / hw) ** 2)
    np.testing.assert_allclose(out, ils, rtol=0, atol=2e-6 * ils.max())
    # half width at half maximum
    k = np.argmax(out)
    half = out[k] / 2
    right = k + np.argmax(out[k:] < half)
    vh = vo[right - 1] + (vo[right] - vo[right - 1]) * (out[right - 1] - half) / (out[right - 1] - out[right])
    assert abs((vh - vo[k]) - hw) < 1e-3 * hw


def test_sinc_line_shape():
    """A delta scans into the sinc of the equivalent interferometer: peak
    2/A per unit area, first zero at A/2 from the line (A = C4 * HWHM)."""
    v, dv = _grid(dv=0.005)
    x = np.zeros_like(v)
    i0 = len(v) // 2
    x[i0] = 1.0
    opd = 0.8
    hw = 1.0 / (opd * S.C[4])
    out, v1s, dvs = S.fftscn(x, v[0], dv, 5, hw, 1040.0, 1060.0)
    vo = v1s + dvs * np.arange(len(out))
    A = S.C[4] * hw
    k = np.argmax(out)
    assert abs(vo[k] - v[i0]) < 1e-9
    assert abs(out[k] / dv - 2.0 / A) < 2e-3 * (2.0 / A)
    u = 2 * math.pi * (vo - v[i0]) / A
    sinc = np.where(u == 0, 1.0, np.sin(u) / np.where(u == 0, 1.0, u)) * dv * 2.0 / A
    near = np.abs(vo - v[i0]) < 5.0
    np.testing.assert_allclose(out[near], sinc[near], rtol=0, atol=5e-3 * sinc.max())


def test_boxcar_only_averages():
    v, dv = _grid(dv=0.01)
    rng = np.random.default_rng(0)
    x = rng.uniform(0.5, 1.0, len(v))
    out, v1s, dvs = S.fftscn(x, v[0], dv, 1, 0.05, 1030.0, 1070.0)
    M = int(2.0 * 0.05 / dv)
    assert dvs == pytest.approx(M * dv)
    # every output point is the mean of M consecutive inputs
    j = int(round((v1s - (dvs - dv) / 2 - v[0]) / dv))
    np.testing.assert_allclose(out[:10], [x[j + M * k:j + M * k + M].mean() for k in range(10)], rtol=1e-14)


def test_prebox_with_deconvolution():
    """Pre-boxing with M points then deconvolving: the reference divides by
    the transform of a boxcar of width 2*M*DV (Scntrn(-1, DV, ...) with the
    new DV, clblm_FFT.f90:726-733), twice the M*DV it averaged over, so an
    oscillation of frequency f comes out scaled by sinc(pi f W)/sinc(2 pi f W)
    relative to the direct scan, W = M*DV."""
    v, dv = _grid(dv=0.002)
    f = 1.0 / 3.0
    x = 1.0 + 0.5 * np.sin(2 * math.pi * f * (v - v[0]))
    direct, v1a, dva = S.fftscn(x, v[0], dv, 3, 0.3, 1030.0, 1070.0, fill=1.0)
    boxed, v1b, dvb = S.fftscn(x, v[0], dv, 3, 0.3, 1030.0, 1070.0, fill=1.0, prebox_hw=0.02, deconv_prebox=True)
    W = dvb
    sinc = lambda z: math.sin(z) / z
    factor = sinc(math.pi * f * W) / sinc(2 * math.pi * f * W)
    vb = v1b + dvb * np.arange(len(boxed))
    ref = 1.0 + (np.interp(vb, v1a + dva * np.arange(len(direct)), direct) - 1.0) * factor
    inner = (vb > 1031) & (vb < 1069)
    np.testing.assert_allclose(boxed[inner], ref[inner], atol=5e-6)


def test_records_padding():
    assert S.records(1) == 4 and S.records(65536) == 4 and S.records(65537) == 8
    assert S.records(3 * 65536) == 16 and S.records(4 * 65536) == 16

"""The oracle's nadir ALAYER + FPACK against closed forms: in an isothermal
exponential atmosphere the layer air column, the absorber columns and the
density-weighted pressure are exponential integrals, and the weighted
temperature is the temperature."""
import math

import numpy as np
import pytest

from oracle import oracle as O

GCAIR = 1.0e-3 * 8.314472e7 / 6.02214199e23


def _isothermal(z, T=250.0, P0=1013.0, H=7.5, q=(1e-2, 3e-6)):
    p = P0 * np.exp(-z / H)
    t = np.full_like(z, T)
    rho = p / (GCAIR * t)
    den = np.outer(rho, q)
    return p, t, rho, den


@pytest.mark.parametrize("z", [np.linspace(0.0, 60.0, 31), np.array([0.0, 1.0, 12.0, 30.0, 31.0, 80.0])])
def test_isothermal_closed_forms(z):
    T, H, q = 250.0, 7.5, (1e-2, 3e-6)
    p, t, rho, den = _isothermal(z, T=T, H=H, q=q)
    out = O.layer_amounts(z, p, t, den)
    dz = np.diff(z)
    col = rho[:-1] * H * (1 - np.exp(-dz / H)) * 1e5  # molec/cm2
    np.testing.assert_allclose(out["wtot"], col, rtol=1e-12)
    np.testing.assert_allclose(out["w"], np.outer(col, q), rtol=1e-12)
    np.testing.assert_allclose(out["tave"], T, rtol=1e-12)
    pbar = p[:-1] * (1 - np.exp(-2 * dz / H)) / (2 * (1 - np.exp(-dz / H)))
    np.testing.assert_allclose(out["pave"], pbar, rtol=1e-12)
    np.testing.assert_allclose(out["secant"], 1.0, rtol=1e-13)


def test_equal_densities_take_the_linear_rule():
    z = np.array([0.0, 2.0, 4.0])
    p = np.array([1000.0, 800.0, 640.0])
    t = np.array([280.0, 270.0, 260.0])
    den = np.array([[5e17, 0.0], [5e17, 1e12], [2e17, 1e12]])
    out = O.layer_amounts(z, p, t, den)
    # layer 0: equal end values -> straight line; the second absorber is zero at
    # the bottom -> straight line too
    assert out["w"][0, 0] == pytest.approx(5e17 * 2.0 * 1e5, rel=1e-12)
    assert out["w"][0, 1] == pytest.approx(0.5 * 1e12 * 2.0 * 1e5, rel=1e-12)
    # layer 1: exponential
    hd = -2.0 / math.log(2e17 / 5e17)
    assert out["w"][1, 0] == pytest.approx(hd * (5e17 - 2e17) * 1e5, rel=1e-12)


def test_equal_pressures_are_rejected():
    z = np.array([0.0, 1.0])
    with pytest.raises(O.OracleError):
        O.layer_amounts(z, np.array([500.0, 500.0]), np.array([250.0, 250.0]), np.ones((2, 1)))

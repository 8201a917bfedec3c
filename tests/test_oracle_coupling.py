"""Line coupling in the oracle (LNCORQ, CNVFNQ's coupling loop, LINF4Q,
SHRINQ and CNVF4Q with SPP): the coefficient records after coupled lines,
zero coefficients, linearity in Y, G as a strength factor, GAMMA as a width
factor and the temperature interpolation of the coefficients."""
import numpy as np
import pytest

from clblm_gb300 import capi_types as T
from clblm_gb300 import synth


def _od(oracle_mod, lines, pave=500.0, tave=250.0, v1=600.0, v2=700.0, mol=2, wabs=1e18):
    col = T.Column(np.array([mol], np.int32), [pave], [tave], [tave], [tave], np.full((1, 1), wabs), [2.479e24],
                   [1.67 * 2.479e24], v1, v2, tave, 1.0)
    dn, df, _ = oracle_mod.Session().setdv(col)
    g = T.grid_struct(col.v1, col.v2, dn[0], df[0])
    od, _, st = oracle_mod.Session().odlay(lines, col.layer(0), g, T.od_ctrl(precision=1, contnm_off=1), None)
    return od, st


@pytest.fixture(scope="module")
def base():
    return synth.line_list(200, 600.0, 700.0, seed=3, mols=(2,))


IDX = np.arange(0, 200, 7)
Y = np.array((0.02, 0.015, 0.01, 0.008))


def test_zero_coefficients_change_nothing(oracle_mod, base):
    r0, s0 = _od(oracle_mod, base)
    r1, s1 = _od(oracle_mod, synth.with_coupling(base, IDX, a=(0.0,) * 4, b=(0.0,) * 4))
    np.testing.assert_array_equal(r1, r0)
    assert s1["nlin"] == s0["nlin"] and s1["nshrunk"] == s0["nshrunk"]


def test_coupled_lines_are_not_shrunk(oracle_mod, base):
    _, s0 = _od(oracle_mod, base)
    _, s1 = _od(oracle_mod, synth.with_coupling(base, IDX, a=Y, b=(0.0,) * 4))
    assert s1["nshrunk"] > s0["nshrunk"]


def test_linear_in_y(oracle_mod, base):
    """Y scaled by 1, 2, 4 (exact in the float fields): the coupling term
    doubles with Y"""
    r = [_od(oracle_mod, synth.with_coupling(base, IDX, a=k * Y, b=(0.0,) * 4))[0] for k in (1.0, 2.0, 4.0)]
    d1, d2 = r[1] - r[0], r[2] - r[1]
    assert np.max(np.abs(d1)) > 1e-3 * np.max(np.abs(r[0]))
    np.testing.assert_allclose(d2, 2.0 * d1, rtol=0, atol=1e-9 * np.max(np.abs(d1)))


def test_y_is_a_dispersion_term(oracle_mod):
    """one coupled line centred on a point of all the nested grids: the Y
    term is odd about the centre"""
    lines = synth.line_list(1, 650.0, 650.0, seed=1, mols=(2,))
    lines.pshift[:] = 0.0
    col = T.Column(np.array([2], np.int32), [500.0], [250.0], [250.0], [250.0], np.full((1, 1), 1e18), [2.479e24],
                   [1.67 * 2.479e24], 640.0, 660.0, 250.0, 1.0)
    dn, df, _ = oracle_mod.Session().setdv(col)
    dv = df[0]
    c = 64 * int(round(10.0 / (64 * dv)))  # the R4 grid's points lie 64 DV apart from V1
    lines.vnu[:] = 640.0 + c * dv
    r0, _ = _od(oracle_mod, lines, v1=640.0, v2=660.0)
    r1, _ = _od(oracle_mod, synth.with_coupling(lines, [0], a=Y, b=(0.0,) * 4), v1=640.0, v2=660.0)
    d = r1 - r0
    k = np.arange(1, min(c, len(d) - 1 - c))
    assert np.max(np.abs(d)) > 1e-3 * np.max(r0)
    np.testing.assert_allclose(d[c + k], -d[c - k], rtol=0, atol=1e-3 * np.max(np.abs(d)))


def test_g_scales_the_strength(oracle_mod, base):
    """IFLG 1 with Y = 0: SP = SUI (1 + G PAVP2), as an uncoupled line of
    that strength (to the float rounding of the strength field)"""
    pave, tave = 500.0, 296.0
    g = np.array((1e-2, 8e-3, 5e-3, 4e-3))
    rg, _ = _od(oracle_mod, synth.with_coupling(base, IDX, a=(0.0,) * 4, b=g), pave=pave, tave=tave)
    scaled = base.subset(0, base.n)
    scaled.sp = scaled.sp.copy()
    scaled.sp[IDX] = (scaled.sp[IDX].astype(np.float64) * (1.0 + g[2] * (pave / 1013.25) ** 2)).astype(np.float32)
    rs, _ = _od(oracle_mod, scaled, pave=pave, tave=tave)
    np.testing.assert_allclose(rg, rs, rtol=2e-6)


def test_gamma_scales_the_width(oracle_mod, base):
    """IFLG 3: the Lorentz width times 1 - GAMMA1 PAVP0 - GAMMA2 PAVP2, as
    an uncoupled line with both widths scaled"""
    pave, tave = 500.0, 296.0
    g1, g2 = 0.05, 0.01
    r3, _ = _od(oracle_mod, synth.with_coupling(base, IDX, iflg=3, a=(g1,) * 4, b=(g2,) * 4), pave=pave, tave=tave)
    f = 1.0 - g1 * (pave / 1013.25) - g2 * (pave / 1013.25) ** 2
    scaled = base.subset(0, base.n)
    scaled.alfa, scaled.hwhm = scaled.alfa.copy(), scaled.hwhm.copy()
    scaled.alfa[IDX] = (scaled.alfa[IDX].astype(np.float64) * f).astype(np.float32)
    scaled.hwhm[IDX] = (scaled.hwhm[IDX].astype(np.float64) * f).astype(np.float32)
    rs, _ = _od(oracle_mod, scaled, pave=pave, tave=tave)
    np.testing.assert_allclose(r3, rs, rtol=2e-5)


@pytest.mark.parametrize("tave", [205.0, 230.0, 270.0, 320.0, 345.0])
def test_coefficients_interpolate_linearly_in_temperature(oracle_mod, base, tave):
    """coefficients linear in T at the four TEMPLC: LNCORQ (from the lower
    node) and LINF4Q (from the upper) both give the line's value at TAVE"""
    t4 = np.array(synth.TEMPLC)
    a_lin = 0.03 - 5e-5 * t4
    ra, _ = _od(oracle_mod, synth.with_coupling(base, IDX, a=a_lin, b=(0.0,) * 4), tave=tave)
    rc, _ = _od(oracle_mod, synth.with_coupling(base, IDX, a=(0.03 - 5e-5 * tave,) * 4, b=(0.0,) * 4), tave=tave)
    np.testing.assert_allclose(ra, rc, rtol=0, atol=1e-9 * np.max(np.abs(ra)))

"""Known-answer tests of the FP64 oracle (CPU only).

The reference ships no tests or golden vectors for this path, so the oracle
is pinned by the reference's own data (the MT_CKD table under tests/golden)
and by answers the mathematics fixes: Planck and radiation-term limits, the
partition-sum ratio at 296 K, the line-shape normalisation, exact linearity
in the line strengths, and the polynomial exactness of the grid
interpolation."""
import numpy as np
import pytest

RADCN1 = 1.191042722e-12
RADCN2 = 1.4387752


def test_golden_fixture_shape(mtckd):
    assert mtckd.v1 == 0.0 and mtckd.dv == 10.0
    assert len(mtckd.self_absco_ref) == 301
    assert mtckd.ref_press == 1013.0 and mtckd.ref_temp == 296.0
    assert np.all(mtckd.self_absco_ref > 0) and np.all(mtckd.for_absco_ref > 0)


@pytest.mark.parametrize("pave,tave,jrad", [(1013.0, 296.0, 0), (612.4, 261.7, 0), (101.3, 231.0, 1)])
def test_continuum_at_table_nodes(oracle_mod, mtckd, pave, tave, jrad):
    """ABSRB at the table's 10 cm-1 nodes is the MT_CKD assembly of the table
    values themselves (mt_ckd_h2o_module.f90:141-160, CONTNM :389-405)."""
    v1, v2, wtot, w1 = 1000.0, 1100.0, 2.0e24, 3.0e22
    v1abs, absrb = oracle_mod.contnm_h2o(mtckd, v1, v2, pave, tave, wtot, w1, jrad=jrad)
    h2o = w1 / wtot
    rho = (pave / mtckd.ref_press) * (mtckd.ref_temp / tave)
    for nu in np.arange(1000.0, 1101.0, 10.0):
        k = int(round((nu - mtckd.v1) / mtckd.dv))
        s = mtckd.self_absco_ref[k] * (mtckd.ref_temp / tave) ** mtckd.self_texp[k] * h2o * rho
        f = mtckd.for_absco_ref[k] * (1 - h2o) * rho
        if jrad:
            x = nu * RADCN2 / tave
            rad = nu * (1 - np.exp(-x)) / (1 + np.exp(-x)) if x <= 10 else nu
            s, f = s * rad, f * rad
        want = w1 * s + w1 * f
        got = absrb[int(nu - v1abs)]
        assert got == pytest.approx(want, rel=1e-13), nu


MAXISO = (6, 10, 9, 5, 6, 4, 3, 3, 2, 1, 2, 2, 3, 2, 4, 4, 2, 2, 5, 3, 2, 2, 3, 2,
          1, 3, 2, 1, 2, 1, 3, 1, 1, 1, 2, 1, 2, 2, 1, 2, 1, 1, 1, 1, 2, 4, 1)
Q_ONE = (34, 39, 47)  # O, CH3OH, SO3: TIPS_2003 takes Q = 1


def test_tips_ratio_is_one_at_296(oracle_mod):
    for mol in range(1, 48):
        for iso in range(1, MAXISO[mol - 1] + 1):
            assert oracle_mod.tips_scor(mol, 296.0, iso) == 1.0, (mol, iso)


def test_tips_ratio_decreases_with_temperature(oracle_mod):
    for mol in range(1, 48):
        for iso in range(1, MAXISO[mol - 1] + 1):
            s = [oracle_mod.tips_scor(mol, t, iso) for t in np.arange(150.0, 351.0, 10.0)]
            if mol in Q_ONE:
                assert np.all(np.array(s) == 1.0)
            else:
                assert np.all(np.diff(s) < 0), (mol, iso)


def test_tips_fallbacks_to_the_first_isotopologue(oracle_mod):
    """TIPS_2003 reads isotopologue 1's table for HNO3 2, HF 2, HCl 3-4,
    HBr 3-4, HI 2, N2 2 and COF2 2 (clblm_ODLAY_TIPS.f90:150-260)"""
    for mol, isos in ((12, (2,)), (14, (2,)), (15, (3, 4)), (16, (3, 4)), (17, (2,)), (22, (2,)), (29, (2,))):
        for t in (200.0, 250.0, 310.0):
            for iso in isos:
                assert oracle_mod.tips_scor(mol, t, iso) == oracle_mod.tips_scor(mol, t, 1)
    # HCl 2 and HBr 2 have tables of their own
    assert oracle_mod.tips_scor(15, 250.0, 2) != oracle_mod.tips_scor(15, 250.0, 1)
    assert oracle_mod.tips_scor(16, 250.0, 2) != oracle_mod.tips_scor(16, 250.0, 1)
    # a classical rotor's Q ~ T^(3/2) (CH4) and T (CO): the ratio's slope
    for mol, expo in ((6, 1.5), (5, 1.0)):
        s = oracle_mod.tips_scor(mol, 250.0, 2)
        assert s == pytest.approx((296.0 / 250.0) ** expo, rel=0.03), mol


def test_planck(oracle_mod):
    for v in (10.0, 500.0, 1234.5, 2500.0, 3500.0):
        for t in (180.0, 250.0, 296.0, 320.0):
            xkt = t / RADCN2
            want = RADCN1 * v ** 3 / np.expm1(v / xkt)
            assert oracle_mod.planck(v, xkt) == pytest.approx(want, rel=1e-13)


def test_radiation_term_branches(oracle_mod):
    """RADFN = v tanh(x/2), x = v/kT, with the reference's small- and
    large-x branches (clblm_ODLAY_CommonSub.f90:293-330)."""
    t = 250.0
    xkt = t / RADCN2
    for x in (1e-4, 5e-3, 0.01, 0.5, 3.0, 9.9, 10.5, 40.0):
        v = x * xkt
        exact = v * np.tanh(x / 2)
        got = oracle_mod.radfn(v, xkt)
        if x <= 0.01:
            assert abs(got / exact - 1) <= x * x / 12 * 1.01
        elif x <= 10:
            assert got == pytest.approx(exact, rel=1e-13)
        else:
            assert abs(got / exact - 1) <= 2.2 * np.exp(-x)


def test_rlin_weight(oracle_mod):
    """hlf = 1/tau - 1/(e^tau - 1) with 1/2 - tau/12 below 1e-3 and 1/tau
    above 20 (clblm_EMLAY.f90:187-223)."""
    for tau in (1e-6, 5e-4, 2e-3, 0.1, 1.0, 7.0, 19.0):
        # the closed form cancels below ~1e-2: take the series there
        exact = 0.5 - tau / 12 + tau ** 3 / 720 if tau < 1e-2 else 1 / tau - 1 / np.expm1(tau)
        got = oracle_mod.rlin(tau)
        tol = 1e-12 if tau < 1e-3 else 1e-10
        assert got == pytest.approx(exact, rel=tol), tau
    assert oracle_mod.rlin(25.0) == 1 / 25.0


def _one_line(nu0=2000.0, sp=1e-20, alfa=0.07):
    from clblm_gb300.capi_types import Lines
    return Lines(vnu=[nu0], sp=[sp], alfa=[alfa], epp=[100.0], mol=[101], hwhm=[0.25], tmpalf=[0.7],
                 pshift=[0.0], iflg=[0])


def _layer_and_grid(v1, v2, dv):
    from clblm_gb300 import capi_types as T
    lay = T.layer_struct([1], [1e20], 2.479e24, 1013.25, 296.0)
    g = T.grid_struct(v1, v2, dv, dv)
    return lay, g


@pytest.mark.parametrize("alfa", [0.02, 0.07, 0.3])
def test_line_area(oracle_mod, alfa):
    """An isolated line integrates to S W RADFN(v)(1 + e^-x) times the area of
    its shape inside the 25 cm-1 cut-off less the far-wing pedestal."""
    from clblm_gb300 import capi_types as T
    nu0, sp = 2000.0, 1e-20
    lines = _one_line(nu0, sp, alfa)
    lay, g = _layer_and_grid(nu0 - 40.0, nu0 + 40.0, 0.002)
    od, dv, _ = oracle_mod.Session().odlay(lines, lay, g, T.od_ctrl(precision=1, contnm_off=1))
    area = np.trapezoid(od, dx=dv)
    xkt = 296.0 / RADCN2
    strength = sp * 1e20 * oracle_mod.radfn(nu0, xkt) * (1 + np.exp(-nu0 / xkt))
    shape = (2 / np.pi) * np.arctan(25.0 / alfa) - 50.0 * alfa / (np.pi * (alfa ** 2 + 625.0))
    assert area == pytest.approx(strength * shape, rel=5e-5)


def test_od_linear_in_strength(oracle_mod):
    """Doubling every line strength doubles the line OD exactly."""
    from clblm_gb300 import capi_types as T, synth
    lines = synth.line_list(3000, 600.0, 640.0, seed=3)
    twice = T.Lines(**{name: getattr(lines, name) for name, _ in T.Lines.FIELDS})
    twice.sp = (lines.sp * np.float32(2)).astype(np.float32)
    lay = T.layer_struct([1], [1e22], 2.479e24, 1013.25, 296.0)
    g = T.grid_struct(605.0, 635.0, 0.0101, 0.0101)
    ctrl = T.od_ctrl(precision=1, contnm_off=1)
    a, _, _ = oracle_mod.Session().odlay(lines, lay, g, ctrl)
    b, _, _ = oracle_mod.Session().odlay(twice, lay, g, ctrl)
    assert np.array_equal(b, 2 * a)


def test_interp_fixed_ratio_is_cubic_exact(oracle_mod):
    """n/(n+1) grid ratios use 4-point Lagrange weights: cubics come out
    exact away from the two extrapolated edge points."""
    dvin, n = 0.01, 400
    x = np.arange(n) * dvin
    f = 1.0 + x - 3 * x ** 2 + 0.5 * x ** 3
    for ratio in (2 / 3, 3 / 4, 3 / 2):
        dvout = dvin * ratio
        nout = int((n - 1) * dvin / dvout)
        out = oracle_mod.interp_spectrum(f, dvin, 500.0, dvout, 500.0, nout)
        xo = np.arange(nout) * dvout
        want = 1.0 + xo - 3 * xo ** 2 + 0.5 * xo ** 3
        inner = slice(4, nout - 4)
        np.testing.assert_allclose(out[inner], want[inner], rtol=1e-12)


def test_interp_general_ratio_linear_within_phase_step(oracle_mod):
    """A general ratio uses a 201-step phase table: a linear spectrum is
    reproduced to within one phase step (1/200 of an input interval)."""
    dvin, n = 0.01, 500
    f = 3.0 + 2.0 * np.arange(n)
    dvout = dvin * 0.7574
    nout = int((n - 1) * dvin / dvout)
    out = oracle_mod.interp_spectrum(f, dvin, 500.0, dvout, 500.0, nout)
    want = 3.0 + 2.0 * np.arange(nout) * dvout / dvin
    inner = slice(2, nout - 3)
    assert np.max(np.abs(out[inner] - want[inner])) <= 2.0 / 200 + 1e-9


def test_co2_continuum_at_table_nodes():
    """At T = 246 K (band-head factor 1) and ABSRB points on FRNCO2's 2 cm-1
    nodes, XINT returns the node value: S(I) * XFACCO2 * W(CO2) RHOAVE 1e-20
    (clblm_ODLAY_Continuum.f90:408-451, :1333-1410)."""
    from pathlib import Path
    txt = (Path(__file__).resolve().parents[1] / "clblm_gb300/csrc/clblm_ref_tables.h").read_text()

    def table(name, n):
        body = txt.split("static const double %s[%d] = {" % (name, n))[1].split("};")[0]
        return np.array([float(x) for x in body.replace("\n", " ").split(",") if x.strip()])

    S = table("CLBLM_CO2_S", 5003)
    XF = table("CLBLM_XFACCO2", 500)
    pave, tave, wco2 = 500.0, 246.0, 3e21
    v1abs, dvabs, n = 1996.0, 1.0, 1010
    a = oracle_mod_contnm(0, v1abs, dvabs, n, 1.0, 2000.0, 3000.0, pave, tave, wco2)
    rho = (pave / 1013.) * (296. / tave)
    w = wco2 * rho * 1e-20
    for v in (2000.0, 2100.0, 2386.0, 2400.0, 2434.0, 2998.0):
        i = int(round((v - v1abs) / dvabs)) + 1
        idx = int(round((v + 4.0) / 2.0)) + 1         # FRNCO2 index I: V = -4 + 2 (I - 1)
        jfac = int((v - 1998.) / 2. + 0.00001)
        want = S[idx - 1] * XF[jfac - 1] * w
        assert a[i] == pytest.approx(want, rel=1e-13), v


def _ref_table(name, n):
    from pathlib import Path
    txt = (Path(__file__).resolve().parents[1] / "clblm_gb300/csrc/clblm_ref_tables.h").read_text()
    body = txt.split("static const double %s[%d] = {" % (name, n))[1].split("};")[0]
    return np.array([float(x) for x in body.replace("\n", " ").split(",") if x.strip()])


def test_n2_rotation_continuum_at_table_nodes():
    """At T = 296 K (temperature factor 1) and ABSRB points on xn2_r's 5 cm-1
    nodes, XINT returns the node value C_296 * XN2CN (Wn2/XLOSMT) amagat
    (x_n2 + f_o2 x_o2 + x_h2o), f_o2 = (SF_296 - 1) 0.79/0.21
    (clblm_ODLAY_Continuum.f90:805-860, :2533-2600)."""
    from oracle import oracle as O
    C296 = _ref_table("CLBLM_N2R_C_296", 73)
    SF296 = _ref_table("CLBLM_N2R_SF_296", 73)
    pave, tave, wtot, wh2o, wo2 = 700.0, 296.0, 1.5e24, 4.0e21, 3.1e23
    v1abs, dvabs, n = 17.0, 1.0, 330
    a = O.contnm_n2(0, v1abs, dvabs, n, 1.0, 20.0, 340.0, pave, tave, wtot, wh2o, wo2)
    xh, xo = wh2o / wtot, wo2 / wtot
    xn = 1. - xh - xo
    tau = (xn * wtot / 2.68675e19) * (pave / 1013.) * (273. / tave)
    for v in (25.0, 50.0, 100.0, 200.0, 300.0, 335.0):
        i = int(round((v - v1abs) / dvabs)) + 1
        k = int(round((v + 10.0) / 5.0))              # xn2_r node: V = -10 + 5 (I - 1)
        fo2 = (SF296[k] - 1.) * 0.79 / 0.21
        want = tau * C296[k] * (xn + fo2 * xo + xh)
        assert a[i] == pytest.approx(want, rel=1e-13), v


def test_n2_continuum_linear_and_absent_for_derivative_od():
    """The N2 blocks scale exactly with XN2CN, vanish for the molecule
    derivative OD (CONTNM sets Wn2 = 0 when icflg > 0) and add nothing
    outside their bands (rotation < 350, fundamental 2001.77-2897.59 cm-1)."""
    from oracle import oracle as O
    args = (700.0, 250.0, 1.5e24, 4.0e21, 0.0)
    v1abs, dvabs, n = 1997.0, 1.0, 1000
    a1 = O.contnm_n2(1, v1abs, dvabs, n, 1.0, 2000.0, 2990.0, *args)
    a2 = O.contnm_n2(1, v1abs, dvabs, n, 2.0, 2000.0, 2990.0, *args)
    assert np.max(a1) > 0
    np.testing.assert_array_equal(a2, 2.0 * a1)
    a0 = O.contnm_n2(1, v1abs, dvabs, n, 1.0, 2000.0, 2990.0, *args, icflg=1)
    assert not np.any(a0)
    gap = O.contnm_n2(1, 497.0, 1.0, 1000, 1.0, 500.0, 1490.0, *args)
    assert not np.any(gap)


def oracle_mod_contnm(*args):
    from oracle import oracle as O
    return O.contnm_co2(*args)

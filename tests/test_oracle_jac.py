"""The oracle's Jacobian recurrence (Jacobians, clblm_noScattJac.f90:346-716)
against central finite differences of its own radiance (CPU only), and a
small end-to-end run of noScattJacob."""
import numpy as np
import pytest


def _column(nl, seed):
    rng = np.random.default_rng(seed)
    od = rng.uniform(0.01, 2.0, nl)
    amf_down = rng.uniform(1.2, 2.0, nl)
    tlev = np.linspace(288.0, 230.0, nl + 1) + rng.normal(0, 2, nl + 1)
    tlay = 0.5 * (tlev[:-1] + tlev[1:]) + rng.normal(0, 0.5, nl)
    return od, amf_down, tlev, tlay


@pytest.mark.parametrize("lin_in_tau", [0, 1, 2])
def test_recurrence_derivatives_match_central_differences(oracle_mod, lin_in_tau):
    nl, vn, tsfc, emis = 6, 900.0, 290.0, 0.93
    od, amfd, tlev, tlay = _column(nl, 3 + lin_in_tau)
    amfv = np.ones(nl)
    zero = np.zeros(nl)

    def rad_of(tau, tl=tlev, ts=tsfc, em=emis):
        return oracle_mod.jac_point(tau * amfv, tau * amfd, amfv, amfd, tlay, tl, ts, em, vn, lin_in_tau,
                                    zero, zero)[0]

    r, dta, dtl, dts, dem = oracle_mod.jac_point(od * amfv, od * amfd, amfv, amfd, tlay, tlev, tsfc, emis, vn,
                                                 lin_in_tau, zero, zero)
    assert r == pytest.approx(rad_of(od), rel=1e-15)
    for l in range(nl):
        h = 1e-5 * od[l]
        p, m = od.copy(), od.copy()
        p[l] += h
        m[l] -= h
        fd = (rad_of(p) - rad_of(m)) / (2 * h)
        assert dta[l] == pytest.approx(fd, rel=1e-6, abs=1e-12 * abs(r)), (l, dta[l], fd)
    if lin_in_tau != 0:  # level temperatures enter through the level Planck terms
        for lv in range(nl + 1):
            p, m = tlev.copy(), tlev.copy()
            p[lv] += 1e-3
            m[lv] -= 1e-3
            fd = (rad_of(od, tl=p) - rad_of(od, tl=m)) / 2e-3
            assert dtl[lv] == pytest.approx(fd, rel=1e-6, abs=1e-12 * abs(r)), (lv, dtl[lv], fd)
    fd = (rad_of(od, ts=tsfc + 1e-3) - rad_of(od, ts=tsfc - 1e-3)) / 2e-3
    assert dts == pytest.approx(fd, rel=1e-6)
    fd = (rad_of(od, em=emis + 1e-6) - rad_of(od, em=emis - 1e-6)) / 2e-6
    assert dem == pytest.approx(fd, rel=1e-6)


def test_small_jacobian_run(oracle_mod, mtckd):
    from clblm_gb300 import synth, capi_types as T
    lines, col, cont = synth.config1(n_lines=20000)
    # layers 10-12 (about 240-150 hPa): below the H2O floor, so the mixing
    # ratio differs between levels (level2layer divides by its log ratio)
    c = col.sub([10, 11, 12]).with_window(1000.0, 1004.0)
    prof = synth.jac_profile(col).sub(10, 3)
    ctrl = T.rt_ctrl(precision=T.CLBLM_PREC_PLAIN, grid_type=1)
    out = oracle_mod.jac_mode2(oracle_mod.Session(), lines, c, ctrl, prof, mtckd)
    n = len(out["rad"])
    assert n > 1000 and np.all(np.isfinite(out["rad"])) and np.all(out["rad"] > 0)
    for k in ("dtlev", "dqlev"):
        assert out[k].shape == (4, n) and np.all(np.isfinite(out[k]))
    # a warmer surface and a warmer top level raise the upwelling radiance
    assert np.all(out["dtsfc"] >= 0)
    assert np.median(out["dtlev"][3]) > 0


def _level2layer(plev, tlev, tave, q):
    """level2layer (clblm_noScattJac.f90:1208-1279), one molecule."""
    nl = len(tave)
    out = np.zeros((4, nl))
    for l in range(nl):
        rhoU = plev[l + 1] / (tlev[l + 1] * 1.3806503e-19)
        rhoL = plev[l] / (tlev[l] * 1.3806503e-19)
        alpha = rhoU / rhoL
        alphaT = -(tlev[l + 1] - tlev[l]) / np.log(alpha)
        out[1, l] = ((tave[l] - alphaT) / tlev[l]) * (rhoL / (rhoL - rhoU)) + (1.0 - alphaT / tlev[l]) / np.log(alpha)
        out[0, l] = ((tave[l] - alphaT) / tlev[l + 1]) * (-rhoU / (rhoL - rhoU)) - (1.0 - alphaT / tlev[l + 1]) / np.log(alpha)
        ratU, ratL = q[l + 1] / rhoU, q[l] / rhoL
        out[3, l] = (ratL / (ratL - alpha * ratU)) + 1.0 / np.log(alpha * ratU / ratL)
        out[2, l] = ((-alpha * ratU) / (ratL - alpha * ratU)) - 1.0 / np.log(alpha * ratU / ratL)
    return out  # dT_dTup, dT_dTlo, dW_dQup, dW_dQlo


def test_level_derivatives_compose_from_layer_ods(oracle_mod, mtckd):
    """drv_LevelTemp / drv_LevelConc rebuilt from separately computed ODs
    (viewing path, T+1 K, Wtot*1.01, H2O alone) and the per-point recurrence."""
    from clblm_gb300 import synth, capi_types as T
    lines, col, _ = synth.config1(n_lines=20000)
    first, nl = 10, 3
    c = col.sub(list(range(first, first + nl))).with_window(1000.0, 1001.0)
    prof = synth.jac_profile(col).sub(first, nl)
    ctrl = T.rt_ctrl(precision=T.CLBLM_PREC_PLAIN, grid_type=1, lin_in_tau=1)
    out = oracle_mod.jac_mode2(oracle_mod.Session(), lines, c, ctrl, prof, mtckd)
    dn, df, do = oracle_mod.Session().setdv(c, grid_type=1)
    tlev = np.append(c.tbot, c.ttop[-1])
    dTu, dTl, dWu, dWl = _level2layer(prof.plev, tlev, c.tave, prof.qlev)
    ods = {}
    for il in range(nl):
        g = T.grid_struct(c.v1, c.v2, dn[il], df[il], do)
        w_h2o = np.where(c.mol_id == 1, c.w[il], 0.0)
        for key, wtot, tave, w, jm in (("m", c.wtot[il], c.tave[il], c.w[il], 0),
                                       ("t", c.wtot[il], c.tave[il] + 1.0, c.w[il], 0),
                                       ("w", c.wtot[il] * 1.01, c.tave[il], c.w[il], 0),
                                       ("q", c.wtot[il], c.tave[il], w_h2o, 1)):
            lay = T.layer_struct(c.mol_id, w, wtot, c.pave[il], tave, lay_no=il + 1)
            od, dv, _ = oracle_mod.Session().odlay(lines, lay, g, T.od_ctrl(precision=1, jac_mol=jm), mtckd)
            ods[key, il] = od
    n = len(out["rad"])
    amfv, amfd = np.ones(nl), c.wtot_down / c.wtot
    for iv in range(0, n, 97):
        tau = np.array([ods["m", l][iv] for l in range(nl)])
        r, dta, dtl, _, _ = oracle_mod.jac_point(tau, tau * amfd, amfv, amfd, c.tave, tlev, c.tskin, c.emis,
                                                 c.v1 + iv * out["dv"], 1, dTu, dTl)
        assert r == pytest.approx(out["rad"][iv], rel=1e-13)
        lo = 0.0
        loq = 0.0
        for l in range(nl):
            dtau_dt = (ods["t", l][iv] - tau[l]) - (ods["w", l][iv] - tau[l]) / (0.01 * c.wtot[l]) * (c.wtot[l] / c.tave[l])
            up = dta[l] * dtau_dt * dTu[l]
            lo = lo + dta[l] * dtau_dt * dTl[l] + dtl[l]
            assert out["dtlev"][l, iv] == pytest.approx(lo, rel=1e-9, abs=1e-30)
            dq = dta[l] * ods["q", l][iv]
            upq = dq * dWu[l]
            loq = loq + dq * dWl[l]
            assert out["dqlev"][l, iv] == pytest.approx(loq, rel=1e-9, abs=1e-30)
            lo, loq = up, upq
        assert out["dtlev"][nl, iv] == pytest.approx(lo + dtl[nl], rel=1e-9, abs=1e-30)
        assert out["dqlev"][nl, iv] == pytest.approx(loq, rel=1e-9, abs=1e-30)

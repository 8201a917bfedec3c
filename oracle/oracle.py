"""ctypes binding of the CPU FP64 oracle (oracle/_build/libclblm_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, always as the checker.  The product never
imports this module.
"""
import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from clblm_gb300 import capi_types as T

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libclblm_oracle.so"


def build():
    """Compile the oracle with its Makefile (gcc)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("oracle error %d: %s" % (code, msg))
        self.code = code


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        P = C.POINTER
        L.ocl_create.restype = C.c_void_p
        L.ocl_destroy.argtypes = [C.c_void_p]
        L.ocl_reset.argtypes = [C.c_void_p]
        L.ocl_last_error.restype = C.c_char_p
        L.ocl_last_error.argtypes = [C.c_void_p]
        L.ocl_odlay.argtypes = [C.c_void_p, P(T.clblm_lines_t), P(T.clblm_cont_t), P(T.clblm_layer_t),
                                P(T.clblm_grid_t), P(T.clblm_od_ctrl_t), P(C.c_double), C.c_int64,
                                P(C.c_int64), P(C.c_double), P(T.clblm_od_stats_t)]
        L.ocl_set_trace.argtypes = [C.c_void_p, P(C.c_int32)] + [P(C.c_double)] * 4 + [P(C.c_int32), P(C.c_int64),
                                                                                     C.c_int64, P(C.c_int64)]
        L.ocl_rt_mode2.argtypes = [C.c_void_p, P(T.clblm_lines_t), P(T.clblm_cont_t), P(T.clblm_column_t),
                                   P(T.clblm_rt_ctrl_t), P(C.c_double), C.c_int64, P(C.c_int64),
                                   P(C.c_double)]
        L.ocl_rt_mode2_par.argtypes = [C.c_void_p, P(T.clblm_lines_t), P(T.clblm_cont_t), P(T.clblm_column_t),
                                       P(T.clblm_rt_ctrl_t), P(C.c_double), C.c_int64, P(C.c_int64),
                                       P(C.c_double), C.c_int]
        L.ocl_setdv.argtypes = [C.c_void_p, P(T.clblm_column_t), C.c_double, C.c_double, C.c_double,
                                C.c_int32, C.c_double, P(C.c_double), P(C.c_double), P(C.c_double)]
        L.ocl_shape_tables.argtypes = [P(C.c_double)] * 5
        L.ocl_radfn.restype = C.c_double
        L.ocl_radfn.argtypes = [C.c_double, C.c_double]
        L.ocl_planck.restype = C.c_double
        L.ocl_planck.argtypes = [C.c_double, C.c_double]
        L.ocl_rlin.argtypes = [C.c_double, P(C.c_double)]
        L.ocl_tips_scor.argtypes = [C.c_int, C.c_int, C.c_double, P(C.c_double)]
        L.ocl_interp_spectrum.argtypes = [P(C.c_double), C.c_double, C.c_double, C.c_int64, P(C.c_double),
                                          C.c_double, C.c_double, C.c_int64]
        L.ocl_jac_mode2.argtypes = [C.c_void_p, P(T.clblm_lines_t), P(T.clblm_cont_t), P(T.clblm_column_t),
                                    P(T.clblm_rt_ctrl_t), P(T.clblm_jac_t)] + [P(C.c_double)] * 5 + [
                                    C.c_int64, P(C.c_int64), P(C.c_double), C.c_int]
        L.ocl_contnm_co2.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, P(C.c_double)] + \
            [C.c_double] * 6
        L.ocl_contnm_n2.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, P(C.c_double)] + \
            [C.c_double] * 8 + [C.c_int]
        L.ocl_layer_amounts.argtypes = [C.c_int, C.c_int] + [P(C.c_double)] * 4 + [C.c_double] + [P(C.c_double)] * 5
        L.ocl_jac_point.argtypes = [P(C.c_double)] * 6 + [C.c_double] * 3 + [C.c_int, C.c_int] + [P(C.c_double)] * 7
        L.ocl_contnm_h2o.argtypes = [P(T.clblm_cont_t), C.c_int] + [C.c_double] * 8 + [P(C.c_double),
                                                                                    P(C.c_double), P(C.c_int)]
        L.ocl_contnm_o3o2.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, P(C.c_double)] + \
            [C.c_double] * 11
        L.ocl_path_amounts.argtypes = [C.c_int, C.c_int] + [P(C.c_double)] * 4 + [C.c_int, C.c_int] + \
            [C.c_double] * 4 + [C.c_int, P(C.c_double), C.c_int, C.c_int, P(C.c_int)] + [P(C.c_double)] * 9 + \
            [P(C.c_int), P(C.c_double)]
        L.ocl_fltrfn.argtypes = [P(C.c_double), C.c_double, C.c_double, C.c_int64, C.c_double, C.c_double, C.c_int,
                                 P(C.c_double), C.c_int, P(C.c_double)]
        L.ocl_scanfn.argtypes = [P(C.c_double), C.c_double, C.c_double, C.c_int64, C.c_int, C.c_double,
                                 C.c_double, C.c_double, C.c_double, P(P(C.c_double)), P(C.c_int64),
                                 P(C.c_double), P(C.c_double)]
        L.ocl_sf_interp.restype = C.c_int64
        L.ocl_sf_interp.argtypes = [P(C.c_double), C.c_double, C.c_double, C.c_int64, C.c_double, C.c_double,
                                    C.c_double, P(P(C.c_double))]
        L.ocl_sf_table.argtypes = [C.c_int, P(C.c_double)]
        L.ocl_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Session:
    """One reference 'process': holds the sticky JRAD state."""

    def __init__(self):
        self.h = lib().ocl_create()

    def __del__(self):
        if getattr(self, "h", None):
            lib().ocl_destroy(self.h)
            self.h = None

    def reset(self):
        lib().ocl_reset(self.h)

    def _check(self, rc):
        if rc != 0:
            raise OracleError(rc, lib().ocl_last_error(self.h).decode())

    def setdv(self, col, sample=4.0, alfal0=0.04, alfal0_fine=0.005, grid_type=0, dv_user=-1.0):
        n = col.nlay
        dn, df, do = np.zeros(n), np.zeros(n), C.c_double()
        cs = col.struct()
        self._check(lib().ocl_setdv(self.h, C.byref(cs), sample, alfal0, alfal0_fine, grid_type, dv_user,
                                    _dp(dn), _dp(df), C.byref(do)))
        return dn, df, do.value

    def odlay(self, lines, layer, grid, ctrl, cont=None):
        ls = lines.struct()
        cs = cont.struct() if cont is not None else None
        ns, dv, st = C.c_int64(), C.c_double(), T.clblm_od_stats_t()
        cap = int(np.ceil((grid.v2 - grid.v1) / min(grid.dv_normal, grid.dv_narrow,
                                                     grid.dv_out if grid.dv_out > 0 else 1e9))) + 64
        out = np.zeros(cap)
        rc = lib().ocl_odlay(self.h, C.byref(ls), C.byref(cs) if cs is not None else None, C.byref(layer),
                             C.byref(grid), C.byref(ctrl), _dp(out), cap, C.byref(ns), C.byref(dv),
                             C.byref(st))
        self._check(rc)
        return out[:ns.value].copy(), dv.value, st.as_dict()

    def odlay_trace(self, lines, layer, grid, ctrl, cont=None, shr_cap=None):
        """odlay plus the reference's line bookkeeping of the call: dict of
        line_panel [lines.n] (panel whose CNVFNQ pass convolved each line, -1
        none) and the TAPE9 pseudo-lines shr_vnu, shr_sp, shr_alfl, shr_alfd,
        shr_mol."""
        shr_cap = shr_cap or lines.n + 16
        tr = {"line_panel": np.full(lines.n, -1, dtype=np.int32), "shr_mol": np.zeros(shr_cap, dtype=np.int32),
              "shr_last": np.zeros(shr_cap, dtype=np.int64)}
        for k in ("shr_vnu", "shr_sp", "shr_alfl", "shr_alfd"):
            tr[k] = np.zeros(shr_cap)
        ns = C.c_int64()
        i32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
        lib().ocl_set_trace(self.h, i32(tr["line_panel"]), _dp(tr["shr_vnu"]), _dp(tr["shr_sp"]),
                            _dp(tr["shr_alfl"]), _dp(tr["shr_alfd"]), i32(tr["shr_mol"]),
                            tr["shr_last"].ctypes.data_as(C.POINTER(C.c_int64)), shr_cap, C.byref(ns))
        od, dv, st = self.odlay(lines, layer, grid, ctrl, cont)
        m = ns.value
        for k in ("shr_vnu", "shr_sp", "shr_alfl", "shr_alfd", "shr_mol", "shr_last"):
            tr[k] = tr[k][:m].copy()
        return od, dv, st, tr

    def rt_mode2(self, lines, col, ctrl, cont=None, nthreads=1, cap=None):
        """Radiance of a fresh reference process (the sticky JRAD is reset)."""
        ls, cols = lines.struct(), col.struct()
        cs = cont.struct() if cont is not None else None
        n, dv = C.c_int64(), C.c_double()
        if cap is None:
            dn, df, _ = self.setdv(col, ctrl.sample, ctrl.alfal0, ctrl.alfal0_fine, ctrl.grid_type, ctrl.dv_user)
            cap = int(np.ceil((col.v2 - col.v1) / min(dn.min(), df.min()))) + 64
        out = np.zeros(cap)
        self.reset()
        self._check(lib().ocl_rt_mode2_par(self.h, C.byref(ls), C.byref(cs) if cs is not None else None,
                                           C.byref(cols), C.byref(ctrl), _dp(out), cap, C.byref(n),
                                           C.byref(dv), int(nthreads)))
        return out[:n.value].copy(), dv.value


def jac_mode2(session, lines, col, ctrl, jac, cont=None, nthreads=1, cap=None):
    """noScattJacob on the uniform grid: dict of rad, dtlev [nlay+1, n],
    dqlev [nlay+1, n], dtsfc, demis and the grid (v1, dv)."""
    if cap is None:
        dn, df, do = session.setdv(col, ctrl.sample, ctrl.alfal0, ctrl.alfal0_fine, 1, ctrl.dv_user)
        cap = int(np.ceil((col.v2 - col.v1) / do)) + 64
    nl = col.nlay
    rad, dts, dem = np.zeros(cap), np.zeros(cap), np.zeros(cap)
    dtl, dql = np.zeros((nl + 1, cap)), np.zeros((nl + 1, cap))
    n, dv = C.c_int64(), C.c_double()
    ls, cs, js = lines.struct(), col.struct(), jac.struct()
    conts = cont.struct() if cont is not None else None
    session.reset()
    session._check(lib().ocl_jac_mode2(session.h, C.byref(ls), C.byref(conts) if conts is not None else None,
                                       C.byref(cs), C.byref(ctrl), C.byref(js), _dp(rad), _dp(dtl), _dp(dql),
                                       _dp(dts), _dp(dem), cap, C.byref(n), C.byref(dv), int(nthreads)))
    k = n.value
    return {"rad": rad[:k].copy(), "dtlev": dtl[:, :k].copy(), "dqlev": dql[:, :k].copy(), "dtsfc": dts[:k].copy(),
            "demis": dem[:k].copy(), "v1": col.v1, "dv": dv.value}


def jac_point(view_od, down_od, amf_view, amf_down, tlay, tlev, tsfc, emis, vn, lin_in_tau, dt_dtup, dt_dtlo):
    """The per-point recurrence of Jacobians: (rad, dRad_dTau, dRad_dTlev, dRad_dTsfc, dRad_dEmis)."""
    nl = len(view_od)
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (view_od, down_od, amf_view, amf_down, tlay, tlev,
                                                              dt_dtup, dt_dtlo)]
    dtl, dta = np.zeros(nl + 1), np.zeros(nl)
    r, ts, em = C.c_double(), C.c_double(), C.c_double()
    rc = lib().ocl_jac_point(_dp(a[0]), _dp(a[1]), _dp(a[2]), _dp(a[3]), _dp(a[4]), _dp(a[5]), float(tsfc),
                             float(emis), float(vn), nl, int(lin_in_tau), _dp(a[6]), _dp(a[7]), _dp(dtl), _dp(dta),
                             C.byref(r), C.byref(ts), C.byref(em))
    if rc:
        raise OracleError(rc, "jac_point")
    return r.value, dta, dtl, ts.value, em.value


def shape_tables():
    arrs = [np.zeros(3001) for _ in range(5)]
    lib().ocl_shape_tables(*[_dp(a) for a in arrs])
    return dict(zip(("F1", "F2", "F3", "FG", "XVER"), arrs))


def radfn(v, xkt):
    return lib().ocl_radfn(float(v), float(xkt))


def planck(v, xkt):
    return lib().ocl_planck(float(v), float(xkt))


def rlin(od):
    h = C.c_double()
    lib().ocl_rlin(float(od), C.byref(h))
    return h.value


def tips_scor(mol, t, iso=1):
    s = C.c_double()
    rc = lib().ocl_tips_scor(int(mol), int(iso), float(t), C.byref(s))
    if rc:
        raise OracleError(rc, "tips")
    return s.value


def interp_spectrum(spin, dvin, v1in, dvout, v1out, nout):
    spin = np.ascontiguousarray(spin, dtype=np.float64)
    out = np.zeros(nout)
    rc = lib().ocl_interp_spectrum(_dp(spin), dvin, v1in, len(spin), _dp(out), dvout, v1out, nout)
    if rc:
        raise OracleError(rc, "interp")
    return out


N_ABSRB = 5050


def contnm_h2o(cont, v1, v2, pave, tave, wtot, wk1, jrad=0, xself=1.0, xfrgn=1.0):
    """(V1ABS, ABSRB[:NPTABS]) of the H2O continuum on OPDPTH's 1 cm-1 grid."""
    out = np.zeros(N_ABSRB)
    v1abs, npt = C.c_double(), C.c_int()
    cs = cont.struct()
    rc = lib().ocl_contnm_h2o(C.byref(cs), int(jrad), v1, v2, pave, tave, wtot, wk1, xself, xfrgn, _dp(out),
                              C.byref(v1abs), C.byref(npt))
    if rc:
        raise OracleError(rc, "contnm_h2o")
    return v1abs.value, out[:npt.value].copy()


def layer_amounts(z, p, t, den, re=6371.23):
    """ALAYER + FPACK for a nadir path between the profile's levels: dict of
    pave, tave, wtot, w [nlay, nmol], secant."""
    z, p, t = (np.ascontiguousarray(a, dtype=np.float64) for a in (z, p, t))
    den = np.ascontiguousarray(den, dtype=np.float64)
    nlev, nmol = den.shape
    nl = nlev - 1
    out = {k: np.zeros(nl) for k in ("pave", "tave", "wtot", "secant")}
    out["w"] = np.zeros((nl, nmol))
    rc = lib().ocl_layer_amounts(nlev, nmol, _dp(z), _dp(p), _dp(t), _dp(den), float(re), _dp(out["pave"]),
                                 _dp(out["tave"]), _dp(out["wtot"]), _dp(out["w"]), _dp(out["secant"]))
    if rc:
        raise OracleError(rc, "layer amounts")
    return out


def contnm_n2(jrad, v1abs, dvabs, nptabs, xn2cn, v1, v2, pave, tave, wtot, wkh2o=0.0, wko2=0.0, icflg=0):
    """ABSRB(1..nptabs) of the N2 continua alone (1-based array, [0] unused)."""
    a = np.zeros(nptabs + 8)
    v2abs = v1abs + dvabs * (nptabs - 1)
    rc = lib().ocl_contnm_n2(jrad, v1abs, v2abs, dvabs, nptabs, _dp(a), xn2cn, v1, v2, pave, tave, wtot, wkh2o, wko2,
                             icflg)
    if rc:
        raise OracleError(rc, "contnm_n2")
    return a


def contnm_co2(jrad, v1abs, dvabs, nptabs, xco2c, v1, v2, pave, tave, wkco2):
    """ABSRB(1..nptabs) of the CO2 continuum alone (1-based array, [0] unused)."""
    a = np.zeros(nptabs + 8)
    v2abs = v1abs + dvabs * (nptabs - 1)
    rc = lib().ocl_contnm_co2(jrad, v1abs, v2abs, dvabs, nptabs, _dp(a), xco2c, v1, v2, pave, tave, wkco2)
    if rc:
        raise OracleError(rc, "contnm_co2")
    return a


def scanfn(spect, v1, dv, funct_id, hwhm, v1out, v2out, dvout=0.0):
    """clblm_SCANFN_array (clblm_ScanFilter.f90:33-67): (out, v1, dv) of the
    wavenumber-space scan of `spect` on v1 + i*dv.  funct_id 1..5
    (rectangle, triangle, Gaussian, sinc**2, sinc; negative: a sinc or
    sinc**2 given by its first zero), dvout <= 0: the function's default
    sampling."""
    sp = np.ascontiguousarray(spect, dtype=np.float64)
    out = C.POINTER(C.c_double)()
    n, v1o, dvo = C.c_int64(), C.c_double(), C.c_double()
    rc = lib().ocl_scanfn(_dp(sp), v1, dv, len(sp), funct_id, hwhm, v1out, v2out, dvout, C.byref(out), C.byref(n),
                          C.byref(v1o), C.byref(dvo))
    if rc:
        raise OracleError(rc, "SCANFN: %s" % {-1: "invalid functID", -2: "beyond the reference's buffers",
                                              -3: "no data"}.get(rc, "failed"))
    try:
        res = np.ctypeslib.as_array(out, shape=(n.value,)).copy() if n.value > 0 else np.zeros(0)
    finally:
        lib().ocl_free(out)
    return res, v1o.value, dvo.value


def sf_interp(spect, v1, dv, v1out, v2out, dvout):
    """clblm_INTERP (clblm_ScanFilter.f90:1975-2316), four-point scheme."""
    sp = np.ascontiguousarray(spect, dtype=np.float64)
    out = C.POINTER(C.c_double)()
    n = lib().ocl_sf_interp(_dp(sp), v1, dv, len(sp), v1out, v2out, dvout, C.byref(out))
    if n < 0:
        raise OracleError(int(n), "INTERP: no data")
    try:
        return np.ctypeslib.as_array(out, shape=(n,)).copy()
    finally:
        lib().ocl_free(out)


def sf_table(jfn):
    """SCANFN's function table XF(1..NFMAX) of JFN 1..4 (index 0 unused)."""
    xf = np.zeros(6020)
    lib().ocl_sf_table(jfn, _dp(xf))
    return xf


def contnm_o3o2(jrad, v1abs, dvabs, nptabs, v1, v2, pave, tave, wtot, wkh2o, wko3, wko2, xo3cn=1.0, xo2cn=1.0,
                xrayl=1.0):
    """CONTNM's O3 and O2 blocks and the Rayleigh extinction on ABSRB
    (1-based, v1abs + (i-1)*dvabs), alone."""
    a = np.zeros(nptabs + 8)
    v2abs = v1abs + dvabs * (nptabs - 1)
    rc = lib().ocl_contnm_o3o2(jrad, v1abs, v2abs, dvabs, nptabs, _dp(a), xo3cn, xo2cn, xrayl, v1, v2, pave, tave,
                               wtot, wkh2o, wko3, wko2)
    if rc:
        raise OracleError(rc, "contnm_o3o2")
    return a


def fltrfn(spect, v1, dv, v1f, dvf, xf, nfltpt=3001):
    """clblm_FLTRFN (clblm_ScanFilter.f90:1702-1897) of one channel."""
    sp = np.ascontiguousarray(spect, dtype=np.float64)
    x = np.ascontiguousarray(xf, dtype=np.float64)
    out = C.c_double()
    rc = lib().ocl_fltrfn(_dp(sp), v1, dv, len(sp), v1f, dvf, len(x), _dp(x), nfltpt, C.byref(out))
    if rc:
        raise OracleError(rc, "FLTRFN")
    return out.value


PATH_ERRORS = {-1: "bad arguments", -2: "impossible geometry (FSCGEO)", -3: "AMERGE", -4: "equal pressures",
               -5: "capacity", -6: "FPACK", -7: "zeroAbsAmt cut in the first layer"}


def path_amounts(z, p, t, den, h_obs, view_ang, z_rt=None, h2o=0, o2=-1, re=6371.23, xvbar=1000.0,
                 zero_abs_amt=0):
    """calculatePath (clblm_AtmPath.f90:871-964) for an observer at h_obs
    [km] looking at zenith angle view_ang [deg]: the output layers' dict
    (zlev, plev, tlev, qlev [nlay+1, nmol], pave, tave, wtot, w [nlay,
    nmol], secant, ipath) and the geometry (Hobs, Hend, ANGLE, PHI, HMIN,
    LEN as standardPathGeometry leaves them; RFPATH's RANGE, BETA, BENDNG
    and PHI_END)."""
    z, p, t = (np.ascontiguousarray(a, dtype=np.float64) for a in (z, p, t))
    den = np.ascontiguousarray(den, dtype=np.float64)
    nlev, nmol = den.shape
    zr = np.ascontiguousarray(z if z_rt is None else z_rt, dtype=np.float64)
    cap = nlev + len(zr) + 4
    zl, pl, tl = np.zeros(cap + 1), np.zeros(cap + 1), np.zeros(cap + 1)
    ql = np.zeros((cap + 1) * max(nmol, 1))
    pave, tave, wtot, sec = np.zeros(cap), np.zeros(cap), np.zeros(cap), np.zeros(cap)
    w = np.zeros(cap * max(nmol, 1))
    ipath = np.zeros(cap, dtype=np.int32)
    geom = np.zeros(10)
    n = C.c_int()
    rc = lib().ocl_path_amounts(nlev, nmol, _dp(z), _dp(p), _dp(t), _dp(den), h2o, o2, re, h_obs, view_ang, xvbar,
                                len(zr), _dp(zr), zero_abs_amt, cap, C.byref(n), _dp(zl), _dp(pl), _dp(tl), _dp(ql),
                                _dp(pave), _dp(tave), _dp(wtot), _dp(w), _dp(sec),
                                ipath.ctypes.data_as(C.POINTER(C.c_int)), _dp(geom))
    if rc:
        raise OracleError(rc, "path: " + PATH_ERRORS.get(rc, "failed"))
    k = n.value
    out = dict(zlev=zl[:k + 1], plev=pl[:k + 1], tlev=tl[:k + 1], qlev=ql[:(k + 1) * nmol].reshape(k + 1, nmol),
               pave=pave[:k], tave=tave[:k], wtot=wtot[:k], w=w[:k * nmol].reshape(k, nmol), secant=sec[:k],
               ipath=ipath[:k])
    names = ("Hobs", "Hend", "ANGLE", "PHI", "HMIN", "LEN", "RANGE", "BETA", "BENDNG", "PHI_END")
    return out, dict(zip(names, geom))

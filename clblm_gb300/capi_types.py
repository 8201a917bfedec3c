"""ctypes mirrors of the C-ABI structs declared in include/clblm_gb300.h.

Only plain data lives here: the structs, the status codes and helpers that
build a struct from numpy arrays while keeping the arrays alive.
"""
import ctypes as C

import numpy as np

CLBLM_OK = 0
CLBLM_ERR_ARG = 1
CLBLM_ERR_UNSORTED = 2
CLBLM_ERR_GRID = 3
CLBLM_ERR_DV_RATIO = 4
CLBLM_ERR_RANGE = 5
CLBLM_ERR_UNSUPPORTED = 6
CLBLM_ERR_OOM = 7
CLBLM_ERR_CUDA = 8
CLBLM_ERR_CAPACITY = 9
CLBLM_ERR_NO_DEVICE = 10

CLBLM_OUT_HOST = 0
CLBLM_OUT_DEVICE = 1
CLBLM_PREC_MIXED = 0
CLBLM_PREC_PLAIN = 1
LINES_PER_RECORD = 250

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)


class clblm_lines_t(C.Structure):
    _fields_ = [("n", C.c_int64), ("vnu", _dp), ("sp", _fp), ("alfa", _fp), ("epp", _fp),
                ("mol", _ip), ("hwhm", _fp), ("tmpalf", _fp), ("pshift", _fp), ("iflg", _ip)]


class clblm_cont_t(C.Structure):
    _fields_ = [("n", C.c_int32), ("v1", C.c_double), ("dv", C.c_double),
                ("self_absco_ref", _dp), ("for_absco_ref", _dp), ("self_texp", _dp),
                ("ref_press", C.c_double), ("ref_temp", C.c_double)]


class clblm_layer_t(C.Structure):
    _fields_ = [("nmol", C.c_int32), ("mol_id", _ip), ("w", _dp), ("wtot", C.c_double),
                ("pave", C.c_double), ("tave", C.c_double), ("zbot", C.c_double),
                ("ztop", C.c_double), ("lay_no", C.c_int32)]


class clblm_grid_t(C.Structure):
    _fields_ = [("v1", C.c_double), ("v2", C.c_double), ("dv_normal", C.c_double),
                ("dv_narrow", C.c_double), ("dv_out", C.c_double), ("sample", C.c_double),
                ("alfal0", C.c_double)]


class clblm_od_ctrl_t(C.Structure):
    _fields_ = [("jrad", C.c_int32), ("line_rejec", C.c_int32), ("dptmin", C.c_double),
                ("dptfac", C.c_double), ("xself", C.c_double), ("xfrgn", C.c_double),
                ("contnm_off", C.c_int32), ("line_off", C.c_int32), ("precision", C.c_int32),
                ("jac_mol", C.c_int32), ("reserved", C.c_int32), ("xco2c", C.c_double), ("xn2cn", C.c_double),
                ("xo3cn", C.c_double), ("xo2cn", C.c_double), ("xrayl", C.c_double)]


class clblm_column_t(C.Structure):
    _fields_ = [("nlay", C.c_int32), ("nmol", C.c_int32), ("mol_id", _ip), ("pave", _dp),
                ("tave", _dp), ("tbot", _dp), ("ttop", _dp), ("w", _dp), ("wtot", _dp),
                ("wtot_down", _dp), ("v1", C.c_double), ("v2", C.c_double),
                ("tskin", C.c_double), ("emis", C.c_double)]


class clblm_jac_t(C.Structure):
    _fields_ = [("plev", _dp), ("qlev", _dp), ("jac_mol", C.c_int32), ("do_temp", C.c_int32)]


class clblm_profile_t(C.Structure):
    _fields_ = [("col", C.POINTER(clblm_column_t)), ("jac", C.POINTER(clblm_jac_t)),
                ("rad", _dp), ("dr_dtlev", _dp), ("dr_dqlev", _dp), ("dr_dtskin", _dp), ("dr_demis", _dp),
                ("cap", C.c_int64), ("status", C.c_int32), ("reserved", C.c_int32)]


CLBLM_BATCH_GRAPH = 0x10


class clblm_scan_t(C.Structure):
    _fields_ = [("funct_id", C.c_int32), ("deconv_prebox", C.c_int32), ("hwhm", C.c_double),
                ("padding", C.c_double), ("prebox_hw", C.c_double), ("v1out", C.c_double), ("v2out", C.c_double),
                ("dvout", C.c_double), ("parms", C.c_double * 3)]


def scan_struct(funct_id, hwhm, v1out, v2out, padding=0.0, prebox_hw=-1.0, deconv_prebox=0, dvout=0.0,
                parms=(0.0, 0.0, 0.0)):
    return clblm_scan_t(funct_id, deconv_prebox, hwhm, padding, prebox_hw, v1out, v2out, dvout,
                        (C.c_double * 3)(*parms))


class clblm_scanfn_t(C.Structure):
    _fields_ = [("funct_id", C.c_int32), ("reserved", C.c_int32), ("hwhm", C.c_double), ("v1out", C.c_double),
                ("v2out", C.c_double), ("dvout", C.c_double)]


def scanfn_struct(funct_id, hwhm, v1out, v2out, dvout=0.0):
    return clblm_scanfn_t(funct_id, 0, hwhm, v1out, v2out, dvout)


class clblm_path_in_t(C.Structure):
    _fields_ = [("nlev", C.c_int32), ("nmol", C.c_int32), ("z", C.POINTER(C.c_double)),
                ("p", C.POINTER(C.c_double)), ("t", C.POINTER(C.c_double)), ("den", C.POINTER(C.c_double)),
                ("h2o", C.c_int32), ("o2", C.c_int32), ("earth_radius", C.c_double), ("obs_alt", C.c_double),
                ("view_ang", C.c_double), ("v_refrac", C.c_double), ("nrt", C.c_int32),
                ("z_rt", C.POINTER(C.c_double)), ("zero_abs_amt", C.c_int32)]


class clblm_path_t(C.Structure):
    _fields_ = [("cap", C.c_int32), ("nlay", C.c_int32)] + \
        [(f, C.POINTER(C.c_double)) for f in ("z", "p", "t", "q", "pave", "tave", "wtot", "w", "secant")] + \
        [("ipath", C.POINTER(C.c_int32))] + [(f, C.c_double) for f in ("hobs", "hend", "angle", "phi", "hmin")] + \
        [("len", C.c_int32)] + [(f, C.c_double) for f in ("range", "beta", "bendng", "phi_end")]


class JacProfile:
    """Level pressures [mb] and Jacobian-molecule number densities [molec/cm3]
    (level 0 at the surface) and the clblm_jac_t view of them."""

    def __init__(self, plev, qlev, jac_mol=1, do_temp=1):
        self.plev = np.ascontiguousarray(plev, dtype=np.float64)
        self.qlev = np.ascontiguousarray(qlev, dtype=np.float64)
        self.jac_mol, self.do_temp = int(jac_mol), int(do_temp)

    def struct(self):
        j = clblm_jac_t()
        j.plev = _ptr(self.plev, C.c_double)
        j.qlev = _ptr(self.qlev, C.c_double)
        j.jac_mol, j.do_temp = self.jac_mol, self.do_temp
        j._keep = self
        return j

    def sub(self, first, count):
        """Levels of layers first .. first+count-1."""
        return JacProfile(self.plev[first:first + count + 1], self.qlev[first:first + count + 1],
                          self.jac_mol, self.do_temp)


class clblm_rt_ctrl_t(C.Structure):
    _fields_ = [("lin_in_tau", C.c_int32), ("grid_type", C.c_int32), ("sample", C.c_double),
                ("alfal0", C.c_double), ("alfal0_fine", C.c_double), ("dv_user", C.c_double),
                ("od", clblm_od_ctrl_t)]


class clblm_od_stats_t(C.Structure):
    _fields_ = [("nlin", C.c_int64), ("lincnt", C.c_int64), ("nminus", C.c_int64),
                ("nplus", C.c_int64), ("nshrunk", C.c_int64), ("npanels", C.c_int64),
                ("nsamp", C.c_int64), ("dv", C.c_double), ("dvr4", C.c_double),
                ("jrad", C.c_int32), ("launches", C.c_int64), ("cnvfnq_steps", C.c_int64),
                ("cnvf4q_steps", C.c_int64), ("ms_panel", C.c_double), ("ms_f4conv", C.c_double),
                ("ms_line_chain", C.c_double), ("ms_f4_chain", C.c_double),
                ("f4_stage_records", C.c_int32), ("rt_threads", C.c_int32), ("jac_threads", C.c_int32),
                ("reserved", C.c_int32), ("ms_rt", C.c_double), ("rt_bytes", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class Lines:
    """A line list held as contiguous numpy arrays with TAPE3 precision and
    the clblm_lines_t view of it."""

    FIELDS = (("vnu", np.float64), ("sp", np.float32), ("alfa", np.float32),
              ("epp", np.float32), ("mol", np.int32), ("hwhm", np.float32),
              ("tmpalf", np.float32), ("pshift", np.float32), ("iflg", np.int32))

    def __init__(self, **arrays):
        n = len(arrays["vnu"])
        for name, dt in self.FIELDS:
            a = np.ascontiguousarray(arrays[name], dtype=dt)
            if a.shape != (n,):
                raise ValueError("line field %s has shape %s, want (%d,)" % (name, a.shape, n))
            setattr(self, name, a)
        self.n = n

    def subset(self, lo, hi):
        return Lines(**{name: getattr(self, name)[lo:hi] for name, _ in self.FIELDS})

    def keys(self):
        """The centres as sort keys: a coefficient record (IFLG < 0, after a
        coupled line) takes its line's centre."""
        k = np.where(self.iflg >= 0, self.vnu, -np.inf)
        return np.maximum.accumulate(k) if self.n else k

    def window(self, v1, v2):
        lo, hi = np.searchsorted(self.keys(), [v1, v2])
        return self.subset(int(lo), int(hi))

    def struct(self):
        s = clblm_lines_t()
        s.n = self.n
        s.vnu = _ptr(self.vnu, C.c_double)
        for name in ("sp", "alfa", "epp", "hwhm", "tmpalf", "pshift"):
            setattr(s, name, _ptr(getattr(self, name), C.c_float))
        s.mol = _ptr(self.mol, C.c_int32)
        s.iflg = _ptr(self.iflg, C.c_int32)
        s._keep = self
        return s

    def nbytes(self):
        return sum(getattr(self, name).nbytes for name, _ in self.FIELDS)


class Continuum:
    """MT_CKD-style continuum table (wavenumbers v1 + i*dv)."""

    def __init__(self, v1, dv, self_absco_ref, for_absco_ref, self_texp, ref_press=1013.0,
                 ref_temp=296.0):
        self.v1 = float(v1)
        self.dv = float(dv)
        self.self_absco_ref = np.ascontiguousarray(self_absco_ref, dtype=np.float64)
        self.for_absco_ref = np.ascontiguousarray(for_absco_ref, dtype=np.float64)
        self.self_texp = np.ascontiguousarray(self_texp, dtype=np.float64)
        self.ref_press = float(ref_press)
        self.ref_temp = float(ref_temp)

    def struct(self):
        s = clblm_cont_t()
        s.n = len(self.self_absco_ref)
        s.v1, s.dv = self.v1, self.dv
        s.self_absco_ref = _ptr(self.self_absco_ref, C.c_double)
        s.for_absco_ref = _ptr(self.for_absco_ref, C.c_double)
        s.self_texp = _ptr(self.self_texp, C.c_double)
        s.ref_press, s.ref_temp = self.ref_press, self.ref_temp
        s._keep = self
        return s


def layer_struct(mol_id, w, wtot, pave, tave, lay_no=1, zbot=0.0, ztop=0.0):
    mol_id = np.ascontiguousarray(mol_id, dtype=np.int32)
    w = np.ascontiguousarray(w, dtype=np.float64)
    s = clblm_layer_t()
    s.nmol = len(mol_id)
    s.mol_id = _ptr(mol_id, C.c_int32)
    s.w = _ptr(w, C.c_double)
    s.wtot, s.pave, s.tave = float(wtot), float(pave), float(tave)
    s.zbot, s.ztop, s.lay_no = float(zbot), float(ztop), int(lay_no)
    s._keep = (mol_id, w)
    return s


def grid_struct(v1, v2, dv_normal, dv_narrow, dv_out=-999.9, sample=4.0, alfal0=0.04):
    g = clblm_grid_t()
    g.v1, g.v2 = float(v1), float(v2)
    g.dv_normal, g.dv_narrow, g.dv_out = float(dv_normal), float(dv_narrow), float(dv_out)
    g.sample, g.alfal0 = float(sample), float(alfal0)
    return g


def od_ctrl(precision=CLBLM_PREC_MIXED, jrad=1, line_rejec=1, dptmin=0.0, dptfac=0.0,
            xself=1.0, xfrgn=1.0, contnm_off=0, line_off=0, jac_mol=0, xco2c=1.0, xn2cn=1.0, xo3cn=1.0,
            xo2cn=1.0, xrayl=1.0):
    """CLBLM_OD_Ctrl with the reference's defaults (clblm_Config.f90:88-110)."""
    c = clblm_od_ctrl_t()
    c.jrad, c.line_rejec, c.dptmin, c.dptfac = jrad, line_rejec, dptmin, dptfac
    c.xself, c.xfrgn, c.contnm_off, c.line_off = xself, xfrgn, contnm_off, line_off
    c.precision, c.jac_mol, c.xco2c, c.xn2cn = precision, jac_mol, xco2c, xn2cn
    c.xo3cn, c.xo2cn, c.xrayl = xo3cn, xo2cn, xrayl
    return c


def rt_ctrl(precision=CLBLM_PREC_MIXED, lin_in_tau=1, grid_type=0, sample=4.0, alfal0=0.04,
            alfal0_fine=0.005, dv_user=-1.0, contnm_off=0):
    r = clblm_rt_ctrl_t()
    r.lin_in_tau, r.grid_type, r.sample = lin_in_tau, grid_type, sample
    r.alfal0, r.alfal0_fine, r.dv_user = alfal0, alfal0_fine, dv_user
    r.od = od_ctrl(precision=precision, contnm_off=contnm_off)
    return r


class Column:
    """A nadir column (layer 0 at the bottom) and its clblm_column_t view."""

    def __init__(self, mol_id, pave, tave, tbot, ttop, w, wtot, wtot_down, v1, v2, tskin,
                 emis):
        self.mol_id = np.ascontiguousarray(mol_id, dtype=np.int32)
        self.pave = np.ascontiguousarray(pave, dtype=np.float64)
        self.tave = np.ascontiguousarray(tave, dtype=np.float64)
        self.tbot = np.ascontiguousarray(tbot, dtype=np.float64)
        self.ttop = np.ascontiguousarray(ttop, dtype=np.float64)
        self.w = np.ascontiguousarray(w, dtype=np.float64)
        self.wtot = np.ascontiguousarray(wtot, dtype=np.float64)
        self.wtot_down = np.ascontiguousarray(wtot_down, dtype=np.float64)
        self.v1, self.v2, self.tskin, self.emis = float(v1), float(v2), float(tskin), float(emis)
        self.nlay = len(self.pave)
        assert self.w.shape == (self.nlay, len(self.mol_id))

    def struct(self):
        s = clblm_column_t()
        s.nlay, s.nmol = self.nlay, len(self.mol_id)
        s.mol_id = _ptr(self.mol_id, C.c_int32)
        for name in ("pave", "tave", "tbot", "ttop", "w", "wtot", "wtot_down"):
            setattr(s, name, _ptr(getattr(self, name), C.c_double))
        s.v1, s.v2, s.tskin, s.emis = self.v1, self.v2, self.tskin, self.emis
        s._keep = self
        return s

    def layer(self, il):
        return layer_struct(self.mol_id, self.w[il], self.wtot[il], self.pave[il], self.tave[il],
                            lay_no=il + 1)

    # optional level profiles ([nlay+1, ...], level 0 at the bottom)
    LEVEL_FIELDS = ("p_lev", "q_h2o_lev", "z_lev", "vmr_lev")

    def sub(self, layers):
        idx = np.asarray(layers)
        c = Column(self.mol_id, self.pave[idx], self.tave[idx], self.tbot[idx], self.ttop[idx],
                   self.w[idx], self.wtot[idx], self.wtot_down[idx], self.v1, self.v2,
                   self.tskin, self.emis)
        if len(idx) and np.all(np.diff(idx) == 1):  # contiguous layers keep their levels
            for f in self.LEVEL_FIELDS:
                if hasattr(self, f):
                    setattr(c, f, getattr(self, f)[idx[0]:idx[-1] + 2])
        return c

    def with_window(self, v1, v2):
        c = Column(self.mol_id, self.pave, self.tave, self.tbot, self.ttop, self.w, self.wtot,
                   self.wtot_down, v1, v2, self.tskin, self.emis)
        for f in self.LEVEL_FIELDS:
            if hasattr(self, f):
                setattr(c, f, getattr(self, f))
        return c

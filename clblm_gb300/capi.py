"""ctypes binding of the GB300 C-ABI (libclblm_gb300.so, include/clblm_gb300.h)
and a host-side mirror of the reference's interface for this path:

  ODLAY(...)               -> clblm_gpu_od          (ODLAY_nonStruct, clblm_ODLAY.f90:129)
  setDV(...)               -> clblm_setdv           (setDV_struct, clblm_setDV.f90:114)
  mode2_lookDn_mergeUp(...)-> clblm_gpu_rt_mode2    (clblm_noScattRT.f90:1134)

The library is loaded from the package directory; if it has not been built,
or no CUDA device is usable, calls fail loudly (there is no CPU fallback).
"""
import ctypes as C
from pathlib import Path

import numpy as np

from . import capi_types as T

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libclblm_gb300.so"

EXPORTS = ("clblm_gpu_create", "clblm_gpu_set_lines", "clblm_gpu_destroy", "clblm_gpu_last_error",
           "clblm_gpu_stream",
           "clblm_setdv", "clblm_gpu_od_size", "clblm_gpu_od", "clblm_gpu_od_stats",
           "clblm_gpu_rt_mode2_size", "clblm_gpu_rt_mode2", "clblm_gpu_jac_size", "clblm_gpu_jac",
           "clblm_tape3_read", "clblm_gpu_interp_spectrum_noalloc", "clblm_gpu_batch_size", "clblm_gpu_batch",
           "clblm_gpu_fftscn_size", "clblm_gpu_fftscn", "clblm_gpu_scanfn_size", "clblm_gpu_scanfn",
           "clblm_gpu_layer_amounts", "clblm_gpu_od_lines", "clblm_gpu_jac_vjp", "clblm_gpu_filter", "clblm_path")

NOALLOC_MAX_POINTS = 1 << 20  # CLBLM_NOALLOC_MAX_POINTS


class ClblmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("clblm error %d: %s" % (code, msg))
        self.code = code


_lib = None


def lib():
    """Load libclblm_gb300.so (raises if it is missing)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ClblmError(T.CLBLM_ERR_NO_DEVICE,
                             "%s not built: run `python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
        L = C.CDLL(str(LIB_PATH))
        P = C.POINTER
        L.clblm_gpu_create.argtypes = [P(T.clblm_lines_t), P(T.clblm_cont_t), C.c_int, P(C.c_void_p)]
        L.clblm_gpu_set_lines.argtypes = [C.c_void_p, P(T.clblm_lines_t)]
        L.clblm_gpu_destroy.argtypes = [C.c_void_p]
        L.clblm_gpu_last_error.argtypes = [C.c_void_p]
        L.clblm_gpu_last_error.restype = C.c_char_p
        L.clblm_gpu_stream.argtypes = [C.c_void_p]
        L.clblm_gpu_stream.restype = C.c_void_p
        L.clblm_setdv.argtypes = [P(T.clblm_column_t), C.c_double, C.c_double, C.c_double, C.c_int32,
                                  C.c_double, P(C.c_double), P(C.c_double), P(C.c_double)]
        L.clblm_gpu_od_size.argtypes = [C.c_void_p, P(T.clblm_layer_t), P(T.clblm_grid_t),
                                        P(T.clblm_od_ctrl_t), P(C.c_int64), P(C.c_double)]
        L.clblm_gpu_od.argtypes = [C.c_void_p, P(T.clblm_layer_t), P(T.clblm_grid_t), P(T.clblm_od_ctrl_t),
                                   C.c_void_p, C.c_int64, C.c_int32]
        L.clblm_gpu_od_stats.argtypes = [C.c_void_p, P(T.clblm_od_stats_t)]
        L.clblm_gpu_od_lines.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int64), P(C.c_int32), C.c_int64,
                                         P(C.c_int64)] + [P(C.c_double)] * 4 + [P(C.c_int32), P(C.c_int64),
                                                                                 C.c_int64]
        L.clblm_gpu_rt_mode2_size.argtypes = [C.c_void_p, P(T.clblm_column_t), P(T.clblm_rt_ctrl_t),
                                              P(C.c_int64), P(C.c_double)]
        L.clblm_gpu_rt_mode2.argtypes = [C.c_void_p, P(T.clblm_column_t), P(T.clblm_rt_ctrl_t), C.c_void_p,
                                         C.c_int64, C.c_int32]
        L.clblm_gpu_jac_size.argtypes = [C.c_void_p, P(T.clblm_column_t), P(T.clblm_rt_ctrl_t), P(T.clblm_jac_t),
                                         P(C.c_int64), P(C.c_double)]
        L.clblm_gpu_jac.argtypes = [C.c_void_p, P(T.clblm_column_t), P(T.clblm_rt_ctrl_t), P(T.clblm_jac_t)] + \
            [C.c_void_p] * 5 + [C.c_int64, C.c_int32]
        L.clblm_gpu_jac_vjp.argtypes = [C.c_void_p, P(T.clblm_column_t), P(T.clblm_rt_ctrl_t), P(T.clblm_jac_t),
                                        C.c_void_p, C.c_int64] + [P(C.c_double)] * 4 + [C.c_int32]
        L.clblm_gpu_batch_size.argtypes = [C.c_void_p, P(T.clblm_profile_t), C.c_int32, P(T.clblm_rt_ctrl_t),
                                           P(C.c_int64), P(C.c_double)]
        L.clblm_gpu_batch.argtypes = [C.c_void_p, P(T.clblm_profile_t), C.c_int32, P(T.clblm_rt_ctrl_t), C.c_int32]
        L.clblm_gpu_fftscn_size.argtypes = [P(T.clblm_scan_t), C.c_double, C.c_double, C.c_int64, P(C.c_double),
                                            P(C.c_double), P(C.c_int64)]
        L.clblm_gpu_fftscn.argtypes = [C.c_void_p, P(T.clblm_scan_t), C.c_void_p, C.c_double, C.c_double, C.c_int64,
                                       C.c_void_p, C.c_int64, C.c_int32]
        L.clblm_gpu_scanfn_size.argtypes = [P(T.clblm_scanfn_t), C.c_double, C.c_double, C.c_int64, P(C.c_double),
                                            P(C.c_double), P(C.c_int64)]
        L.clblm_gpu_scanfn.argtypes = [C.c_void_p, P(T.clblm_scanfn_t), C.c_void_p, C.c_double, C.c_double, C.c_int64,
                                       C.c_void_p, C.c_int64, C.c_int32]
        L.clblm_gpu_filter.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int64, C.c_int32,
                                       P(C.c_double), P(C.c_double), P(C.c_int32), P(C.c_double), P(C.c_double)]
        L.clblm_gpu_layer_amounts.argtypes = [C.c_void_p, C.c_int32, C.c_int32] + [P(C.c_double)] * 4 + \
            [C.c_double] + [P(C.c_double)] * 5
        L.clblm_path.argtypes = [P(T.clblm_path_in_t), P(T.clblm_path_t), C.c_char_p, C.c_int32]
        L.clblm_tape3_read.argtypes = [C.c_char_p, C.c_double, C.c_double, P(T.clblm_lines_t), C.c_int64,
                                       P(C.c_int64), C.c_char_p, C.c_int32]
        L.clblm_gpu_interp_spectrum_noalloc.argtypes = [C.c_void_p, C.c_int64, C.c_double, C.c_double,
                                                        C.c_void_p, C.c_int64, C.c_double, C.c_void_p]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Handle:
    """A device-resident line list (+ continuum table) and the reference's
    per-process state (the sticky JRAD)."""

    def __init__(self, lines, cont=None, device=0):
        self.lines = lines
        self.cont = cont
        ls = lines.struct()
        cs = cont.struct() if cont is not None else None
        h = C.c_void_p()
        rc = lib().clblm_gpu_create(C.byref(ls), C.byref(cs) if cs is not None else None, device, C.byref(h))
        if rc:
            raise ClblmError(rc, lib().clblm_gpu_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().clblm_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise ClblmError(rc, lib().clblm_gpu_last_error(self.h).decode())

    def stream(self):
        """cudaStream_t of the handle (as an int)."""
        return lib().clblm_gpu_stream(self.h)

    def set_lines(self, lines):
        self.lines = lines
        ls = lines.struct()
        self._check(lib().clblm_gpu_set_lines(self.h, C.byref(ls)))

    def od_size(self, layer, grid, ctrl):
        n, dv = C.c_int64(), C.c_double()
        self._check(lib().clblm_gpu_od_size(self.h, C.byref(layer), C.byref(grid), C.byref(ctrl), C.byref(n),
                                            C.byref(dv)))
        return n.value, dv.value

    def odlay(self, layer, grid, ctrl, out=None):
        """Layer OD (binary64) on v1 + i*dv; returns (od, dv)."""
        n, dv = self.od_size(layer, grid, ctrl)
        if out is None:
            out = np.empty(n)
        self._check(lib().clblm_gpu_od(self.h, C.byref(layer), C.byref(grid), C.byref(ctrl),
                                       out.ctypes.data_as(C.c_void_p), len(out), T.CLBLM_OUT_HOST))
        return out[:n], dv

    def od_device(self, layer, grid, ctrl, dptr, cap):
        """Layer OD written to a device buffer (e.g. torch tensor data_ptr())."""
        self._check(lib().clblm_gpu_od(self.h, C.byref(layer), C.byref(grid), C.byref(ctrl), C.c_void_p(dptr),
                                       cap, T.CLBLM_OUT_DEVICE))

    def od_lines(self):
        """Line selection of the last odlay call (clblm_gpu_od_lines): dict of
        line_lo, line_panel [n_lines] (panel that convolved each line of the
        window, -1 rejected) and the far-wing pseudo-lines shr_vnu, shr_sp,
        shr_alfl, shr_alfd, shr_mol in TAPE9 order."""
        lo, nl, ns = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(lib().clblm_gpu_od_lines(self.h, C.byref(lo), C.byref(nl), None, 0, C.byref(ns), None, None, None,
                                             None, None, None, 0))
        n, m = nl.value, ns.value
        out = {"line_lo": lo.value, "line_panel": np.zeros(n, dtype=np.int32)}
        for k in ("shr_vnu", "shr_sp", "shr_alfl", "shr_alfd"):
            out[k] = np.zeros(m)
        out["shr_mol"] = np.zeros(m, dtype=np.int32)
        out["shr_last"] = np.zeros(m, dtype=np.int64)
        i32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
        self._check(lib().clblm_gpu_od_lines(self.h, C.byref(lo), C.byref(nl), i32(out["line_panel"]), n,
                                             C.byref(ns), _dp(out["shr_vnu"]), _dp(out["shr_sp"]),
                                             _dp(out["shr_alfl"]), _dp(out["shr_alfd"]), i32(out["shr_mol"]),
                                             out["shr_last"].ctypes.data_as(C.POINTER(C.c_int64)), m))
        return out

    def stats(self):
        s = T.clblm_od_stats_t()
        self._check(lib().clblm_gpu_od_stats(self.h, C.byref(s)))
        return s.as_dict()

    def rt_size(self, col, ctrl):
        n, dv = C.c_int64(), C.c_double()
        cs = col.struct()
        self._check(lib().clblm_gpu_rt_mode2_size(self.h, C.byref(cs), C.byref(ctrl), C.byref(n), C.byref(dv)))
        return n.value, dv.value

    def rt_mode2(self, col, ctrl, out=None):
        """Nadir upwelling radiance at the top of `col`; returns (rad, dv)."""
        n, dv = self.rt_size(col, ctrl)
        if out is None:
            out = np.empty(n)
        cs = col.struct()
        self._check(lib().clblm_gpu_rt_mode2(self.h, C.byref(cs), C.byref(ctrl), out.ctypes.data_as(C.c_void_p),
                                             len(out), T.CLBLM_OUT_HOST))
        return out[:n], dv

    def rt_mode2_device(self, col, ctrl, dptr, cap):
        cs = col.struct()
        self._check(lib().clblm_gpu_rt_mode2(self.h, C.byref(cs), C.byref(ctrl), C.c_void_p(dptr), cap,
                                             T.CLBLM_OUT_DEVICE))


def _jac_methods():
    def jac_size(self, col, ctrl, jac):
        n, dv = C.c_int64(), C.c_double()
        cs, js = col.struct(), jac.struct()
        self._check(lib().clblm_gpu_jac_size(self.h, C.byref(cs), C.byref(ctrl), C.byref(js), C.byref(n),
                                             C.byref(dv)))
        return n.value, dv.value

    def jac(self, col, ctrl, jac):
        """Radiance and Jacobians (noScattJacob) on the uniform grid: dict of
        rad, dtlev [nlay+1, n], dqlev [nlay+1, n], dtsfc, demis, v1, dv."""
        n, dv = self.jac_size(col, ctrl, jac)
        nl = col.nlay
        out = {"rad": np.empty(n), "dtsfc": np.empty(n), "demis": np.empty(n),
               "dtlev": np.empty((nl + 1, n)), "dqlev": np.empty((nl + 1, n))}
        cs, js = col.struct(), jac.struct()
        ptr = lambda a: a.ctypes.data_as(C.c_void_p)
        self._check(lib().clblm_gpu_jac(self.h, C.byref(cs), C.byref(ctrl), C.byref(js), ptr(out["rad"]),
                                        ptr(out["dtlev"]), ptr(out["dqlev"]), ptr(out["dtsfc"]), ptr(out["demis"]),
                                        n, T.CLBLM_OUT_HOST))
        out["v1"], out["dv"] = col.v1, dv
        return out

    def jac_device(self, col, ctrl, jac, rad=0, dtlev=0, dqlev=0, dtsfc=0, demis=0, cap=0):
        """The same into device buffers (device addresses, level-major rows of `cap`)."""
        cs, js = col.struct(), jac.struct()
        self._check(lib().clblm_gpu_jac(self.h, C.byref(cs), C.byref(ctrl), C.byref(js), C.c_void_p(rad or None),
                                        C.c_void_p(dtlev or None), C.c_void_p(dqlev or None),
                                        C.c_void_p(dtsfc or None), C.c_void_p(demis or None), cap,
                                        T.CLBLM_OUT_DEVICE))

    def jac_vjp(self, col, ctrl, jac, g, n=None):
        """Sums over the spectrum of g times each Jacobian (clblm_gpu_jac_vjp):
        dict of g_tlev [nlay+1], g_qlev [nlay+1], g_tskin, g_emis.  `g` is a
        numpy array (host) or a device address with its length `n`."""
        nl = col.nlay
        out = {"g_tlev": np.zeros(nl + 1), "g_qlev": np.zeros(nl + 1)}
        ts, em = C.c_double(), C.c_double()
        cs, js = col.struct(), jac.struct()
        if isinstance(g, np.ndarray):
            g = np.ascontiguousarray(g, dtype=np.float64)
            ptr, n, flags = g.ctypes.data_as(C.c_void_p), len(g), T.CLBLM_OUT_HOST
        else:
            ptr, flags = C.c_void_p(g), T.CLBLM_OUT_DEVICE
        self._check(lib().clblm_gpu_jac_vjp(self.h, C.byref(cs), C.byref(ctrl), C.byref(js), ptr, n,
                                            _dp(out["g_tlev"]), _dp(out["g_qlev"]), C.byref(ts), C.byref(em),
                                            flags))
        out["g_tskin"], out["g_emis"] = ts.value, em.value
        return out

    return jac_size, jac, jac_device, jac_vjp


Handle.jac_size, Handle.jac, Handle.jac_device, Handle.jac_vjp = _jac_methods()


def _profiles(cols, jacs):
    arr = (T.clblm_profile_t * len(cols))()
    keep = []
    for i, (c, j) in enumerate(zip(cols, jacs)):
        cs, js = c.struct(), j.struct()
        keep += [cs, js]
        arr[i].col = C.pointer(cs)
        arr[i].jac = C.pointer(js)
    return arr, keep


def _batch_methods():
    def batch_size(self, cols, ctrl, jacs):
        """Points and DVout of every profile's spectra."""
        arr, keep = _profiles(cols, jacs)
        n = len(cols)
        npts, dv = (C.c_int64 * n)(), (C.c_double * n)()
        self._check(lib().clblm_gpu_batch_size(self.h, arr, n, C.byref(ctrl), npts, dv))
        return list(npts), list(dv)

    def batch(self, cols, ctrl, jacs):
        """Radiance and Jacobians of many profiles in one call (the scene loop
        of the reference's main program): a list of dicts as Handle.jac."""
        npts, dvs = self.batch_size(cols, ctrl, jacs)
        arr, keep = _profiles(cols, jacs)
        outs = []
        for i, c in enumerate(cols):
            n, nl = npts[i], c.nlay
            o = {"rad": np.empty(n), "dtsfc": np.empty(n), "demis": np.empty(n),
                 "dtlev": np.empty((nl + 1, n)), "dqlev": np.empty((nl + 1, n)), "v1": c.v1, "dv": dvs[i]}
            for f, k in (("rad", "rad"), ("dr_dtlev", "dtlev"), ("dr_dqlev", "dqlev"), ("dr_dtskin", "dtsfc"),
                         ("dr_demis", "demis")):
                setattr(arr[i], f, o[k].ctypes.data_as(C.POINTER(C.c_double)))
            arr[i].cap = n
            outs.append(o)
        self._check(lib().clblm_gpu_batch(self.h, arr, len(cols), C.byref(ctrl), T.CLBLM_OUT_HOST))
        return outs

    def batch_device(self, cols, ctrl, jacs, outs, graph=False):
        """The same into device buffers: outs[i] = dict of device addresses
        (rad, dtlev, dqlev, dtsfc, demis; 0 for none) and cap; with graph=True
        the launches are captured once and replayed for the same batch.
        Returns the per-profile status codes."""
        arr, keep = _profiles(cols, jacs)
        for i, o in enumerate(outs):
            for f, k in (("rad", "rad"), ("dr_dtlev", "dtlev"), ("dr_dqlev", "dqlev"), ("dr_dtskin", "dtsfc"),
                         ("dr_demis", "demis")):
                setattr(arr[i], f, C.cast(C.c_void_p(o.get(k) or None), C.POINTER(C.c_double)))
            arr[i].cap = o["cap"]
        flags = T.CLBLM_OUT_DEVICE | (T.CLBLM_BATCH_GRAPH if graph else 0)
        self._check(lib().clblm_gpu_batch(self.h, arr, len(cols), C.byref(ctrl), flags))
        return [arr[i].status for i in range(len(cols))]

    return batch_size, batch, batch_device


Handle.batch_size, Handle.batch, Handle.batch_device = _batch_methods()


def noScattJacob(handle, col, ctrl, jac):
    """Radiance and level Jacobians of a nadir column (clblm_noScattJac.f90:20)."""
    return handle.jac(col, ctrl, jac)


def fftscn_size(scan, v1, dv, n):
    """(V1S, DV, points) of the scanned spectrum (host arithmetic)."""
    v1s, dvs, ns = C.c_double(), C.c_double(), C.c_int64()
    rc = lib().clblm_gpu_fftscn_size(C.byref(scan), v1, dv, n, C.byref(v1s), C.byref(dvs), C.byref(ns))
    if rc:
        raise ClblmError(rc, "FFTSCN size")
    return v1s.value, dvs.value, ns.value


def _scan_methods():
    def fftscn(self, scan, spect, v1, dv):
        """clblm_FFTSCN of a binary64 spectrum on v1 + i*dv: (scanned, V1S, DV)."""
        spect = np.ascontiguousarray(spect, dtype=np.float64)
        v1s, dvs, ns = fftscn_size(scan, v1, dv, len(spect))
        out = np.empty(ns)
        self._check(lib().clblm_gpu_fftscn(self.h, C.byref(scan), spect.ctypes.data_as(C.c_void_p), v1, dv,
                                           len(spect), out.ctypes.data_as(C.c_void_p), ns, T.CLBLM_OUT_HOST))
        return out, v1s, dvs

    def fftscn_device(self, scan, dspect, n, v1, dv, dout, cap):
        """The same on device buffers (addresses)."""
        self._check(lib().clblm_gpu_fftscn(self.h, C.byref(scan), C.c_void_p(dspect), v1, dv, n, C.c_void_p(dout),
                                           cap, T.CLBLM_OUT_DEVICE))

    return fftscn, fftscn_device


Handle.fftscn, Handle.fftscn_device = _scan_methods()


def scanfn_size(scan, v1, dv, n):
    """(V1out, DVout, NPout) of the wavenumber-space scan (host arithmetic)."""
    v1o, dvo, no = C.c_double(), C.c_double(), C.c_int64()
    rc = lib().clblm_gpu_scanfn_size(C.byref(scan), v1, dv, n, C.byref(v1o), C.byref(dvo), C.byref(no))
    if rc:
        raise ClblmError(rc, "SCANFN size")
    return v1o.value, dvo.value, no.value


def _scanfn_methods():
    def scanfn(self, scan, spect, v1, dv):
        """clblm_SCANFN of a binary64 spectrum on v1 + i*dv: (scanned, V1out, DVout)."""
        spect = np.ascontiguousarray(spect, dtype=np.float64)
        v1o, dvo, no = scanfn_size(scan, v1, dv, len(spect))
        out = np.empty(max(no, 1))
        self._check(lib().clblm_gpu_scanfn(self.h, C.byref(scan), spect.ctypes.data_as(C.c_void_p), v1, dv,
                                           len(spect), out.ctypes.data_as(C.c_void_p), no, T.CLBLM_OUT_HOST))
        return out[:no], v1o, dvo

    def scanfn_device(self, scan, dspect, n, v1, dv, dout, cap):
        """The same on device buffers (addresses)."""
        self._check(lib().clblm_gpu_scanfn(self.h, C.byref(scan), C.c_void_p(dspect), v1, dv, n, C.c_void_p(dout),
                                           cap, T.CLBLM_OUT_DEVICE))

    return scanfn, scanfn_device


Handle.scanfn, Handle.scanfn_device = _scanfn_methods()


def _layer_amounts(self, z, p, t, den, earth_radius=6371.23):
    """Layer Pave, Tave, Wtot, W [nlay, nmol] and secant of a nadir path
    between the levels of a profile (rayTraceAndLayerPack: ALAYER + FPACK)."""
    z, p, t = (np.ascontiguousarray(a, dtype=np.float64) for a in (z, p, t))
    den = np.ascontiguousarray(den, dtype=np.float64)
    nlev, nmol = den.shape
    nl = nlev - 1
    out = {k: np.zeros(nl) for k in ("pave", "tave", "wtot", "secant")}
    out["w"] = np.zeros((nl, nmol))
    self._check(lib().clblm_gpu_layer_amounts(self.h, nlev, nmol, _dp(z), _dp(p), _dp(t), _dp(den), earth_radius,
                                              _dp(out["pave"]), _dp(out["tave"]), _dp(out["wtot"]), _dp(out["w"]),
                                              _dp(out["secant"])))
    return out


Handle.layer_amounts = _layer_amounts


def read_tape3(path, v1=-1e30, v2=1e30):
    """Line list of an LNFL TAPE3 file (whole 250-line blocks meeting
    [v1, v2]); host code, no device needed."""
    err = C.create_string_buffer(512)
    n = C.c_int64()
    p = str(path).encode()
    rc = lib().clblm_tape3_read(p, v1, v2, None, 0, C.byref(n), err, 512)
    if rc:
        raise ClblmError(rc, err.value.decode())
    arrays = {name: np.empty(n.value, dtype=dt) for name, dt in T.Lines.FIELDS}
    lines = T.Lines(**arrays)
    ls = lines.struct()
    rc = lib().clblm_tape3_read(p, v1, v2, C.byref(ls), n.value, C.byref(n), err, 512)
    if rc:
        raise ClblmError(rc, err.value.decode())
    return lines


def path(z, p, t, den, obs_alt, view_ang, z_rt=None, h2o=0, o2=-1, earth_radius=6371.23, v_refrac=1000.0,
         zero_abs_amt=0, cap=None):
    """calculatePath (clblm_AtmPath.f90:871-964): the layers of the line of
    sight from an observer at obs_alt [km] at zenith angle view_ang [deg]
    through the level profile (z [km], p [mb], t [K], den [nlev, nmol]
    number densities), with the RT boundaries z_rt (default: the profile's
    levels).  Returns (layers, geometry): layers holds the path's levels
    (z, p, t, q [nlay+1, nmol]) and layers (pave, tave, wtot, w [nlay,
    nmol], secant, ipath); geometry the standard form (hobs, hend, angle,
    phi, hmin, len) and the traced ray's range, beta, bendng, phi_end.
    Host code, no device needed."""
    z, p, t = (np.ascontiguousarray(a, dtype=np.float64) for a in (z, p, t))
    den = np.ascontiguousarray(den, dtype=np.float64)
    nlev, nmol = den.shape
    zr = np.ascontiguousarray(z if z_rt is None else z_rt, dtype=np.float64)
    cap = nlev + len(zr) + 4 if cap is None else int(cap)
    o = dict(z=np.zeros(cap + 1), p=np.zeros(cap + 1), t=np.zeros(cap + 1), q=np.zeros((cap + 1) * max(nmol, 1)),
             pave=np.zeros(cap), tave=np.zeros(cap), wtot=np.zeros(cap), w=np.zeros(cap * max(nmol, 1)),
             secant=np.zeros(cap), ipath=np.zeros(cap, dtype=np.int32))
    pin = T.clblm_path_in_t(nlev, nmol, _dp(z), _dp(p), _dp(t), _dp(den), h2o, o2, earth_radius, obs_alt, view_ang,
                            v_refrac, len(zr), _dp(zr), zero_abs_amt)
    pout = T.clblm_path_t()
    pout.cap = cap
    for k in ("z", "p", "t", "q", "pave", "tave", "wtot", "w", "secant"):
        setattr(pout, k, _dp(o[k]))
    pout.ipath = o["ipath"].ctypes.data_as(C.POINTER(C.c_int32))
    err = C.create_string_buffer(512)
    rc = lib().clblm_path(C.byref(pin), C.byref(pout), err, 512)
    if rc:
        raise ClblmError(rc, err.value.decode())
    n = pout.nlay
    layers = dict(z=o["z"][:n + 1], p=o["p"][:n + 1], t=o["t"][:n + 1], q=o["q"][:(n + 1) * nmol].reshape(n + 1, nmol),
                  pave=o["pave"][:n], tave=o["tave"][:n], wtot=o["wtot"][:n], w=o["w"][:n * nmol].reshape(n, nmol),
                  secant=o["secant"][:n], ipath=o["ipath"][:n])
    geom = {k: getattr(pout, k) for k in ("hobs", "hend", "angle", "phi", "hmin", "len", "range", "beta", "bendng",
                                          "phi_end")}
    return layers, geom


def setDV(col, sample=4.0, alfal0=0.04, alfal0_fine=0.005, grid_type=0, dv_user=-1.0):
    """DVnormal, DVnarrow per layer and the output DV (setDV_struct)."""
    n = col.nlay
    dn, df, do = np.zeros(n), np.zeros(n), C.c_double()
    cs = col.struct()
    rc = lib().clblm_setdv(C.byref(cs), sample, alfal0, alfal0_fine, grid_type, dv_user, _dp(dn), _dp(df),
                           C.byref(do))
    if rc:
        raise ClblmError(rc, "setDV")
    return dn, df, do.value


def ODLAY(handle, layer, grid, ctrl):
    """monoOD, nSamp, DVout of ODLAY_nonStruct (clblm_ODLAY.f90:129-177)."""
    od, dv = handle.odlay(layer, grid, ctrl)
    return od, len(od), dv


def mode2_lookDn_mergeUp(handle, col, ctrl):
    """totalRadUp of mode2_lookDn_mergeUp (clblm_noScattRT.f90:1134)."""
    return handle.rt_mode2(col, ctrl)


def interp_spectrum_noalloc(d_in, nin, v1, dvin, d_out, nout, dvout, stream=0):
    """Device spectrum (v1, dvin, nin) -> (v1, dvout, nout) with interpSpectrum's
    rules, allocating no device memory (clblm_gpu_interp_spectrum_noalloc).

    d_in, d_out: device addresses (e.g. torch tensor data_ptr()); stream: a
    cudaStream_t as an int.  The work is queued, not waited for.  Calls share
    one scratch array per device: order them on one stream."""
    rc = lib().clblm_gpu_interp_spectrum_noalloc(C.c_void_p(d_in), nin, v1, dvin, C.c_void_p(d_out), nout,
                                                 dvout, C.c_void_p(stream))
    if rc:
        raise ClblmError(rc, "clblm_gpu_interp_spectrum_noalloc")


def _filter_method():
    def filter(self, spect, v1, dv, channels):
        """clblm_FLTRFN for every channel: `channels` is a list of (start_freq,
        delta_freq, values); returns the channels' filtered values."""
        spect = np.ascontiguousarray(spect, dtype=np.float64)
        sf = np.array([c[0] for c in channels], dtype=np.float64)
        df = np.array([c[1] for c in channels], dtype=np.float64)
        ns = np.array([len(c[2]) for c in channels], dtype=np.int32)
        vals = np.ascontiguousarray(np.concatenate([np.asarray(c[2], dtype=np.float64) for c in channels]))
        out = np.zeros(len(channels))
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self._check(lib().clblm_gpu_filter(self.h, spect.ctypes.data_as(C.c_void_p), v1, dv, len(spect),
                                           len(channels), dp(sf), dp(df), ns.ctypes.data_as(C.POINTER(C.c_int32)),
                                           dp(vals), dp(out)))
        return out

    return filter


Handle.filter = _filter_method()

"""Many profiles in one call (clblm_gpu_batch): equal to clblm_gpu_jac on each
profile in turn with the same handle, eagerly and through the captured CUDA
graph, with a failing profile failing alone."""
import ctypes as C

import numpy as np
import pytest

from clblm_gb300 import capi_types as T
from clblm_gb300 import synth

pytestmark = pytest.mark.gpu

# uneven layer counts and windows, as in the batched-profiles workload
CASES = [(10, 3, (1000.0, 1004.0)), (0, 5, (1100.0, 1101.5)), (30, 2, (700.0, 712.0)), (5, 4, (1000.5, 1003.0))]


def _profiles(n_lines=20000):
    lines, col, _ = synth.config1(n_lines=n_lines)
    prof = synth.jac_profile(col)
    cols, jacs = [], []
    for first, count, window in CASES:
        cols.append(col.sub(list(range(first, first + count))).with_window(*window))
        jacs.append(prof.sub(first, count))
    return lines, cols, jacs


KEYS = ("rad", "dtlev", "dqlev", "dtsfc", "demis")


@pytest.mark.parametrize("precision", [T.CLBLM_PREC_MIXED, T.CLBLM_PREC_PLAIN])
def test_batch_equals_profile_calls(gpu_lib, mtckd, precision):
    lines, cols, jacs = _profiles()
    ctrl = T.rt_ctrl(precision=precision, grid_type=1)
    h = gpu_lib.Handle(lines, mtckd)
    want = [h.jac(c, ctrl, j) for c, j in zip(cols, jacs)]
    h.close()
    h = gpu_lib.Handle(lines, mtckd)
    got = h.batch(cols, ctrl, jacs)
    h.close()
    for w, g in zip(want, got):
        assert g["dv"] == w["dv"] and len(g["rad"]) == len(w["rad"])
        for k in KEYS:
            np.testing.assert_array_equal(g[k], w[k], err_msg=k)


def test_batch_graph_replay(gpu_lib, mtckd):
    import torch
    lines, cols, jacs = _profiles()
    ctrl = T.rt_ctrl(precision=T.CLBLM_PREC_MIXED, grid_type=1)
    h = gpu_lib.Handle(lines, mtckd)
    # the first call settles the sticky JRAD (OPDPTH zeroes it below 5 kT and
    # it stays zero); every later call of the same batch then has one plan
    h.batch(cols, ctrl, jacs)
    want = h.batch(cols, ctrl, jacs)
    npts, _ = h.batch_size(cols, ctrl, jacs)
    bufs, outs = [], []
    for c, n in zip(cols, npts):
        b = {"rad": torch.zeros(n, dtype=torch.float64, device="cuda"),
             "dtlev": torch.zeros((c.nlay + 1, n), dtype=torch.float64, device="cuda"),
             "dqlev": torch.zeros((c.nlay + 1, n), dtype=torch.float64, device="cuda"),
             "dtsfc": torch.zeros(n, dtype=torch.float64, device="cuda"),
             "demis": torch.zeros(n, dtype=torch.float64, device="cuda")}
        bufs.append(b)
        outs.append({k: v.data_ptr() for k, v in b.items()} | {"cap": n})
    torch.cuda.synchronize()
    # the first graph call captures, the others replay
    for _ in range(3):
        for b in bufs:
            for v in b.values():
                v.zero_()
        torch.cuda.synchronize()
        st = h.batch_device(cols, ctrl, jacs, outs, graph=True)
        assert st == [0] * len(cols)
        torch.cuda.synchronize()
        for w, b in zip(want, bufs):
            for k in KEYS:
                np.testing.assert_array_equal(b[k].cpu().numpy(), w[k], err_msg=k)
    h.close()


def test_batch_failing_profile(gpu_lib, mtckd):
    lines, cols, jacs = _profiles()
    ctrl = T.rt_ctrl(precision=T.CLBLM_PREC_MIXED, grid_type=1)
    bad = T.JacProfile(jacs[1].plev, jacs[1].qlev, jac_mol=40)  # not one of the column's molecules
    h = gpu_lib.Handle(lines, mtckd)
    want = [h.jac(c, ctrl, j) for i, (c, j) in enumerate(zip(cols, jacs)) if i != 1]
    h.close()
    h = gpu_lib.Handle(lines, mtckd)
    arr_cols = cols
    arr_jacs = [jacs[0], bad, jacs[2], jacs[3]]
    npts = []
    for c, j in zip(arr_cols, arr_jacs):
        try:
            npts.append(h.jac_size(c, ctrl, j)[0])
        except Exception:
            npts.append(1)
    from clblm_gb300 import capi
    arr, keep = capi._profiles(arr_cols, arr_jacs)
    outs = []
    for i, (c, n) in enumerate(zip(arr_cols, npts)):
        o = {"rad": np.empty(n), "dtlev": np.empty((c.nlay + 1, n)), "dqlev": np.empty((c.nlay + 1, n)),
             "dtsfc": np.empty(n), "demis": np.empty(n)}
        for f, k in (("rad", "rad"), ("dr_dtlev", "dtlev"), ("dr_dqlev", "dqlev"), ("dr_dtskin", "dtsfc"),
                     ("dr_demis", "demis")):
            setattr(arr[i], f, o[k].ctypes.data_as(C.POINTER(C.c_double)))
        arr[i].cap = n
        outs.append(o)
    rc = capi.lib().clblm_gpu_batch(h.h, arr, len(arr_cols), C.byref(ctrl), T.CLBLM_OUT_HOST)
    assert rc == T.CLBLM_ERR_ARG
    assert [arr[i].status for i in range(4)] == [0, T.CLBLM_ERR_ARG, 0, 0]
    for w, o in zip(want, [outs[0], outs[2], outs[3]]):
        for k in KEYS:
            np.testing.assert_array_equal(o[k], w[k], err_msg=k)
    h.close()

"""Failure paths of the C boundary: the reference STOPs the process on these
conditions (fixDVRatio's 'DV RATIO .GT. 2.5', clblm_setDV.f90:318-320; the
unsorted or unreadable line file and bad layer input, clblm_ODLAY.f90:277,703);
the library returns a status code instead and stays usable.  No GPU fault is
involved: every case is refused on the host before any device work."""
import copy

import numpy as np
import pytest

from clblm_gb300 import capi_types as T


def _two_layer_jump():
    """Two adjacent layers whose DVs differ by more than 2.5x: 1013 hPa at the
    surface, 0.5 hPa above it."""
    from clblm_gb300 import synth
    _, col, _ = synth.config1(n_lines=10)
    c = col.sub([0, 59])
    return c


def test_setdv_dv_ratio_refused(gpu_lib, oracle_mod):
    col = _two_layer_jump()
    with pytest.raises(gpu_lib.ClblmError) as e:
        gpu_lib.setDV(col)
    assert e.value.code == T.CLBLM_ERR_DV_RATIO
    with pytest.raises(oracle_mod.OracleError) as eo:
        oracle_mod.Session().setdv(col)
    assert eo.value.code == T.CLBLM_ERR_DV_RATIO


@pytest.mark.parametrize("field,value", [("pave", np.nan), ("tave", np.nan), ("wtot", np.inf), ("tave", -5.0),
                                         ("w", np.nan)])
def test_setdv_bad_layer_input_refused(gpu_lib, field, value):
    from clblm_gb300 import synth
    _, col, _ = synth.config1(n_lines=10)
    c = copy.deepcopy(col.sub([10, 11, 12]))
    arr = getattr(c, field)
    if arr.ndim == 2:
        arr[1, 0] = value
    else:
        arr[1] = value
    with pytest.raises(gpu_lib.ClblmError) as e:
        gpu_lib.setDV(c)
    assert e.value.code == T.CLBLM_ERR_ARG


@pytest.mark.gpu
def test_unsorted_lines_refused(gpu_lib):
    from clblm_gb300 import synth
    lines = synth.line_list(600, 600.0, 610.0, seed=3)
    bad = T.Lines(**{name: getattr(lines, name).copy() for name, _ in T.Lines.FIELDS})
    bad.vnu[300], bad.vnu[301] = bad.vnu[301], bad.vnu[300]
    with pytest.raises(gpu_lib.ClblmError) as e:
        gpu_lib.Handle(bad)
    assert e.value.code == T.CLBLM_ERR_UNSORTED
    h = gpu_lib.Handle(lines)  # the library is still usable
    with pytest.raises(gpu_lib.ClblmError) as e:
        h.set_lines(bad)
    assert e.value.code == T.CLBLM_ERR_UNSORTED
    h.close()


@pytest.mark.gpu
def test_nan_layer_and_column_refused(gpu_lib):
    from clblm_gb300 import synth
    lines, col, cont = synth.config1(n_lines=20000)
    col = col.with_window(1000.0, 1002.0).sub([20, 21, 22])
    h = gpu_lib.Handle(lines.window(970.0, 1032.0), cont)
    try:
        dn, df, _ = gpu_lib.setDV(col)
        g = T.grid_struct(col.v1, col.v2, dn[0], df[0])
        ctrl = T.od_ctrl()
        for field in ("pave", "tave", "wtot"):
            lay = col.layer(0)
            setattr(lay, field, float("nan"))
            with pytest.raises(gpu_lib.ClblmError) as e:
                h.odlay(lay, g, ctrl)
            assert e.value.code == T.CLBLM_ERR_ARG
        c = copy.deepcopy(col)
        c.w[0, 0] = np.nan
        with pytest.raises(gpu_lib.ClblmError) as e:
            h.odlay(c.layer(0), g, ctrl)
        assert e.value.code == T.CLBLM_ERR_ARG
        rctrl = T.rt_ctrl()
        for field, val in (("tbot", np.nan), ("ttop", -1.0), ("wtot_down", np.nan)):
            c = copy.deepcopy(col)
            getattr(c, field)[1] = val
            with pytest.raises(gpu_lib.ClblmError) as e:
                h.rt_mode2(c, rctrl)
            assert e.value.code == T.CLBLM_ERR_ARG
        for field, val in (("tskin", float("nan")), ("emis", 1.5)):
            c = copy.deepcopy(col)
            setattr(c, field, val)
            with pytest.raises(gpu_lib.ClblmError) as e:
                h.rt_mode2(c, rctrl)
            assert e.value.code == T.CLBLM_ERR_ARG
        # and the handle still computes the good column
        rad, _ = h.rt_mode2(col, rctrl)
        assert np.all(np.isfinite(rad)) and np.all(rad > 0)
    finally:
        h.close()

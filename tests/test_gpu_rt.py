"""Nadir radiance (mode2_lookDn_mergeUp) on the GPU against the FP64 oracle."""
import numpy as np
import pytest

from clblm_gb300 import capi_types as T
from clblm_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [(T.CLBLM_PREC_MIXED, 1e-4), (T.CLBLM_PREC_PLAIN, 1e-8)])
def test_rt_small_column(gpu_lib, oracle_mod, precision, tol):
    lines, col, cont = synth.config1(n_lines=40000)
    # adjacent layers: the reference stops on a DV ratio > 2.5 between neighbours
    col = col.sub(list(range(20, 32))).with_window(1200.0, 1230.0)
    ctrl = T.rt_ctrl(precision=precision)
    h = gpu_lib.Handle(lines, cont)
    rad, dv = h.rt_mode2(col, ctrl)
    h.close()
    ref, dvr = oracle_mod.Session().rt_mode2(lines, col, ctrl, cont)
    assert dv == dvr and len(rad) == len(ref)
    rel = np.max(np.abs(rad - ref) / np.abs(ref))
    assert rel <= tol, rel


@pytest.mark.parametrize("precision,tol", [(T.CLBLM_PREC_MIXED, 1e-4), (T.CLBLM_PREC_PLAIN, 1e-8)])
def test_rt_slant_view(gpu_lib, oracle_mod, precision, tol):
    """A slant view at 140 deg through levels 20-32 of the column's profile:
    the view and downwelling paths traced by clblm_path, the radiance of
    mode2 on the GPU against the oracle on the same layers"""
    from clblm_gb300 import scene
    lines, col, cont = synth.config1(n_lines=40000)
    t_lev = np.append(col.tbot, col.ttop[-1])
    den = synth.level_density(col.p_lev[:, None], t_lev[:, None], col.vmr_lev)
    lv = slice(20, 33)
    z = col.z_lev[lv]
    scol = scene.slant_column(col.mol_id, z, col.p_lev[lv], t_lev[lv], den[lv], z[-1], 140.0, 1200.0, 1230.0,
                              t_lev[20], col.emis)
    assert scol.nlay == 12 and np.all(scol.wtot > col.wtot[20:32])
    ctrl = T.rt_ctrl(precision=precision)
    h = gpu_lib.Handle(lines, cont)
    rad, dv = h.rt_mode2(scol, ctrl)
    h.close()
    ref, dvr = oracle_mod.Session().rt_mode2(lines, scol, ctrl, cont)
    assert dv == dvr and len(rad) == len(ref)
    rel = np.max(np.abs(rad - ref) / np.abs(ref))
    assert rel <= tol, rel

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

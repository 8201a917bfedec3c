"""The autotuner's launch shapes change no result: the layer OD is bit-equal
for every far-wing stage size, and the chosen shapes are reported."""
import os

import numpy as np
import pytest

from clblm_gb300 import capi
from clblm_gb300 import capi_types as T
from clblm_gb300 import synth

pytestmark = pytest.mark.gpu


def _layer_od(lines, cont, col, precision, stage=None):
    old = os.environ.get("CLBLM_F4_STAGE_RECORDS")
    if stage is not None:
        os.environ["CLBLM_F4_STAGE_RECORDS"] = str(stage)
    try:
        h = capi.Handle(lines, cont)
    finally:
        if stage is None or old is not None:
            if old is not None:
                os.environ["CLBLM_F4_STAGE_RECORDS"] = old
        else:
            del os.environ["CLBLM_F4_STAGE_RECORDS"]
    dn, df, _ = capi.setDV(col)
    g = T.grid_struct(col.v1, col.v2, dn[0], df[0])
    od, _ = h.odlay(col.layer(0), g, T.od_ctrl(precision=precision))
    st = h.stats()
    h.close()
    return od, st


@pytest.mark.parametrize("precision", [T.CLBLM_PREC_MIXED, T.CLBLM_PREC_PLAIN])
def test_stage_size_does_not_change_od(gpu_lib, mtckd, precision):
    lines, col, _ = synth.config1(n_lines=60000)
    c = col.sub([45]).with_window(900.0, 960.0)
    ref, st = _layer_od(lines, mtckd, c, precision)
    assert st["f4_stage_records"] in (64, 128, 256)
    for stage in (64, 128, 256):
        od, st = _layer_od(lines, mtckd, c, precision, stage)
        assert st["f4_stage_records"] == stage
        np.testing.assert_array_equal(od, ref)


def test_tuned_shapes_reported(gpu_lib, mtckd):
    lines, col, _ = synth.config1(n_lines=20000)
    c = col.sub([10, 11, 12]).with_window(1000.0, 1004.0)
    h = capi.Handle(lines, mtckd)
    ctrl = T.rt_ctrl(precision=T.CLBLM_PREC_MIXED, grid_type=1)
    h.jac(c, ctrl, synth.jac_profile(col).sub(10, 3))
    st = h.stats()
    assert st["jac_threads"] in (64, 128) and st["f4_stage_records"] in (64, 128, 256)
    h.close()

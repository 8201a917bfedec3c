"""Radiance Jacobians on the GPU (clblm_gpu_jac) against the FP64 oracle's
noScattJacob restatement."""
import numpy as np
import pytest

from clblm_gb300 import capi_types as T
from clblm_gb300 import synth

pytestmark = pytest.mark.gpu


def _case(first=10, count=3, window=(1000.0, 1004.0), n_lines=20000):
    lines, col, _ = synth.config1(n_lines=n_lines)
    c = col.sub(list(range(first, first + count))).with_window(*window)
    prof = synth.jac_profile(col).sub(first, count)
    return lines, c, prof


def _rel(a, b):
    """max |a - b| over the largest |b| of the spectrum (per row for 2-D)."""
    scale = np.max(np.abs(b), axis=-1, keepdims=True)
    return float(np.max(np.abs(a - b) / np.where(scale > 0, scale, 1.0)))


@pytest.mark.parametrize("precision,tol", [(T.CLBLM_PREC_PLAIN, 1e-8), (T.CLBLM_PREC_MIXED, 2e-3)])
@pytest.mark.parametrize("lin_in_tau", [1, 0])
def test_jacobians_match_oracle(gpu_lib, oracle_mod, mtckd, precision, tol, lin_in_tau):
    lines, col, prof = _case()
    ctrl = T.rt_ctrl(precision=precision, grid_type=1, lin_in_tau=lin_in_tau)
    h = gpu_lib.Handle(lines, mtckd)
    got = h.jac(col, ctrl, prof)
    h.close()
    want = oracle_mod.jac_mode2(oracle_mod.Session(), lines, col, ctrl, prof, mtckd)
    assert len(got["rad"]) == len(want["rad"]) and got["dv"] == want["dv"]
    rtol = 1e-9 if precision == T.CLBLM_PREC_PLAIN else 1e-4
    np.testing.assert_allclose(got["rad"], want["rad"], rtol=rtol)
    for k in ("dtlev", "dqlev", "dtsfc", "demis"):
        assert _rel(got[k], want[k]) <= tol, (k, _rel(got[k], want[k]))

"""Parity at the workloads' own sizes: the GPU path against the FP64 oracle
on full-width sub-columns and whole spectral windows, not on slices.

  * the 60-layer column (500,000 lines): full 500-2500 cm-1 radiance of the
    ten uppermost layers (the finest grids, 5.4 M points) and of twelve
    middle layers;
  * the Jacobian workload: radiance and level T / ln q(H2O) Jacobians over
    the whole 600-1100 cm-1 window (the 120,000 lines there) on six layers
    at the bottom and six at the top of the column;
  * a dozen of the 256 batched profiles (every 21st), each through
    clblm_gpu_batch, against the oracle's noScattJacob;
  * the broadband column (3,000,000 lines): the three lowest layers at
    10-60 cm-1, where the far-wing mirror lines of CNVF4Q are active.

Bounds: radiance 1e-4 relative per point (mixed) and 1e-8 (FP64).
Jacobians, per point and level l:
    |got - want| <= JAC_RTOL |want| + JAC_ATOL S_l,
    S_l = max(max|want_l|, 1e-6 max over all levels |want|).
Where the bound comes from (mixed path): the reference forms dtau/dT as
tau(T+1) - tau(T) - (Wtot/T) [tau(1.01 W) - tau(W)] / 0.01, a difference of
ODs whose relative error is eps <= 1e-6, so its absolute error is at most
2 eps tau (1 + 100/T) < 3 eps tau.  A layer's OD changes by no less than
about 2.3e-3 per K at its line peaks (the Doppler width's T^1/2 at 217 K),
so the error is at most ~1.3e-3 of the level's largest Jacobian wherever it
falls (JAC_ATOL, with room for level2layer's two-layer sums), and
about 3e-4 of the value itself where dtau/dT is typical (JAC_RTOL 1e-3).
Levels below an opaque lower atmosphere have Jacobians of 1e-40 to 1e-320,
below FP32's range, where the mixed path returns 0: S_l's floor at 1e-6 of
the column's largest Jacobian makes those levels count as zero.  FP64: the
same form with 1e-9 and 1e-10.
"""
import os

import numpy as np
import pytest

from clblm_gb300 import capi_types as T
from clblm_gb300 import synth

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
JAC_TOL = {T.CLBLM_PREC_MIXED: (1e-3, 2.5e-3), T.CLBLM_PREC_PLAIN: (1e-9, 1e-10)}
JAC_FLOOR = 1e-6
RAD_TOL = {T.CLBLM_PREC_MIXED: 1e-4, T.CLBLM_PREC_PLAIN: 1e-8}


def _rad_err(got, want):
    assert got.shape == want.shape
    return float(np.max(np.abs(got - want) / np.abs(want)))


def _jac_check(got, want, precision, what):
    """The per-point bound of the module docstring, level by level; a level
    that is not finite in the oracle must be non-finite in both."""
    rt, at = JAC_TOL[precision]
    g2, w2 = np.atleast_2d(got), np.atleast_2d(want)
    assert g2.shape == w2.shape, what
    fin = [bool(np.all(np.isfinite(w))) for w in w2]
    top = max((float(np.max(np.abs(w))) for w, f in zip(w2, fin) if f), default=0.0)
    worst, where = 0.0, None
    for lev in range(w2.shape[0]):
        w, g = w2[lev], g2[lev]
        if not fin[lev]:
            assert not np.all(np.isfinite(g)), (what, lev)
            continue
        scale = max(float(np.max(np.abs(w))), JAC_FLOOR * top)
        excess = np.abs(g - w) / (rt * np.abs(w) + at * scale + 1e-300)
        i = int(np.argmax(excess))
        if excess[i] > worst:
            worst, where = float(excess[i]), (lev, i, float(w[i]), float(g[i]), scale, top)
    assert worst <= 1.0, (what, worst, where)
    return worst


@pytest.fixture(scope="module")
def config1():
    return synth.config1()


@pytest.mark.parametrize("precision", [T.CLBLM_PREC_MIXED, T.CLBLM_PREC_PLAIN])
@pytest.mark.parametrize("layers", [(50, 60), (20, 32)])
def test_config1_radiance_full_width(gpu_lib, oracle_mod, config1, precision, layers):
    lines, col, cont = config1
    sub = col.sub(list(range(*layers)))
    ctrl = T.rt_ctrl(precision=precision)
    h = gpu_lib.Handle(lines, cont)
    try:
        got, dv = h.rt_mode2(sub, ctrl)
    finally:
        h.close()
    want, dvw = oracle_mod.Session().rt_mode2(lines, sub, T.rt_ctrl(precision=T.CLBLM_PREC_PLAIN), cont,
                                             nthreads=THREADS)
    assert dv == dvw and len(got) == len(want) > 1_000_000
    err = _rad_err(got, want)
    assert err <= RAD_TOL[precision], err


@pytest.mark.parametrize("precision", [T.CLBLM_PREC_MIXED, T.CLBLM_PREC_PLAIN])
@pytest.mark.parametrize("first", [0, 54])
def test_config2_jacobians_whole_window(gpu_lib, oracle_mod, config1, precision, first):
    lines, col, cont = config1
    lines = lines.window(600.0, 1100.0)
    full = col.with_window(600.0, 1100.0)
    sub = full.sub(list(range(first, first + 6)))
    prof = synth.jac_profile(full).sub(first, 6)
    ctrl = T.rt_ctrl(precision=precision, grid_type=1)
    h = gpu_lib.Handle(lines, cont)
    try:
        got = h.jac(sub, ctrl, prof)
    finally:
        h.close()
    want = oracle_mod.jac_mode2(oracle_mod.Session(), lines, sub, T.rt_ctrl(precision=T.CLBLM_PREC_PLAIN,
                                                                            grid_type=1), prof, cont,
                                nthreads=THREADS)
    assert got["dv"] == want["dv"] and len(got["rad"]) == len(want["rad"]) > 100_000
    assert _rad_err(got["rad"], want["rad"]) <= RAD_TOL[precision]
    for k in ("dtlev", "dqlev", "dtsfc", "demis"):
        _jac_check(got[k], want[k], precision, k)


@pytest.mark.parametrize("precision", [T.CLBLM_PREC_MIXED, T.CLBLM_PREC_PLAIN])
def test_config3_dozen_profiles(gpu_lib, oracle_mod, precision):
    lines, cont, cols, jacs = synth.config3()
    ctrl = T.rt_ctrl(precision=precision, grid_type=1)
    octrl = T.rt_ctrl(precision=T.CLBLM_PREC_PLAIN, grid_type=1)
    for i in range(0, 252, 21):
        # a handle per profile, as the oracle starts a fresh process per
        # profile (the sticky JRAD would otherwise run from profile to profile)
        h = gpu_lib.Handle(lines, cont)
        try:
            got = h.batch([cols[i]], ctrl, [jacs[i]])[0]
        finally:
            h.close()
        want = oracle_mod.jac_mode2(oracle_mod.Session(), lines, cols[i], octrl, jacs[i], cont, nthreads=THREADS)
        assert got["dv"] == want["dv"] and len(got["rad"]) == len(want["rad"]), i
        err = _rad_err(got["rad"], want["rad"])
        assert err <= RAD_TOL[precision], (i, err)
        for k in ("dtlev", "dqlev", "dtsfc", "demis"):
            _jac_check(got[k], want[k], precision, (i, k))


@pytest.mark.parametrize("precision", [T.CLBLM_PREC_MIXED, T.CLBLM_PREC_PLAIN])
def test_config4_lowest_layers_far_wing_mirror(gpu_lib, oracle_mod, precision):
    lines, col, cont = synth.config4()
    sub = col.sub([0, 1, 2]).with_window(10.0, 60.0)
    ctrl = T.rt_ctrl(precision=precision)
    h = gpu_lib.Handle(lines, cont)
    try:
        got, dv = h.rt_mode2(sub, ctrl)
    finally:
        h.close()
    want, dvw = oracle_mod.Session().rt_mode2(lines, sub, T.rt_ctrl(precision=T.CLBLM_PREC_PLAIN), cont,
                                             nthreads=THREADS)
    assert dv == dvw and len(got) == len(want)
    err = _rad_err(got, want)
    assert err <= RAD_TOL[precision], err

"""The torch.autograd binding of the radiance Jacobians (GPU): the backward
pass applies the analytic Jacobians, checked against central finite
differences of the radiance computed through the same C-ABI."""
import numpy as np
import pytest

from clblm_gb300 import capi_types as T
from clblm_gb300 import synth

pytestmark = pytest.mark.gpu


def _problem(gpu_lib, mtckd, col=None, precision=T.CLBLM_PREC_PLAIN, first=10):
    from clblm_gb300 import torch_ops
    lines, full, _ = synth.config1(n_lines=20000)
    nl = 3
    c = col if col is not None else full.sub(list(range(first, first + nl))).with_window(1000.0, 1002.0)
    prof = synth.jac_profile(full).sub(first, nl)
    h = gpu_lib.Handle(lines, mtckd)
    ctrl = T.rt_ctrl(precision=precision, grid_type=1, lin_in_tau=1)
    return torch_ops.RadianceProblem(h, c, ctrl, prof), c, prof, h


def _radiance(gpu_lib, mtckd, col):
    p, _, _, h = _problem(gpu_lib, mtckd, col)
    out = h.jac(col, p.ctrl, p.prof)
    h.close()
    return out["rad"]


def test_backward_is_jacobian_transpose(gpu_lib, mtckd):
    import torch
    from clblm_gb300 import torch_ops
    p, c, prof, h = _problem(gpu_lib, mtckd)
    t, q, ts, em = [x.requires_grad_() for x in p.levels()]
    rad = torch_ops.NadirRadiance.apply(t, q, ts, em, p)
    ref = h.jac(c, p.ctrl, prof)
    np.testing.assert_allclose(rad.detach().cpu().numpy(), ref["rad"], rtol=1e-12)
    g = torch.rand_like(rad)
    (rad * g).sum().backward()
    gn = g.cpu().numpy()
    np.testing.assert_allclose(t.grad.cpu().numpy(), ref["dtlev"] @ gn, rtol=1e-10)
    np.testing.assert_allclose(q.grad.cpu().numpy(), ref["dqlev"] @ gn, rtol=1e-10)
    assert float(ts.grad) == pytest.approx(float(ref["dtsfc"] @ gn), rel=1e-10)
    assert float(em.grad) == pytest.approx(float(ref["demis"] @ gn), rel=1e-10)
    h.close()


def _shift_col(c, **kw):
    a = dict(mol_id=c.mol_id, pave=c.pave, tave=c.tave, tbot=c.tbot, ttop=c.ttop, w=c.w, wtot=c.wtot,
             wtot_down=c.wtot_down, v1=c.v1, v2=c.v2, tskin=c.tskin, emis=c.emis)
    a.update(kw)
    return T.Column(**a)


def test_surface_derivatives_match_central_differences(gpu_lib, mtckd):
    # layers 40-42 (a few hPa): thin enough that the surface is seen
    p, c, prof, h = _problem(gpu_lib, mtckd, first=40)
    ref = h.jac(c, p.ctrl, prof)
    h.close()
    for key, field, step in (("dtsfc", "tskin", 0.01), ("demis", "emis", 1e-4)):
        rp = _radiance(gpu_lib, mtckd, _shift_col(c, **{field: getattr(c, field) + step}))
        rm = _radiance(gpu_lib, mtckd, _shift_col(c, **{field: getattr(c, field) - step}))
        fd = (rp - rm) / (2 * step)
        scale = np.max(np.abs(ref[key]))
        assert np.max(np.abs(fd - ref[key])) <= 1e-5 * scale, key


def _level_shift(c, prof, k, dT=0.0, dlnq=0.0):
    """The column after level k's temperature or ln q moves, carried into the
    layers through level2layer's own maps (the reference's linearisation)."""
    sys_ = __import__("test_oracle_jac")
    tlev = np.append(c.tbot, c.ttop[-1])
    dTu, dTl, dWu, dWl = sys_._level2layer(prof.plev, tlev, c.tave, prof.qlev)
    tave, w = c.tave.copy(), c.w.copy()
    tlev2 = tlev.copy()
    tlev2[k] += dT
    ih = int(np.where(c.mol_id == 1)[0][0])
    if k < c.nlay:  # layer k has level k at its bottom
        tave[k] += dTl[k] * dT
        w[k, ih] *= np.exp(dWl[k] * dlnq)
    if k > 0:       # layer k-1 has level k at its top
        tave[k - 1] += dTu[k - 1] * dT
        w[k - 1, ih] *= np.exp(dWu[k - 1] * dlnq)
    return _shift_col(c, tave=tave, w=w, tbot=tlev2[:-1], ttop=tlev2[1:], tskin=c.tskin)


def test_level_derivatives_against_central_differences(gpu_lib, mtckd):
    """Central differences in level T (0.01 K) and ln q (1e-4) against the
    analytic Jacobians.  The reference's dTau/dT is a 1 K forward difference
    and its dTau/dln q leaves the self-broadening unchanged, so the agreement
    is that of those approximations (a few per cent), not of rounding."""
    p, c, prof, h = _problem(gpu_lib, mtckd)
    ref = h.jac(c, p.ctrl, prof)
    h.close()
    worst = {}
    for k in range(1, c.nlay + 1):
        for key, kw, step in (("dtlev", "dT", 0.01), ("dqlev", "dlnq", 1e-4)):
            rp = _radiance(gpu_lib, mtckd, _level_shift(c, prof, k, **{kw: step}))
            rm = _radiance(gpu_lib, mtckd, _level_shift(c, prof, k, **{kw: -step}))
            fd = (rp - rm) / (2 * step)
            a = ref[key][k]
            err = np.linalg.norm(fd - a) / np.linalg.norm(fd)
            worst[key, k] = err
    print("relative differences", worst)
    assert max(worst.values()) <= 0.1, worst

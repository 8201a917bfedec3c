"""The radiance as a differentiable function of the level profile (GPU):
clblm_gpu_jac_vjp against clblm_gpu_jac's Jacobians contracted with the same
cotangent, the torch.autograd binding at states other than the profile's
own, and the gradient against central finite differences of the forward
pass (levels -> ALAYER/FPACK layers -> radiance)."""
import numpy as np
import pytest

from clblm_gb300 import capi_types as T
from clblm_gb300 import synth

pytestmark = pytest.mark.gpu


def _problem(gpu_lib, mtckd, precision=T.CLBLM_PREC_PLAIN, first=10, nl=3, window=(1000.0, 1002.0)):
    from clblm_gb300 import torch_ops
    lines, full, _ = synth.config1(n_lines=20000)
    col = full.sub(list(range(first, first + nl))).with_window(*window)
    h = gpu_lib.Handle(lines, mtckd)
    ctrl = T.rt_ctrl(precision=precision, grid_type=1, lin_in_tau=1)
    return torch_ops.RadianceProblem.from_column(h, ctrl, col), col, h


def _tlev(col):
    return np.append(col.tbot, col.ttop[-1])


@pytest.mark.parametrize("precision,rtol", [(T.CLBLM_PREC_PLAIN, 1e-10), (T.CLBLM_PREC_MIXED, 1e-9)])
def test_vjp_is_jacobian_transpose(gpu_lib, mtckd, precision, rtol):
    """The product reduces exactly the derivatives clblm_gpu_jac writes; the
    whole 600-1100 cm-1 window of six layers, several 100000-point blocks."""
    p, col, h = _problem(gpu_lib, mtckd, precision, first=30, nl=6, window=(600.0, 1100.0))
    try:
        c, prof = p.state(_tlev(col), np.log(col.vmr_lev[:, 0]), col.tskin, col.emis)
        ref = h.jac(c, p.ctrl, prof)
        n = len(ref["rad"])
        assert n > 200000
        g = np.random.default_rng(5).standard_normal(n)
        got = h.jac_vjp(c, p.ctrl, prof, g)
        again = h.jac_vjp(c, p.ctrl, prof, g)
    finally:
        h.close()
    for k, j in (("g_tlev", "dtlev"), ("g_qlev", "dqlev")):
        np.testing.assert_allclose(got[k], ref[j] @ g, rtol=rtol, atol=0, err_msg=k)
        assert np.array_equal(got[k], again[k])  # a fixed summation order
    assert got["g_tskin"] == pytest.approx(float(ref["dtsfc"] @ g), rel=rtol)
    assert got["g_emis"] == pytest.approx(float(ref["demis"] @ g), rel=rtol)


def test_autograd_at_a_perturbed_state(gpu_lib, mtckd):
    """Forward at a state other than the profile's own (the layers are formed
    from the level tensors); backward equals the Jacobians at that state
    contracted with the incoming gradient."""
    import torch
    from clblm_gb300 import torch_ops
    p, col, h = _problem(gpu_lib, mtckd)
    try:
        t0, q0 = p.levels(_tlev(col))
        t = (t0 + torch.tensor([1.5, -0.7, 2.0, 0.3], dtype=torch.float64, device="cuda")).requires_grad_()
        q = (q0 + 0.05).requires_grad_()
        ts = torch.tensor(col.tskin + 1.0, dtype=torch.float64, device="cuda", requires_grad=True)
        em = torch.tensor(0.95, dtype=torch.float64, device="cuda", requires_grad=True)
        rad = torch_ops.nadir_radiance(p, t, q, ts, em)
        c, prof = p.state(t.detach().cpu().numpy(), q.detach().cpu().numpy(), float(ts), float(em))
        ref = h.jac(c, p.ctrl, prof)
        np.testing.assert_allclose(rad.detach().cpu().numpy(), ref["rad"], rtol=1e-12)
        c0, prof0 = p.state(_tlev(col), np.log(col.vmr_lev[:, 0]), col.tskin, col.emis)
        base = h.jac(c0, p.ctrl, prof0)["rad"]
        assert len(base) == len(ref["rad"])  # one grid for every state
        assert np.max(np.abs(ref["rad"] / base - 1)) > 1e-3  # the state moved the radiance
        g = torch.rand_like(rad)
        (rad * g).sum().backward()
    finally:
        h.close()
    gn = g.cpu().numpy()
    np.testing.assert_allclose(t.grad.cpu().numpy(), ref["dtlev"] @ gn, rtol=1e-10)
    np.testing.assert_allclose(q.grad.cpu().numpy(), ref["dqlev"] @ gn, rtol=1e-10)
    assert float(ts.grad) == pytest.approx(float(ref["dtsfc"] @ gn), rel=1e-10)
    assert float(em.grad) == pytest.approx(float(ref["demis"] @ gn), rel=1e-10)


def test_gradient_against_central_differences(gpu_lib, mtckd):
    """Directional derivatives of sum(g * radiance) by central differences of
    the forward pass (0.01 K in the level temperatures, 1e-4 in ln q, 0.01 K
    in Tskin, 1e-4 in the emissivity) against the gradient.  The reference's
    dtau/dT is a 1 K forward difference with the Wtot/T correction and its
    dtau/dln q keeps the self-broadening fixed, and its level maps linearise
    ALAYER's integrals, so the level terms agree to a few per cent; the
    surface terms are exact derivatives."""
    import torch
    from clblm_gb300 import torch_ops
    # layers 40-42 (a few hPa): thin enough that the surface is seen
    p, col, h = _problem(gpu_lib, mtckd, first=40)
    try:
        t0, q0 = p.levels(_tlev(col))
        ts0, em0 = col.tskin, col.emis
        rng = np.random.default_rng(11)
        gvec = None

        def f(t, q, ts, em):
            nonlocal gvec
            r = torch_ops.nadir_radiance(p, t, q, ts, em)
            if gvec is None:
                gvec = torch.tensor(rng.uniform(0.5, 1.5, len(r)), dtype=torch.float64, device="cuda")
            return (r * gvec).sum()

        t = t0.clone().requires_grad_()
        q = q0.clone().requires_grad_()
        ts = torch.tensor(ts0, dtype=torch.float64, device="cuda", requires_grad=True)
        em = torch.tensor(em0, dtype=torch.float64, device="cuda", requires_grad=True)
        f(t, q, ts, em).backward()
        worst = {}
        for name, grad, step, shift in (
                ("t_lev", t.grad, 0.01, lambda s, d: (t0 + s * d, q0, ts0, em0)),
                ("lnq_lev", q.grad, 1e-4, lambda s, d: (t0, q0 + s * d, ts0, em0))):
            d = torch.tensor(rng.choice([-1.0, 1.0], len(t0)), dtype=torch.float64, device="cuda")
            fd = (f(*shift(step, d)) - f(*shift(-step, d))).item() / (2 * step)
            an = float((grad * d).sum())
            worst[name] = abs(fd - an) / abs(fd)
        for name, grad, step, x0 in (("tskin", ts.grad, 0.01, ts0), ("emis", em.grad, 1e-4, em0)):
            args = lambda s: (t0, q0, x0 + s, em0) if name == "tskin" else (t0, q0, ts0, x0 + s)
            fd = (f(*args(step)) - f(*args(-step))).item() / (2 * step)
            assert float(grad) == pytest.approx(fd, rel=1e-5), name
    finally:
        h.close()
    print("relative differences", worst)
    assert max(worst.values()) <= 0.1, worst

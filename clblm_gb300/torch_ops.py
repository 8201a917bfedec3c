"""PyTorch binding of the nadir radiance and its Jacobians.

`NadirRadiance.apply(t_lev, lnq_lev, tskin, emis, problem)` returns the top of
atmosphere radiance of `problem`'s column on the uniform Jacobian grid; its
backward pass applies the analytic Jacobians of noScattJacob
(clblm_noScattJac.f90:20-339) computed by clblm_gpu_jac in the same call:

    d rad / d t_lev    level temperatures (K)
    d rad / d lnq_lev  log mixing ratio of the Jacobian molecule at levels
    d rad / d tskin    surface skin temperature
    d rad / d emis     surface emissivity

The tensors passed in must describe the problem's column (they are checked);
the radiance is computed from the column itself, so the function is the
linearisation of the radiance about that state, which is what gradient-based
retrievals use.  All outputs stay on the device.
"""
import numpy as np
import torch

from . import capi
from . import capi_types as T


class RadianceProblem:
    """A handle (device-resident lines), a column, RT controls and the level
    profile of the Jacobian inputs."""

    def __init__(self, handle, col, ctrl, prof):
        self.handle, self.col, self.ctrl, self.prof = handle, col, ctrl, prof
        self.npts, self.dv = handle.jac_size(col, ctrl, prof)

    def levels(self, device="cuda"):
        """(t_lev, lnq_lev, tskin, emis) tensors of the column's state."""
        t = np.append(self.col.tbot, self.col.ttop[-1])
        q = np.log(self.prof.qlev)
        f = lambda a: torch.tensor(a, dtype=torch.float64, device=device)
        return f(t), f(q), f(self.col.tskin), f(self.col.emis)


class NadirRadiance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, t_lev, lnq_lev, tskin, emis, problem):
        p = problem
        t_ref, q_ref, ts_ref, em_ref = p.levels("cpu")
        if not (torch.allclose(t_lev.detach().cpu(), t_ref) and torch.allclose(lnq_lev.detach().cpu(), q_ref)
                and float(tskin) == float(ts_ref) and float(emis) == float(em_ref)):
            raise ValueError("NadirRadiance: the tensors do not describe the problem's column")
        n, nl = p.npts, p.col.nlay
        dev = t_lev.device
        rad = torch.empty(n, dtype=torch.float64, device=dev)
        dtl = torch.empty((nl + 1, n), dtype=torch.float64, device=dev)
        dql = torch.empty((nl + 1, n), dtype=torch.float64, device=dev)
        dts = torch.empty(n, dtype=torch.float64, device=dev)
        dem = torch.empty(n, dtype=torch.float64, device=dev)
        torch.cuda.current_stream(dev).synchronize()
        p.handle.jac_device(p.col, p.ctrl, p.prof, rad.data_ptr(), dtl.data_ptr(), dql.data_ptr(), dts.data_ptr(),
                            dem.data_ptr(), n)
        ctx.save_for_backward(dtl, dql, dts, dem)
        return rad

    @staticmethod
    def backward(ctx, g):
        dtl, dql, dts, dem = ctx.saved_tensors
        g = g.to(torch.float64)
        return dtl @ g, dql @ g, (dts * g).sum(), (dem * g).sum(), None


def nadir_radiance(problem, t_lev=None, lnq_lev=None, tskin=None, emis=None):
    """Radiance with autograd through the analytic Jacobians."""
    t, q, ts, em = problem.levels()
    return NadirRadiance.apply(t if t_lev is None else t_lev, q if lnq_lev is None else lnq_lev,
                               ts if tskin is None else tskin, em if emis is None else emis, problem)

"""PyTorch binding: the nadir radiance as a differentiable function of the
level profile.

A `RadianceProblem` holds a handle (device-resident lines), the radiative-
transfer controls and a level profile: altitudes, pressures and the
absorbers' volume mixing ratios.  `nadir_radiance(problem, t_lev, lnq_lev,
tskin, emis)` takes the level temperatures, the log mixing ratio of the
Jacobian molecule at the levels, the skin temperature and the emissivity as
tensors and

  forward   builds the layers from them as the reference does
            (rayTraceAndLayerPack: ALAYER's integrals and FPACK's averages,
            clblm_AtmPath.f90:1135-1301, through clblm_gpu_layer_amounts) and
            returns the top-of-atmosphere radiance on noScattJacob's uniform
            grid (clblm_gpu_jac with no derivative asked for: only the
            viewing-path layer ODs are formed);
  backward  is the vector-Jacobian product at the same state
            (clblm_gpu_jac_vjp): the layer ODs of noScattJacob (viewing path,
            T + 1 K, Wtot * 1.01, the molecule alone) are formed again block
            by block and each block's analytic derivatives (Jacobians,
            drv_LevelTemp, drv_LevelConc, level2layer; clblm_noScattJac.f90:
            346-1279) are reduced against the incoming gradient on the device,
            so nothing of size (levels x points) is kept between the passes or
            formed in the backward one.

The gradient is the reference's linearisation: its dtau/dT is a 1 K forward
difference with the Wtot/T correction and its dtau/dln q holds the self-
broadening fixed, so it agrees with finite differences of the forward pass
to within those approximations (a few per cent), and exactly with
clblm_gpu_jac's Jacobians contracted with the same gradient.
"""
import numpy as np
import torch

from . import capi_types as T
from .synth import BOLTZ_MB


class RadianceProblem:
    """A handle, RT controls (grid_type 1: the uniform grid) and a level
    profile: z_lev [km], p_lev [mb] (level 0 at the surface), vmr_lev
    [nlev, nmol] volume mixing ratios of the absorbers `mol_id`, the spectral
    window and the Jacobian molecule (HITRAN number)."""

    def __init__(self, handle, ctrl, z_lev, p_lev, vmr_lev, mol_id, v1, v2, t_lev, tskin, emis, jac_mol=1,
                 earth_radius=6371.23):
        self.handle = handle
        self.z = np.ascontiguousarray(z_lev, dtype=np.float64)
        self.p = np.ascontiguousarray(p_lev, dtype=np.float64)
        self.vmr = np.ascontiguousarray(vmr_lev, dtype=np.float64)
        self.mol_id = np.ascontiguousarray(mol_id, dtype=np.int32)
        self.v1, self.v2, self.jac_mol, self.re = float(v1), float(v2), int(jac_mol), float(earth_radius)
        self.jm = int(np.nonzero(self.mol_id == self.jac_mol)[0][0])
        self.ctrl = T.clblm_rt_ctrl_t.from_buffer_copy(ctrl)
        if self.ctrl.dv_user <= 0.0:
            # the uniform grid is the one of the profile's own state for every
            # state (a user DV, as setDV takes it), so that the radiance of
            # nearby states is on the same points
            col, prof = self.state(t_lev, np.log(self.vmr[:, self.jm]), tskin, emis)
            _, self.ctrl.dv_user = handle.jac_size(col, self.ctrl, prof)

    @classmethod
    def from_column(cls, handle, ctrl, col, jac_mol=1):
        """The level profile of a column made by synth.atmosphere()."""
        return cls(handle, ctrl, col.z_lev, col.p_lev, col.vmr_lev, col.mol_id, col.v1, col.v2,
                   np.append(col.tbot, col.ttop[-1]), col.tskin, col.emis, jac_mol)

    def state(self, t_lev, lnq_lev, tskin, emis):
        """The column and the Jacobian inputs of a state: layers from the
        levels by ALAYER + FPACK on the device; the downwelling path's columns
        at the diffusivity secant 1.67."""
        t = np.ascontiguousarray(t_lev, dtype=np.float64)
        vmr = self.vmr.copy()
        vmr[:, self.jm] = np.exp(np.asarray(lnq_lev, dtype=np.float64))
        rho = self.p / (t * BOLTZ_MB)  # air number density at the levels
        la = self.handle.layer_amounts(self.z, self.p, t, rho[:, None] * vmr, earth_radius=self.re)
        col = T.Column(self.mol_id, la["pave"], la["tave"], t[:-1], t[1:], la["w"], la["wtot"], 1.67 * la["wtot"],
                       self.v1, self.v2, float(tskin), float(emis))
        prof = T.JacProfile(self.p, rho * vmr[:, self.jm], jac_mol=self.jac_mol, do_temp=1)
        return col, prof

    def levels(self, t_lev, device="cuda"):
        """Tensors (t_lev, lnq_lev) of the profile at level temperatures t_lev."""
        f = lambda a: torch.tensor(np.asarray(a, dtype=np.float64), device=device)
        return f(t_lev), f(np.log(self.vmr[:, self.jm]))


class NadirRadiance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, t_lev, lnq_lev, tskin, emis, problem):
        p = problem
        col, prof = p.state(t_lev.detach().cpu().numpy(), lnq_lev.detach().cpu().numpy(), float(tskin),
                            float(emis))
        rad_only = T.JacProfile(prof.plev, prof.qlev, jac_mol=0, do_temp=0)
        n, _ = p.handle.jac_size(col, p.ctrl, rad_only)
        dev = t_lev.device
        rad = torch.empty(n, dtype=torch.float64, device=dev)
        torch.cuda.current_stream(dev).synchronize()
        p.handle.jac_device(col, p.ctrl, rad_only, rad=rad.data_ptr(), cap=n)
        ctx.problem, ctx.col, ctx.prof, ctx.n = p, col, prof, n
        return rad

    @staticmethod
    def backward(ctx, g):
        p = ctx.problem
        g = g.detach().to(torch.float64).contiguous()
        torch.cuda.current_stream(g.device).synchronize()  # g is formed on torch's stream
        out = p.handle.jac_vjp(ctx.col, p.ctrl, ctx.prof, g.data_ptr(), ctx.n)
        f = lambda a: torch.tensor(a, dtype=torch.float64, device=g.device)
        return f(out["g_tlev"]), f(out["g_qlev"]), f(out["g_tskin"]), f(out["g_emis"]), None


def nadir_radiance(problem, t_lev, lnq_lev, tskin, emis):
    """Radiance of the state (t_lev, lnq_lev, tskin, emis) of `problem`, with
    autograd through the vector-Jacobian product."""
    as_t = lambda x: x if torch.is_tensor(x) else torch.tensor(float(x), dtype=torch.float64, device="cuda")
    return NadirRadiance.apply(t_lev, lnq_lev, as_t(tskin), as_t(emis), problem)

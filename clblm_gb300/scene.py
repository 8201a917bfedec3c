"""The paths of a down-looking scene, as the nadir radiance takes them.

calcCLBLMPaths (clblm_AtmPath.f90:478-660) for an observer at or above the
top of the profile looking down to the ground: the line of sight (the view
path), and the path of the reflected downwelling radiance from the end of
the view path upwards (at the diffusivity angle acos(1/1.67) for a
Lambertian surface, ThmReflMode 0, or at the view path's zenith angle at
the ground for a specular one, ThmReflMode 1) on the view path's RT levels.
Both come from the library's clblm_path (host code).

mode2_lookDn_mergeUp (clblm_noScattRT.f90:1340-1360) with the default
AMscalingThermal and refPath = 1 computes each layer's OD on the view
path's layer and scales it by the ratio of the downwelling path's air
column to the view path's for the reflected term: that is the Column's
wtot_down over wtot, so slant_column's result goes straight to
Handle.rt_mode2 / Handle.jac.  An observer inside the profile (extendPath,
:670-751), up-looking and limb views (mode3) are not on this path."""
import math

import numpy as np

from . import capi
from .capi_types import Column

SECANT_DIFFUSE = 1.67       # secant_diffuse, clblm_ConstParam.f90:120
PI = 3.1415926535898        # PI as clblm_ConstParam.f90 writes it
TOL = 5.e-4                 # calcCLBLMPaths' altitude tolerance [km]


def scene_paths(z, p, t, den, obs_alt, view_ang, z_rt=None, h2o=0, o2=-1, earth_radius=6371.23,
                v_refrac=1000.0, thm_refl_mode=0, zero_abs_amt=0):
    """(view, down, geometry): the two paths' layer dicts (capi.path) and the
    view path's geometry."""
    view, g = capi.path(z, p, t, den, obs_alt, view_ang, z_rt=z_rt, h2o=h2o, o2=o2, earth_radius=earth_radius,
                        v_refrac=v_refrac, zero_abs_amt=zero_abs_amt)
    if g["hend"] > g["hmin"]:
        raise ValueError("the line of sight goes back to space (a limb view): not a down-looking scene")
    if obs_alt < z[-1] - TOL:
        raise ValueError("the observer is inside the profile: the view path would be extended above it")
    if thm_refl_mode == 0:
        ang = math.acos(1. / SECANT_DIFFUSE) * 180. / PI
    elif thm_refl_mode == 1:
        ang = g["phi"]
    else:
        raise ValueError("thm_refl_mode is 0 (Lambertian) or 1 (specular)")
    down, _ = capi.path(z, p, t, den, g["hend"], ang, z_rt=view["z"], h2o=h2o, o2=o2, earth_radius=earth_radius,
                        v_refrac=v_refrac, zero_abs_amt=zero_abs_amt)
    if len(down["z"]) != len(view["z"]) or np.any(np.abs(down["z"] - view["z"]) > TOL):
        raise ValueError("the altitude grids of the view and downwelling paths are not consistent")
    return view, down, g


def slant_column(mol_id, z, p, t, den, obs_alt, view_ang, v1, v2, tskin, emis, v_refrac=None, **kw):
    """The Column of a down-looking slant view from obs_alt at zenith angle
    view_ang (> 90 deg) through the level profile (z, p, t, den [nlev,
    nmol] number densities of the absorbers mol_id): the view path's layer
    amounts, its level temperatures, and the downwelling path's air column.
    V_refrac defaults to (v1 + v2) / 2 (clblm_Config.f90:412)."""
    vr = 0.5 * (v1 + v2) if v_refrac is None else v_refrac
    view, down, _ = scene_paths(z, p, t, den, obs_alt, view_ang, v_refrac=vr, **kw)
    return Column(mol_id, view["pave"], view["tave"], view["t"][:-1], view["t"][1:], view["w"], view["wtot"],
                  down["wtot"], v1, v2, tskin, emis)

"""Slant and refracted paths (calculatePath, clblm_AtmPath.f90:871-964).

The oracle's restatement (oracle/path.c) is pinned by properties the
geometry must have: a path straight down is the nadir layer integral, a
line of sight through a profile without refractivity is the straight chord
of the spherical shells, a limb path is twice the path that starts
horizontally at its tangent point, and the path up from the ground is the
path down from its end at the zenith angle it arrives with.  The library's
clblm_path (host code) must equal the oracle bit for bit on every case."""
import numpy as np
import pytest

from clblm_gb300 import synth

RE = 6371.23


@pytest.fixture(scope="module")
def profile():
    col = synth.atmosphere(60, 0.1, 500., 2500.)
    z, p = col.z_lev.copy(), col.p_lev.copy()
    z[0] = 0.0
    t = np.append(col.tbot, col.ttop[-1])
    den = synth.level_density(p[:, None], t[:, None], col.vmr_lev)
    return z, p, t, den


def _chord(h1, ang, h2):
    """straight line from altitude h1 at zenith angle ang down to altitude h2"""
    r1, r2, th = RE + h1, RE + h2, np.radians(ang)
    return -r1 * np.cos(th) - np.sqrt(r2 ** 2 - (r1 * np.sin(th)) ** 2)


def test_vertical_path_is_the_nadir_integral(oracle_mod, profile):
    z, p, t, den = profile
    out, g = oracle_mod.path_amounts(z, p, t, den, z[-1], 180.0)
    ref = oracle_mod.layer_amounts(z, p, t, den)
    for k in ("pave", "tave", "wtot", "w"):
        np.testing.assert_allclose(out[k], ref[k], rtol=1e-14, err_msg=k)
    np.testing.assert_allclose(out["secant"], 1.0, rtol=1e-12)
    assert np.all(out["ipath"] == 1) and g["LEN"] == 0 and g["Hend"] == 0.0
    np.testing.assert_array_equal(out["zlev"], z)
    np.testing.assert_allclose(out["qlev"], den, rtol=1e-15)  # x1 * (x2 / x1)**1


@pytest.mark.parametrize("ang", [160.0, 135.0, 110.0, 100.0])
def test_without_refractivity_the_path_is_the_chord(oracle_mod, profile, ang):
    z, p, t, den = profile
    # the refractivity is the dry term ~ p plus a water vapour term: scale p
    # down and leave H2O out of it (the densities are given apart)
    ps = p * 1e-12
    out, g = oracle_mod.path_amounts(z, ps, t, den, z[-1], ang, h2o=-1)
    assert g["BENDNG"] < 1e-9
    assert g["RANGE"] == pytest.approx(_chord(z[-1], ang, 0.0), rel=1e-9)
    # per layer: the chord between the shells at zenith angle sin(i) r = const
    c = (RE + z[-1]) * np.sin(np.radians(ang))
    seg = np.sqrt((RE + z[1:]) ** 2 - c ** 2) - np.sqrt((RE + z[:-1]) ** 2 - c ** 2)
    np.testing.assert_allclose(out["secant"] * np.diff(z), seg, rtol=1e-8)
    assert g["PHI"] == pytest.approx(np.degrees(np.arcsin(c / RE)), rel=1e-9)


def test_refraction_shortens_and_bends(oracle_mod, profile):
    z, p, t, den = profile
    prev = 0.0
    for ang in (150.0, 120.0, 100.0):
        out, g = oracle_mod.path_amounts(z, p, t, den, z[-1], ang)
        assert g["BENDNG"] > prev
        prev = g["BENDNG"]
        # refraction bends the ray towards the ground: it arrives steeper
        assert 0 < _chord(z[-1], ang, 0.0) - g["RANGE"] < 0.01 * g["RANGE"]
        assert np.all(np.diff(out["secant"]) < 0)


def test_limb_path_doubles_the_tangent_path(oracle_mod, profile):
    z, p, t, den = profile
    limb, g = oracle_mod.path_amounts(z, p, t, den, z[-1], 95.0)
    assert g["LEN"] == 1 and 0 < g["HMIN"] < z[-1] and g["Hend"] == z[-1]
    assert np.all(limb["ipath"] == 2)
    up, gu = oracle_mod.path_amounts(z, p, t, den, g["HMIN"], 90.0)
    assert np.all(up["ipath"] == 3)
    for k in ("pave", "tave", "wtot", "w", "secant", "zlev"):
        np.testing.assert_allclose(limb[k], up[k], rtol=1e-13, err_msg=k)
    assert g["RANGE"] == pytest.approx(2.0 * gu["RANGE"], rel=1e-13)
    assert g["BENDNG"] == pytest.approx(2.0 * gu["BENDNG"], rel=1e-13)


def test_limb_below_the_observer(oracle_mod, profile):
    """observer inside the profile looking just below the horizon: layers
    under it are crossed twice (IPATH 2), those above once going up (3)"""
    z, p, t, den = profile
    out, g = oracle_mod.path_amounts(z, p, t, den, 30.0, 92.0)
    assert g["LEN"] == 1 and g["HMIN"] < 30.0
    below = out["zlev"][:-1] < 30.0 - 1e-9
    assert np.all(out["ipath"][below] == 2) and np.all(out["ipath"][~below] == 3)
    assert out["zlev"][0] == g["HMIN"] and 30.0 in out["zlev"]


def test_up_and_down_paths_agree(oracle_mod, profile):
    z, p, t, den = profile
    up, gu = oracle_mod.path_amounts(z, p, t, den, 0.0, 30.0)
    dn, gd = oracle_mod.path_amounts(z, p, t, den, z[-1], gu["PHI"])
    assert gd["PHI"] == pytest.approx(30.0, abs=1e-10)
    for k in ("pave", "tave", "wtot", "w", "secant"):
        np.testing.assert_allclose(up[k], dn[k], rtol=1e-10, err_msg=k)
    assert np.all(up["ipath"] == 3) and np.all(dn["ipath"] == 1)


def test_rt_boundaries_between_levels(oracle_mod, profile):
    """RT boundaries off the profile's levels: the output layers sum the
    merged layers, so their columns add up to the profile-level path's"""
    z, p, t, den = profile
    zr = np.array([0.0, 1.23, 5.0, 17.77, 40.0, z[-1]])
    coarse, _ = oracle_mod.path_amounts(z, p, t, den, z[-1], 140.0, z_rt=zr)
    np.testing.assert_array_equal(coarse["zlev"], zr)
    fine, _ = oracle_mod.path_amounts(z, p, t, den, z[-1], 140.0, z_rt=np.union1d(z, zr))
    edges = np.searchsorted(fine["zlev"], zr)
    for k in ("wtot", "w"):
        sums = np.add.reduceat(fine[k], edges[:-1], axis=0)
        np.testing.assert_allclose(coarse[k], sums, rtol=1e-12, err_msg=k)
    # levels between the profile's: densities interpolated exponentially
    i = np.searchsorted(z, 1.23)
    a = (1.23 - z[i - 1]) / (z[i] - z[i - 1])
    np.testing.assert_allclose(coarse["qlev"][1], den[i - 1] * (den[i] / den[i - 1]) ** a, rtol=1e-13)


def test_zero_abs_amt_upward(oracle_mod, profile):
    z, p, t, den = profile
    full, _ = oracle_mod.path_amounts(z, p, t, den, 0.0, 30.0)
    cut, _ = oracle_mod.path_amounts(z, p, t, den, 0.0, 30.0, zero_abs_amt=1)
    n = len(cut["pave"])
    assert 0 < n < len(full["pave"])
    for k in ("pave", "tave", "wtot", "secant"):
        np.testing.assert_array_equal(cut[k], full[k][:n])
    tot = full["w"].sum(axis=0)
    for m in range(den.shape[1]):
        zeroed = cut["w"][:, m] == 0
        if not zeroed.any():
            np.testing.assert_array_equal(cut["w"][:, m], full["w"][:n, m])
            continue
        first = int(np.argmax(zeroed))
        assert np.all(zeroed[first:])  # once exhausted, zero above
        assert full["w"][:first, m].sum() >= 0.999 * tot[m]
    # a downward path keeps everything
    dn, _ = oracle_mod.path_amounts(z, p, t, den, z[-1], 150.0, zero_abs_amt=1)
    assert len(dn["pave"]) == len(z) - 1 and np.all(dn["w"] > 0)


@pytest.mark.parametrize("h,ang", [(0.0, 120.0), (z_top := 64.0, 30.0), (80.0, 30.0)])
def test_rejected_geometries(oracle_mod, profile, h, ang):
    """FSCGEO's IERROR: looking down from the ground, up from the top or
    above it"""
    z, p, t, den = profile
    with pytest.raises(oracle_mod.OracleError):
        oracle_mod.path_amounts(z, p, t, den, z[-1] if h == z_top else h, ang)


def test_observer_above_the_profile_is_reduced(oracle_mod, profile):
    """REDUCE: an observer above the profile's top starts there, at the
    zenith angle the ray has when it reaches it"""
    z, p, t, den = profile
    out, g = oracle_mod.path_amounts(z, p, t, den, 100.0, 150.0)
    assert g["Hobs"] == z[-1]
    s = (RE + 100.0) * np.sin(np.radians(150.0)) / (RE + z[-1])
    assert g["ANGLE"] == pytest.approx(180.0 - np.degrees(np.arcsin(s)), rel=1e-6)
    ref, _ = oracle_mod.path_amounts(z, p, t, den, z[-1], g["ANGLE"])
    np.testing.assert_allclose(out["w"], ref["w"], rtol=1e-10)


CASES = [
    (None, 180.0, {}), (None, 150.0, {}), (None, 100.0, {}), (None, 95.0, {}), (0.0, 30.0, {}),
    (0.0, 30.0, dict(zero_abs_amt=1)), (10.0, 60.0, {}), (10.0, 120.0, {}), (100.0, 150.0, {}), (30.0, 92.0, {}),
    (None, 180.0, dict(z_rt=np.array([0., 1.23, 5.0, 17.77, 40.0, 64.0]))),
    (12.3456, 140.0, dict(z_rt=np.linspace(0, 60.0, 17))), (5.0, 45.0, dict(xvbar=25000.0, o2=2)),
    (None, 170.0, dict(h2o=-1)),
]


@pytest.mark.parametrize("h,ang,kw", CASES)
def test_library_equals_oracle(gpu_lib, oracle_mod, profile, h, ang, kw):
    z, p, t, den = profile
    h = z[-1] if h is None else h
    kw = dict(kw)
    if "z_rt" in kw:
        kw["z_rt"] = np.append(kw["z_rt"][kw["z_rt"] < z[-1] - 1.0], z[-1])
    o, go = oracle_mod.path_amounts(z, p, t, den, h, ang, **kw)
    kl = dict(kw)
    if "xvbar" in kl:
        kl["v_refrac"] = kl.pop("xvbar")
    layers, gl = gpu_lib.path(z, p, t, den, h, ang, **kl)
    for ko, kl_ in (("zlev", "z"), ("plev", "p"), ("tlev", "t"), ("qlev", "q"), ("pave", "pave"), ("tave", "tave"),
                    ("wtot", "wtot"), ("w", "w"), ("secant", "secant"), ("ipath", "ipath")):
        np.testing.assert_array_equal(layers[kl_], o[ko], err_msg=kl_)
    for ko, kl_ in (("Hobs", "hobs"), ("Hend", "hend"), ("ANGLE", "angle"), ("PHI", "phi"), ("HMIN", "hmin"),
                    ("LEN", "len"), ("RANGE", "range"), ("BETA", "beta"), ("BENDNG", "bendng"),
                    ("PHI_END", "phi_end")):
        assert gl[kl_] == go[ko], kl_


def test_library_errors(gpu_lib, profile):
    z, p, t, den = profile
    with pytest.raises(gpu_lib.ClblmError) as e:
        gpu_lib.path(z, p, t, den, 0.0, 120.0)
    assert e.value.code == 1 and "FSCGEO" in str(e.value)
    with pytest.raises(gpu_lib.ClblmError) as e:
        gpu_lib.path(z, p, t, den, z[-1], 150.0, cap=10)
    assert e.value.code == 9
    with pytest.raises(gpu_lib.ClblmError):
        gpu_lib.path(z[::-1], p, t, den, z[0], 150.0)
    p2 = p.copy()
    p2[5] = p2[4]
    with pytest.raises(gpu_lib.ClblmError) as e:
        gpu_lib.path(z, p2, t, den, z[-1], 150.0)
    assert "pressures" in str(e.value)


def test_scene_paths_of_a_slant_view(gpu_lib, profile):
    """calcCLBLMPaths' view and downwelling paths: the downwelling path runs
    up from the view path's end on its levels; with a Lambertian surface its
    air columns are the diffusivity secant's, with a specular one the view
    path's own"""
    from clblm_gb300 import scene
    z, p, t, den = profile
    view, down, g = scene.scene_paths(z, p, t, den, z[-1], 150.0)
    nadir, _ = gpu_lib.path(z, p, t, den, z[-1], 180.0)
    np.testing.assert_array_equal(down["z"], view["z"])
    assert np.all(view["ipath"] == 1) and np.all(down["ipath"] == 3)
    # air columns over the vertical ones: the secants of straight chords
    # through the shells (sin(i) r = c), to the refraction's bending
    for path, c in ((down, RE * np.sqrt(1 - 1 / scene.SECANT_DIFFUSE ** 2)),
                    (view, (RE + z[-1]) * np.sin(np.radians(150.0)))):
        sec = (np.sqrt((RE + z[1:]) ** 2 - c ** 2) - np.sqrt((RE + z[:-1]) ** 2 - c ** 2)) / np.diff(z)
        np.testing.assert_allclose(path["wtot"] / nadir["wtot"], sec, rtol=2e-3)
    _, spec, _ = scene.scene_paths(z, p, t, den, z[-1], 150.0, thm_refl_mode=1)
    np.testing.assert_allclose(spec["wtot"], view["wtot"], rtol=1e-10)
    col = scene.slant_column(np.arange(1, den.shape[1] + 1), z, p, t, den, z[-1], 150.0, 600.0, 700.0, 290.0, 0.98)
    assert col.nlay == len(z) - 1
    np.testing.assert_array_equal(col.ttop[:-1], col.tbot[1:])
    with pytest.raises(ValueError):
        scene.scene_paths(z, p, t, den, z[-1], 95.0)  # limb
    with pytest.raises(ValueError):
        scene.scene_paths(z, p, t, den, 20.0, 150.0)  # observer inside

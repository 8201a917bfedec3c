"""The radiance and Jacobian output files (clblm_Drivers.f90 writeRadiance,
writeJacobians, writeSpectFileHeader): names, format, header and layout."""
import numpy as np
import pytest

pytest.importorskip("scipy")
from clblm_gb300 import ncout  # noqa: E402


def test_names_follow_the_driver():
    assert ncout.radiance_name(1) == "rad_mono_s001.nc"
    assert ncout.radiance_name(12, obs_alt=10.0, view_ang=40.0) == "rad_mono_a010km-o040deg_s012.nc"
    # without an altitude the angle follows `_mono` directly, as the driver's
    # trim(altStr)//trim(angStr) makes it
    assert ncout.radiance_name(3, view_ang=0.0) == "rad_monoo000deg_s003.nc"
    assert ncout.jacobian_name("T", 2) == "drad-dT_mono_s002.nc"
    assert ncout.jacobian_name("H2O", 2, obs_alt=705.0) == "drad-dH2O_mono_a705km-_s002.nc"


def test_radiance_file(tmp_path):
    rad = np.linspace(1e-7, 2e-7, 1001)
    p = ncout.write_radiance(tmp_path, rad, 600.0, 0.01, scene_no=4, uid=77, scene_file="scene.nc")
    assert p.name == "rad_mono_s004.nc"
    assert p.read_bytes()[:4] == b"CDF\x02"  # 64-bit offset classic format
    attrs, vars_ = ncout.read(p)
    assert list(attrs) == ["title", "sceneFileName", "UID", "sceneNumber", "productName", "spectralDataType",
                           "V1", "V2", "DV", "NSAMP"]
    assert attrs["title"] == "CLBLM Output File"
    assert len(attrs["sceneFileName"]) == 256 and attrs["sceneFileName"].rstrip() == "scene.nc"
    assert attrs["productName"].rstrip() == "Radiance" and len(attrs["productName"]) == 32
    assert attrs["spectralDataType"].rstrip() == "Monochromatic"
    assert attrs["UID"] == 77 and attrs["sceneNumber"] == 4 and attrs["NSAMP"] == 1001
    assert attrs["V1"] == 600.0 and attrs["DV"] == 0.01 and attrs["V2"] == 600.0 + 0.01 * 1000
    np.testing.assert_array_equal(vars_["radiance"], rad)
    assert vars_["radiance"].dtype == np.float64


def test_jacobian_files(tmp_path):
    nlev, n = 7, 500
    dt = np.arange(nlev * n, dtype=np.float64).reshape(nlev, n)
    dq = -dt
    ts, em = np.ones(n), np.full(n, 2.0)
    paths = ncout.write_jacobians(tmp_path, 1000.0, 0.002, dtlev=dt, dqlev=dq, dtsfc=ts, demis=em)
    assert [p.name for p in paths] == ["drad-dT_mono_s001.nc", "drad-dH2O_mono_s001.nc",
                                       "drad-dTskin_mono_s001.nc", "drad-demis_mono_s001.nc"]
    attrs, v = ncout.read(paths[0])
    assert attrs["productName"].rstrip() == "Concentration_Jacobians" and attrs["NSAMP"] == n
    np.testing.assert_array_equal(v["dRad_dT"], dt)  # (numLayers, numPoints): Fortran (numPoints, numLayers)
    _, v = ncout.read(paths[1])
    np.testing.assert_array_equal(v["dRad_dH2O"], dq)
    _, v = ncout.read(paths[2])
    np.testing.assert_array_equal(v["dRad_dTskin"], ts)
    _, v = ncout.read(paths[3])
    np.testing.assert_array_equal(v["dRad_dEmis"], em)


@pytest.mark.gpu
def test_gpu_results_round_trip(gpu_lib, mtckd, tmp_path):
    """Radiance and Jacobians of a GPU call written in the driver's files and
    read back unchanged."""
    from clblm_gb300 import capi_types as T
    from clblm_gb300 import synth
    lines, col, _ = synth.config1(n_lines=5000)
    c = col.sub([0, 1, 2]).with_window(1000.0, 1004.0)
    h = gpu_lib.Handle(lines, mtckd)
    r = h.jac(c, T.rt_ctrl(grid_type=1), synth.jac_profile(c))
    h.close()
    v1 = r["v1"]
    p = ncout.write_radiance(tmp_path, r["rad"], v1, r["dv"])
    _, v = ncout.read(p)
    np.testing.assert_array_equal(v["radiance"], r["rad"])
    paths = ncout.write_jacobians(tmp_path, v1, r["dv"], dtlev=r["dtlev"], dqlev=r["dqlev"], dtsfc=r["dtsfc"],
                                  demis=r["demis"])
    for path, key, var in zip(paths, ("dtlev", "dqlev", "dtsfc", "demis"),
                              ("dRad_dT", "dRad_dH2O", "dRad_dTskin", "dRad_dEmis")):
        _, v = ncout.read(path)
        np.testing.assert_array_equal(v[var], r[key])


def test_od_and_transmittance_names():
    # writeOD: root, altitude/angle, _sNNN_LLL (no _mono)
    assert ncout.od_name(7, 2) == "od_s002_007.nc"
    assert ncout.od_name(12, 1, obs_alt=705.0, view_ang=0.0) == "od_a705km-o000deg_s001_012.nc"
    assert ncout.transmittance_name(3) == "tx-total_mono_s003.nc"
    assert ncout.transmittance_name(3, convolved=True) == "tx-total_convolved_s003.nc"
    assert ncout.transmittance_name(3, lay_no=14) == "tx-prfl_mono_s003_014.nc"
    assert ncout.transmittance_name(1, lay_no=2, convolved=True, view_ang=40.0) == "tx-prfl_convolvedo040deg_s001_002.nc"


def test_od_and_transmittance_files(tmp_path):
    od = np.geomspace(1e-4, 3.0, 777)
    p = ncout.write_od(tmp_path, od, 600.0, 0.005, lay_no=5, scene_no=2, uid=9)
    assert p.name == "od_s002_005.nc" and p.read_bytes()[:4] == b"CDF\x02"
    attrs, v = ncout.read(p)
    assert attrs["productName"].rstrip() == "Layer_OD" and attrs["spectralDataType"].rstrip() == "Monochromatic"
    assert attrs["NSAMP"] == 777 and attrs["V2"] == 600.0 + 0.005 * 776
    np.testing.assert_array_equal(v["layerOD"], od)
    tx = np.exp(-od)
    p = ncout.write_transmittance(tmp_path, tx, 600.0, 0.005, scene_no=2)
    attrs, v = ncout.read(p)
    assert p.name == "tx-total_mono_s002.nc" and attrs["productName"].rstrip() == "Total_transmittance"
    np.testing.assert_array_equal(v["transmittance"], tx)
    p = ncout.write_transmittance(tmp_path, tx, 600.0, 0.005, scene_no=2, lay_no=4, convolved=True)
    attrs, _ = ncout.read(p)
    assert attrs["productName"].rstrip() == "Transmittance_profile"
    assert attrs["spectralDataType"].rstrip() == "Convolved"


@pytest.mark.gpu
def test_gpu_od_file_round_trip(gpu_lib, tmp_path):
    """A layer OD of clblm_gpu_od written as writeOD's file and read back."""
    from clblm_gb300 import capi_types as T
    from clblm_gb300 import synth
    lines, col = synth.config0()
    dn, df, _ = gpu_lib.setDV(col)
    h = gpu_lib.Handle(lines)
    od, dv = h.odlay(col.layer(0), T.grid_struct(col.v1, col.v2, dn[0], df[0]), T.od_ctrl(contnm_off=1))
    h.close()
    p = ncout.write_od(tmp_path, od, col.v1, dv, lay_no=1)
    attrs, v = ncout.read(p)
    np.testing.assert_array_equal(v["layerOD"], od)
    assert attrs["DV"] == dv and attrs["NSAMP"] == len(od)

"""CLBLM's spectral output files: the radiance and Jacobian netCDF files the
reference's driver writes (src/clblm_src/clblm_Drivers.f90), for results
computed through the C-ABI.

The reference creates each file in the 64-bit-offset classic format
(createNetCDFFile, clblm_FileIO.f90:300-313), writes the global header of
writeSpectFileHeader (clblm_Drivers.f90:2312-2367), one or two dimensions and
one binary64 variable (writeSpectFile_1D_array :2039-2076,
writeSpectFile_2D_array :2111-2153).  Its build promotes REAL to binary64
(-fdefault-real-8, Makefile:28), so DV is binary64 like V1 and V2; integers
are 32-bit; the CHARACTER header fields keep their declared lengths, blank
padded (sceneFile 256, productName and productSpectType 32,
clblm_FileIO.f90:33-47).  A Fortran variable dimensioned (numPoints,
numLayers) is stored as (numLayers, numPoints) in the file's C order, the
layout of this package's level-major Jacobian arrays.

File names follow writeRadiance (:1342-1462) and writeJacobians
(:1668-1908): root name, product, `_mono`, the observer altitude and view
angle when set, `_sNNN`, `.nc`, with the default root names of
clblm_Config.f90:255-259.  The layer OD file of writeOD (:1914-2016) is
`od` + altitude/angle + `_sNNN_LLL.nc` with variable `layerOD`; the
transmittance files of writeTransmittance (:1469-1666) are
`tx-total_<mono|convolved>..._sNNN.nc` and, per layer of a profile,
`tx-prfl_<mono|convolved>..._sNNN_LLL.nc`, with variable `transmittance`.
"""
from pathlib import Path

import numpy as np
from scipy.io import netcdf_file

ROOT_OD = "od"          # clblm_Config.f90:255
ROOT_RAD = "rad"        # clblm_Config.f90:256
ROOT_TXTOT = "tx-total"  # clblm_Config.f90:257
ROOT_TXPRFL = "tx-prfl"  # clblm_Config.f90:258
ROOT_JAC = "drad-d"     # clblm_Config.f90:259


def _pad(s, n):
    """A CHARACTER(n) value: blank padded or cut to n."""
    return (str(s) + " " * n)[:n]


def _alt_ang(obs_alt, view_ang):
    """`_aNNNkm-` and `oNNNdeg` of writeRadiance (:1372-1376), each only when set."""
    alt = "_a%03dkm-" % int(obs_alt) if obs_alt is not None and obs_alt >= 0. else ""
    ang = "o%03ddeg" % int(view_ang) if view_ang is not None and view_ang >= 0. else ""
    return alt + ang


def radiance_name(scene_no=1, obs_alt=None, view_ang=None, extra="", root=ROOT_RAD):
    """The monochromatic radiance file's name (writeRadiance :1386-1392)."""
    ext = "_" + extra if extra else ""
    return "%s_mono%s_s%03d%s.nc" % (root, _alt_ang(obs_alt, view_ang), scene_no, ext)


def jacobian_name(jac, scene_no=1, obs_alt=None, view_ang=None, root=ROOT_JAC):
    """The monochromatic Jacobian file's name for `jac` ('T', 'Tskin', 'emis'
    or a molecule name; writeJacobians :1813-1817)."""
    return "%s%s_mono%s_s%03d.nc" % (root, jac, _alt_ang(obs_alt, view_ang), scene_no)


def od_name(lay_no, scene_no=1, obs_alt=None, view_ang=None, root=ROOT_OD):
    """The layer OD file's name (writeOD :1968-1980): no `_mono` tag."""
    return "%s%s_s%03d_%03d.nc" % (root, _alt_ang(obs_alt, view_ang), scene_no, lay_no)


def transmittance_name(scene_no=1, lay_no=None, convolved=False, obs_alt=None, view_ang=None):
    """The total (lay_no None) or profile-layer transmittance file's name
    (writeTransmittance :1535, :1554, :1611, :1626)."""
    kind = "_convolved" if convolved else "_mono"
    if lay_no is None:
        return "%s%s%s_s%03d.nc" % (ROOT_TXTOT, kind, _alt_ang(obs_alt, view_ang), scene_no)
    return "%s%s%s_s%03d_%03d.nc" % (ROOT_TXPRFL, kind, _alt_ang(obs_alt, view_ang), scene_no, lay_no)


def _write(path, var, data, dims, v1, v2, dv, product, scene_no, uid, scene_file, spect_type="Monochromatic"):
    data = np.ascontiguousarray(data, dtype=np.float64)
    f = netcdf_file(str(path), "w", version=2)
    try:
        # writeSpectFileHeader, in its order
        f.title = "CLBLM Output File"
        f.sceneFileName = _pad(scene_file, 256)
        f.UID = np.int32(uid)
        f.sceneNumber = np.int32(scene_no)
        f.productName = _pad(product, 32)
        f.spectralDataType = _pad(spect_type, 32)
        f.V1 = np.float64(v1)
        f.V2 = np.float64(v2)
        f.DV = np.float64(dv)
        f.NSAMP = np.int32(data.shape[-1])
        for name, n in zip(dims, data.shape):
            f.createDimension(name, n)
        v = f.createVariable(var, "d", dims)
        v[...] = data
    finally:
        f.close()
    return Path(path)


def write_radiance(directory, rad, v1, dv, scene_no=1, uid=0, scene_file="", obs_alt=None, view_ang=None,
                   extra=""):
    """`radiance` on numPoints, with the header of a monochromatic radiance
    (writeRadiance, radFlag = 1).  Returns the file's path."""
    rad = np.asarray(rad, dtype=np.float64)
    v2 = v1 + dv * (len(rad) - 1)
    path = Path(directory) / radiance_name(scene_no, obs_alt, view_ang, extra)
    return _write(path, "radiance", rad, ("numPoints",), v1, v2, dv, "Radiance", scene_no, uid, scene_file)


def write_jacobians(directory, v1, dv, dtlev=None, dqlev=None, dtsfc=None, demis=None, jac_mol_name="H2O",
                    scene_no=1, uid=0, scene_file="", obs_alt=None, view_ang=None):
    """The monochromatic Jacobian files of writeJacobians (JacFlag = 1):
    dRad_dT and dRad_d<MOL> on (numLayers, numPoints) from level-major arrays
    [level, point], dRad_dTskin and dRad_dEmis on numPoints.  Returns the
    paths written."""
    out = []
    items = (("T", "dRad_dT", dtlev), (jac_mol_name.upper(), "dRad_d" + jac_mol_name.upper(), dqlev),
             ("Tskin", "dRad_dTskin", dtsfc), ("emis", "dRad_dEmis", demis))
    for tag, var, arr in items:
        if arr is None:
            continue
        arr = np.asarray(arr, dtype=np.float64)
        dims = ("numLayers", "numPoints") if arr.ndim == 2 else ("numPoints",)
        v2 = v1 + dv * (arr.shape[-1] - 1)
        path = Path(directory) / jacobian_name(tag, scene_no, obs_alt, view_ang)
        out.append(_write(path, var, arr, dims, v1, v2, dv, "Concentration_Jacobians", scene_no, uid, scene_file))
    return out


def write_od(directory, od, v1, dv, lay_no, scene_no=1, uid=0, scene_file="", obs_alt=None, view_ang=None):
    """A layer's monochromatic optical depth (ODLAY's monoOD) as writeOD
    writes it: `layerOD` on numPoints, product Layer_OD.  Returns the path."""
    od = np.asarray(od, dtype=np.float64)
    v2 = v1 + dv * (len(od) - 1)
    path = Path(directory) / od_name(lay_no, scene_no, obs_alt, view_ang)
    return _write(path, "layerOD", od, ("numPoints",), v1, v2, dv, "Layer_OD", scene_no, uid, scene_file)


def write_transmittance(directory, tx, v1, dv, scene_no=1, lay_no=None, convolved=False, uid=0, scene_file="",
                        obs_alt=None, view_ang=None):
    """A total transmittance (lay_no None: product Total_transmittance) or
    one layer of a transmittance profile (Transmittance_profile), on its own
    grid, monochromatic or convolved, as writeTransmittance writes them
    (TxFlag 1, -1 with a scanning function, 2, -2).  Returns the path."""
    tx = np.asarray(tx, dtype=np.float64)
    v2 = v1 + dv * (len(tx) - 1)
    path = Path(directory) / transmittance_name(scene_no, lay_no, convolved, obs_alt, view_ang)
    product = "Total_transmittance" if lay_no is None else "Transmittance_profile"
    return _write(path, "transmittance", tx, ("numPoints",), v1, v2, dv, product, scene_no, uid, scene_file,
                  "Convolved" if convolved else "Monochromatic")


def read(path):
    """(global attributes, {variable: array}) of a file written here or by the reference."""
    f = netcdf_file(str(path), "r", mmap=False)
    try:
        attrs = {k: (v.decode() if isinstance(v, bytes) else v) for k, v in f._attributes.items()}
        return attrs, {k: np.array(v[...], dtype=v[...].dtype.newbyteorder("=")) for k, v in f.variables.items()}
    finally:
        f.close()

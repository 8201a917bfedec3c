"""Seeded synthetic inputs of the benchmark workloads.

No public dataset or line database is involved: the line lists, atmospheres
and continuum table are drawn from numpy's PCG64 generator with the seed
equal to the workload index, using the distributions the workloads specify:

  * lines: centres uniform on the window (sorted), intensities log-uniform on
    1e-26..1e-19 cm/molecule at 296 K, air half-widths uniform 0.05-0.10
    cm-1/atm, self half-widths 1.5-5x air, temperature exponents 0.5-0.8,
    lower-state energies 0-3000 cm-1, pressure shifts +-0.005 cm-1/atm.
    Precision as on TAPE3: centre binary64, the rest binary32.
  * atmosphere: pressure falling exponentially (levels equally spaced in
    ln p), temperature 288 K at the surface, lapse to 217 K at 11 km, warming
    linearly to 270 K at 50 km and constant above; altitudes from a 7 km
    scale height.  Layer pressure is the geometric mean of its levels,
    temperature the arithmetic mean.  Layer air columns from hydrostatics.
    H2O volume mixing ratio 1e-2 exp(-z / 2 km), floored at 4e-6.
  * continuum: a smooth self/foreign table on the MT_CKD grid (-20..20000
    cm-1 by 10) with log-normal magnitudes and self T-exponents in 2..4.
"""
import numpy as np

from .capi_types import Column, Continuum, Lines

# HITRAN numbers of the seven synthetic absorbers (iso 1 each).  O2 (7) is left
# out: the reference turns an O2 air width into a foreign width as
# (alfa - 0.21 hwhm) / 0.79 (RDLIN, clblm_ODLAY.f90:2705-2712), which goes
# negative for the workload's self widths of up to 5x air.
SEVEN = np.array([1, 2, 3, 4, 5, 6, 8], dtype=np.int32)
# constant volume mixing ratio of absorbers 2..7 (absorber 1 is H2O-like)
OTHER_VMR = 1.0e-5
AIR_COLUMN_PER_HPA = 100.0 / (9.80665 * 28.964e-3 / 6.02214199e23) / 1.0e4  # molec/cm2/hPa
SECANT_DIFFUSE = 1.67  # clblm_ConstParam.f90:124


# isotopologues of each HITRAN molecule 1..47 (MaxISOTPL_smass, clblm_ConstParam.f90:246-251)
MAXISO = (6, 10, 9, 5, 6, 4, 3, 3, 2, 1, 2, 2, 3, 2, 4, 4, 2, 2, 5, 3, 2, 2, 3, 2,
          1, 3, 2, 1, 2, 1, 3, 1, 1, 1, 2, 1, 2, 2, 1, 2, 1, 1, 1, 1, 2, 4, 1)


def line_list(n, v1, v2, seed, mols=(1,), isotopologues=False):
    """n lines on [v1, v2] with the workload distributions; molecules drawn
    uniformly from `mols` (HITRAN numbers), isotopologue 1, or with
    isotopologues=True each molecule's isotopologues drawn uniformly (the
    line file's MOL field is molecule + 100 * isotopologue, 10 written as 0)
    and O2 and N2 given self widths near their air widths."""
    rng = np.random.Generator(np.random.PCG64(seed))
    vnu = np.sort(rng.uniform(v1, v2, n))
    sp = 10.0 ** rng.uniform(-26.0, -19.0, n)
    alfa = rng.uniform(0.05, 0.10, n)
    hwhm = alfa * rng.uniform(1.5, 5.0, n)
    tmpalf = rng.uniform(0.5, 0.8, n)
    epp = rng.uniform(0.0, 3000.0, n)
    pshift = rng.uniform(-0.005, 0.005, n)
    mols = np.asarray(mols, dtype=np.int32)
    m = mols[rng.integers(0, len(mols), n)]
    mol = m + 100
    if isotopologues:
        iso = 1 + np.floor(rng.uniform(0.0, 1.0, n) * np.asarray(MAXISO)[m - 1]).astype(np.int32)
        mol = m + 100 * (iso % 10)
        # O2 and N2: self widths near the air widths, as in HITRAN, so that
        # the reference's foreign width (air - vmr * self) / (1 - vmr) stays
        # positive
        o2n2 = (m == 7) | (m == 22)
        hwhm = np.where(o2n2, alfa * rng.uniform(0.8, 1.2, n), hwhm)
    return Lines(vnu=vnu, sp=sp.astype(np.float32), alfa=alfa.astype(np.float32),
                 epp=epp.astype(np.float32), mol=mol.astype(np.int32),
                 hwhm=hwhm.astype(np.float32), tmpalf=tmpalf.astype(np.float32),
                 pshift=pshift.astype(np.float32), iflg=np.zeros(n, np.int32))


# temperatures of the line-coupling coefficients (LNCORQ's TEMPLC)
TEMPLC = (200.0, 250.0, 296.0, 340.0)


def with_coupling(lines, idx, iflg=1, a=(0.02, 0.015, 0.01, 0.008), b=(1.0e-3, 8.0e-4, 5.0e-4, 4.0e-4)):
    """The line list with line-coupling coefficients for the lines idx: each
    gets IFLG = iflg (1: first-order coupling Y and second-order G; 3:
    reduced widths GAMMA1, GAMMA2; one value, or one per line) and is
    followed by a coefficient record
    (IFLG -1) holding a = Y or GAMMA1 at the four TEMPLC in VNU, ALFA, MOL
    (the bits of a float) and TMPALF, and b = G or GAMMA2 in SP, EPP, HWHM
    and PSHIFT, as LNFL writes them (LNCORQ clblm_ODLAY.f90:1822-1832).
    a and b: four values, or one row of four per line."""
    from .capi_types import Lines
    idx = np.asarray(idx, dtype=np.int64)
    order = np.argsort(idx, kind="stable")
    idx = idx[order]
    m = len(idx)
    iflg = np.broadcast_to(np.asarray(iflg, dtype=np.int32), (m,))[order] if np.ndim(iflg) else np.full(m, iflg, np.int32)
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    a = a[order] if a.ndim == 2 else a
    b = b[order] if b.ndim == 2 else b
    a = np.broadcast_to(np.asarray(a, dtype=np.float64), (m, 4))
    b = np.broadcast_to(np.asarray(b, dtype=np.float64), (m, 4))
    total = lines.n + m
    pos = idx + np.arange(m) + 1              # the coefficient records in the new list
    keep = np.ones(total, bool)
    keep[pos] = False
    out = {}
    for name, dt in Lines.FIELDS:
        arr = np.zeros(total, dtype=dt)
        arr[keep] = getattr(lines, name)
        out[name] = arr
    out["iflg"][pos - 1] = iflg
    out["iflg"][pos] = -1
    out["vnu"][pos] = a[:, 0]
    out["alfa"][pos] = a[:, 1].astype(np.float32)
    out["mol"][pos] = a[:, 2].astype(np.float32).view(np.int32)
    out["tmpalf"][pos] = a[:, 3].astype(np.float32)
    out["sp"][pos] = b[:, 0].astype(np.float32)
    out["epp"][pos] = b[:, 1].astype(np.float32)
    out["hwhm"][pos] = b[:, 2].astype(np.float32)
    out["pshift"][pos] = b[:, 3].astype(np.float32)
    return Lines(**out)


def continuum(seed=7):
    """Smooth synthetic self/foreign coefficients on the MT_CKD 10 cm-1 grid."""
    rng = np.random.Generator(np.random.PCG64(1000 + seed))
    n = 2003
    v = -20.0 + 10.0 * np.arange(n)

    def smooth_lognormal(mean_log10, sigma):
        z = rng.standard_normal(n + 64)
        k = np.exp(-0.5 * (np.arange(-32, 33) / 8.0) ** 2)
        z = np.convolve(z, k / np.sqrt((k * k).sum()), mode="same")[32:32 + n]
        return 10.0 ** (mean_log10 + sigma * z)

    self_ref = smooth_lognormal(-22.0, 0.6)
    for_ref = smooth_lognormal(-24.0, 0.5)
    texp = 2.0 + 2.0 * rng.uniform(0.0, 1.0, n)
    texp = np.convolve(texp, np.ones(9) / 9.0, mode="same")
    texp[:4] = texp[4]
    texp[-4:] = texp[-5]
    return Continuum(v[0], 10.0, self_ref, for_ref, texp, 1013.0, 296.0)


def temperature(z_km):
    z = np.asarray(z_km, dtype=np.float64)
    t = np.where(z <= 11.0, 288.0 + (217.0 - 288.0) * z / 11.0,
                 np.where(z <= 50.0, 217.0 + (270.0 - 217.0) * (z - 11.0) / 39.0, 270.0))
    return t


def atmosphere(nlay, p_top, v1, v2, mols=SEVEN, p_sfc=1013.0, scale_height=7.0,
               other_vmr=OTHER_VMR, emis=0.98, dt_lev=None):
    """Layered nadir column, layer 0 at the surface; dt_lev [nlay+1] (K) is
    added to the level temperatures of the lapse profile."""
    k = np.arange(nlay + 1)
    p_lev = p_sfc * (p_top / p_sfc) ** (k / nlay)
    z_lev = -scale_height * np.log(p_lev / p_sfc)
    t_lev = temperature(z_lev)
    if dt_lev is not None:
        t_lev = t_lev + np.asarray(dt_lev, dtype=np.float64)
    pave = np.sqrt(p_lev[:-1] * p_lev[1:])
    tave = 0.5 * (t_lev[:-1] + t_lev[1:])
    zmid = 0.5 * (z_lev[:-1] + z_lev[1:])
    wair = (p_lev[:-1] - p_lev[1:]) * AIR_COLUMN_PER_HPA
    mols = np.asarray(mols, dtype=np.int32)
    w = np.zeros((nlay, len(mols)))
    for j, m in enumerate(mols):
        if m == 1:
            vmr = np.maximum(1.0e-2 * np.exp(-zmid / 2.0), 4.0e-6)
        else:
            vmr = np.full(nlay, other_vmr)
        w[:, j] = vmr * wair
    col = Column(mols, pave, tave, t_lev[:-1], t_lev[1:], w, wair, SECANT_DIFFUSE * wair,
                 v1, v2, t_lev[0], emis)
    col.p_lev = p_lev
    col.z_lev = z_lev
    col.q_h2o_lev = np.maximum(1.0e-2 * np.exp(-z_lev / 2.0), 4.0e-6)
    # volume mixing ratios of every absorber at the levels [nlay+1, nmol]
    col.vmr_lev = np.stack([col.q_h2o_lev if m == 1 else np.full(nlay + 1, other_vmr) for m in mols], axis=1)
    return col


# Boltzmann's constant in the units of level2layer's air density P/(T k)
# with P in mb (clblm_noScattJac.f90:1243-1244)
BOLTZ_MB = 1.3806503E-19


def level_density(p_lev, t_lev, vmr_lev):
    """Number density [molec/cm3] of an absorber at levels: vmr P/(k T), the
    level concentrations the reference's Jacobians take (viewPath%Q,
    densityOnPathLevel, clblm_AtmPath.f90:1278,1306-1313)."""
    return np.asarray(vmr_lev) * np.asarray(p_lev) / (np.asarray(t_lev) * BOLTZ_MB)


def jac_profile(col, jac_mol=1, do_temp=1):
    """Level pressures and H2O number densities of a column made by
    atmosphere(), as the Jacobian inputs (level 0 at the surface)."""
    from .capi_types import JacProfile
    t_lev = np.append(col.tbot, col.ttop[-1])
    return JacProfile(col.p_lev, level_density(col.p_lev, t_lev, col.q_h2o_lev), jac_mol=jac_mol, do_temp=do_temp)


# ---- the benchmark workloads --------------------------------------------

def config0():
    """One homogeneous layer, 20,000 H2O-like lines on 600-700 cm-1."""
    lines = line_list(20000, 600.0, 700.0, seed=0, mols=(1,))
    wabs = 1.0e22
    wtot = 2.479e24  # 1 km of air at 1013.25 hPa, 296 K (not given by the workload)
    col = Column(np.array([1], np.int32), [1013.25], [296.0], [296.0], [296.0],
                 np.array([[wabs]]), [wtot], [SECANT_DIFFUSE * wtot], 600.0, 700.0, 296.0, 1.0)
    return lines, col


def config1(n_lines=500000):
    """60 layers 1013->0.1 hPa, seven absorbers, 500,000 lines on 500-2500."""
    lines = line_list(n_lines, 500.0, 2500.0, seed=1, mols=SEVEN)
    col = atmosphere(60, 0.1, 500.0, 2500.0)
    return lines, col, continuum()


def config2():
    """config 1's atmosphere and lines over 600-1100 cm-1."""
    lines, col, cont = config1()
    return lines.window(600.0, 1100.0), col.with_window(600.0, 1100.0), cont


def config3(n_profiles=256, n_lines=500000):
    """Batched profiles: layer counts uniform on 20..100, level temperatures
    of the config 1 lapse profile plus N(0, 3 K), each with its own window of
    log-uniform width 10..1000 cm-1 inside 500-2500 cm-1, config 1's lines.
    Returns the lines, the continuum and lists of columns and Jacobian
    profiles (radiance + T and H2O Jacobians for each)."""
    lines, _, cont = config1(n_lines)
    rng = np.random.default_rng(3)
    cols, jacs = [], []
    for _ in range(n_profiles):
        nlay = int(rng.integers(20, 101))
        width = 10.0 ** rng.uniform(1.0, 3.0)
        v1 = float(np.round(rng.uniform(500.0, 2500.0 - width), 3))
        col = atmosphere(nlay, 0.1, v1, float(np.round(v1 + width, 3)), dt_lev=rng.normal(0.0, 3.0, nlay + 1))
        cols.append(col)
        jacs.append(jac_profile(col))
    return lines, cont, cols, jacs


def config4(n_lines=3000000):
    """100 layers 1013->0.01 hPa, 3,000,000 lines on 10-3500 cm-1."""
    lines = line_list(n_lines, 10.0, 3500.0, seed=4, mols=SEVEN)
    col = atmosphere(100, 0.01, 10.0, 3500.0)
    return lines, col, continuum()

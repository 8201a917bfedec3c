"""Layer optical depth on the GPU against the FP64 oracle (ODLAY_nonStruct)."""
import numpy as np
import pytest

from clblm_gb300 import capi_types as T
from clblm_gb300 import synth

pytestmark = pytest.mark.gpu


def _layer_case(n_lines, v1, v2, seed, mols=(1,), pave=1013.25, tave=296.0, wabs=1e22, wtot=2.479e24,
                isotopologues=False):
    lines = synth.line_list(n_lines, v1, v2, seed=seed, mols=mols, isotopologues=isotopologues)
    mol = np.array(mols, np.int32)
    w = np.full((1, len(mols)), wabs)
    col = T.Column(mol, [pave], [tave], [tave], [tave], w, [wtot], [1.67 * wtot], v1, v2, tave, 1.0)
    return lines, col


def _compare(gpu_lib, oracle_mod, lines, col, cont=None, contnm_off=1, precision=T.CLBLM_PREC_MIXED, xn2cn=1.0,
             **scales):
    dn, df, _ = gpu_lib.setDV(col)
    lay = col.layer(0)
    g = T.grid_struct(col.v1, col.v2, dn[0], df[0])
    ctrl = T.od_ctrl(precision=precision, contnm_off=contnm_off, xn2cn=xn2cn, **scales)
    h = gpu_lib.Handle(lines, cont)
    od, dv = h.odlay(lay, g, ctrl)
    st = h.stats()
    h.close()
    ref, dvr, sr = oracle_mod.Session().odlay(lines, lay, g, ctrl, cont)
    assert dv == dvr
    assert len(od) == len(ref)
    for k in ("nlin", "lincnt", "nminus", "nplus", "nshrunk", "npanels", "nsamp"):
        assert st[k] == sr[k], (k, st[k], sr[k])
    return od, ref


@pytest.mark.parametrize("precision,tol", [(T.CLBLM_PREC_MIXED, 1e-5), (T.CLBLM_PREC_PLAIN, 1e-9)])
def test_config0_full(gpu_lib, oracle_mod, precision, tol):
    lines, col = synth.config0()
    od, ref = _compare(gpu_lib, oracle_mod, lines, col, precision=precision)
    rel = np.max(np.abs(od - ref) / np.abs(ref))
    assert rel <= tol, rel


@pytest.mark.parametrize("precision,tol", [(T.CLBLM_PREC_MIXED, 1e-5), (T.CLBLM_PREC_PLAIN, 1e-9)])
def test_isotopologues_and_molecules_past_nine(gpu_lib, oracle_mod, precision, tol):
    """Lines of every isotopologue of H2O, CO2, O3 and O2 and of HNO3, OCS,
    N2 (foreign width from the air width), O, CH3OH and SO3 (Q = 1): each
    isotopologue's partition-sum ratio and Doppler mass"""
    mols = (1, 2, 3, 7, 12, 19, 22, 34, 39, 47)
    lines, col = _layer_case(30000, 600.0, 700.0, seed=11, mols=mols, pave=400.0, tave=240.0, wabs=1e17,
                             isotopologues=True)
    iso = (lines.mol // 100) % 10
    assert len(set(iso.tolist())) == 10  # isotopologues 1-9 and 10 (written as 0)
    od, ref = _compare(gpu_lib, oracle_mod, lines, col, precision=precision)
    rel = np.max(np.abs(od - ref) / np.abs(ref))
    assert rel <= tol, rel


def test_continuum_and_seven_absorbers(gpu_lib, oracle_mod):
    lines, col, cont = synth.config1(n_lines=20000)
    lines = lines.window(900.0, 1000.0)
    col = col.sub([5]).with_window(900.0, 1000.0)
    od, ref = _compare(gpu_lib, oracle_mod, lines, col, cont=cont, contnm_off=0)
    rel = np.max(np.abs(od - ref) / np.abs(ref))
    assert rel <= 1e-5, rel


@pytest.mark.parametrize("precision", [T.CLBLM_PREC_MIXED, T.CLBLM_PREC_PLAIN])
@pytest.mark.parametrize("v1,v2,contnm_off", [(1000.0, 1010.0, 1), (1000.0, 1010.0, 0), (720.0, 730.0, 1)])
def test_window_without_line_centres(gpu_lib, oracle_mod, precision, v1, v2, contnm_off):
    """A window that no line centre reaches: far from every line the OD is
    zero, or the continuum alone; 20-30 cm-1 past the last line only the far
    wings (BOUND4 = 25 cm-1) reach it"""
    lines, col = _layer_case(5000, 600.0, 700.0, seed=4, wabs=1e21)
    col = col.with_window(v1, v2)
    cont = synth.continuum() if contnm_off == 0 else None
    od, ref = _compare(gpu_lib, oracle_mod, lines, col, cont=cont, contnm_off=contnm_off, precision=precision)
    st_zero = v1 >= 1000.0 and contnm_off == 1
    if st_zero:
        assert np.all(od == 0.0) and np.all(ref == 0.0)
    else:
        assert np.max(np.abs(ref)) > 0.0
        tol = 1e-5 if precision == T.CLBLM_PREC_MIXED else 1e-9
        rel = np.max(np.abs(od - ref)) / np.max(np.abs(ref))
        assert rel <= tol, rel


@pytest.mark.parametrize("layer", [0, 30, 59])
def test_config1_layers_narrow_window(gpu_lib, oracle_mod, layer):
    lines, col, cont = synth.config1(n_lines=50000)
    col = col.sub([layer]).with_window(1000.0, 1040.0)
    od, ref = _compare(gpu_lib, oracle_mod, lines, col, cont=cont, contnm_off=0)
    rel = np.max(np.abs(od - ref) / np.abs(ref))
    assert rel <= 1e-5, rel


@pytest.mark.parametrize("precision,tol", [(T.CLBLM_PREC_MIXED, 1e-5), (T.CLBLM_PREC_PLAIN, 1e-9)])
@pytest.mark.parametrize("layer", [0, 12])
def test_reference_mtckd_table(gpu_lib, oracle_mod, mtckd, precision, tol, layer):
    """The H2O continuum from the reference's own MT_CKD table (golden fixture)
    on a water-rich lower layer, 1300-1400 cm-1 (the 6.3 um band wing).  A
    sparse line list (500 lines on 500-2500 cm-1) leaves the continuum up to
    99 % of the layer OD between lines."""
    lines, col, _ = synth.config1(n_lines=500)
    col = col.sub([layer]).with_window(1300.0, 1400.0)
    od, ref = _compare(gpu_lib, oracle_mod, lines, col, cont=mtckd, contnm_off=0, precision=precision)
    rel = np.max(np.abs(od - ref) / np.abs(ref))
    assert rel <= tol, rel


@pytest.mark.parametrize("precision,tol", [(T.CLBLM_PREC_MIXED, 1e-5), (T.CLBLM_PREC_PLAIN, 1e-9)])
@pytest.mark.parametrize("window", [(150.0, 250.0), (2050.0, 2150.0)])
def test_n2_continua(gpu_lib, oracle_mod, precision, tol, window):
    """The N2 collision-induced continua (pure rotation below 350 cm-1, the
    fundamental at 2000-2900 cm-1) on a water-rich lower layer of the
    broadband atmosphere with a sparse line list, against the oracle (there
    the N2 part reaches 13 % and 2e-5 of the OD); on the FP64 path also the
    N2 part itself (XN2CN = 1 minus XN2CN = 0) against the oracle's."""
    lines, col, cont = synth.config4(n_lines=3000)
    col = col.sub([2]).with_window(*window)
    od1, ref1 = _compare(gpu_lib, oracle_mod, lines, col, cont=cont, contnm_off=0, precision=precision)
    rel = np.max(np.abs(od1 - ref1) / np.abs(ref1))
    assert rel <= tol, rel
    if precision == T.CLBLM_PREC_PLAIN:
        od0, ref0 = _compare(gpu_lib, oracle_mod, lines, col, cont=cont, contnm_off=0, precision=precision,
                             xn2cn=0.0)
        dref = ref1 - ref0
        assert np.max(dref) > 0.0
        err = np.max(np.abs((od1 - od0) - dref)) / np.max(dref)
        assert err <= 1e-6, err


def _o2_atmosphere():
    """The broadband atmosphere's levels with H2O, CO2, O3 and O2 at 0.21."""
    col = synth.atmosphere(100, 0.01, 10.0, 3500.0, mols=(1, 2, 3, 7))
    col.w[:, 3] *= 0.21 / synth.OTHER_VMR
    return col


@pytest.mark.parametrize("precision,tol", [(T.CLBLM_PREC_MIXED, 1e-5), (T.CLBLM_PREC_PLAIN, 1e-9)])
@pytest.mark.parametrize("window,what", [
    ((1400.0, 1500.0), "xo2cn"),      # O2 collision-induced fundamental
    ((7600.0, 7700.0), "xo2cn"),      # O2 1.27 um
    ((9300.0, 9400.0), "xo2cn"),      # O2 1.06 um (and the O3 Chappuis band)
    ((13000.0, 13100.0), "xo2cn"),    # O2 A band, over pre_xint's range
    ((20000.0, 20100.0), "xo3cn"),    # O3 Chappuis (and the O2 visible)
    ((27300.0, 27450.0), "xo3cn"),    # O3 Hartley-Huggins from its first point
    ((40700.0, 40900.0), "xo3cn"),    # Hartley-Huggins handing over to the UV at 40800 cm-1
    ((38000.0, 38100.0), "xo2cn"),    # O2 Herzberg
    ((57000.0, 57100.0), "xo2cn"),    # O2 far UV, over pre_xint's range
    ((2500.0, 2600.0), "xrayl"),      # Rayleigh extinction
])
def test_o3_o2_rayleigh_continua(gpu_lib, oracle_mod, precision, tol, window, what):
    """The O3 and O2 continua and Rayleigh extinction of CONTNM on a lower
    layer of the broadband atmosphere with O2 at 0.21, in windows where each
    band lives, against the oracle; on the FP64 path also that continuum
    alone (scale 1 minus scale 0) against the oracle's, which pins it where
    lines or other continua would hide it."""
    lines, _, cont = synth.config4(n_lines=3000)
    col = _o2_atmosphere().sub([2]).with_window(*window)
    od1, ref1 = _compare(gpu_lib, oracle_mod, lines, col, cont=cont, contnm_off=0, precision=precision)
    rel = np.max(np.abs(od1 - ref1) / np.abs(ref1))
    assert rel <= tol, rel
    if precision == T.CLBLM_PREC_PLAIN:  # the part alone: below the mixed path's FP32 noise at line centres
        od0, ref0 = _compare(gpu_lib, oracle_mod, lines, col, cont=cont, contnm_off=0, precision=precision,
                             **{what: 0.0})
        dref = ref1 - ref0
        assert np.max(np.abs(dref)) > 0.0
        # to 1e-6 of the part, or to binary64 rounding of the whole OD where
        # the part is that small (Rayleigh: 3e-6 beside line centres of 1e7)
        err = np.max(np.abs((od1 - od0) - dref))
        assert err <= max(1e-6 * np.max(np.abs(dref)), 1e-13 * np.max(np.abs(ref1))), err


def test_od_from_tape3_file_is_identical(gpu_lib, tmp_path):
    """Lines written as an LNFL TAPE3 file and read back by the library give
    the same OD bit for bit."""
    from clblm_gb300 import tape3
    lines, col = _layer_case(6000, 600.0, 640.0, seed=21)
    p = tmp_path / "TAPE3"
    tape3.write_tape3(p, lines)
    back = gpu_lib.read_tape3(p)
    dn, df, _ = gpu_lib.setDV(col)
    g = T.grid_struct(col.v1, col.v2, dn[0], df[0])
    ctrl = T.od_ctrl(precision=T.CLBLM_PREC_MIXED, contnm_off=1)
    h1, h2 = gpu_lib.Handle(lines), gpu_lib.Handle(back)
    a, _ = h1.odlay(col.layer(0), g, ctrl)
    b, _ = h2.odlay(col.layer(0), g, ctrl)
    h1.close()
    h2.close()
    assert np.array_equal(a, b)


def _selection(gpu_lib, oracle_mod, lines, col, cont, precision, contnm_off=0):
    """OD, the per-line panel of every line of the layer's window and the
    far-wing pseudo-lines, from the library and the oracle."""
    dn, df, _ = gpu_lib.setDV(col)
    lay = col.layer(0)
    g = T.grid_struct(col.v1, col.v2, dn[0], df[0])
    ctrl = T.od_ctrl(precision=precision, contnm_off=contnm_off)
    h = gpu_lib.Handle(lines, cont)
    try:
        od, dv = h.odlay(lay, g, ctrl)
        sel = h.od_lines()
    finally:
        h.close()
    ref, dvr, sr, tr = oracle_mod.Session().odlay_trace(lines, lay, g, ctrl, cont)
    return od, ref, sel, tr, sr


@pytest.mark.parametrize("precision", [T.CLBLM_PREC_MIXED, T.CLBLM_PREC_PLAIN])
@pytest.mark.parametrize("case", ["config0", "config1_top", "config1_surface", "config4_lowest"])
def test_line_selection_bit_exact(gpu_lib, oracle_mod, case, precision):
    """Line selection and panel index ranges equal the reference's bookkeeping
    line by line: every line of the window is convolved in the same panel (or
    rejected by both), so each panel's line range is the same; SHRINQ merges
    the same lines into the same far-wing pseudo-lines in the same order
    (the last line of every group is the same line).  Their values: FP64
    path to 1e-14 (the device exp and the C library's may differ in the last
    bit); mixed path, whose strengths are FP32 (relative error below 2e-6):
    centres, the strength-weighted means of a group no wider than DVR4/2,
    within 2e-6 DVR4, strengths and widths within 2e-6."""
    if case == "config0":
        lines, col = synth.config0()
        cont = None
        contnm_off = 1
    elif case.startswith("config1"):
        lines, col, cont = synth.config1(n_lines=100000)
        col = col.sub([59 if case.endswith("top") else 0]).with_window(1000.0, 1100.0)
        contnm_off = 0
    else:  # the lowest layer of the broadband column at 10-60 cm-1: far-wing mirror lines
        lines, col, cont = synth.config4(n_lines=300000)
        col = col.sub([0]).with_window(10.0, 60.0)
        contnm_off = 0
    od, ref, sel, tr, sr = _selection(gpu_lib, oracle_mod, lines, col, cont, precision, contnm_off)
    lo, lp = sel["line_lo"], sel["line_panel"]
    want = tr["line_panel"]
    assert np.array_equal(lp, want[lo:lo + len(lp)])
    assert np.all(want[:lo] == -1) and np.all(want[lo + len(lp):] == -1)
    assert (lp >= 0).sum() == sr["lincnt"]
    # per-panel line ranges follow: first and last line of each panel
    for q in range(int(sr["npanels"])):
        idx = np.nonzero(lp == q)[0]
        widx = np.nonzero(want == q)[0]
        assert len(idx) == len(widx)
        if len(idx):
            assert idx[0] + lo == widx[0] and idx[-1] + lo == widx[-1]
    assert len(sel["shr_vnu"]) == len(tr["shr_vnu"]) == sr["nshrunk"]
    assert np.array_equal(sel["shr_mol"], tr["shr_mol"])
    # the same lines merge: each pseudo-line's group ends at the same line
    bad = np.nonzero(sel["shr_last"] != tr["shr_last"])[0]
    assert len(bad) == 0, (len(bad), bad[:5], sel["shr_last"][bad[:5]], tr["shr_last"][bad[:5]])
    if precision == T.CLBLM_PREC_PLAIN:
        for k in ("shr_vnu", "shr_sp", "shr_alfl", "shr_alfd"):
            np.testing.assert_allclose(sel[k], tr[k], rtol=1e-14, atol=0, err_msg=k)
    else:
        np.testing.assert_allclose(sel["shr_vnu"], tr["shr_vnu"], rtol=0, atol=2e-6 * sr["dvr4"])
        for k in ("shr_sp", "shr_alfl", "shr_alfd"):
            np.testing.assert_allclose(sel[k], tr[k], rtol=2e-6, atol=0, err_msg=k)
    tol = 1e-9 if precision == T.CLBLM_PREC_PLAIN else 1e-5
    assert np.max(np.abs(od - ref) / np.abs(ref)) <= tol


def _coupled(lines, every, seed):
    """every `every`-th line coupled: IFLG 1 with Y and G of either sign
    and size, every fifth of them IFLG 3 (reduced widths)"""
    rng = np.random.default_rng(seed)
    idx = np.arange(3, lines.n, every)
    m = len(idx)
    iflg = np.where(np.arange(m) % 5 == 4, 3, 1)
    t4 = np.array(synth.TEMPLC)
    y = rng.uniform(-0.05, 0.05, (m, 1)) * (1.0 + 0.3 * (296.0 - t4) / 100.0)
    g = rng.uniform(-0.01, 0.01, (m, 1)) * (1.0 + 0.2 * (296.0 - t4) / 100.0)
    return synth.with_coupling(lines, idx, iflg=iflg, a=np.abs(y) * (iflg[:, None] == 3) + y * (iflg[:, None] == 1),
                               b=np.abs(g) * (iflg[:, None] == 3) + g * (iflg[:, None] == 1))


@pytest.mark.parametrize("precision,tol", [(T.CLBLM_PREC_MIXED, 1e-5), (T.CLBLM_PREC_PLAIN, 1e-9)])
@pytest.mark.parametrize("tave", [215.0, 288.0])
def test_line_coupling(gpu_lib, oracle_mod, precision, tol, tave):
    """Coupled H2O and CO2 lines (each followed by its coefficient record):
    the dispersion term on the three line-centre grids, G and the reduced
    widths, coupled far-wing lines kept out of SHRINQ's groups and their
    dispersion term in CNVF4Q, lines outside the window through the wings"""
    lines = _coupled(synth.line_list(20000, 550.0, 750.0, seed=5, mols=(1, 2)), 13, seed=6)
    col = T.Column(np.array([1, 2], np.int32), [400.0], [tave], [tave], [tave], np.array([[3e17, 3e17]]), [2.479e24],
                   [1.67 * 2.479e24], 600.0, 700.0, tave, 1.0)
    od, ref = _compare(gpu_lib, oracle_mod, lines, col, precision=precision)
    rel = np.max(np.abs(od - ref) / np.abs(ref))
    assert rel <= tol, rel


@pytest.mark.parametrize("precision,tol", [(T.CLBLM_PREC_MIXED, 1e-5), (T.CLBLM_PREC_PLAIN, 1e-9)])
def test_line_coupling_near_zero(gpu_lib, oracle_mod, precision, tol):
    """Coupled O2-like lines from 0.02 cm-1 in a window starting near zero:
    the dispersion term in the folded first panel (RSYM) and in the far
    wings' Van Vleck-Weisskopf mirror records (SPP negated)"""
    lines = _coupled(synth.line_list(3000, 0.02, 90.0, seed=10, mols=(7,), isotopologues=True), 7, seed=11)
    col = T.Column(np.array([7], np.int32), [1013.25], [296.0], [296.0], [296.0], np.array([[5e18]]), [2.479e24],
                   [1.67 * 2.479e24], 0.0005, 60.0, 296.0, 1.0)
    od, ref = _compare(gpu_lib, oracle_mod, lines, col, precision=precision)
    rel = np.max(np.abs(od - ref) / np.abs(ref))
    assert rel <= tol, rel


@pytest.mark.parametrize("precision,tol", [(T.CLBLM_PREC_MIXED, 1e-5), (T.CLBLM_PREC_PLAIN, 1e-9)])
@pytest.mark.parametrize("v2", [12.0, 60.0])
def test_window_starting_at_zero_rsym(gpu_lib, oracle_mod, precision, tol, v2):
    """A window starting at 0.0005 cm-1: the first panel's origin
    VFT = V1 - 32 DV lies below zero, where HIRACQ folds the panel's line
    sums about zero (RSYM, clblm_ODLAY.f90:3020-3085); one panel (v2 = 12)
    and three (v2 = 60), lines from 0.02 cm-1, the MT_CKD-style continuum."""
    lines = synth.line_list(6000, 0.02, 90.0, seed=9, mols=(1,))
    cont = synth.continuum()
    col = T.Column(np.array([1], np.int32), [1013.25], [296.0], [296.0], [296.0], np.array([[1e22]]), [2.479e24],
                   [1.67 * 2.479e24], 0.0005, v2, 296.0, 1.0)
    od, ref = _compare(gpu_lib, oracle_mod, lines, col, cont=cont, contnm_off=0, precision=precision)
    rel = np.max(np.abs(od - ref) / np.abs(ref))
    assert rel <= tol, rel

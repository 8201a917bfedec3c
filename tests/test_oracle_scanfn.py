"""The oracle's clblm_SCANFN restatement pinned by properties (the reference
ships no test of the scan), and the library's host plan of the scan's grid
against it (no device needed)."""
import numpy as np
import pytest

from clblm_gb300 import capi_types as T


def _flat(v1=1000.0, dv=0.001, n=30000, level=2.5):
    return np.full(n, level), v1, dv


@pytest.mark.parametrize("fid,hw,dvout", [(1, 0.05, 0.01), (2, 0.05, 0.01), (3, 0.05, 0.01), (3, 0.3, 0.05),
                                          (2, 0.1, 0.02)])
def test_constant_stays_constant(oracle_mod, fid, hw, dvout):
    """The rectangle and the triangle integrate to one at their sampling, so
    a constant spectrum is kept to rounding; the Gaussian's table ends at
    4 HWHM, which loses 2.5e-6 of its area."""
    x, v1, dv = _flat()
    out, v1o, dvo = oracle_mod.scanfn(x, v1, dv, fid, hw, 1005.0, 1020.0, dvout)
    assert v1o == 1005.0
    np.testing.assert_allclose(out, 2.5 * (1 - 2.48e-6 if fid == 3 else 1.0), rtol=1e-8 if fid == 3 else 1e-14)


def test_narrow_line_gives_the_gaussian(oracle_mod):
    """A line one input point wide (no shrink: HWHM/12 is one input spacing)
    scans to the tabulated Gaussian of unit area: the scan's samples sum to
    the line's area over DVout, and peak where the line is."""
    v1, dv, n = 1000.0, 0.001, 20001
    x = np.zeros(n)
    k = 10000
    x[k] = 1.0
    out, v1o, dvo = oracle_mod.scanfn(x, v1, dv, 3, 0.012, 1009.0, 1011.0, 0.001)
    v = v1o + dvo * np.arange(len(out))
    assert abs(v[np.argmax(out)] - (v1 + k * dv)) < 1e-9
    assert abs(out.sum() * dvo - dv) < 1e-3 * dv
    xf = oracle_mod.sf_table(2)
    assert out.max() == pytest.approx(dv / 0.012 * xf[1], rel=1e-12)


def test_interp_keeps_a_linear_spectrum(oracle_mod):
    """clblm_INTERP's four-point scheme reproduces a straight line up to its
    tabulated coefficients: P is taken as INT(201 P)/200, at most 1/100 of an
    input step away, so the error stays within slope * DV / 100."""
    v1, dv, n = 500.0, 0.01, 5000
    x = 3.0 + 0.2 * (np.arange(n) * dv)
    out = oracle_mod.sf_interp(x, v1, dv, v1 + 1.0, v1 + 40.0, 0.0013)
    v = v1 + 1.0 + 0.0013 * np.arange(len(out))
    np.testing.assert_allclose(out, 3.0 + 0.2 * (v - v1), rtol=0, atol=0.2 * dv / 100)


def test_plan_grid_matches_oracle(oracle_mod):
    """The library's host plan (clblm_gpu_scanfn_size) gives the oracle's
    V1out, DVout and point count, and its errors, over functions, widths,
    spacings, ranges and inputs finer and coarser than HWHM/12."""
    from clblm_gb300 import capi
    rng = np.random.default_rng(1)
    n_cases = 0
    for fid in (1, 2, 3, 4, 5, -4, -5, 0, 6, -2):
        for (v1, dv, n) in [(1000.0, 0.001, 30000), (10.0, 0.02, 4000), (1000.0, 0.01, 9000)]:
            for hw in (0.01, 0.05, 0.2):
                for dvout in (0.0, 0.004, 0.05):
                    v2s = v1 + dv * (n - 1)
                    for (a, b) in [(v1 + 0.1 * (v2s - v1), v1 + 0.8 * (v2s - v1)), (v1 + 0.3 * (v2s - v1), v2s)]:
                        sp = rng.random(n)
                        try:
                            ref = oracle_mod.scanfn(sp, v1, dv, fid, hw, a, b, dvout)
                        except oracle_mod.OracleError:
                            ref = None
                        try:
                            got = capi.scanfn_size(T.scanfn_struct(fid, hw, a, b, dvout), v1, dv, n)
                        except capi.ClblmError:
                            got = None
                        assert (ref is None) == (got is None), (fid, v1, dv, hw, dvout, a, b)
                        if ref is not None:
                            assert (len(ref[0]), ref[1], ref[2]) == (got[2], got[0], got[1])
                        n_cases += 1
    assert n_cases == 540


def test_filter_keeps_a_constant_and_a_line(oracle_mod):
    """FLTRFN over a smooth filter keeps a constant and a straight line
    through the filter's centre to 2e-5 (its trapezoid edges and the
    reference's one-point shift of the spectrum's grid against the
    filter's)."""
    v1, dv, n = 900.0, 0.001, 200001
    v = v1 + dv * np.arange(n)
    g = np.exp(-np.linspace(-3, 3, 61) ** 2)
    assert oracle_mod.fltrfn(np.full(n, 3.0), v1, dv, 1000.0, -0.1, g) == pytest.approx(3.0, rel=2e-5)
    assert oracle_mod.fltrfn(1 + (v - 1000) / 100, v1, dv, 1000.0, -0.1, g) == pytest.approx(1.0, rel=2e-5)


def test_filter_stops_where_the_reference_does(oracle_mod):
    """A filter whose last point falls exactly on the first point of a
    2400-point input panel leaves CNVFLT no point to keep in that panel: the
    reference stops (subscript beyond XF); so do the oracle and the library."""
    from clblm_gb300 import capi
    v1, dv, n = 900.0, 0.001, 200001
    with pytest.raises(oracle_mod.OracleError):
        oracle_mod.fltrfn(np.full(n, 3.0), v1, dv, 950.0, 0.5, np.ones(21))
    with pytest.raises(oracle_mod.OracleError):
        oracle_mod.fltrfn(np.full(n, 3.0), v1, dv, 950.0, -0.5, np.ones(20))  # even count about a centre

"""The oracle's O3, O2 and Rayleigh blocks of CONTNM pinned by their closed
forms and the reference's hand-over rules (no device needed)."""
import numpy as np

from oracle import oracle as O


def test_rayleigh_closed_form():
    """ray_ext = x^3/(938.076 - 10.8426 x^2) * Wtot * 1e-20/2.68675e4 with
    x = v/1e4, times x with the radiation term (JRAD = 1), over 1e4 without
    (JRAD = 0) (clblm_ODLAY_Continuum.f90:1040-1056)."""
    v1abs, n, wtot = 997.0, 1500, 2.1e24
    v = v1abs + np.arange(n)
    x = v / 1e4
    base = (x ** 3 / (9.38076e2 - 10.8426 * x ** 2)) * (wtot * 1e-20 / (2.68675e-1 * 1e5))
    for jrad, want in ((1, base * x), (0, base / 1e4)):
        a = O.contnm_o3o2(jrad, v1abs, 1.0, n, 1000.0, 2500.0, 500.0, 250.0, wtot, 0.0, 0.0, 0.0, xo3cn=0.0,
                          xo2cn=0.0)
        np.testing.assert_allclose(a[1:n + 1], want, rtol=1e-13)
    # below 820 cm-1 at V2: none
    a = O.contnm_o3o2(1, 97.0, 1.0, 500, 100.0, 600.0, 500.0, 250.0, wtot, 0.0, 0.0, 0.0)
    assert not np.any(a)


def test_hartley_huggins_hands_over_at_40800():
    """Below 40800 cm-1 the Hartley-Huggins band alone, from 40800 on the UV
    table alone: the reference saves and restores ABSRB on either side, so a
    window across 40800 equals, point for point, a window below it (no UV)
    and one above it (no Hartley-Huggins)."""
    kw = dict(xo2cn=0.0, xrayl=0.0)
    args = (500.0, 250.0, 2e24, 0.0, 1e18, 0.0)
    v1abs, n = 40597.0, 400
    both = O.contnm_o3o2(0, v1abs, 1.0, n, 40600.0, 40990.0, *args, **kw)[1:n + 1]
    ifix = int((40800.0 - v1abs) / 1.0 + 1.001)  # the first point the UV part keeps (1-based)
    lo = O.contnm_o3o2(0, v1abs, 1.0, 190, 40600.0, 40780.0, *args, **kw)[1:191]
    np.testing.assert_array_equal(both[:150], lo[:150])
    hi_v1abs = 40797.0
    hi = O.contnm_o3o2(0, hi_v1abs, 1.0, 200, 40801.0, 40990.0, *args, **kw)[1:201]
    k0 = ifix - 1 + 3  # a few points past the hand-over
    np.testing.assert_array_equal(both[k0:k0 + 150], hi[(k0 - int(hi_v1abs - v1abs)):(k0 - int(hi_v1abs - v1abs)) + 150])
    assert np.all(both > 0)


def test_o2_scales_linearly_with_xo2cn():
    v1abs, n = 1297.0, 600
    a1 = O.contnm_o3o2(1, v1abs, 1.0, n, 1300.0, 1890.0, 700.0, 260.0, 1.5e24, 1e21, 0.0, 3.1e23, xrayl=0.0)
    a2 = O.contnm_o3o2(1, v1abs, 1.0, n, 1300.0, 1890.0, 700.0, 260.0, 1.5e24, 1e21, 0.0, 3.1e23, xo2cn=2.0,
                       xrayl=0.0)
    assert np.max(a1) > 0
    np.testing.assert_allclose(a2, 2 * a1, rtol=1e-14, atol=0)

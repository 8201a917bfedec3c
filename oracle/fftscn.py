"""FP64 restatement of CLBLM's FFT instrument-function scan (clblm_FFTSCN,
src/clblm_src/clblm_FFT.f90), numpy.

TEST INFRASTRUCTURE ONLY: the checker of the GPU scan.  PARITY UNPINNED by
the reference's own tests (it has none); pinned instead by properties: a
constant spectrum stays constant, the scan of one narrow line is the
instrument line shape of the requested half width.

The reference keeps the spectrum in 65536-point records (LPTSMX) and,
since the padding was raised fourfold (clblm_FFT.f90:1173-1186), always
takes its disk-based FFT (REALBG/BIGFFT, :2605-2736).  Its transform pair
is normalised (the inverse is divided by the record count in BIGFFT and by
the record size inside), so the scan is the circular convolution of the
FILL-padded spectrum with the unit-area scanning function.  Any correct FFT
gives the same values up to rounding; numpy's is used here.

Covered: functID 1 (boxcar only), 2..11 and 14 (triangle, Gaussian,
sinc**2, sinc, Beer, Hamming, Hanning, Norton-Beer weak/medium/strong,
Kiruna) with the apodization computed analytically (IVX = 1: (V2Z-V1Z)/HWHM
> CRATIO) or as the transform of the sampled scanning function (IVX = -1,
Scntrn :2097-2163), optional pre-boxing with deconvolution, the
deconvolution of an external pre-boxing (functID 102..114) or alone
(functID -1), the interpolation of a spectrum coarser than 2*HWHM/12 before
the scan and onto DVOUT after it (Intpdr :2392-2443, clblm_INTERP through
the C oracle).  As in the reference, Brault and Kaiser-Bessel (functID 12,
13) stop for want of an optical path difference, and the Norton-Beer
functions have no spectral-domain form (IVX = -1 stops).
"""
import math

import numpy as np

LPTSMX = 65536  # clblm_FFT.f90:91

# scanning-function constants, clblm_FFT.f90:108-131 (index JFN = functID-1)
C = [0.0, 2.0, 0.849322, 2.257609, 3.314800, 2.100669, 2.195676, 2.0, 2.570274, 2.367714, 2.071759,
     -3.3, -2.5, 3.314800]
CRATIO = [0.0, 40., 10., 40., 160., 20., 20., 20., 40., 40., 20., 100., 10., float(np.finfo(np.float64).max)]
CLIMIT = [1., 2., 3., 40., 160., 20., 20., 20., 40., 40., 20., 100., 10., 160.]
ARGMIN = 34.0  # src/common/clblm_ConstParam.f90:51
MDVHW = 12     # clblm_FFT.f90:415


class ScanError(ValueError):
    pass


def records(ltotal):
    """Records of LPTSMX points for LTOTAL points, padded fourfold to a power
    of two (LoadSpect, clblm_FFT.f90:1160-1186; Boxcar, :902-925)."""
    ardata = float(ltotal) / float(LPTSMX)
    lrdata = int(ardata) if ardata - int(ardata) == 0.0 else int(ardata + 1.0)
    power = math.log(float(lrdata)) / math.log(2.0)
    return 2 ** (int(power) + 2) if power - int(power) == 0 else 2 ** (int(power) + 3)


def apodization(jfn, A, dv, nrec, deconv_a=None):
    """The apodization function on the complex points k = 0 .. N/2 of the
    N = nrec * LPTSMX point transform (Scntrn with IVX = 1, :2170-2185, and
    Scnfnt, :1445-1990): x = k * DX, DX = 1/(N*DV), accumulated per record
    as the reference does; the Nyquist point is 0 (the imaginary slot of the
    first packed element).  With deconv_a, the boxcar deconvolution factor
    Z/sin(Z), Z = 2 pi x deconv_a (Scnfnt function -1, :1935-1958), follows."""
    lpts = LPTSMX
    n = nrec * lpts
    half = lpts // 2
    DX = 1.0 / (float(lpts * nrec) * dv)
    PI = 2.0 * math.asin(1.0)
    H = np.zeros(n // 2 + 1)
    D = np.ones(n // 2 + 1) if deconv_a is not None else None
    kk = np.arange(half, dtype=np.float64)
    X0 = 0.0
    for j in range(nrec):
        x = X0 + kk * DX  # X = X0 + (L+1)*DX/2: round((L+1)*DX)/2 = round(k*DX)
        sl = slice(j * half, (j + 1) * half)
        if jfn == 0:    # no scanning function (the deconvolution alone)
            h = np.ones_like(x)
        elif jfn == 1:    # triangle: sinc**2
            z = PI * x * A
            with np.errstate(invalid="ignore", divide="ignore"):
                h = np.where(x == 0, 1.0, (np.sin(z) / z) ** 2)
        elif jfn == 2:  # Gaussian
            h = np.exp(-np.minimum(2.0 * (PI * x * A) ** 2, ARGMIN))
        elif jfn == 3:  # sinc**2: triangle
            h = np.where(x < 1.0 / A, 1.0 - x * A, 0.0)
        elif jfn == 4:  # sinc: rectangle with an interpolated end point
            alen = 1.0 / A
            h = np.where(x < alen, 1.0, 0.0)
            xstart = X0
            nn = int((alen - xstart) / DX) + 1
            r = (alen - xstart) / DX + 1 - nn
            if r <= 0.5:
                r = r + 1.0
                nn = nn - 1
            if 1 <= nn <= lpts // 2 - 1:
                h[nn] = r - 0.5
        elif jfn == 5:  # Beer
            h = np.where(x < 1.0 / A, (1.0 - (x * A) ** 2) ** 2, 0.0)
        elif jfn == 6:  # Hamming
            h = np.where(x < 1.0 / A, 0.53835685 * (1.0 + 0.857504 * np.cos(PI * x * A)), 0.0)
        elif jfn == 7:  # Hanning
            h = np.where(x < 1.0 / A, 0.5 * (1.0 + np.cos(PI * x * A)), 0.0)
        elif jfn in (8, 9, 10):  # Norton-Beer weak, medium, strong (:1774-1813)
            u = 1.0 - (x * A) ** 2
            if jfn == 8:
                f = 0.384093 - 0.087577 * u + 0.703484 * u ** 2
            elif jfn == 9:
                f = 0.152442 - 0.136176 * u + 0.983734 * u ** 2
            else:
                f = 0.045355 + 0.554883 * u ** 2 + 0.399782 * u ** 4
            h = np.where(x < 1.0 / A, f, 0.0)
        else:
            raise ScanError("scanning function %d is not covered" % jfn)
        H[sl] = h
        if D is not None:
            z = 2.0 * PI * x * deconv_a
            with np.errstate(invalid="ignore", divide="ignore"):
                D[sl] = np.where(z != 0, z / np.sin(z), 1.0)
        X0 = X0 + (lpts - 1 + 1) * DX / 2.0
    H[n // 2] = 0.0
    if D is not None:
        D[n // 2] = 0.0
    return H, D


def scanning_function(jfn, A, x, parms=(0.0, 0.0, 0.0)):
    """The scanning function of JFN at wavenumber offsets x (Scnfnt with
    IAPSC = -1, :1499-1921): triangle, Gaussian, sinc**2, sinc, Beer,
    Hamming, Hanning, Kiruna."""
    PI = 2.0 * math.asin(1.0)
    x = np.asarray(x, dtype=np.float64)
    with np.errstate(invalid="ignore", divide="ignore"):
        if jfn == 1:
            return np.where(x > A, 0.0, 1.0 - x / A)
        if jfn == 2:
            return np.exp(-np.minimum(0.5 * (x / A) ** 2, ARGMIN))
        if jfn == 3:
            z = PI * x / A
            return np.where(x != 0, (np.sin(z) / z) ** 2, 1.0)
        if jfn == 4:
            z = 2.0 * PI * x / A
            return np.where(x != 0, np.sin(z) / z, 1.0)
        if jfn == 5:
            u = 2.0 * PI * x / A
            return np.where(u >= 0.5, 15. * ((3.0 - u ** 2) * np.sin(u) - 3.0 * u * np.cos(u)) / (u ** 5),
                            1.0 - 15.0 / 210 * u ** 2)
        if jfn in (6, 7):
            c = 0.428752 if jfn == 6 else 0.5
            u = 2.0 * PI * x / A
            f = np.sin(u) / u + c * (np.sin(u + PI) / (u + PI) + np.sin(u - PI) / (u - PI))
            f = np.where(u == 0, 1.0, f)
            return np.where(np.abs(u) == PI, c, f)
        if jfn == 13:
            u1 = 2.0 * PI * x / A
            u2 = 2.0 * PI * (x - parms[0]) / A
            f1 = np.where(u1 == 0.0, 1.0, np.sin(u1) / u1)
            f2 = np.where(u2 == 0.0, 1.0, np.sin(u2) / u2)
            return parms[1] * f1 + parms[2] * f2
    raise ScanError("scanning function %d has no spectral-domain form" % jfn)


def numeric_apodization(jfn, A, dv, nrec, parms=(0.0, 0.0, 0.0)):
    """IVX = -1 (Scntrn :2097-2163): the scanning function sampled at DV in
    the transform's circular layout, transformed, over its first coefficient
    (its area).  The symmetric functions hold f(g DV) at g < N/2 and
    f((N-g) DV) above; the asymmetric Kiruna function's negative blocks are
    written as the reference writes them, from X = VSAVE + DV downwards and
    reversed: block J (of 65536 points, counted from the end) holds
    f(((2J-2)*65536 - (N-g) + 2) DV)."""
    lpts = LPTSMX
    n = nrec * lpts
    g = np.arange(n, dtype=np.int64)
    if jfn == 13:
        ng = n - g
        J = (ng + lpts - 1) // lpts
        xneg = ((2 * J - 2) * lpts - ng + 2).astype(np.float64) * dv
        x = np.where(g < n // 2, g.astype(np.float64) * dv, xneg)
    else:
        x = np.minimum(g, n - g).astype(np.float64) * dv
    F = np.fft.rfft(scanning_function(jfn, A, x, parms))
    return F / F[0].real


def intpdr(spect, v1c, dv, vv1, vv2, dvv):
    """Intpdr (:2392-2443): the requested limits pulled inside the data by
    whole steps, then clblm_INTERP onto vv1 + j*dvv.  Returns (spectrum, V1)."""
    from oracle import oracle as O
    v2c = v1c + dv * (len(spect) - 1)
    if vv1 < v1c:
        an = (v1c - vv1) / dvv
        vv1 = vv1 + dvv * int(an) if an == int(an) else vv1 + dvv * (int(an) + 1)
    if vv2 > v2c:
        an = (vv2 - v2c) / dvv
        vv2 = vv2 - dvv * int(an) if an == int(an) else vv2 - dvv * (int(an) + 1)
    return O.sf_interp(spect, v1c, dv, vv1, vv2, dvv), vv1


def fftscn(spect, v1c, dv, funct_id, hwhm, v1out, v2out, fill=0.0, prebox_hw=-1.0, deconv_prebox=False,
           dvout=0.0, parms=(0.0, 0.0, 0.0)):
    """clblm_FFTSCN_struct (:352-844) for the cases above.  Returns
    (scanned spectrum, V1S, DV) on the scan grid."""
    spect = np.asarray(spect, dtype=np.float64)
    np_in = len(spect)
    v2c = v1c + dv * (np_in - 1)
    if not (0.0 <= fill <= 1.0):
        raise ScanError("FILL out of range")
    if not (1 <= funct_id <= 14 or 102 <= funct_id <= 114 or funct_id == -1):
        raise ScanError("functID must be in [1,14] or [102,114], or -1")
    jfn = funct_id - 1
    deconv_only = False
    deconv_hw = None
    if jfn == 0:
        do_prebox, do_deconv, boxcar_hw = True, False, hwhm
    elif 1 <= jfn <= 13:
        if prebox_hw <= 0.0:
            do_prebox, do_deconv, boxcar_hw = False, False, 0.0
        else:
            do_prebox, do_deconv, boxcar_hw = True, bool(deconv_prebox), prebox_hw
    elif 101 <= jfn <= 113:  # pre-boxed outside: the scan and the deconvolution
        jfn -= 100
        do_prebox, do_deconv, boxcar_hw, deconv_hw = False, True, 0.0, prebox_hw
    else:  # -1: the deconvolution alone
        deconv_only = True
        jfn = 0
        do_prebox, do_deconv, boxcar_hw, deconv_hw = False, True, 0.0, prebox_hw
    if jfn > 0:
        if C[jfn] <= 0:
            raise ScanError("scanning function needs an optical path difference")
        A = C[jfn] * hwhm
    else:
        A = 0.0
    if v1out >= v2out or v1out >= v2c or v2out <= v1c:
        raise ScanError("V1out..V2out outside the data")
    # limits of the internal calculation (:527-578)
    if deconv_only:
        V1Z, V2Z = v1c, v2c
    else:
        V1Z = v1out - hwhm * CLIMIT[jfn]
        V2Z = v2out + hwhm * CLIMIT[jfn]
        V1Z = v1c + float(int((V1Z - v1c) / dv)) * dv
        V2Z = v1c + float(int((V2Z - v1c) / dv + 1.01)) * dv
    if V1Z < v1c:
        V1Z = v1c
    if V2Z > v2c:
        V2Z = v2c
    if (V2Z - V1Z) / hwhm < CLIMIT[jfn]:
        raise ScanError("insufficient data for an accurate calculation")
    DVN = 2.0 * hwhm / MDVHW
    if dv > DVN and jfn != 0:  # a coarse grid: onto 2*HWHM/12 first (:592-610)
        spect, v1c = intpdr(spect, v1c, dv, V1Z, V2Z, DVN)
        dv = DVN
        np_in = len(spect)
        v2c = v1c + dv * (np_in - 1)
        V1Z, V2Z = v1c, v2c
    ivx = 1 if (V2Z - V1Z) / hwhm > CRATIO[jfn] else -1
    if jfn == 0:
        ivx = 0
    if ivx == -1 and jfn in (8, 9, 10):
        raise ScanError("Norton-Beer apodization has no spectral-domain form (IVX = -1)")
    # LoadSpect (:1113-1290)
    ltotal = int((V2Z - V1Z) / dv + 1.1)
    V2Z = V1Z + dv * (ltotal - 1)
    nrec = records(ltotal)
    n1 = int((V1Z - v1c) / dv + 1.00001)
    if n1 - 1 + ltotal > np_in:
        raise ScanError("ran out of data")
    x = np.full(nrec * LPTSMX, fill)
    x[:ltotal] = spect[n1 - 1:n1 - 1 + ltotal]
    # pre-boxing (:665-697, Boxcar :862-1012)
    deconv_a = None
    DV = dv
    if do_prebox:
        M = int(2.0 * boxcar_hw / DV)
        if M >= 2:
            V1Z = V1Z + DV * (M - 1) / 2.0
            ktotal = ltotal // M
            DV = M * DV
            V2Z = V1Z + DV * (ktotal - 1)
            box = np.zeros(ktotal)
            for k in range(ktotal):  # sequential sums, as the reference
                s = 0.0
                for m in range(M):
                    s = s + x[k * M + m]
                box[k] = s / float(M)
            nrec = records(ktotal)
            x = np.full(nrec * LPTSMX, fill)
            x[:ktotal] = box
            ltotal = ktotal
            deconv_a = DV
        else:
            do_deconv = False
    if deconv_hw is not None:
        deconv_a = deconv_hw
    if not do_deconv:
        deconv_a = None
    if jfn != 0 or do_deconv:
        F = np.fft.rfft(x)
        H, D = apodization(jfn if ivx == 1 else 0, A, DV, nrec, deconv_a)
        if jfn != 0:
            F = F * (H if ivx == 1 else numeric_apodization(jfn, A, DV, nrec, parms))
        if D is not None:
            F = F * D
        x = np.fft.irfft(F, n=nrec * LPTSMX)
    # output limits (:767-784)
    N1 = int((v1out - V1Z) / DV)
    V1S = V1Z + (N1 - 1) * DV
    if V1S < V1Z:
        N1 = 1
        V1S = V1Z
    N2 = int((v2out - V1Z) / DV + 3.01)
    V2S = V1Z + (N2 - 1) * DV
    if V2S > V2Z:
        N2 = int((V2Z - V1Z) / DV + 1.01)
    ntotal = N2 - N1 + 1
    out = x[N1 - 1:N1 - 1 + ntotal].copy()
    if dvout > 0:  # onto the requested grid (:804-820)
        out, V1S = intpdr(out, V1S, DV, v1out, v2out, dvout)
        DV = dvout
    return out, V1S, DV

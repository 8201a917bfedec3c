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

Covered: functID 1 (boxcar only) and 2..8 (triangle, Gaussian, sinc**2,
sinc, Beer, Hamming, Hanning) with the apodization computed analytically
(IVX = 1: (V2Z-V1Z)/HWHM > CRATIO), optional pre-boxing with deconvolution,
output on the scan grid (DVOUT <= 0).
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
        if jfn == 1:    # triangle: sinc**2
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


def fftscn(spect, v1c, dv, funct_id, hwhm, v1out, v2out, fill=0.0, prebox_hw=-1.0, deconv_prebox=False):
    """clblm_FFTSCN_struct (:352-844) for the cases above.  Returns
    (scanned spectrum, V1S, DV) on the scan grid."""
    spect = np.asarray(spect, dtype=np.float64)
    np_in = len(spect)
    v2c = v1c + dv * (np_in - 1)
    if not (0.0 <= fill <= 1.0):
        raise ScanError("FILL out of range")
    jfn = funct_id - 1
    if jfn == 0:
        do_prebox, do_deconv, boxcar_hw = True, False, hwhm
    elif 1 <= jfn <= 13:
        if prebox_hw <= 0.0:
            do_prebox, do_deconv, boxcar_hw = False, False, 0.0
        else:
            do_prebox, do_deconv, boxcar_hw = True, bool(deconv_prebox), prebox_hw
    else:
        raise ScanError("functID %d is not covered" % funct_id)
    if jfn > 0:
        if C[jfn] <= 0:
            raise ScanError("scanning function needs an optical path difference")
        A = C[jfn] * hwhm
    else:
        A = 0.0
    if v1out >= v2out or v1out >= v2c or v2out <= v1c:
        raise ScanError("V1out..V2out outside the data")
    # limits of the internal calculation (:527-578)
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
    if dv > DVN and jfn != 0:
        raise ScanError("input grid coarser than 2*HWHM/12: the interpolation step is not covered")
    if jfn != 0 and not ((V2Z - V1Z) / hwhm > CRATIO[jfn]):
        raise ScanError("apodization from the scanning function's transform (IVX = -1) is not covered")
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
    if not do_deconv:
        deconv_a = None
    if jfn != 0 or do_deconv:
        F = np.fft.rfft(x)
        H, D = apodization(jfn, A, DV, nrec, deconv_a)
        F = F * H
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
    return x[N1 - 1:N1 - 1 + ntotal].copy(), V1S, DV

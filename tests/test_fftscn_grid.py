"""The library's scan grid (clblm_gpu_fftscn_size: host arithmetic, no GPU)
equals the oracle's restatement of clblm_FFTSCN's limits."""
import numpy as np
import pytest

from oracle import fftscn as S
from clblm_gb300 import capi
from clblm_gb300 import capi_types as T

CASES = [
    # funct_id, hwhm, v1out, v2out, prebox_hw, deconv, dvout, input dv
    (5, 0.3771, 1030.0, 1070.0, -1.0, 0, 0.0, 0.002),   # sinc
    (3, 0.3771, 1030.0, 1070.0, -1.0, 0, 0.0, 0.002),   # Gaussian
    (2, 0.5, 1020.0, 1080.0, -1.0, 0, 0.0, 0.002),      # triangle
    (8, 0.25, 1001.0, 1099.0, -1.0, 0, 0.0, 0.002),     # Hanning, clipped at the data
    (3, 0.3, 1030.0, 1070.0, 0.02, 1, 0.0, 0.002),      # pre-boxing + deconvolution
    (1, 0.05, 1030.0, 1070.0, -1.0, 0, 0.0, 0.002),     # boxcar only
    (9, 0.3, 1030.0, 1070.0, -1.0, 0, 0.0, 0.002),      # Norton-Beer weak
    (11, 0.3, 1030.0, 1070.0, -1.0, 0, 0.0, 0.002),     # Norton-Beer strong
    (2, 4.0, 1040.0, 1060.0, -1.0, 0, 0.0, 0.002),      # triangle from its transform (IVX = -1)
    (3, 12.0, 1040.0, 1060.0, -1.0, 0, 0.0, 0.002),     # Gaussian, IVX = -1
    (14, 0.1, 1030.0, 1070.0, -1.0, 0, 0.0, 0.002),     # Kiruna (always IVX = -1)
    (3, 0.3, 1030.0, 1070.0, -1.0, 0, 0.0, 0.1),        # coarse input: interpolated first
    (5, 0.3771, 1030.0, 1070.0, -1.0, 0, 0.01, 0.002),  # onto DVOUT
    (103, 0.3, 1030.0, 1070.0, 0.01, 0, 0.0, 0.002),    # boxed outside: scan + deconvolution
    (-1, 0.3, 1030.0, 1070.0, 0.01, 0, 0.0, 0.002),     # the deconvolution alone
]


@pytest.mark.parametrize("funct_id,hwhm,v1o,v2o,prebox,deconv,dvout,dv", CASES)
def test_scan_grid_matches_oracle(funct_id, hwhm, v1o, v2o, prebox, deconv, dvout, dv):
    v1 = 1000.0
    n = int(round(100.0 / dv)) + 1
    x = np.ones(n)
    want, v1s, dvs = S.fftscn(x, v1, dv, funct_id, hwhm, v1o, v2o, fill=1.0, prebox_hw=prebox,
                              deconv_prebox=bool(deconv), dvout=dvout, parms=(0.05, 0.9, 0.1))
    sc = T.scan_struct(funct_id, hwhm, v1o, v2o, padding=1.0, prebox_hw=prebox, deconv_prebox=deconv, dvout=dvout,
                       parms=(0.05, 0.9, 0.1))
    g1, gdv, gn = capi.fftscn_size(sc, v1, dv, n)
    assert (g1, gdv, gn) == (v1s, dvs, len(want))


@pytest.mark.parametrize("funct_id", [12, 13, 15, 0, -2])
def test_scan_rejects_as_the_reference_stops(funct_id):
    """Brault and Kaiser-Bessel need an optical path difference the
    reference's FFTSCN does not take; functID outside its ranges."""
    sc = T.scan_struct(funct_id, 0.3, 1030.0, 1070.0)
    with pytest.raises(capi.ClblmError) as e:
        capi.fftscn_size(sc, 1000.0, 0.002, 50001)
    assert e.value.code == T.CLBLM_ERR_ARG
    with pytest.raises(S.ScanError):
        S.fftscn(np.ones(50001), 1000.0, 0.002, funct_id, 0.3, 1030.0, 1070.0)

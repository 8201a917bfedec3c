"""The library's scan grid (clblm_gpu_fftscn_size: host arithmetic, no GPU)
equals the oracle's restatement of clblm_FFTSCN's limits."""
import numpy as np
import pytest

from oracle import fftscn as S
from clblm_gb300 import capi
from clblm_gb300 import capi_types as T

CASES = [
    (5, 0.3771, 1030.0, 1070.0, -1.0, 0),   # sinc
    (3, 0.3771, 1030.0, 1070.0, -1.0, 0),   # Gaussian
    (2, 0.5, 1020.0, 1080.0, -1.0, 0),      # triangle
    (8, 0.25, 1001.0, 1099.0, -1.0, 0),     # Hanning, clipped at the data
    (3, 0.3, 1030.0, 1070.0, 0.02, 1),      # pre-boxing + deconvolution
    (1, 0.05, 1030.0, 1070.0, -1.0, 0),     # boxcar only
]


@pytest.mark.parametrize("funct_id,hwhm,v1o,v2o,prebox,deconv", CASES)
def test_scan_grid_matches_oracle(funct_id, hwhm, v1o, v2o, prebox, deconv):
    v1, dv, n = 1000.0, 0.002, 50001
    x = np.ones(n)
    want, v1s, dvs = S.fftscn(x, v1, dv, funct_id, hwhm, v1o, v2o, fill=1.0, prebox_hw=prebox,
                              deconv_prebox=bool(deconv))
    sc = T.scan_struct(funct_id, hwhm, v1o, v2o, padding=1.0, prebox_hw=prebox, deconv_prebox=deconv)
    g1, gdv, gn = capi.fftscn_size(sc, v1, dv, n)
    assert (g1, gdv, gn) == (v1s, dvs, len(want))


def test_scan_rejects_what_is_not_on_the_path():
    sc = T.scan_struct(12, 0.3, 1030.0, 1070.0)  # Brault
    with pytest.raises(capi.ClblmError) as e:
        capi.fftscn_size(sc, 1000.0, 0.002, 50001)
    assert e.value.code == T.CLBLM_ERR_UNSUPPORTED

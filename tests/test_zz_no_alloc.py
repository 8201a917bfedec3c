"""clblm_gpu_interp_spectrum_noalloc (the grid interpolation that allocates
nothing) against the DVout interpolation of clblm_gpu_od on the same layer.

Both run the same interpolation kernel on the same binary64 values, so the
outputs are expected to agree to the last bit; the tolerance is the FP64
path's 1e-12."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _column():
    from clblm_gb300 import synth
    lines, col, cont = synth.config1(n_lines=40000)
    return lines, col.with_window(1200.0, 1230.0), cont


def test_noalloc_matches_od_dvout_twice(gpu_lib):
    import torch
    from clblm_gb300 import capi_types as T
    lines, col, cont = _column()
    dn, df, _ = gpu_lib.setDV(col)
    h = gpu_lib.Handle(lines, cont)
    try:
        stream = torch.cuda.current_stream()
        # two calls in a row on one stream: a coarser and then a finer output
        # grid, both general ratios (the case that uses the scratch map)
        for il, factor in ((30, 1.2345), (31, 0.8123)):
            lay = col.layer(il)
            ctrl = T.od_ctrl(precision=T.CLBLM_PREC_PLAIN)
            g = T.grid_struct(col.v1, col.v2, dn[il], df[il])
            od, dv = h.odlay(lay, g, ctrl)
            dvout = dv * factor
            gout = T.grid_struct(col.v1, col.v2, dn[il], df[il], dv_out=dvout)
            want, dv_used = h.odlay(lay, gout, ctrl)
            assert dv_used == dvout
            d_in = torch.from_numpy(od).to("cuda")
            d_out = torch.full((len(want),), float("nan"), dtype=torch.float64, device="cuda")
            gpu_lib.interp_spectrum_noalloc(d_in.data_ptr(), len(od), col.v1, dv, d_out.data_ptr(), len(want),
                                            dvout, stream.cuda_stream)
            torch.cuda.synchronize()
            got = d_out.cpu().numpy()
            assert np.all(np.isfinite(got))
            np.testing.assert_allclose(got, want, rtol=RTOL, atol=0)
    finally:
        h.close()


def test_noalloc_rejects_oversize(gpu_lib):
    import torch
    from clblm_gb300 import capi_types as T
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    with pytest.raises(gpu_lib.ClblmError) as e:
        gpu_lib.interp_spectrum_noalloc(x.data_ptr(), 16, 1000.0, 0.01, x.data_ptr(),
                                        gpu_lib.NOALLOC_MAX_POINTS + 1, 0.007)
    assert e.value.code == T.CLBLM_ERR_CAPACITY

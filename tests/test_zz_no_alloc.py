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


def test_noalloc_other_grid_kinds_and_no_allocation(gpu_lib):
    """The same grid, a 2:1 grid (aligned copy) and a 5:4 grid (fixed ratio),
    each called twice in a row, equal the DVout interpolation of
    clblm_gpu_od; once every kernel the call uses has run, two more calls
    leave the device's free memory unchanged (they allocate nothing)."""
    import torch
    from clblm_gb300 import capi_types as T
    lines, col, cont = _column()
    dn, df, _ = gpu_lib.setDV(col)
    h = gpu_lib.Handle(lines, cont)
    try:
        il = 30
        lay = col.layer(il)
        ctrl = T.od_ctrl(precision=T.CLBLM_PREC_PLAIN)
        od, dv = h.odlay(lay, T.grid_struct(col.v1, col.v2, dn[il], df[il]), ctrl)
        d_in = torch.from_numpy(od).to("cuda")
        stream = torch.cuda.current_stream().cuda_stream
        cases = []
        for factor in (1.0, 2.0, 1.25, 1.2345):
            dvout = dv * factor
            want, _ = h.odlay(lay, T.grid_struct(col.v1, col.v2, dn[il], df[il], dv_out=dvout), ctrl)
            cases.append((dvout, want))
        torch.cuda.synchronize()
        outs = [torch.full((len(w),), float("nan"), dtype=torch.float64, device="cuda") for _, w in cases]
        for _ in range(2):
            for (dvout, want), d_out in zip(cases, outs):
                d_out.fill_(float("nan"))
                gpu_lib.interp_spectrum_noalloc(d_in.data_ptr(), len(od), col.v1, dv, d_out.data_ptr(), len(want),
                                                dvout, stream)
                torch.cuda.synchronize()
                got = d_out.cpu().numpy()
                assert np.all(np.isfinite(got))
                np.testing.assert_allclose(got, want, rtol=RTOL, atol=0)
        free_before, _ = torch.cuda.mem_get_info()
        for (dvout, want), d_out in zip(cases, outs):
            gpu_lib.interp_spectrum_noalloc(d_in.data_ptr(), len(od), col.v1, dv, d_out.data_ptr(), len(want),
                                            dvout, stream)
        torch.cuda.synchronize()
        free_after, _ = torch.cuda.mem_get_info()
        assert free_after >= free_before, (free_before, free_after)
    finally:
        h.close()


def test_noalloc_rejects_host_pointer(gpu_lib):
    import torch
    from clblm_gb300 import capi_types as T
    host = np.zeros(64, dtype=np.float64)
    dev = torch.zeros(64, dtype=torch.float64, device="cuda")
    for d_in, d_out in ((host.ctypes.data, dev.data_ptr()), (dev.data_ptr(), host.ctypes.data)):
        with pytest.raises(gpu_lib.ClblmError) as e:
            gpu_lib.interp_spectrum_noalloc(d_in, 64, 1000.0, 0.01, d_out, 64, 0.01)
        assert e.value.code == T.CLBLM_ERR_ARG

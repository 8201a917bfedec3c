"""TAPE3 line files: the package's writer and the library's reader
(clblm_tape3_read, host code) round-trip a line list exactly."""
import numpy as np
import pytest

from clblm_gb300 import synth
from clblm_gb300 import capi_types as T


def test_round_trip(gpu_lib, tmp_path):
    from clblm_gb300 import tape3
    lines = synth.line_list(1234, 600.0, 640.0, seed=11, mols=synth.SEVEN)
    p = tmp_path / "TAPE3"
    tape3.write_tape3(p, lines)
    back = gpu_lib.read_tape3(p)
    assert back.n == lines.n
    for name, _ in T.Lines.FIELDS:
        np.testing.assert_array_equal(getattr(back, name), getattr(lines, name))


def test_window_keeps_whole_records(gpu_lib, tmp_path):
    from clblm_gb300 import tape3
    lines = synth.line_list(2000, 600.0, 700.0, seed=12)
    p = tmp_path / "TAPE3"
    tape3.write_tape3(p, lines)
    back = gpu_lib.read_tape3(p, 650.0, 660.0)
    lo = int(np.searchsorted(lines.vnu, 650.0, side="right")) - 1
    first_rec, last_rec = max(lo, 0) // 250, int(np.searchsorted(lines.vnu, 660.0)) // 250
    assert back.n == (min(lines.n, (last_rec + 1) * 250) - first_rec * 250)
    np.testing.assert_array_equal(back.vnu, lines.vnu[first_rec * 250:first_rec * 250 + back.n])


def test_bad_file_fails_cleanly(gpu_lib, tmp_path):
    p = tmp_path / "bad"
    p.write_bytes(b"\x10\x00\x00\x00garbage")
    with pytest.raises(gpu_lib.ClblmError):
        gpu_lib.read_tape3(p)


def test_round_trip_with_line_coupling(gpu_lib, tmp_path):
    """coupled lines and their coefficient records (IFLG -1, no centre in
    VNU) survive the file; a window keeps a coupled line with its record"""
    from clblm_gb300 import tape3
    base = synth.line_list(1500, 600.0, 700.0, seed=13, mols=(2,))
    lines = synth.with_coupling(base, np.arange(5, base.n, 11))
    p = tmp_path / "TAPE3"
    tape3.write_tape3(p, lines)
    back = gpu_lib.read_tape3(p)
    for name, _ in T.Lines.FIELDS:
        np.testing.assert_array_equal(getattr(back, name), getattr(lines, name))
    win = gpu_lib.read_tape3(p, 650.0, 660.0)
    k = win.keys()
    assert np.all(np.diff(k) >= 0) and k[0] <= 650.0 and k[-1] >= 660.0

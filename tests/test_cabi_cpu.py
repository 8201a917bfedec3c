"""The C-ABI library builds, loads and exports every symbol of include/*.h (no GPU)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_exports_match_header(gpu_lib):
    header = (ROOT / "include" / "clblm_gb300.h").read_text()
    declared = set(re.findall(r"^(?:int|const char \*|void \*)\s*(clblm_\w+)\s*\(", header, re.M))
    assert declared, "no entry points parsed"
    lib = ctypes.CDLL(str(gpu_lib.LIB_PATH))
    for name in sorted(declared):
        assert hasattr(lib, name), name
    assert declared == set(gpu_lib.EXPORTS)


def test_create_without_device_fails_cleanly(gpu_lib):
    import torch
    if torch.cuda.is_available():
        return
    from clblm_gb300 import synth
    lines = synth.line_list(10, 600.0, 601.0, seed=0)
    try:
        gpu_lib.Handle(lines)
    except gpu_lib.ClblmError as e:
        assert e.code in (10, 8)
    else:
        raise AssertionError("create succeeded without a device")

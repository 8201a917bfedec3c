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


def test_every_template_kernel_instance_has_device_code(gpu_lib):
    """each explicit instantiation of a template kernel has its launch stub
    in the library: an instantiation whose declaration differs from the
    definition (nvcc takes a __restrict__ difference for another template)
    has none and fails at launch with 'invalid device function'"""
    import subprocess
    from collections import Counter
    csrc = ROOT / "clblm_gb300" / "csrc"
    want = Counter()
    for src in csrc.glob("*.cu"):
        for name in re.findall(r"^template __global__ void (\w+)<", src.read_text(), re.M):
            want[name] += 1
    assert want, "no explicit instantiations found"
    out = subprocess.run(["nm", str(gpu_lib.LIB_PATH)], capture_output=True, text=True).stdout
    for name, n in want.items():
        # the stub, or the static variables of an inlined stub, name the
        # instance: its template arguments run from I to the EEv before the
        # parameters
        have = set(re.findall(r"__device_stub__ZN5clblm%d%s(I\w*?E)Ev" % (len(name), name), out))
        assert len(have) == n, (name, n, sorted(have))

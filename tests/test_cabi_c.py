"""The C boundary as a C program sees it.

- Layout (CPU): a C file generated from the ctypes mirrors in
  clblm_gb300/capi_types.py is compiled with gcc against
  include/clblm_gb300.h; it prints sizeof and offsetof of every struct and
  field, which must equal the ctypes layout (a field missing from the header
  fails the compile).
- Call (GPU): tests/c/od_call.c, a plain C caller linked against
  libclblm_gb300.so, runs create -> od_size -> od -> od_stats -> destroy on the
  one-layer, 20,000-line workload; its optical depth and line counts are
  compared with the FP64 oracle.
"""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
INCLUDE = ROOT / "include"

STRUCTS = ("clblm_lines_t", "clblm_cont_t", "clblm_layer_t", "clblm_grid_t", "clblm_od_ctrl_t", "clblm_column_t",
           "clblm_jac_t", "clblm_rt_ctrl_t", "clblm_od_stats_t", "clblm_profile_t", "clblm_scan_t",
           "clblm_scanfn_t", "clblm_path_in_t", "clblm_path_t")


def _gcc():
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    return cc


def test_struct_layout_matches_header(tmp_path):
    from clblm_gb300 import capi_types as T
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "clblm_gb300.h"', "int main(void) {"]
    want = {}
    for name in STRUCTS:
        ct = getattr(T, name)
        lines.append('  printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        want[name] = C.sizeof(ct)
        for fname, _ in ct._fields_:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, fname, name, fname))
            want["%s.%s" % (name, fname)] = getattr(ct, fname).offset
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([_gcc(), "-std=c11", "-Wall", "-Werror", "-I", str(INCLUDE), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = {k: int(v) for k, v in (ln.split() for ln in out.splitlines())}
    assert got == want


def test_header_compiles_as_cxx(tmp_path):
    """The header is also usable from C++ (extern "C" block)."""
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no C++ compiler")
    src = tmp_path / "h.cpp"
    src.write_text('#include "clblm_gb300.h"\nint main() { clblm_od_stats_t s{}; return (int)s.nlin; }\n')
    r = subprocess.run([gxx, "-std=c++17", "-Wall", "-Werror", "-I", str(INCLUDE), str(src), "-o",
                        str(tmp_path / "h")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _write_inputs(d, lines, lay, g):
    with open(d / "lines.bin", "wb") as f:
        np.array([lines.n], dtype=np.int64).tofile(f)
        for name, _ in lines.FIELDS:
            getattr(lines, name).tofile(f)
    with open(d / "layer.bin", "wb") as f:
        np.array([lay.nmol], dtype=np.int32).tofile(f)
        np.array([lay.mol_id[i] for i in range(lay.nmol)], dtype=np.int32).tofile(f)
        np.array([lay.w[i] for i in range(lay.nmol)], dtype=np.float64).tofile(f)
        np.array([lay.wtot, lay.pave, lay.tave, g.v1, g.v2, g.dv_normal, g.dv_narrow], dtype=np.float64).tofile(f)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(0, 1e-5), (1, 1e-9)])
def test_c_program_config0_od(tmp_path, gpu_lib, oracle_mod, prec, tol):
    from clblm_gb300 import capi_types as T
    from clblm_gb300 import synth
    lines, col = synth.config0()
    dn, df, _ = gpu_lib.setDV(col)
    lay = col.layer(0)
    g = T.grid_struct(col.v1, col.v2, dn[0], df[0])
    _write_inputs(tmp_path, lines, lay, g)
    exe = tmp_path / "od_call"
    libdir = str(gpu_lib.LIB_PATH.parent)
    r = subprocess.run([_gcc(), "-std=c11", "-O2", "-Wall", "-I", str(INCLUDE), str(ROOT / "tests" / "c" / "od_call.c"),
                        "-o", str(exe), "-L", libdir, "-lclblm_gb300", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(tmp_path / "lines.bin"), str(tmp_path / "layer.bin"), str(tmp_path / "out.bin"),
                        str(prec)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = (tmp_path / "out.bin").read_bytes()
    n, = np.frombuffer(raw[:8], dtype=np.int64)
    dv, = np.frombuffer(raw[8:16], dtype=np.float64)
    cnt = np.frombuffer(raw[16:48], dtype=np.int64)
    od = np.frombuffer(raw[48:], dtype=np.float64)
    assert len(od) == n
    ctrl = T.od_ctrl(precision=prec, contnm_off=1)
    ref, dvr, st = oracle_mod.Session().odlay(lines, lay, g, ctrl)
    assert n == len(ref) and dv == dvr
    assert list(cnt) == [st["nlin"], st["lincnt"], st["nshrunk"], st["npanels"]]
    rel = np.max(np.abs(od - ref) / np.abs(ref))
    assert rel < tol, rel

"""Build the GB300 library libclblm_gb300.so in-tree with nvcc (sm_103a).

Translation units are compiled in parallel; prep.cu, whose FP64 index
arithmetic must round every product and sum separately, is compiled with
--fmad=false.  Host code is compiled with -ffp-contract=off everywhere: the
planning arithmetic (panel and block bounds, grid restarts) must round like
the reference's, and GCC on aarch64 would otherwise fuse a + b*c.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libclblm_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = {
    "prep.cu": ["--fmad=false"],
    "panel.cu": [],
    "rt.cu": [],
    "jac.cu": [],
    "scan.cu": [],
    "scanfn.cu": [],
    "tape3.cpp": [],
    "path.cpp": [],
    "runtime.cu": [],
}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src, extra, verbose_ptxas=False):
    obj = BUILD / (Path(src).stem + ".o")
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-rdc=true", "-I", str(CSRC), "-I", str(HERE.parent / "include"), *extra, "-c", str(CSRC / src),
           "-o", str(obj)]
    if verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose_ptxas=False):
    srcs = [CSRC / s for s in UNITS] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + \
        [HERE.parent / "include" / "clblm_gb300.h", Path(__file__)]
    if LIB.exists() and not force:
        t = LIB.stat().st_mtime
        if all(p.stat().st_mtime <= t for p in srcs):
            return LIB
    BUILD.mkdir(exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose_ptxas), UNITS.items()))
    objs = [str(o) for o, _ in results]
    if verbose_ptxas:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB.with_suffix(".so.tmp")
    cudalib = str(Path(nvcc()).resolve().parent.parent / "lib64")
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", str(tmp), "-lcudart", "-L", cudalib,
           "-lcufft", "-Xlinker", "-rpath," + cudalib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(LIB)

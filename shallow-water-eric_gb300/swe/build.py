"""Build of the native library ``libswe_gpu.so`` (sm_103a) with nvcc/g++.

Translation units are compiled in parallel into ``_build/`` and linked
in-tree next to this package.  The FP64 kernels are compiled without FMA
contraction (they reproduce the FP64 restatement bit for bit); the mixed
kernels use approximate single-precision division and square root, and no
contraction either (their fused multiply-adds are written out, so every
launch variant gives the same bits); host setup code is compiled with
-ffp-contract=off so its matrices are identical on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent                      # shallow-water-eric_gb300/
CSRC = ROOT / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "_lib" / "libswe_gpu.so"
INCLUDE = ROOT.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off",
               f"-I{INCLUDE}", *ARCH]

UNITS = {
    "swe_kernels_f64.cu": ["-fmad=false"],
    # approximate FP32 division and square root, flush-to-zero, and no FMA
    # contraction: the kernels spell out every fused multiply-add, so every
    # launch variant performs the same operations and gives the same bits
    "swe_kernels_mixed.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false", "-fmad=false",
                             "-Xptxas", "-warn-spills"],
    "swe_api.cu": [],
    "swe_noalloc.cu": ["-fmad=false"],
    "swe_setup_gpu.cu": ["-fmad=false"],
    "swe_diag.cu": ["-fmad=false"],
    "swe_setup.cpp": None,   # host C++
    "swe_io.cpp": None,      # host C++
}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (Path(cand).exists() or cand == "nvcc"):
            return cand
    return "nvcc"


def _compile(src: str, extra, verbose=False):
    s = CSRC / src
    o = BUILD / (s.stem + ".o")
    deps = [s] + sorted(CSRC.glob("*.hpp")) + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "swe_gpu.h"]
    if o.exists() and o.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return o
    if extra is None:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-fopenmp",
               f"-I{INCLUDE}", "-c", str(s), "-o", str(o)]
    else:
        cmd = [_nvcc(), *NVCC_COMMON, *extra, "-c", str(s), "-o", str(o)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout, r.stderr)
    return o


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)
    if force:
        for o in BUILD.glob("*.o"):
            o.unlink()
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    if not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_name(f"libswe_gpu.{os.getpid()}.so")
        cmd = [_nvcc(), "-shared", *ARCH, "-Xcompiler", "-fopenmp", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    _build_driver()
    return LIB


DRIVER = LIB.with_name("swe_main")


def _build_driver():
    """swe_main (csrc/swe_main.cpp): the reference's main program (a data
    file's run, or the dam break) over the C++ host interfaces
    include/swe_update.hpp and include/swe_case.hpp (csrc/swe_case.cpp),
    linked against the library next to it.  No FMA contraction (g++
    contracts a*b + c on aarch64 by default): its host arithmetic (init,
    sol_anal, the RK combinations of the per-call loop) follows the
    reference's evaluation order like the Python host side."""
    src = CSRC / "swe_main.cpp"
    case_src = CSRC / "swe_case.cpp"
    deps = [src, case_src, LIB, INCLUDE / "swe_update.hpp", INCLUDE / "swe_case.hpp", INCLUDE / "swe_gpu.h"]
    if DRIVER.exists() and DRIVER.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return DRIVER
    tmp = DRIVER.with_name(f"swe_main.{os.getpid()}")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{INCLUDE}", str(src), str(case_src),
           f"-L{LIB.parent}", "-lswe_gpu",
           "-Wl,-rpath,$ORIGIN", "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(verbose=True))

"""The C++ host side over the C ABI (include/swe_update.hpp) through the
main-program driver (csrc/swe_main.cpp): the dam break it runs equals the
Python host side's run of the same case bit for bit (both drive the same
library), and its VTK movie frames carry the reference's text for the states
they were taken from."""
import subprocess

import numpy as np
import pytest

import oracle
from swe import build as B
from swe import cases as C
from swe import lib as L
from swe.update import from_case

pytestmark = pytest.mark.gpu


def _python_run(n, prec):
    case = C.dam_break_case(n=n, precision=prec)
    upd = from_case(case, precision=prec)
    upd.upload(case.u0)
    upd.set_time(0.0, case.tfinal)
    done = 0
    while True:                      # to time >= Tfinal, as the driver does
        _, _, k = upd.rk3_steps(64)
        done += k
        if k < 64:
            break
    u = upd.download()
    upd.close()
    return case, u, done


@pytest.mark.parametrize("prec", [0, 1])
def test_driver_equals_python_host(tmp_path, monkeypatch, prec):
    """Both processes launch the default variants (SWE_AUTOTUNE=0): the
    autotuner's choice can differ between two runs, and the mixed variants
    agree only to FP32 rounding."""
    import os
    L.load()
    monkeypatch.setenv("SWE_AUTOTUNE", "0")
    out = tmp_path / "state.bin"
    r = subprocess.run([str(B.DRIVER), "--n", "41", "--precision", str(prec), "--out", str(out)],
                       capture_output=True, text=True, timeout=300, env=dict(os.environ))
    assert r.returncode == 0, r.stderr
    case, u, steps = _python_run(41, prec)
    got = np.fromfile(out, np.float64).reshape(u.shape, order="F")
    np.testing.assert_array_equal(got, u)
    assert f"steps {steps} " in r.stdout


def test_driver_frames(tmp_path):
    L.load()
    r = subprocess.run([str(B.DRIVER), "--n", "21", "--frames", "3", "--dir", str(tmp_path), "--out",
                        str(tmp_path / "state.bin")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    names = sorted(p.name for p in tmp_path.glob("*.vtk"))
    assert names == ["h_1.vtk", "h_2.vtk", "h_3.vtk", "hpz_1.vtk", "hpz_2.vtk", "hpz_3.vtk"]
    case = C.dam_break_case(n=21)
    u = np.fromfile(tmp_path / "state.bin", np.float64).reshape(case.u0.shape, order="F")
    hpz, h = oracle.frame_fields(u[0], case.bath, 1.0)   # the last frame is the final state
    for name, f in (("hpz_3.vtk", hpz), ("h_3.vtk", h)):
        assert (tmp_path / name).read_text() == oracle.vtk_2d_text(name.ljust(200), case.mesh["jj"],
                                                                    case.mesh["rr"], f)


def test_cpp_update_interface_bit_exact(tmp_path):
    """tests/cpp/test_update_parity.cpp: construct_matrices, compute_dij,
    euler and FCT_positivity through the C++ host interface against the C++
    oracle, bit for bit, on a dam break and a wet/dry basin."""
    from pathlib import Path
    L.load()
    olib = oracle.build()
    here = Path(__file__).resolve().parent
    exe = tmp_path / "test_update_parity"
    cmd = ["g++", "-O2", "-std=c++17", f"-I{here.parent / 'include'}", str(here / "cpp" / "test_update_parity.cpp"),
           f"-L{B.LIB.parent}", "-lswe_gpu", f"-Wl,-rpath,{B.LIB.parent}", f"-L{olib.parent}", "-lswe_oracle",
           f"-Wl,-rpath,{olib.parent}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert sum(1 for line in r.stdout.splitlines() if line.startswith("ok ")) == 18, r.stdout

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
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{here.parent / 'include'}", str(here / "cpp" / "test_update_parity.cpp"),
           f"-L{B.LIB.parent}", "-lswe_gpu", f"-Wl,-rpath,{B.LIB.parent}", f"-L{olib.parent}", "-lswe_oracle",
           f"-Wl,-rpath,{olib.parent}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert sum(1 for line in r.stdout.splitlines() if line.startswith("ok ")) == 18, r.stdout


@pytest.mark.parametrize("data,mesh,steps", [("ref_data_paraboloid.txt", "ref_cdisk.1_mesh.FEM.gz", 10),
                                             ("ref_data_sources.txt", "ref_rectangle.1.FEM.gz", 6)])
def test_driver_runs_a_reference_data_file(tmp_path, golden, data, mesh, steps):
    """swe_main --data: main.f90 for a reference data file in C++
    (read_my_data, the .FEM reader, init, the Dirichlet lists and bdy) equals
    the Python host side's run of the same data file bit for bit.
    PARABOLOID/data (type 12, 'viscous', dry rim) runs the device loop;
    SOURCES/data (type 13, 'entropy_visc', h at the channel ends moving with
    the wave) runs main.f90's loop over the per-call euler."""
    import gzip
    from swe import data as D, mesh as M, refcases as R
    L.load()
    fem = tmp_path / "mesh.FEM"
    fem.write_bytes(gzip.decompress((golden / mesh).read_bytes()))
    out = tmp_path / "state.bin"
    r = subprocess.run([str(B.DRIVER), "--data", str(golden / data), "--mesh", str(fem), "--steps", str(steps),
                        "--frames", "0", "--out", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = D.read_my_data(golden / data)
    case = R.case_from_data(d, M.load_mesh_free_format(fem, d["list_dom"]))
    if case.bdy_fixed:
        upd = from_case(case)
        upd.upload(case.u0)
        upd.set_time(case.t0, case.tfinal)
        t, _, n = upd.rk3_steps(steps)
        u, t = upd.download(), t[0]
        assert "device-loop" in r.stdout
    else:
        upd = from_case(case, per_call=True)
        u, t, n = R.host_time_loop(R.PerCall(upd), case.bdy, case.u0, case.t0, case.tfinal, steps)
        assert "per-call" in r.stdout
    upd.close()
    got = np.fromfile(out, np.float64).reshape(u.shape, order="F")
    np.testing.assert_array_equal(got, u)
    assert f"steps {n} time {t!r}" in r.stdout or f"steps {n} time {t:.17g}" in r.stdout


@pytest.mark.parametrize("data,mesh", [("ref_data_paraboloid.txt", "ref_cdisk.1_mesh.FEM.gz"),
                                       ("ref_data_sources.txt", "ref_rectangle.1.FEM.gz")])
def test_driver_data_file_frames_and_errors(tmp_path, golden, data, mesh):
    """swe_main --data writes main.f90's files for a run with frames
    (bath.vtk, hexact.vtk = sol_anal(1, rr, Tfinal), then hpz_k / h_k after
    the first step, the next one Tfinal/(nb_frame-1) later) with the
    reference's text, from the device state (device loop) or the host state
    (per-call loop), and prints compute_errors' relative L1 / L2 errors on h
    at the Gauss points."""
    import gzip
    from swe import data as D, mesh as M, refcases as R
    L.load()
    fem = tmp_path / "mesh.FEM"
    fem.write_bytes(gzip.decompress((golden / mesh).read_bytes()))
    r = subprocess.run([str(B.DRIVER), "--data", str(golden / data), "--mesh", str(fem), "--steps", "2",
                        "--frames", "3", "--dir", str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = D.read_my_data(golden / data)
    m = M.load_mesh_free_format(fem, d["list_dom"])
    case = R.case_from_data(d, m)
    jj, rr = m["jj"], m["rr"]
    assert sorted(p.name for p in tmp_path.glob("*.vtk")) == ["bath.vtk", "h_1.vtk", "hexact.vtk", "hpz_1.vtk"]
    assert (tmp_path / "bath.vtk").read_text() == oracle.vtk_2d_text("bath.vtk", jj, rr, case.bath)
    hex_ = case.exact(1, rr, case.tfinal)
    assert (tmp_path / "hexact.vtk").read_text() == oracle.vtk_2d_text("hexact.vtk", jj, rr, hex_)
    hmax0 = case.u0[0].max()
    upd = from_case(case, per_call=not case.bdy_fixed)
    if case.bdy_fixed:
        upd.upload(case.u0)
        upd.set_time(case.t0, case.tfinal)
        upd.rk3_steps(1)
        u1 = upd.download()
        upd.rk3_steps(1)
        t = upd.get_time()[0][0]
    else:
        u1, t1, _ = R.host_time_loop(R.PerCall(upd), case.bdy, case.u0, case.t0, case.tfinal, 1)
        u2, t, _ = R.host_time_loop(R.PerCall(upd), case.bdy, u1, t1, case.tfinal, 1)
        upd.upload(u2)
    hpz, h = oracle.frame_fields(u1[0], case.bath, hmax0)
    for name, f in (("hpz_1.vtk", hpz), ("h_1.vtk", h)):
        assert (tmp_path / name).read_text() == oracle.vtk_2d_text(name.ljust(200), jj, rr, f)
    rj, rg = upd.gauss_points()
    fa = case.exact(1, rg, t)
    e1, e2 = upd.norms(0, fa)
    n1, n2 = np.sum(np.abs(fa) * rj), np.sqrt(np.sum(fa * fa * rj))
    got = {ln.split(" (Gaussian) ")[0].strip(): float(ln.split()[-1]) for ln in r.stdout.splitlines()
           if "(Gaussian)" in ln}
    assert got["Relative L1 error on h"] == pytest.approx(e1 / n1, rel=1e-12)
    assert got["Relative L2 error on h"] == pytest.approx(e2 / n2, rel=1e-12)
    upd.close()



_DATA_TYPE2 = """===Name of directory for mesh file===
'.'
===Name of mesh file===
mesh.FEM
===Test case number===
2
===Final time===
10.
===CFL number===
.25d0
===Viscosity type (galerkin, viscous, entropy_visc, fct)===
'fct'
===Type of first-order viscosity===
'type2'
===Alpha limitation? (True/False)===
.t.
===Lumping the mass matrix? (true/false)===
.t.
===How many Dirichlet boundaries for h?===
0
===List of Dirichlet boundaries for h?===
1
===How many Dirichlet boundaries for ux?===
2
===List of Dirichlet boundaries for ux?===
1 3
===How many Dirichlet boundaries for uy?===
2
===List of Dirichlet boundaries for uy?===
2 4
===Number of subdomains in the mesh===
1
===List of subdomain in the mesh===
1
===Type of finite element===
1
"""


def test_driver_monitor_of_types_1_and_2(tmp_path, golden):
    """Type 2 (lake at rest over the bump of BUMP_3_1/cav_0.3, walls): the
    driver finds the mesh next to its data file, runs the device loop a step
    at a time and writes main.f90's monitor, time and
    0.5 (|qx|_1 + |qy|_1) / (g |h^(3/2)|_1), to fort.10 after every step,
    equal to the same norms taken through the Python host side."""
    import gzip
    from swe import data as D, mesh as M, refcases as R
    L.load()
    (tmp_path / "mesh.FEM").write_bytes(gzip.decompress((golden / "ref_bump_cav_0.3.FEM.gz").read_bytes()))
    (tmp_path / "data").write_text(_DATA_TYPE2)
    r = subprocess.run([str(B.DRIVER), "--data", str(tmp_path / "data"), "--steps", "5", "--dir", str(tmp_path)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    rows = [tuple(float(v) for v in ln.split()) for ln in (tmp_path / "fort.10").read_text().splitlines()]
    d = D.read_my_data(tmp_path / "data")
    case = R.case_from_data(d, M.load_mesh_free_format(tmp_path / "mesh.FEM", d["list_dom"]))
    assert case.bdy_fixed
    upd = from_case(case)
    upd.upload(case.u0)
    upd.set_time(case.t0, case.tfinal)
    want = []
    for _ in range(5):
        t, _, _ = upd.rk3_steps(1)
        q1, q2, q3 = upd.norms(1)[0], upd.norms(2)[0], upd.norms(L.FIELD_H32)[0]
        want.append((t[0], 0.5 * (q1 + q2) / (case.params.gravity * q3)))
    upd.close()
    assert rows == want
    assert not list(tmp_path.glob("*.vtk"))          # type 2 writes no frames

"""Host-side logic and the C-ABI library boundary (CPU only: no kernel runs)."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from swe import cases as C, lib as L, mesh as M

REPO = Path(__file__).resolve().parent.parent


def test_library_builds_and_exports_every_declared_symbol():
    path = L.load()   # builds in-tree (nvcc cross-compiles for sm_103a)
    header = (REPO / "include" / "swe_gpu.h").read_text()
    declared = set(re.findall(r"\b(swe_[a-z0-9_]+)\s*\(", header))
    assert declared == set(L.EXPORTS)
    so = ctypes.CDLL(str(L.library_path()))
    for name in declared:
        assert hasattr(so, name), name


@pytest.mark.parametrize("cc,std,body", [
    ("gcc", "c99", "int main(void) { return swe_last_error(0) == 0; }"),
    ("g++", "c++17", "int main() { return swe_last_error(nullptr) == nullptr; }"),
])
def test_header_is_plain_c(tmp_path, cc, std, body):
    """The C ABI header stands alone (no CUDA or C++ types in the signatures):
    it compiles as C99 and as C++17 with every warning an error."""
    import shutil
    import subprocess
    if shutil.which(cc) is None:
        pytest.skip(f"{cc} not found")
    src = tmp_path / ("t.c" if cc == "gcc" else "t.cpp")
    src.write_text('#include "swe_gpu.h"\n' + body + "\n")
    r = subprocess.run([cc, f"-std={std}", "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only",
                        f"-I{REPO / 'include'}", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_no_cpu_fallback_without_device():
    """Without a CUDA device the library refuses to create a context."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = L.load()
    mesh = M.lattice_mesh(3, 3)
    p = L.swe_params(*C.Params().fields())
    h = ctypes.c_void_p()
    jj = np.asfortranarray(mesh["jj"], np.int32).ravel(order="F")
    rr = np.asfortranarray(mesh["rr"]).ravel(order="F")
    bath = np.zeros(9)
    rc = lib.swe_create(ctypes.byref(h), 9, mesh["jj"].shape[1], L.ip(jj), L.dp(rr), L.dp(bath), ctypes.byref(p))
    assert rc == L.SWE_ERR_CUDA
    assert b"no CUDA device" in lib.swe_last_error(h)
    lib.swe_destroy(h)


def test_reader_matches_committed_mesh(golden):
    """The .FEM reader on the reference's shipped cav_0.2.FEM (copied under
    tests/golden/) reproduces the committed mesh fixture."""
    m = M.load_mesh_free_format(golden / "ref_cav_0.2.FEM")
    g = np.load(golden / "mesh_cav_0.2.npz")
    np.testing.assert_array_equal(m["jj"], g["jj"])
    np.testing.assert_array_equal(m["rr"], g["rr"])


def test_fem_write_read_roundtrip(tmp_path):
    m = M.jittered_mesh(9, 7, 0.0, 2.0, 0.0, 1.0, seed=1)
    M.write_fem(tmp_path / "x.FEM", m)
    r = M.load_mesh_free_format(tmp_path / "x.FEM")
    # first-touch renumbering: mapping old->new must reproduce coordinates
    assert r["rr"].shape == m["rr"].shape and r["jj"].shape == m["jj"].shape
    np.testing.assert_array_equal(np.sort(r["rr"][0]), np.sort(m["rr"][0]))
    x_old = m["rr"][:, m["jj"] - 1]
    x_new = r["rr"][:, r["jj"] - 1]
    np.testing.assert_array_equal(x_old, x_new)


@pytest.mark.parametrize("gen", ["lattice", "jitter"])
def test_generators_ccw_and_boundary(gen):
    m = M.lattice_mesh(11, 6, 0.0, 2.0, 0.0, 1.0) if gen == "lattice" else \
        M.jittered_mesh(11, 6, 0.0, 2.0, 0.0, 1.0, jitter=0.3, seed=4)
    jj, rr = m["jj"] - 1, m["rr"]
    x, y = rr
    area = 0.5 * ((x[jj[1]] - x[jj[0]]) * (y[jj[2]] - y[jj[0]]) - (y[jj[1]] - y[jj[0]]) * (x[jj[2]] - x[jj[0]]))
    assert (area > 0).all()
    assert area.sum() == pytest.approx(2.0, rel=1e-12)
    assert set(np.unique(m["sides"])) == {1, 2, 3, 4}
    xs = M.dirichlet_nodes(m["jjs"], m["sides"], [1])
    assert np.allclose(x[xs - 1], 0.0)
    if gen == "lattice":
        assert m["rr"].shape[1] == 66 and jj.shape[1] == 2 * 10 * 5


def test_dirichlet_nodes_sorted_unique():
    m = M.lattice_mesh(5, 5)
    js = M.dirichlet_nodes(m["jjs"], m["sides"], [1, 2, 3, 4])
    assert list(js) == sorted(set(js)) and len(js) == 16


def test_cases_shapes():
    c = C.dam_break_case(n=11)
    assert c.u0.shape == (3, 121) and c.u0.flags.f_contiguous
    t = C.thacker_case(C.thacker_mesh(0.4), periods=1.0)
    assert t.params.htiny == pytest.approx(4e-4) and t.u0[0].min() >= 4e-4
    s = C.sgn_case(nx=21, ny=3)
    assert s.u0.shape == (5, 63)
    np.testing.assert_allclose(s.u0[3], s.u0[0] ** 2)


def test_cpp_driver_builds_and_stops_without_device():
    """The C++ host side (include/swe_update.hpp) and the main-program driver
    over it build with the library; with no CUDA device the driver reports
    the library's refusal and stops with a nonzero status (no CPU path)."""
    import subprocess
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from swe import build as B
    L.load()
    r = subprocess.run([str(B.DRIVER), "--n", "5"], capture_output=True, text=True)
    assert r.returncode == 3
    assert "no CUDA device" in r.stderr

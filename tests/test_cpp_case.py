"""The C++ set-up (include/swe_case.hpp, csrc/swe_case.cpp: read_my_data,
the .FEM reader with the reference's renumbering, dirichlet_nodes, init and
sol_anal) against the Python host side on the reference's data files and
meshes: readers, node lists, bathymetry, initial and exact fields identical
bit for bit (both sides evaluate exp, cos, acos, cosh, tanh and real powers
with the C library, as the reference's compiled code does).  No GPU."""
import gzip
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN
from swe import data as D, mesh as M, refcases as R

HERE = Path(__file__).resolve().parent
REPO = HERE.parent


@pytest.fixture(scope="module")
def dump_case(tmp_path_factory):
    out = tmp_path_factory.mktemp("cpp") / "dump_case"
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{REPO / 'include'}", str(HERE / "cpp" / "dump_case.cpp"),
           str(REPO / "shallow-water-eric_gb300" / "csrc" / "swe_case.cpp"), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _plain(tmp_path, name):
    src = GOLDEN / name
    if src.suffix != ".gz":
        return src
    dst = tmp_path / src.stem
    dst.write_bytes(gzip.decompress(src.read_bytes()))
    return dst


def _run(exe, data, mesh, tt=None):
    args = [str(exe), str(data), str(mesh)] + ([str(tt)] if tt is not None else [])
    r = subprocess.run(args, capture_output=True, text=True)
    out = {}
    for line in r.stdout.splitlines():
        key, _, rest = line.partition(" ")
        out[key] = rest
    return r.returncode, out


def _ints(s):
    return np.array([int(x) for x in s.split()], np.int64)


def _reals(s):
    return np.array([float(x) for x in s.split()])


def _close(a, b):
    np.testing.assert_array_equal(a, b)          # NaN (a Cardano branch with no real cube root) equals NaN


CASES = [("ref_data_sources.txt", "ref_rectangle.1.FEM.gz", None),
         ("ref_data_paraboloid.txt", "ref_cdisk.1_mesh.FEM.gz", None),
         ("ref_data_paraboloid.txt", "ref_cav_0.2.FEM", 5),
         ("ref_data_paraboloid.txt", "ref_cav_0.2.FEM", 11),
         ("ref_data_paraboloid.txt", "ref_bump_cav_0.3.FEM.gz", 2),
         ("ref_data_paraboloid.txt", "ref_bump_cav_0.3.FEM.gz", 3),
         ("ref_data_paraboloid.txt", "ref_bump_cav_0.3.FEM.gz", 6),
         ("ref_data_paraboloid.txt", "ref_bump_cav_0.3.FEM.gz", 7),
         ("ref_data_paraboloid.txt", "ref_dam_cav_0.25.FEM.gz", 4),
         ("ref_data_paraboloid.txt", "ref_dam_cav_0.25.FEM.gz", 1),
         ("ref_data_paraboloid.txt", "ref_dam_cav_0.25.FEM.gz", 8)]


@pytest.mark.parametrize("data,mesh,tt", CASES)
def test_cpp_setup_matches_python(dump_case, tmp_path, data, mesh, tt):
    rc, out = _run(dump_case, GOLDEN / data, _plain(tmp_path, mesh), tt)
    assert rc == 0, out
    d = D.read_my_data(GOLDEN / data)
    assert out["strings"].split("|") == [d["directory"], d["file_name"], d["viscosity_type"], d["viscous_type"]]
    sc = out["scalars"].split()
    assert [int(sc[0]), int(sc[1]), float(sc[2]), float(sc[3])] == [d["nb_dom"], d["type_fe"], d["Tfinal"], d["CFL"]]
    assert [bool(int(sc[4])), bool(int(sc[5])), int(sc[6])] == [d["if_alpha_limit"], d["if_lumped"], d["type_test"]]
    assert float(sc[7]) == d["mannings"] and float(sc[8]) == d.get("lambdaSGN", 0.0)
    for key, comp in (("list_dom", "list_dom"), ("h_dir", "h_Dir_list"), ("ux_dir", "ux_Dir_list"),
                      ("uy_dir", "uy_Dir_list")):
        np.testing.assert_array_equal(_ints(out[key]), d[comp])
    m = M.load_mesh_free_format(_plain(tmp_path, mesh), d["list_dom"])
    np.testing.assert_array_equal(_ints(out["jj"]), m["jj"].ravel(order="F"))
    np.testing.assert_array_equal(_ints(out["jjs"]), m["jjs"].ravel(order="F"))
    np.testing.assert_array_equal(_ints(out["sides"]), m["sides"])
    np.testing.assert_array_equal(_reals(out["rr"]), m["rr"].ravel(order="F"))
    for key, lst in (("h_js", "h_Dir_list"), ("ux_js", "ux_Dir_list"), ("uy_js", "uy_Dir_list")):
        np.testing.assert_array_equal(_ints(out[key]), M.dirichlet_nodes(m["jjs"], m["sides"], d[lst]))
    tt = d["type_test"] if tt is None else tt
    ini = R.init(tt, m["rr"])
    _close(_reals(out["bath"]), ini["bath"])
    g, mwh, htiny, t0, tf, sets = out["init"].split()
    assert (float(g), float(mwh), float(htiny), float(t0)) == (ini["gravity"], ini["max_water_h"], ini["htiny"],
                                                               ini["t0"])
    assert bool(int(sets)) == (ini["tfinal"] is not None)
    if ini["tfinal"] is not None:
        assert float(tf) == ini["tfinal"]
    S = 5 if tt == 13 else 3
    with np.errstate(invalid="ignore"):
        for k in range(1, S + 1):
            _close(_reals(out[f"u0_{k}"]), R.sol_anal(tt, k, m["rr"], ini["t0"], ini["bath"], ini["gravity"],
                                                      ini["htiny"]))
        for k in (1, 2, 3):
            _close(_reals(out[f"sol_{k}"]), R.sol_anal(tt, k, m["rr"], ini["t0"] + 0.75, ini["bath"],
                                                       ini["gravity"], ini["htiny"]))


def test_cpp_setup_refuses_what_the_reference_cannot_run(dump_case, tmp_path):
    mesh = _plain(tmp_path, "ref_cav_0.2.FEM")
    for tt, msg in ((9, "Malpasset"), (10, "BUG in init")):
        rc, out = _run(dump_case, GOLDEN / "ref_data_paraboloid.txt", mesh, tt)
        assert rc == 1 and msg in out["error"]
    bad = tmp_path / "data"
    bad.write_text((GOLDEN / "ref_data_paraboloid.txt").read_text().replace("===CFL number===", "===CFL==="))
    rc, out = _run(dump_case, bad, mesh)
    assert rc == 1 and "===CFL number=== not found" in out["error"]
    trunc = tmp_path / "short.FEM"
    trunc.write_bytes(mesh.read_bytes()[:1000])
    rc, out = _run(dump_case, GOLDEN / "ref_data_paraboloid.txt", trunc)
    assert rc == 1 and "corrupt" in out["error"]

"""VTK output (vtk_2d, SFEMaNS/FEMSUB/sub_plot.f90:1036-1095) against the
reference's own files (SOURCES/BACKUP/{bath,h_1,hpz_1}.vtk on cav_0.2,
committed gzipped): the oracle's restatement of the Fortran edit descriptors
and the library's C++ writer must reproduce them byte for byte.  CPU only:
the writer is host code."""
import gzip
import math

import numpy as np
import pytest

import oracle
from swe.update import write_vtk_2d

REF_FILES = ("bath", "h_1", "hpz_1")


def _ref(golden, name):
    with gzip.open(golden / f"ref_{name}.vtk.gz", "rb") as f:
        return f.read()


def _field(text):
    lines = text.split("\n")
    i = lines.index("LOOKUP_TABLE default")
    return np.array([float(v) for v in lines[i + 1:] if v.strip()])


def _title(name):
    # bath.vtk is written with a literal name; frames with main.f90's
    # CHARACTER(LEN=200) header, blank-padded
    return f"{name}.vtk" if name == "bath" else f"{name}.vtk".ljust(200)


@pytest.mark.parametrize("name", REF_FILES)
def test_oracle_vtk_text_matches_reference_files(golden, name):
    ref = _ref(golden, name).decode()
    m = np.load(golden / "mesh_cav_0.2.npz")
    assert oracle.vtk_2d_text(_title(name), m["jj"], m["rr"], _field(ref)) == ref


@pytest.mark.parametrize("name", REF_FILES)
def test_library_writer_matches_reference_files(golden, tmp_path, name):
    ref = _ref(golden, name)
    m = np.load(golden / "mesh_cav_0.2.npz")
    out = tmp_path / f"{name}.vtk"
    write_vtk_2d(out, m["jj"], m["rr"], _field(ref.decode()), title=_title(name))
    assert out.read_bytes() == ref


def test_writer_edge_values_match_oracle(tmp_path):
    """Signs, zeros, carries into the next decade, 3-digit exponents and
    non-finite values: the C++ E13.7 against the oracle's."""
    vals = [0.0, -0.0, 1.0, -1.0, 0.99999995, 9.9999999e-5, -3.347705e-3, 1e-100, -2.5e120, 1.7976931348623157e308,
            5e-324, 123456789.0, -0.1, math.nan, math.inf, -math.inf, 0.5, 0.05, 1e99, 1e100]
    n = len(vals)
    rr = np.vstack([np.linspace(-1, 1, n), np.linspace(2e-5, -3e5, n)])
    jj = np.array([[1, 2, 3], [2, 3, 4]]).T
    out = tmp_path / "edge.vtk"
    write_vtk_2d(out, jj, rr, np.array(vals), title="edge.vtk")
    assert out.read_text() == oracle.vtk_2d_text("edge.vtk", jj, rr, vals)
    assert oracle.fortran_e13_7(-0.003347705) == "-.3347705E-02"
    assert oracle.fortran_e13_7(0.99999996) == "0.1000000E+01"
    assert oracle.fortran_e13_7(2.5e120) == "0.2500000+121"


def test_writer_reports_unwritable_path(tmp_path):
    from swe import lib as L
    m_rr = np.zeros((2, 3)); jj = np.array([[1], [2], [3]])
    with pytest.raises(L.SweError):
        write_vtk_2d(tmp_path / "no_such_dir" / "x.vtk", jj, m_rr, np.zeros(3))

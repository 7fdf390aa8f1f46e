"""The reference's ``data`` files (read_my_data, SOURCES/read_data.f90:35-100,
with read_until of SOURCES/tools.f90:3-19) read by swe.data, on the files the
reference ships (committed under tests/golden/)."""
import pytest

from swe import data as D


def test_sources_data(golden):
    d = D.read_my_data(golden / "ref_data_sources.txt")
    assert d["directory"] == "../MESHES/SGN_CANAL" and d["file_name"] == "rectangle.6.FEM"
    assert d["type_test"] == 13 and d["Tfinal"] == 5.0 and d["CFL"] == 0.08
    # only the first line after the marker is read: reordering selects the mode
    assert d["viscosity_type"] == "entropy_visc" and d["viscous_type"] == "type2"
    assert d["if_alpha_limit"] is True and d["if_lumped"] is True
    assert d["h_Dir_list"] == [1, 3] and d["ux_Dir_list"] == [] and d["uy_Dir_list"] == []
    assert d["nb_dom"] == 1 and d["list_dom"] == [1] and d["type_fe"] == 1
    assert d["lambdaSGN"] == 9.0 and d["mannings"] == 0.0
    p = D.params_from_data(d, htiny=1e-4)
    assert (p.syst_size, p.viscosity_type, p.viscous_type, p.type_test) == (5, 2, 2, 13)
    assert p.lambda_sgn == 9.0 and p.cfl == 0.08


def test_paraboloid_data(golden):
    d = D.read_my_data(golden / "ref_data_paraboloid.txt")
    assert d["file_name"] == "cdisk.5_mesh.FEM" and d["type_test"] == 12
    assert d["Tfinal"] == 8.0 and d["CFL"] == 0.3 and d["viscosity_type"] == "viscous"
    assert d["h_Dir_list"] == [1, 2, 3, 4] and d["ux_Dir_list"] == [1, 2, 3, 4] and d["uy_Dir_list"] == [2, 4, 1, 3]
    assert "lambdaSGN" not in d and d["mannings"] == 0.0
    p = D.params_from_data(d, htiny=1e-4)
    assert (p.syst_size, p.viscosity_type, p.if_alpha_limit) == (3, 1, 1)


def test_backup_data_lacks_a_marker(golden):
    """SOURCES/BACKUP/data is an older format without the viscosity-type
    marker: the current read_my_data cannot read it."""
    with pytest.raises(D.DataFileError, match="Viscosity type"):
        D.read_my_data(golden / "ref_data_backup.txt")


def test_list_directed_forms(tmp_path):
    text = "\n".join([
        "  ===Name of directory for mesh file===  ", "'a dir', ignored", "===Name of mesh file===", "m.FEM",
        "===Number of subdomains in the mesh===", "2", "===List of subdomain in the mesh===", "1", "3",
        "===Type of finite element===", "1", "===Final time===", "1.5D-1", "===CFL number===", "2*0.25",
        "===Viscosity type (galerkin, viscous, entropy_visc, fct)===", "fct", "===Type of first-order viscosity===",
        "'type1'", "===Alpha limitation? (True/False)===", ".false.", "===Lumping the mass matrix? (true/false)===",
        "T", "===Test case number===", "10", "===How many Dirichlet boundaries for h?===", "0",
        "===List of Dirichlet boundaries for h?===", "1 2", "===How many Dirichlet boundaries for ux?===", "2",
        "===List of Dirichlet boundaries for ux?===", "4,2 / 9", "===How many Dirichlet boundaries for uy?===", "1",
        "===List of Dirichlet boundaries for uy?===", "3", "===Mannings coefficient===", "3.d-2"]) + "\n"
    f = tmp_path / "data"
    f.write_text(text)
    d = D.read_my_data(f)
    assert d["directory"] == "a dir" and d["list_dom"] == [1, 3] and d["Tfinal"] == 0.15 and d["CFL"] == 0.25
    assert d["if_alpha_limit"] is False and d["if_lumped"] is True and d["ux_Dir_list"] == [4, 2]
    assert d["mannings"] == 0.03 and d["viscous_type"] == "type1"
    assert D.params_from_data(d, htiny=1e-3).viscous_type == 1

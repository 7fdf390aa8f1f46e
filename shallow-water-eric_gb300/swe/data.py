"""Reader of the reference's ``data`` files: ``read_my_data``
(SOURCES/read_data.f90:35-100) with the marker search of ``read_until``
(SOURCES/tools.f90:3-19) and Fortran list-directed input for the values.

    d = read_my_data("PARABOLOID/data")      # the ``inputs`` record as a dict
    p = params_from_data(d, htiny=1e-4)      # swe.cases.Params for the C ABI

``read_until`` rewinds and returns at the first line whose trimmed, left-
adjusted first 128 characters equal the marker, so markers may come in any
order; the value is then read list-directed from the following line(s): a
quoted or blank-delimited string, an integer, a real with ``d`` or ``e``
exponent, a logical (``.t.``, ``T``, ``.false.``, ...), ``r*c`` repeats.  A
missing marker raises ``DataFileError`` (the reference prints a message and
then fails on the next READ).
"""
from __future__ import annotations

import re
from pathlib import Path

from .cases import Params

VISCOSITY_TYPES = {"galerkin": 0, "viscous": 1, "entropy_visc": 2, "fct": 3}


class DataFileError(ValueError):
    pass


def _read_until(lines, marker):
    """Index of the line after the first line equal to marker
    (tools.f90:3-19: control is CHARACTER(LEN=128), compared trimmed and
    left-adjusted)."""
    for i, line in enumerate(lines):
        if line[:128].strip() == marker:
            return i + 1
    raise DataFileError(f"Data string {marker} not found")


_TOKEN = re.compile(r"""\s*(?:'((?:[^']|'')*)'|"((?:[^"]|"")*)"|([^\s,/]+))\s*,?""")


def _tokens(line):
    """Values of one record, list-directed: quoted strings keep blanks,
    others end at a blank, comma or slash; ``r*c`` repeats c r times; a
    slash ends the record."""
    out = []
    pos = 0
    line = line.rstrip("\n")
    while pos < len(line):
        if line[pos:].lstrip().startswith("/"):
            break
        m = _TOKEN.match(line, pos)
        if not m or m.end() == pos:
            break
        pos = m.end()
        if m.group(1) is not None:
            out.append(m.group(1).replace("''", "'"))
        elif m.group(2) is not None:
            out.append(m.group(2).replace('""', '"'))
        else:
            tok = m.group(3)
            rep = re.fullmatch(r"(\d+)\*(.*)", tok)
            if rep:
                out.extend([rep.group(2)] * int(rep.group(1)))
            else:
                out.append(tok)
    return out


def _values(lines, i, n):
    """n list-directed values starting at record i (a list may continue on
    the next records); a READ of zero items still consumes one record."""
    vals = []
    while len(vals) < n:
        if i >= len(lines):
            raise DataFileError("end of file while reading values")
        vals.extend(_tokens(lines[i]))
        i += 1
    return vals[:n]


def _real(tok):
    return float(tok.replace("d", "e").replace("D", "e"))


def _logical(tok):
    t = tok.lstrip(".").upper()
    if t.startswith("T"):
        return True
    if t.startswith("F"):
        return False
    raise DataFileError(f"not a logical: {tok}")


def read_my_data(path):
    """The fields read_my_data fills (read_data.f90:35-100), in its order."""
    lines = Path(path).read_text().splitlines()

    def one(marker):
        return _values(lines, _read_until(lines, marker), 1)[0]

    def many(marker, n):
        return _values(lines, _read_until(lines, marker), n) if n else []

    d = {"epsilon": 1.e-4}
    d["directory"] = one("===Name of directory for mesh file===")
    d["file_name"] = one("===Name of mesh file===")
    d["nb_dom"] = int(one("===Number of subdomains in the mesh==="))
    d["list_dom"] = [int(v) for v in many("===List of subdomain in the mesh===", d["nb_dom"])]
    d["type_fe"] = int(one("===Type of finite element==="))
    d["Tfinal"] = _real(one("===Final time==="))
    d["CFL"] = _real(one("===CFL number==="))
    d["viscosity_type"] = one("===Viscosity type (galerkin, viscous, entropy_visc, fct)===")[:15]
    d["viscous_type"] = one("===Type of first-order viscosity===")
    d["if_alpha_limit"] = _logical(one("===Alpha limitation? (True/False)==="))
    d["if_lumped"] = _logical(one("===Lumping the mass matrix? (true/false)==="))
    d["type_test"] = int(one("===Test case number==="))
    for comp in ("h", "ux", "uy"):
        n = int(one(f"===How many Dirichlet boundaries for {comp}?==="))
        d[f"{comp}_nb_Dir_bdy"] = n
        d[f"{comp}_Dir_list"] = [int(v) for v in many(f"===List of Dirichlet boundaries for {comp}?===", n)]
    d["mannings"] = _real(one("===Mannings coefficient===")) if d["type_test"] in (9, 10) else 0.0
    if d["type_test"] == 13:
        d["lambdaSGN"] = _real(one("===Lambda for SGN model==="))
    return d


def params_from_data(d, htiny, gravity=9.81, max_water_h=1.0, dt=0.0, precision=0):
    """swe.cases.Params from a read_my_data record.  htiny, gravity and
    max_water_h are set by the reference's ``init`` per test case
    (SOURCES/condlim.f90:92-242), not by the data file."""
    visc = d["viscosity_type"].strip().lower()
    if visc not in VISCOSITY_TYPES:
        raise DataFileError(f"viscosity type {visc!r}")
    vt = d["viscous_type"].strip().lower()
    if vt not in ("type1", "type2"):
        raise DataFileError(f"first-order viscosity {vt!r}")
    return Params(gravity=gravity, dt=dt, cfl=d["CFL"], htiny=htiny, mannings=d["mannings"],
                  lambda_sgn=d.get("lambdaSGN", 0.0), max_water_h=max_water_h, type_test=d["type_test"],
                  syst_size=5 if d["type_test"] == 13 else 3, viscosity_type=VISCOSITY_TYPES[visc],
                  viscous_type=1 if vt == "type1" else 2, if_alpha_limit=int(d["if_alpha_limit"]),
                  if_lumped=int(d["if_lumped"]), precision=precision)

"""Oracle package — TEST INFRASTRUCTURE ONLY.

This is the FP64 CPU restatement of the reference's explicit P1 Saint-Venant
step (SOURCES/update.f90, SOURCES/fct.f90, SOURCES/condlim.f90,
SOURCES/main.f90 of t-bltg/shallow-water-eric), compiled from
``swe_oracle.cpp``.  Only the tests, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` may import it, and only as the checker or the
timed CPU baseline.  The product library never loads it.

Parity status: partially pinned (see the header of swe_oracle.cpp): the
reference's own initial-state/bathymetry dumps on cav_0.2 pin the setup, the
reference's recorded Thacker L1 errors pin the time stepping loosely.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libswe_oracle.so"
SRC = HERE / "swe_oracle.cpp"

# No FMA contraction and no fast-math: the restatement's evaluation order is
# its contract (identical results on x86-64 and aarch64 hosts).  Row loops are
# OpenMP-parallel; every row is still summed by one thread in CSR order, so
# results do not depend on the thread count.
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp"]


def build(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        tmp = BUILD / f"libswe_oracle.{os.getpid()}.so"
        subprocess.run(["g++", *CXXFLAGS, "-o", str(tmp), str(SRC)], check=True)
        os.replace(tmp, LIB)
    return LIB


class Params(ctypes.Structure):
    """Same layout as ``swe_params`` in include/swe_gpu.h."""
    _fields_ = [
        ("gravity", ctypes.c_double), ("dt", ctypes.c_double), ("cfl", ctypes.c_double),
        ("htiny", ctypes.c_double), ("mannings", ctypes.c_double), ("lambda_sgn", ctypes.c_double),
        ("max_water_h", ctypes.c_double),
        ("type_test", ctypes.c_int), ("syst_size", ctypes.c_int), ("viscosity_type", ctypes.c_int),
        ("viscous_type", ctypes.c_int), ("if_alpha_limit", ctypes.c_int), ("if_lumped", ctypes.c_int),
        ("if_roundoff_fix", ctypes.c_int), ("precision", ctypes.c_int),
    ]


class Dump(ctypes.Structure):
    _fields_ = [(n, ctypes.POINTER(ctypes.c_double)) for n in
                ("dij_low", "muij_low", "alpha", "u_low", "res", "fctmat", "rminus", "lij")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build()))
        L = _lib
        vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [ctypes.c_int, ctypes.c_int, ip, dp]
        L.orc_destroy.argtypes = [vp]
        L.orc_nnz.argtypes = [vp]
        L.orc_get_matrices.argtypes = [vp, ip, ip, dp, dp, ip, dp, dp]
        L.orc_gauss.argtypes = [vp, dp, dp]
        L.orc_norms.argtypes = [vp, dp, dp, dp, dp]
        L.orc_set_params.argtypes = [vp, ctypes.POINTER(Params)]
        L.orc_get_params.argtypes = [vp, ctypes.POINTER(Params)]
        L.orc_set_bath.argtypes = [vp, dp]
        L.orc_set_dirichlet.argtypes = [vp, ctypes.c_int, ctypes.c_int, ip, dp]
        L.orc_compute_dij.argtypes = [vp, dp, dp, dp]
        L.orc_euler.argtypes = [vp, dp, dp, ctypes.POINTER(Dump)]
        L.orc_fct_positivity.argtypes = [vp, dp, dp, dp]
        L.orc_fct_generic.argtypes = [vp, dp, dp, dp, dp, dp]
        L.orc_rk3_step.argtypes = [vp, dp, dp, ctypes.c_double]
        L.orc_run.argtypes = [vp, dp, dp, ctypes.c_double, ctypes.c_int, ip]
        L.orc_last_dt.restype = ctypes.c_double
        L.orc_last_dt.argtypes = [vp]
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class OracleError(RuntimeError):
    def __init__(self, code, where):
        super().__init__(f"oracle {where} failed with code {code}")
        self.code = code


class Oracle:
    """The reference path restated on the CPU, in the reference's node numbering.

    ``jj`` is (3, me) 1-based, ``rr`` is (2, np); states are (S, np) arrays
    (stored column-major like the Fortran ``un(S, np)``).
    """

    def __init__(self, jj, rr):
        L = lib()
        self.jj = np.asfortranarray(jj, dtype=np.int32)
        self.rr = np.asfortranarray(rr, dtype=np.float64)
        self.np = self.rr.shape[1]
        self.me = self.jj.shape[1]
        self.h = L.orc_create(self.np, self.me, _ip(self.jj), _dp(self.rr))
        if not self.h:
            raise OracleError(-1, "create")
        self.nnz = L.orc_nnz(self.h)
        self.params = None

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def matrices(self):
        n, z = self.np, self.nnz
        ia = np.zeros(n + 1, np.int32); ja = np.zeros(z, np.int32)
        mass = np.zeros(z); lumped = np.zeros(n); diag = np.zeros(n, np.int32)
        cx = np.zeros(z); cy = np.zeros(z)
        lib().orc_get_matrices(self.h, _ip(ia), _ip(ja), _dp(mass), _dp(lumped), _ip(diag), _dp(cx), _dp(cy))
        return dict(ia=ia, ja=ja, mass=mass, lumped=lumped, diag=diag, cx=cx, cy=cy)

    def gauss(self):
        rj = np.zeros(3 * self.me); rg = np.zeros(6 * self.me)
        lib().orc_gauss(self.h, _dp(rj), _dp(rg))
        return rj, rg.reshape(-1, 2).T.copy()

    def norms(self, ff, f_anal):
        ff = np.ascontiguousarray(ff, np.float64); fa = np.ascontiguousarray(f_anal, np.float64)
        l1 = ctypes.c_double(); l2 = ctypes.c_double()
        lib().orc_norms(self.h, _dp(ff), _dp(fa), ctypes.byref(l1), ctypes.byref(l2))
        return l1.value, l2.value

    def set_params(self, p: Params):
        rc = lib().orc_set_params(self.h, ctypes.byref(p))
        if rc:
            raise OracleError(rc, "set_params")
        self.params = p

    def get_params(self) -> Params:
        p = Params()
        lib().orc_get_params(self.h, ctypes.byref(p))
        return p

    def set_bath(self, bath):
        b = np.ascontiguousarray(bath, np.float64)
        lib().orc_set_bath(self.h, _dp(b))

    def set_dirichlet(self, comp, js, vals=None):
        js = np.ascontiguousarray(js, np.int32)
        v = None if vals is None else np.ascontiguousarray(vals, np.float64)
        rc = lib().orc_set_dirichlet(self.h, comp, len(js), _ip(js), None if v is None else _dp(v))
        if rc:
            raise OracleError(rc, "set_dirichlet")

    def compute_dij(self, un):
        u = np.asfortranarray(un, np.float64)
        dij = np.zeros(self.nnz); dt = ctypes.c_double()
        rc = lib().orc_compute_dij(self.h, _dp(u), _dp(dij), ctypes.byref(dt))
        if rc:
            raise OracleError(rc, "compute_dij")
        return dij, dt.value

    def euler(self, un, dump=False):
        u = np.asfortranarray(un, np.float64)
        out = np.zeros_like(u, order="F")
        d = None
        if dump:
            z, n = self.nnz, self.np
            arrs = dict(dij_low=np.zeros(z), muij_low=np.zeros(z), alpha=np.zeros(n),
                        u_low=np.zeros_like(u, order="F"), res=np.zeros(n), fctmat=np.zeros(z),
                        rminus=np.zeros(n), lij=np.zeros(z))
            d = Dump(**{k: _dp(v) for k, v in arrs.items()})
        rc = lib().orc_euler(self.h, _dp(u), _dp(out), ctypes.byref(d) if d is not None else None)
        if rc:
            raise OracleError(rc, "euler")
        return (out, arrs) if dump else out

    def fct_positivity(self, unext_scaled, fmat):
        u = np.ascontiguousarray(unext_scaled, np.float64); f = np.ascontiguousarray(fmat, np.float64)
        lij = np.zeros(self.nnz)
        lib().orc_fct_positivity(self.h, _dp(u), _dp(f), _dp(lij))
        return lij

    def fct_generic(self, unext, maxn, minn, fmat, dg):
        """FCT_generic (SAFE/fct.f90:3-43); returns the limited copy of unext."""
        u = np.array(unext, np.float64)
        args = [np.ascontiguousarray(a, np.float64) for a in (maxn, minn, fmat, dg)]
        lib().orc_fct_generic(self.h, _dp(u), *[_dp(a) for a in args])
        return u

    def rk3_step(self, un, time, fixed_dt=0.0):
        t = ctypes.c_double(time)
        rc = lib().orc_rk3_step(self.h, _dp(un), ctypes.byref(t), fixed_dt)
        if rc:
            raise OracleError(rc, "rk3_step")
        return t.value

    def run(self, un, time, tfinal, max_steps=1 << 30):
        """In-place DO WHILE(time < Tfinal) loop; returns (time, nsteps)."""
        assert un.flags.f_contiguous and un.dtype == np.float64
        t = ctypes.c_double(time); n = ctypes.c_int()
        rc = lib().orc_run(self.h, _dp(un), ctypes.byref(t), tfinal, max_steps, ctypes.byref(n))
        if rc:
            raise OracleError(rc, "run")
        return t.value, n.value

    @property
    def last_dt(self):
        return lib().orc_last_dt(self.h)


def frame_fields(h, bath, hmax0):
    """Movie-frame fields of the time loop (SOURCES/main.f90:125-143):
    hpz = h + bath, or -1e-7 hmax0 + bath where h <= 1e-4 hmax0 (hpz_k.vtk);
    h, or 0 there (h_k.vtk).  Each product and sum is one FP64 rounding."""
    h = np.asarray(h, np.float64)
    bath = np.asarray(bath, np.float64)
    dry = h <= 1.e-4 * hmax0
    hpz = np.where(dry, (-1.e-7 * hmax0) + bath, h + bath)
    return hpz, np.where(dry, 0.0, h)


def fortran_e13_7(x):
    """Fortran E13.7 edit descriptor as gfortran writes it (the number format
    of vtk_2d, SFEMaNS/FEMSUB/sub_plot.f90:1059,1093): 0.dddddddE+xx,
    -.dddddddE+xx when negative (no room for the leading zero)."""
    import math
    if math.isnan(x):
        return "NaN".rjust(13)
    if math.isinf(x):
        return ("Infinity" if x > 0 else "-Infinity").rjust(13)
    neg = math.copysign(1.0, x) < 0
    if x == 0:
        digits, e = "0000000", 0
    else:
        m, ex = f"{abs(x):.6E}".split("E")
        digits, e = m.replace(".", ""), int(ex) + 1
    exp = f"E{'-' if e < 0 else '+'}{abs(e):02d}" if abs(e) <= 99 else f"{'-' if e < 0 else '+'}{abs(e):03d}"
    return ("-." if neg else "0.") + digits + exp


def vtk_2d_text(title, jj, rr, field):
    """The text vtk_2d writes (SFEMaNS/FEMSUB/sub_plot.f90:1036-1095, P1
    branch) for a mesh jj (3, me) 1-based, rr (2, np) and a P1 field."""
    np_, me = rr.shape[1], jj.shape[1]
    out = ["# vtk DataFile Version 3.0", f"vtk {title}", "ASCII", "DATASET UNSTRUCTURED_GRID",
           f"POINTS {np_:7d} float"]
    out += [f"{fortran_e13_7(rr[0, i])}  {fortran_e13_7(rr[1, i])}   0.0 " for i in range(np_)]
    out.append(f"CELLS {me:7d}{4 * me:8d}")
    out += [f"3 {jj[0, k] - 1:8d} {jj[1, k] - 1:8d} {jj[2, k] - 1:8d}" for k in range(me)]
    out.append(f"CELL_TYPES {me:7d}")
    out += ["5"] * me
    out += [f"POINT_DATA {np_:7d}", "SCALARS scalars float 1", "LOOKUP_TABLE default"]
    out += [fortran_e13_7(v) for v in field]
    return "\n".join(out) + "\n"


def _pd_scal(a, b):
    return a[0] * b[0] + a[1] * b[1]


def _pd_vect(y):
    return (-y[1], y[0])


def _sub(a, b):
    return (a[0] - b[0], a[1] - b[1])


def gauge_element(jj, rr, r):
    """First element (1-based) where inside(mesh, m, r) holds
    (SFEMaNS/FEMSUB_OBJET/post_interp.f90:492-524, the search of
    SOURCES/condlim.f90:273-278), or 0.  jj (3, me) 1-based, rr (2, np)."""
    r = (float(r[0]), float(r[1]))
    for m in range(jj.shape[1]):
        p = [(float(rr[0, jj[v, m] - 1]), float(rr[1, jj[v, m] - 1])) for v in range(3)]
        s1 = _pd_scal(_pd_vect(_sub(p[2], p[1])), _sub(r, p[1]))
        s2 = _pd_scal(_pd_vect(_sub(p[0], p[2])), _sub(r, p[2]))
        s3 = _pd_scal(_pd_vect(_sub(p[1], p[0])), _sub(r, p[0]))
        if not (min(s1, s2, s3) < -1.e-12):
            return m + 1
    return 0


def gauge_weights(jj, rr, m, r):
    """FE_interpolation(mesh, m, r) for P1 (post_interp.f90:206-255), m
    1-based."""
    r = (float(r[0]), float(r[1]))
    p = [(float(rr[0, jj[v, m - 1] - 1]), float(rr[1, jj[v, m - 1] - 1])) for v in range(3)]
    n2, n3 = _pd_vect(_sub(p[0], p[2])), _pd_vect(_sub(p[1], p[0]))
    x = 1.0 - _pd_scal(n2, _sub(p[1], r)) / _pd_scal(n2, _sub(p[1], p[2]))
    y = 1.0 - _pd_scal(n3, _sub(p[2], r)) / _pd_scal(n3, _sub(p[2], p[0]))
    return ((1.0 - x) - y, x, y)


def gauge_values(jj, m, ff, h, bath):
    """The two sums the Malpasset gauges write (SOURCES/main.f90:112-115):
    SUM(h(jj(:,m)) * ff) and SUM((h + bath)(jj(:,m)) * ff), in order."""
    nodes = [int(jj[v, m - 1]) - 1 for v in range(3)]
    sh = se = 0.0
    for v, n in enumerate(nodes):
        sh = h[n] * ff[v] if v == 0 else sh + h[n] * ff[v]
        se = (h[n] + bath[n]) * ff[v] if v == 0 else se + (h[n] + bath[n]) * ff[v]
    return sh, se

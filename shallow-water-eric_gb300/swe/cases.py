"""Test-case physics on the host: bathymetry, initial state, exact solutions
and Dirichlet data for the workloads.

These restate the host-side routines the reference keeps in
SOURCES/condlim.f90 (``init`` :92-242, ``sol_anal`` :311-831) for the cases
the workloads use, plus new cases written in the same style for workloads the
reference has no case for (unit-square dam break, Gaussian-bump wet/dry basin
with Manning friction, batched dam breaks, SGN solitary wave in a long
channel).  They run once per run (or once per error evaluation), never inside
the time step.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np

from . import mesh as M

VISC = {"galerkin": 0, "viscous": 1, "entropy_visc": 2, "fct": 3}


@dataclass
class Params:
    """Mirror of the ``inputs`` record fields the step reads
    (SOURCES/read_data.f90:4-32) plus module constants; same field order as
    ``swe_params`` in include/swe_gpu.h."""
    gravity: float = 9.81
    dt: float = 0.0
    cfl: float = 0.25
    htiny: float = 1e-4
    mannings: float = 0.0
    lambda_sgn: float = 0.0
    max_water_h: float = 1.0
    type_test: int = 4
    syst_size: int = 3
    viscosity_type: int = 3          # fct
    viscous_type: int = 2            # 'type2'
    if_alpha_limit: int = 1
    if_lumped: int = 1
    if_roundoff_fix: int = 1         # SOURCES/update.f90:15
    precision: int = 0               # 0 = FP64, 1 = mixed FP32/FP64

    def fields(self):
        return [getattr(self, k) for k in self.__dataclass_fields__]


@dataclass
class Case:
    name: str
    mesh: dict
    params: Params
    bath: np.ndarray
    u0: np.ndarray                    # (S, np), Fortran order
    tfinal: float
    dirichlet: list = field(default_factory=list)   # [(comp0, js 1-based, values)]
    nsteps: int | None = None        # fixed step count when the workload names one
    exact: object = None             # callable(k, rr, t) -> values, when known
    t0: float = 0.0                  # inputs%time at the start (1 for the reference's type 4)
    bdy: object = None               # callable(un, t): bdy (main.f90:176-188) on the host, when known
    bdy_fixed: bool = True           # Dirichlet values independent of t: the device loop can run it
    dirichlet_anal: list = field(default_factory=list)   # [(comp0, js)] of sol_anal(t), evaluated on the device


def _walls(mesh, S):
    """qx = 0 on x-normal sides (1, 3), qy = 0 on y-normal sides (2, 4)."""
    jx = M.dirichlet_nodes(mesh["jjs"], mesh["sides"], [1, 3])
    jy = M.dirichlet_nodes(mesh["jjs"], mesh["sides"], [2, 4])
    return [(1, jx, np.zeros(len(jx))), (2, jy, np.zeros(len(jy)))]


# --------------------------------------------------------------------------
# Thacker planar surface in a paraboloid: type_test 5,
# SOURCES/condlim.f90:151-161 (init) and :429-456 (sol_anal).
# --------------------------------------------------------------------------
THACKER = dict(a=1.0, h0=0.1, hL=4.0, eta=0.5)


def thacker_bath(rr):
    a, h0, hL = THACKER["a"], THACKER["h0"], THACKER["hL"]
    return -h0 * (1.0 - ((rr[0] - hL / 2.0) ** 2 + (rr[1] - hL / 2.0) ** 2) / a ** 2)


def thacker_sol(k, rr, t, htiny, g=9.81, film=True):
    """sol_anal type 5.  ``film`` adds the +htiny of the current reference
    (SOURCES/condlim.f90:440); the revision that produced the recorded
    PARABOLOID/lis_* runs had it commented out (SOURCES/BACKUP/condlim.f90:298)."""
    a, h0, hL, eta = THACKER["a"], THACKER["h0"], THACKER["hL"], THACKER["eta"]
    omega = math.sqrt(2 * g * h0) / a
    bathi = -h0 * (1.0 - ((rr[0] - hL / 2.0) ** 2 + (rr[1] - hL / 2.0) ** 2) / a ** 2)
    base = np.maximum((eta * h0 / a ** 2) * (2.0 * (rr[0] - hL / 2.0) * math.cos(omega * t)
                                             + 2.0 * (rr[1] - hL / 2.0) * math.sin(omega * t)) - bathi, 0.0)
    if k == 1:
        return base + htiny if film else base
    if k == 2:
        return -eta * omega * math.sin(omega * t) * base
    if k == 3:
        return eta * omega * math.cos(omega * t) * base
    return np.zeros(rr.shape[1])


def thacker_case(mesh, periods=1.0, cfl=0.2, precision=0, dirichlet=True, film=True):
    """Thacker oscillation.  With ``dirichlet`` the exact h, qx, qy are imposed
    on all four sides (as in the reference's PARABOLOID data file); the box
    boundary is dry, so the imposed values are h = htiny, q = 0 at all times."""
    g = 9.81
    hL = THACKER["hL"]
    p = Params(gravity=g, cfl=cfl, max_water_h=hL, htiny=1e-4 * hL, type_test=5, precision=precision)
    rr = mesh["rr"]
    bath = thacker_bath(rr)
    u0 = np.asfortranarray(np.vstack([thacker_sol(k, rr, 0.0, p.htiny, g, film) for k in (1, 2, 3)]))
    omega = math.sqrt(2 * g * THACKER["h0"]) / THACKER["a"]
    tf = periods * 2 * math.pi / omega
    bc = []
    if dirichlet:
        js = M.dirichlet_nodes(mesh["jjs"], mesh["sides"], [1, 2, 3, 4])
        for k in (1, 2, 3):
            bc.append((k - 1, js, thacker_sol(k, rr[:, js - 1], 0.0, p.htiny, g, film)))
    return Case("thacker", mesh, p, bath, u0, tf, bc,
                exact=lambda k, r, t: thacker_sol(k, r, t, p.htiny, g, film))


def thacker_mesh(spacing, seed=3):
    """Jittered-lattice Delaunay mesh of the Thacker box [0,4]^2."""
    n = int(round(4.0 / spacing)) + 1
    return M.jittered_mesh(n, n, 0.0, 4.0, 0.0, 4.0, jitter=0.3, seed=seed)


# --------------------------------------------------------------------------
# Unit-square dam break (new case): h = 1 for x < 0.5 else 0.1, z = 0, walls.
# --------------------------------------------------------------------------
def dam_break_case(n=101, precision=0, tfinal=0.2, cfl=0.25):
    mesh = M.lattice_mesh(n, n, 0.0, 1.0, 0.0, 1.0)
    rr = mesh["rr"]
    h = np.where(rr[0] < 0.5, 1.0, 0.1)
    u0 = np.asfortranarray(np.vstack([h, np.zeros_like(h), np.zeros_like(h)]))
    p = Params(gravity=9.81, cfl=cfl, max_water_h=1.0, htiny=1e-4 * 1.0, type_test=4, precision=precision)
    return Case("dam_break_unit_square", mesh, p, np.zeros(rr.shape[1]), u0, tfinal, _walls(mesh, 3))


# --------------------------------------------------------------------------
# Wet/dry basin with 32 Gaussian bumps, circular dam and Manning friction
# (new case; friction is the reference's type 9/10 term,
# SOURCES/update.f90:425-452).
# --------------------------------------------------------------------------
def bump_basin_case(n=2000, precision=0, nsteps=200, cfl=0.25, mannings=0.03, seed_mesh=0, seed_bath=1,
                    mesh=None):
    L = 10.0
    if mesh is None:
        mesh = M.jittered_mesh(n, n, 0.0, L, 0.0, L, jitter=0.3, seed=seed_mesh)
    rr = mesh["rr"]
    rng = np.random.default_rng(seed_bath)
    A = rng.uniform(0.1, 0.8, 32)
    w = rng.uniform(0.2, 1.5, 32)
    c = rng.uniform(0.0, L, (32, 2))
    z = np.zeros(rr.shape[1])
    for k in range(32):
        z += A[k] * np.exp(-((rr[0] - c[k, 0]) ** 2 + (rr[1] - c[k, 1]) ** 2) / w[k] ** 2)
    eta = np.where((rr[0] - 5.0) ** 2 + (rr[1] - 5.0) ** 2 < 1.0, 1.5, 0.5)
    h = np.maximum(eta - z, 0.0)
    u0 = np.asfortranarray(np.vstack([h, np.zeros_like(h), np.zeros_like(h)]))
    mwh = float(h.max())
    p = Params(gravity=9.81, cfl=cfl, max_water_h=mwh, htiny=1e-4 * mwh, mannings=mannings,
               type_test=10, precision=precision)
    return Case("bump_basin", mesh, p, z, u0, 1e30, _walls(mesh, 3), nsteps=nsteps)


# --------------------------------------------------------------------------
# Batched dam breaks (new case): log-uniform node counts, rectangles of aspect
# U(1,4), per-instance upstream/downstream depth and Manning coefficient.
# --------------------------------------------------------------------------
def batch_instances(n_inst=512, nmin=2000, nmax=200000, seed=2, precision=0, cfl=0.25):
    rng = np.random.default_rng(seed)
    cases = []
    for b in range(n_inst):
        N = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        asp = rng.uniform(1.0, 4.0)
        ny = max(3, int(round(math.sqrt(N / asp))))
        nx = max(3, int(round(N / ny)))
        hu = rng.uniform(0.5, 2.0)
        hd = rng.uniform(0.0, 0.2)
        nman = rng.uniform(0.01, 0.05)
        mesh = M.jittered_mesh(nx, ny, 0.0, asp, 0.0, 1.0, jitter=0.3, seed=1000 + b)
        rr = mesh["rr"]
        h = np.where(rr[0] < 0.5 * asp, hu, hd)
        u0 = np.asfortranarray(np.vstack([h, np.zeros_like(h), np.zeros_like(h)]))
        p = Params(gravity=9.81, cfl=cfl, max_water_h=hu, htiny=1e-4 * hu, mannings=nman, type_test=10,
                   precision=precision)
        cases.append(Case(f"dam_{b}", mesh, p, np.zeros(rr.shape[1]), u0, 1e30, _walls(mesh, 3)))
    return cases


# --------------------------------------------------------------------------
# Hyperbolised SGN solitary wave: type_test 13 physics
# (SOURCES/condlim.f90:215-226, :751-824) with the channel's own parameters.
# --------------------------------------------------------------------------
def sgn_sol(k, rr, t, h1, h2, x0, g=9.81):
    D = math.sqrt(g * h2)
    z = math.sqrt((3.0 * (h2 - h1)) / (h2 * h1 ** 2.0))
    arg = 1.0 / 2.0 * z * (rr[0] - x0 - D * t)
    ht = np.maximum(h1 + (h2 - h1) * (1.0 / np.cosh(arg)) ** 2.0, 0.0)
    if k == 1:
        return ht
    if k == 2:
        return ht * D - h1 * D
    if k == 3:
        return ht * 0.0
    if k == 4:
        return ht * ht
    if k == 5:
        return -D * h1 * ((h1 - h2) * z * (1.0 / np.cosh(arg)) ** 2.0 * np.tanh(arg))
    raise ValueError(k)


def sgn_case(nx=10001, ny=201, Lx=100.0, Ly=2.0, h1=1.0, h2=1.2, x0=20.0, lambda_sgn=100.0,
             precision=0, nsteps=1000, cfl=0.1, mesh=None):
    if mesh is None:
        mesh = M.lattice_mesh(nx, ny, 0.0, Lx, 0.0, Ly)
    rr = mesh["rr"]
    u0 = np.asfortranarray(np.vstack([sgn_sol(k, rr, 0.0, h1, h2, x0) for k in (1, 2, 3, 4, 5)]))
    p = Params(gravity=9.81, cfl=cfl, max_water_h=h2, htiny=1e-4 * h2, lambda_sgn=lambda_sgn, type_test=13,
               syst_size=5, precision=precision, viscosity_type=VISC["fct"])
    # walls on the long sides (qy = 0), nothing imposed at the channel ends
    jy = M.dirichlet_nodes(mesh["jjs"], mesh["sides"], [2, 4])
    return Case("sgn_solitary", mesh, p, np.zeros(rr.shape[1]), u0, 1e30,
                [(2, jy, np.zeros(len(jy)))], nsteps=nsteps,
                exact=lambda k, r, t: sgn_sol(k, r, t, h1, h2, x0))

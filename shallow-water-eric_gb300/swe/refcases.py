"""The reference's own test cases by number: ``init``
(SOURCES/condlim.f90:92-245) and ``sol_anal`` (:311-831) for every
``type_test``, the Dirichlet node lists of construct_mesh
(SOURCES/mesh.f90:20-36) and the values ``bdy`` imposes after every RK stage
(SOURCES/main.f90:176-188).  With them a reference data file and its mesh
set up the same run on the device:

    d = data.read_my_data("data")
    mesh = M.load_mesh_free_format(d["directory"] + "/" + d["file_name"], d["list_dom"])
    case = refcases.case_from_data(d, mesh)                    # swe.cases.Case
    upd = update.from_case(case)
    upd.upload(case.u0); upd.set_time(case.t0, case.tfinal); upd.rk3_steps(...)

Host-side set-up, run once per run; the step itself is the device's.

Kept as the reference has them:

* ``sol_anal`` reads the module array ``bath`` by the position in ``rr``
  (types 1, 2 and 8 at t = 0): a call on a subset of the nodes (``bdy`` on
  the Dirichlet nodes) reads bath of nodes 1..n, not of the subset.
* Fortran default-real literals are single precision: ``h0 = 0.32`` of
  type 8 (condlim.f90:165, :608) is the float32 nearest 0.32, widened.
* Integer powers ``x**n`` are products (x*x, x*x*x), as Fortran evaluates
  them; real powers (``**(1.d0/3)``) are ``pow``.

Refused with an error:

* type 9 needs the Malpasset data files (malpasset.wh/.jj/.bath), which are
  not shipped with the reference; ``cases`` has a stand-in;
* type 10 has no ``init`` branch (the reference prints ' BUG in init' and
  STOPs);
* components 4 and 5 of type 13 on Dirichlet nodes: ``sol_anal`` leaves them
  undefined for t > 1e-10 (condlim.f90:791-821).

Boundary data: the device loop (``rk3_steps``) imposes fixed Dirichlet
values after every stage.  Where the values bdy writes stay fixed over
(t0, Tfinal] (walls, steady inflow, dry boundaries: checked at set-up) the
case carries them as ``dirichlet`` and runs on the device loop; where they
change with time (the type-13 solitary wave at the channel ends) the case is
marked ``bdy_fixed = False`` and runs through ``host_time_loop``: per-call
euler on the device, bdy on the host at the reference's stage times.
"""
from __future__ import annotations

import math

import numpy as np

from . import cases as C
from . import mesh as M
from .data import params_from_data

EPSILON = 1.e-4                       # inputs%epsilon (SOURCES/read_data.f90:38)
H0_ISLAND = float(np.float32(0.32))   # h0 = 0.32, a default-real literal


def _libm(fn, x, *args):
    """The C library's fn elementwise (Python's math module calls it), as
    the reference's compiled code evaluates exp, cos, acos, cosh, tanh and
    real powers; numpy's own vectorised versions can differ in the last bit.
    A domain error gives NaN and an overflow inf, as in C."""
    def one(v):
        try:
            return fn(v, *args)
        except ValueError:
            return math.nan
        except OverflowError:
            return math.inf
    a = np.asarray(x, np.float64)
    return np.fromiter(map(one, a.ravel().tolist()), np.float64, a.size).reshape(a.shape)


def _bump(x):
    """0.2*(x-8)**3*(12-x)**3/64, the bump of types 2, 3, 6, 7."""
    a = x - 8.0
    b = 12.0 - x
    return 0.2 * ((a * a) * a) * ((b * b) * b) / 64.0


def _paraboloid(rr, h0, hL, a):
    """-h0*(1-((x-hL/2)**2+(y-hL/2)**2)/a**2), types 5, 11, 12."""
    dx = rr[0] - hL / 2.0
    dy = rr[1] - hL / 2.0
    return -h0 * (1.0 - (dx * dx + dy * dy) / (a * a))


def init(type_test, rr, gravity=9.81):
    """init (condlim.f90:92-245) without the state: bath, gravity,
    max_water_h, htiny = epsilon*max_water_h, the start time (1 for type 4,
    else 0) and the final time init imposes (types 5 and 11; None = the data
    file's)."""
    x, y = rr[0], rr[1]
    n = rr.shape[1]
    t0, tfinal = 0.0, None
    if type_test == 1:                                    # :116-133
        gravity, mwh = 1.0, 0.2
        dx1, dy1 = x - 1.2, y - 0.7
        dx2, dy2 = x - 0.45, y - 0.4
        ray1 = 25.0 * (dx1 * dx1) + 50.0 * (dy1 * dy1)
        ray2 = 50.0 * (dx2 * dx2) + 100.0 * (dy2 * dy2)
        e1, e2 = math.exp(-1.0), math.exp(-2.0)
        cone = ((_libm(math.exp, -ray1) - e1) / (e2 - e1) - 1.0) * (-0.2)
        cone = np.where(np.abs(np.sqrt(ray1) - 1.0) < 1.e-10, 0.2, cone)
        bath = np.where(ray1 <= 2.0, cone, np.where(ray2 <= 1.0, -0.5 * (_libm(math.exp, -ray2) - e1), 0.0))
    elif type_test in (2, 3, 6, 7):                       # :134-146
        gravity = 9.81
        mwh = 0.2 if type_test == 2 else 2.0
        bath = np.where((8.0 < x) & (x < 12.0), _bump(x), 0.0)
    elif type_test == 4:                                  # :147-152
        t0, gravity, mwh = 1.0, 9.81, 0.005
        bath = np.zeros(n)
    elif type_test == 5:                                  # :153-163
        gravity, a, h0, hL = 9.81, 1.0, 0.1, 4.0
        mwh = hL
        omega = math.sqrt(2 * gravity * h0) / a
        tfinal = 6.0 * math.acos(-1.0) / omega
        bath = _paraboloid(rr, h0, hL, a)
    elif type_test == 8:                                  # :164-179
        gravity, htop, rcone, scone, hcone = 9.81, 0.625, 3.6, 4.0, 0.9
        mwh = H0_ISLAND
        dx, dy = x - 15.0, y - 13.0
        radius = np.sqrt(dx * dx + dy * dy)
        bath = np.where(radius < rcone, np.minimum(htop, hcone - radius / scone), 0.0)
    elif type_test == 11:                                 # :200-211
        gravity, a, h0, hL, kappa = 9.81, 1.0, 0.1, 4.0, 0.2
        mwh = hL
        p = math.sqrt((8 * gravity * h0) / (a * a))
        s = 1.0 / 2.0 * math.sqrt(p * p - kappa * kappa)
        tfinal = 2 * 2 * math.acos(-1.0) / s
        bath = _paraboloid(rr, h0, hL, a)
    elif type_test == 12:                                 # :212-218
        gravity, a, h0, hL = 9.81, 3.0, 0.5, 0.0
        mwh = 6.0
        bath = _paraboloid(rr, h0, hL, a)
    elif type_test == 13:                                 # :219-229
        gravity, mwh = 9.81, 11.0 / 100.0
        bath = np.zeros(n)
    elif type_test == 9:
        raise ValueError("type_test 9 (Malpasset) needs malpasset.wh/.jj/.bath, which the reference does "
                         "not ship")
    else:
        raise ValueError(f"type_test {type_test}: no init for this case (the reference STOPs: BUG in init)")
    return dict(bath=np.asarray(bath, np.float64), gravity=gravity, max_water_h=mwh, htiny=EPSILON * mwh,
                t0=t0, tfinal=tfinal)


def _cardano(b, d):
    """Roots of x**3 + b*x**2 + d = 0 the way sol_anal writes them
    (condlim.f90:353-364, :477-504): R, Q, D, then the trigonometric roots
    x1, x2, x3 where D < 0 and Cardano's x1, x2 where D >= 0."""
    R = (-27 * d - 2 * ((b * b) * b)) / 54
    Q = -(b * b) / 9
    D = (Q * Q) * Q + R * R
    return R, Q, D


def _trig_roots(R, Q, b):
    tpio3 = 2 * math.acos(-1.0) / 3
    fpio3 = 2 * tpio3
    with np.errstate(invalid="ignore"):
        theta = _libm(math.acos, R / np.sqrt(-((Q * Q) * Q)))
        sq = 2 * np.sqrt(-Q)
        x1 = sq * _libm(math.cos, theta / 3) - b / 3
        x2 = sq * _libm(math.cos, theta / 3 + tpio3) - b / 3
        x3 = sq * _libm(math.cos, theta / 3 + fpio3) - b / 3
    return x1, x2, x3


def _cardano_x2(R, D, b):
    with np.errstate(invalid="ignore"):
        S = -_libm(math.pow, -np.sqrt(D) - R, 1.0 / 3)
        T = -_libm(math.pow, np.sqrt(D) - R, 1.0 / 3)
    return -(S + T) / 2.0 - b / 3.0


def sol_anal(type_test, k, rr, t, bath, gravity, htiny):
    """sol_anal(k, rr, t) (condlim.f90:311-831): component k (1 = h, 2 = qx,
    3 = qy, 4 and 5 the SGN unknowns of type 13) at the points rr (2, n)."""
    x, y = rr[0], rr[1]
    n = rr.shape[1]
    g = gravity
    zero = np.zeros(n)
    if type_test in (1, 2):                               # :327-345
        if k != 1:
            return zero
        lvl = 0.2 if type_test == 1 else 0.1
        bi = bath[:n]
        return np.maximum(np.maximum(bi, lvl) - bi, 0.0)
    if type_test == 3:                                    # :346-379
        q0, hL = 4.42, 2.0
        if k == 1:
            bathi = np.maximum(0.0, _bump(x))
            if t <= 1.e-14:
                return hL - bathi
            b = bathi - (q0 * q0) / (2 * g * (hL * hL)) - hL
            d = (q0 * q0) / (2 * g)
            R, Q, _ = _cardano(b, d)
            return _trig_roots(R, Q, b)[0]
        if k == 2:
            return zero if t <= 1.e-14 else np.full(n, q0)
        return zero
    if type_test == 4:                                    # :380-420
        x0, hL = 5.0, 0.005
        speed = math.sqrt(g * hL)
        if k == 1:
            if t <= 1.e-14:
                return np.where(x <= x0, hL, 0.0)
            xx = x - x0
            s = speed - xx / (2 * t)
            fan = (4.0 / (9.0 * g)) * (s * s)
            return np.where(xx <= -t * speed, hL, np.where(xx <= 2 * t * speed, fan, 0.0 + htiny))
        if k == 2:
            if t <= 1.e-14:
                return zero
            xx = x - x0
            s = speed - xx / (2 * t)
            fan = (8.0 / (27.0 * g)) * (speed + xx / t) * (s * s)
            return np.where(xx <= -t * speed, 0.0, np.where(xx <= 2 * t * speed, fan, 0.0))
        return zero
    if type_test == 5:                                    # :421-456
        if k > 3:
            raise ValueError(f"sol_anal type 5 has no component {k}")
        return C.thacker_sol(k, rr, t, htiny, g, film=True)
    if type_test == 6:                                    # :457-514
        x0, q0, hL = 10.0, 1.53, 0.66
        d = (q0 * q0) / (2 * g)
        eta = -math.pow(27 * d / 4, 1.0 / 3)
        bernoulli = 0.2 - eta
        if k == 1:
            bathi = np.maximum(0.0, _bump(x))
            if t <= 1.e-14:
                return hL - bathi
            b = bathi - bernoulli
            R, Q, D = _cardano(b, d)
            x1, _, x3 = _trig_roots(R, Q, b)
            sub = np.where(x < x0, np.maximum(x1, x3), np.minimum(x1, x3))
            return np.where(D >= 0.0, _cardano_x2(R, D, b), sub)
        if k == 2:
            return zero if t <= 1.e-14 else np.full(n, q0)
        return zero
    if type_test == 7:                                    # :515-603
        x0, xshock, q0 = 10.0, 11.7, 0.18
        d = (q0 * q0) / (2 * g)
        eta = -math.pow(27 * d / 4, 1.0 / 3)
        ber_pre = 0.2 - eta
        bath_shock = float(_bump(xshock)) if 8.0 < xshock < 12.0 else 0.0
        b = bath_shock - ber_pre
        R, Q, D = _cardano(b, d)
        if D >= 0.0:
            raise ValueError("sol_anal type 7: no pre-shock root (the reference prints BUG case(7))")
        x3 = float(_trig_roots(R, Q, b)[2])
        h_post = (-x3 + math.sqrt(x3 * x3 + 8 * (q0 * q0) / (g * x3))) / 2
        if k == 1:
            bathi = np.maximum(0.0, _bump(x))
            if t <= 1.e-14:
                return h_post - bathi
            bb = bathi - ber_pre
            R, Q, D = _cardano(bb, d)
            x1, _, x3v = _trig_roots(R, Q, bb)
            sub = np.where(x < x0, np.maximum(x1, x3v),
                           np.where(x < xshock, np.minimum(x1, x3v), bath_shock + h_post - bathi))
            return np.where(D >= 0.0, _cardano_x2(R, D, bb), sub)
        if k == 2:
            return np.full(n, q0)
        return zero
    if type_test == 8:                                    # :604-628
        h0 = H0_ISLAND
        alpha = 1 * h0
        xs = 15.0 - 12.96
        vel = math.sqrt(3.0 * alpha / (4 * ((h0 * h0) * h0)))
        ch = _libm(math.cosh, vel * (x - xs))
        if k == 1:
            return np.maximum(h0 + alpha / (ch * ch) - bath[:n], 0.0) if t <= 1.e-14 else np.full(n, h0)
        if k == 2:
            return alpha / (ch * ch) * math.sqrt(g / h0) if t <= 1.e-14 else zero
        return zero
    if type_test == 11:                                   # :645-697
        a, h0, hL, kappa, gamma = 1.0, 0.1, 4.0, 0.2, 0.5
        p = math.sqrt((8 * g * h0) / (a * a))
        s = 1.0 / 2.0 * math.sqrt(p * p - kappa * kappa)
        bathi = _paraboloid(rr, h0, hL, a)
        e2 = math.exp(-kappa * t / 2.0)
        cs, sn = math.cos(s * t), math.sin(s * t)
        htilde = (-bathi - (gamma * gamma) / (2 * g) * math.exp(-kappa * t)
                  - gamma / (2.0 * g) * e2 * (x - hL / 2.0) * (2 * s * cs + kappa * sn)
                  - gamma / (2.0 * g) * e2 * (y - hL / 2.0) * (kappa * cs - 2.0 * s * sn))
        h = np.maximum(htilde, 0.0)
        if k == 1:
            return h
        if k == 2:
            return h * gamma * e2 * sn
        if k == 3:
            return h * gamma * e2 * cs
        raise ValueError(f"sol_anal type 11 has no component {k}")
    if type_test == 12:                                   # :698-750
        a, h0, hL, f, eta = 3.0, 0.5, 0.0, 2.0, 0.5
        a2 = a * a
        a4 = a2 * a2
        den = (f * f) * a4 + math.sqrt(8.0 * (f * f) * g * h0 * (a4 * a2) + ((f * f) * (f * f)) * (a4 * a4))
        delta = 2.0 * f * a4 / den
        w = -1.0 / (math.sqrt(2.0) * a2) * math.sqrt(4.0 * g * h0 * a2 + den)
        cs, sn = math.cos(w * t), math.sin(w * t)
        bathi = _paraboloid(rr, h0, hL, a)
        htilde = (-bathi - eta / g * cs * (1 - delta * f) * (y - hL / 2.0)
                  + eta / g * sn * (f / w - delta * w) * (x - hL / 2.0)
                  + (eta * eta) / (2.0 * g) * ((delta * delta) * cs * cs + sn * sn / (w * w)))
        h = np.maximum(htilde, 0.0)
        if k == 1:
            return h
        if k == 2:
            return -h * delta * eta * cs
        if k == 3:
            return h * eta * sn / w
        raise ValueError(f"sol_anal type 12 has no component {k}")
    if type_test == 13:                                   # :751-824
        if k in (4, 5) and t > 1.e-10:
            raise ValueError(f"sol_anal type 13 leaves component {k} undefined for t > 1e-10")
        h1, h2, x0 = 10.0 / 100.0, 11.0 / 100.0, 2.75
        D = math.sqrt(g * h2)
        z = math.sqrt((3.0 * (h2 - h1)) / (h2 * math.pow(h1, 2.0)))
        arg = 1.0 / 2.0 * z * (x - x0 - D * t)
        se = 1.0 / _libm(math.cosh, arg)
        se2 = se * se
        ht = np.maximum(h1 + (h2 - h1) * se2, 0.0)
        if k == 1:
            return ht
        if k == 2:
            return ht * D - h1 * D
        if k == 3:
            return ht * 0.0
        if k == 4:
            return ht * ht
        if k == 5:
            return -D * h1 * ((h1 - h2) * z * se2 * _libm(math.tanh, arg))
        raise ValueError(f"sol_anal type 13 has no component {k}")
    raise ValueError(f"type_test {type_test}: no sol_anal for this case (the reference STOPs)")


def dirichlet_lists(d, mesh):
    """h_js_D, ux_js_D, uy_js_D of construct_mesh (mesh.f90:20-36): the
    nodes of the boundary sides each data-file list names."""
    return [M.dirichlet_nodes(mesh["jjs"], mesh["sides"], d[f"{c}_Dir_list"][: d[f"{c}_nb_Dir_bdy"]])
            for c in ("h", "ux", "uy")]


def _bdy_comps(type_test, lists):
    """(component, nodes) pairs bdy writes (main.f90:180-186): h on h_js_D,
    qx on ux_js_D, qy on uy_js_D, and for type 13 the fourth and fifth
    unknowns on ux_js_D and uy_js_D."""
    comps = [(0, lists[0]), (1, lists[1]), (2, lists[2])]
    if type_test == 13:
        comps += [(3, lists[1]), (4, lists[2])]
    return [(c, np.asarray(js, np.int32)) for c, js in comps if len(js)]


def make_bdy(type_test, lists, rr, bath, gravity, htiny):
    """bdy(uu, t) (main.f90:176-188) on the host: uu(k, js_D) =
    sol_anal(k, rr(:, js_D), t), in place on a (S, np) array."""
    comps = _bdy_comps(type_test, lists)

    def bdy(uu, t):
        for comp, js in comps:
            uu[comp, js - 1] = sol_anal(type_test, comp + 1, rr[:, js - 1], t, bath, gravity, htiny)
    return bdy


def bdy_data(type_test, lists, rr, bath, gravity, htiny, t0, tfinal, nsamples=17):
    """The (component, nodes, values) triples for the device loop, which
    imposes fixed values after every stage, or None when the values bdy
    would write change over (t0, tfinal]."""
    times = [t0 + 1.e-6] + list(np.linspace(t0, tfinal, nsamples)[1:])
    out = []
    for comp, js in _bdy_comps(type_test, lists):
        pts = rr[:, js - 1]
        try:
            vals = [sol_anal(type_test, comp + 1, pts, t, bath, gravity, htiny) for t in times]
        except ValueError:
            return None
        if any(not np.array_equal(v, vals[0]) for v in vals[1:]):
            return None
        out.append((comp, js, np.asarray(vals[-1], np.float64)))
    return out


def host_time_loop(op, bdy, un, time, tfinal, max_steps=1 << 30):
    """The time loop of main.f90:61-91 through per-call operators, for
    Dirichlet data that change with time:

        COMPUTE_DT; uo = un
        un = euler(uo);            bdy(un, time + dt)     ! time = to
        time = to + dt;   ui = euler(un); un = (3*uo + ui)/4; bdy(un, time + dt/2)
        time = to + dt/2; ui = euler(un); un = (uo + 2*ui)/3; bdy(un, time + dt)
        time = to + dt

    (the second and third bdy calls see to + 3dt/2, as in the reference).
    ``op`` has compute_dt(un) -> dt (COMPUTE_DT, main.f90:166-174),
    set_dt(dt) and euler(un) -> unext.  Returns (un, time, steps)."""
    un = np.asfortranarray(un, np.float64).copy(order="F")
    steps = 0
    while time < tfinal and steps < max_steps:
        dt = op.compute_dt(un)
        op.set_dt(dt)
        to = time
        uo = un
        un = np.asfortranarray(op.euler(uo))
        bdy(un, time + dt)
        time = to + dt
        ui = op.euler(un)
        un = np.asfortranarray((3 * uo + ui) / 4)
        bdy(un, time + dt / 2)
        time = to + dt / 2
        ui = op.euler(un)
        un = np.asfortranarray((uo + 2 * ui) / 3)
        bdy(un, time + dt)
        time = to + dt
        steps += 1
    return un, time, steps


class PerCall:
    """host_time_loop's operators over an update.Update (the C ABI's
    swe_compute_dij / swe_set_params / swe_euler)."""

    def __init__(self, upd, inst=0):
        self.upd, self.inst = upd, inst

    def compute_dt(self, un):
        return self.upd.compute_dij(un, self.inst)[1]

    def set_dt(self, dt):
        from dataclasses import replace
        self.upd.set_params(replace(self.upd.params[self.inst], dt=dt), self.inst)

    def euler(self, un):
        return self.upd.euler(un, self.inst)


def reference_case(type_test, mesh, h_dir=(), ux_dir=(), uy_dir=(), tfinal=None, cfl=0.25, precision=0,
                   viscosity_type=3, viscous_type=2, if_alpha_limit=1, if_lumped=1, lambda_sgn=0.0):
    """Case ``type_test`` on ``mesh`` with the Dirichlet sides given like a
    data file's lists (mesh side numbers)."""
    d = {"h_nb_Dir_bdy": len(h_dir), "h_Dir_list": list(h_dir), "ux_nb_Dir_bdy": len(ux_dir),
         "ux_Dir_list": list(ux_dir), "uy_nb_Dir_bdy": len(uy_dir), "uy_Dir_list": list(uy_dir),
         "type_test": type_test, "Tfinal": 1.0 if tfinal is None else tfinal, "CFL": cfl,
         "viscosity_type": ["galerkin", "viscous", "entropy_visc", "fct"][viscosity_type],
         "viscous_type": f"type{viscous_type}", "if_alpha_limit": bool(if_alpha_limit),
         "if_lumped": bool(if_lumped), "mannings": 0.0}
    if type_test == 13:
        d["lambdaSGN"] = lambda_sgn
    return case_from_data(d, mesh, precision=precision, tfinal=tfinal)


def case_from_data(d, mesh, precision=0, tfinal=None):
    """main.f90:19-60 up to the time loop for a read_my_data record ``d``:
    init, the initial state un(k,:) = sol_anal(k, rr, time) and the bdy
    data; ``tfinal`` overrides the data file's final time (init's own
    override for types 5 and 11 wins, as in the reference)."""
    tt = d["type_test"]
    rr = mesh["rr"]
    ini = init(tt, rr)
    p = params_from_data(d, htiny=ini["htiny"], gravity=ini["gravity"], max_water_h=ini["max_water_h"],
                         precision=precision)
    t0 = ini["t0"]
    tf = ini["tfinal"] if ini["tfinal"] is not None else (d["Tfinal"] if tfinal is None else tfinal)
    u0 = np.asfortranarray(np.vstack([sol_anal(tt, k, rr, t0, ini["bath"], ini["gravity"], ini["htiny"])
                                      for k in range(1, p.syst_size + 1)]))
    lists = dirichlet_lists(d, mesh)
    bc = bdy_data(tt, lists, rr, ini["bath"], ini["gravity"], ini["htiny"], t0, tf)
    # values that change with time: the device evaluates sol_anal for types 5
    # and 13 (components h, qx, qy; swe_set_dirichlet_anal)
    comps = _bdy_comps(tt, lists)
    anal = comps if bc is None and tt in (5, 13) and all(comp <= 2 for comp, _ in comps) else []
    return C.Case(f"type{tt}", mesh, p, ini["bath"], u0, tf, bc or [], t0=t0,
                  exact=lambda k, r, t: sol_anal(tt, k, r, t, ini["bath"], ini["gravity"], ini["htiny"]),
                  bdy=make_bdy(tt, lists, rr, ini["bath"], ini["gravity"], ini["htiny"]), bdy_fixed=bc is not None,
                  dirichlet_anal=anal)

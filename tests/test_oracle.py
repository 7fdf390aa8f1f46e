"""The FP64 oracle against the reference's own recorded outputs and against
hand-computable properties (CPU only)."""
import math

import numpy as np
import pytest

import oracle
from swe import cases as C, mesh as M


def _mesh(golden, h):
    d = np.load(golden / f"mesh_cav_{h}.npz")
    return {k: d[k] for k in d.files}


def _oracle_for(case):
    o = oracle.Oracle(case.mesh["jj"], case.mesh["rr"])
    o.set_params(oracle.Params(*case.params.fields()))
    o.set_bath(case.bath)
    for comp, js, vals in case.dirichlet:
        o.set_dirichlet(comp, js, vals)
    return o


def test_backup_dump_pins_reader_and_init(golden):
    """SOURCES/BACKUP/hinit.plt / bath.plt: node numbering, coordinates,
    bathymetry and initial depth of type_test 5 on cav_0.2 (older revision,
    no +htiny)."""
    m = _mesh(golden, "0.2")
    pin = np.load(golden / "pin_backup_cav02.npz")
    idx = pin["node"] - 1
    assert len(idx) == m["rr"].shape[1]
    np.testing.assert_array_equal(m["rr"][0, idx], pin["x"])
    np.testing.assert_array_equal(m["rr"][1, idx], pin["y"])
    np.testing.assert_allclose(C.thacker_bath(m["rr"])[idx], pin["bath"], rtol=0, atol=1e-15)
    h0 = C.thacker_sol(1, m["rr"], 0.0, 4e-4, film=False)
    np.testing.assert_allclose(h0[idx], pin["h0"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("h", ["0.2", "0.1", "0.05"])
def test_initial_dt_pins_it_max(golden, h):
    """it_max = INT(Tfinal/dt0) of the reference's recorded Thacker runs
    (PARABOLOID/lis_{h}_type2_lim, CFL 0.3, three periods): pins
    compute_lambda_vacc, compute_dij and COMPUTE_DT on the initial state."""
    pin = np.load(golden / "pin_lis.npz")
    k = list(pin["h"]).index(float(h))
    m = _mesh(golden, h)
    case = C.thacker_case(m, periods=3.0, cfl=float(pin["cfl"]), film=False)
    o = _oracle_for(case)
    _, dt0 = o.compute_dij(case.u0)
    tfinal = 6.0 * math.acos(-1.0) / math.sqrt(2 * 9.81 * 0.1)
    assert int(tfinal / dt0) == int(pin["it_max"][k])


def test_thacker_error_order_of_magnitude(golden):
    """Relative L1 error after one Thacker period on cav_0.2 / cav_0.1 (CFL 0.3)
    decreases under refinement and sits in the range the recorded runs show."""
    errs = []
    for h in ("0.2", "0.1"):
        m = _mesh(golden, h)
        case = C.thacker_case(m, periods=1.0, cfl=0.3, film=False)
        o = _oracle_for(case)
        u = case.u0.copy(order="F")
        t, _ = o.run(u, 0.0, case.tfinal)
        rj, rg = o.gauss()
        ex = case.exact(1, rg, t)
        e1, _ = o.norms(u[0], ex)
        n1, _ = o.norms(np.zeros(o.np), ex)
        errs.append(e1 / n1)
        assert u[0].min() >= 0.0
    assert errs[1] < 0.6 * errs[0]
    assert 0.02 < errs[0] < 0.3 and 0.005 < errs[1] < 0.1


def test_oracle_regression_vectors(golden):
    """The oracle reproduces its committed trajectories bit for bit."""
    g = np.load(golden / "oracle_thacker_cav02.npz")
    m = _mesh(golden, "0.2")
    case = C.thacker_case(m, periods=1.0, cfl=0.3)
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    t = 0.0
    for s in range(20):
        t = o.rk3_step(u, t)
    np.testing.assert_array_equal(u, g["states"][2])
    g2 = np.load(golden / "oracle_dam21.npz")
    case = C.dam_break_case(n=21, tfinal=0.05)
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    t, n = o.run(u, 0.0, case.tfinal)
    assert n == int(g2["nsteps"])
    np.testing.assert_array_equal(u, g2["u"])


def test_two_triangle_matrices():
    """Hand-computable P1 matrices on the unit square cut in two triangles."""
    rr = np.array([[0.0, 1.0, 1.0, 0.0], [0.0, 0.0, 1.0, 1.0]])
    jj = np.array([[1, 2, 3], [1, 3, 4]]).T
    o = oracle.Oracle(jj, rr)
    mt = o.matrices()
    np.testing.assert_allclose(mt["lumped"].sum(), 1.0, rtol=1e-15)
    np.testing.assert_allclose(mt["lumped"], [1 / 3, 1 / 6, 1 / 3, 1 / 6], rtol=1e-14)
    ia = mt["ia"] - 1
    for i in range(4):
        sl = slice(ia[i], ia[i + 1])
        assert abs(mt["cx"][sl].sum()) < 1e-15 and abs(mt["cy"][sl].sum()) < 1e-15   # sum_j c_ij = 0
    # c_ij + c_ji = boundary integral of phi_i phi_j n (= 0 for the interior diagonal edge 1-3)
    def c(i, j):
        p = [q for q in range(ia[i], ia[i + 1]) if mt["ja"][q] - 1 == j][0]
        return mt["cx"][p], mt["cy"][p]
    cx13, cy13 = c(0, 2)
    cx31, cy31 = c(2, 0)
    assert abs(cx13 + cx31) < 1e-15 and abs(cy13 + cy31) < 1e-15


def _lambda_py(ul, ur, n, g, htiny):
    """Independent restatement of compute_lambda_vacc (SOURCES/condlim.f90:879-957)
    returning (lambda, case)."""
    def ovh(h):
        return 2 * h / (h * h + max(h, htiny) ** 2)

    def phi(h, vl, hl, vr, hr):
        def f(hk):
            if h > hk:
                return (h - hk) * math.sqrt((g / 2) * (ovh(h) + ovh(hk)))
            return 2 * (math.sqrt(g * h) - math.sqrt(g * hk))
        return f(hl) + f(hr) + vr - vl

    hl, hr = ul[0], ur[0]
    vl = (ul[1] * n[0] + ul[2] * n[1]) * ovh(hl)
    vr = (ur[1] * n[0] + ur[2] * n[1]) * ovh(hr)
    sql, sqr = math.sqrt(g * abs(hl)), math.sqrt(g * abs(hr))
    x0 = (2 * math.sqrt(2) - 1) ** 2
    hmin, hmax = (hl, hr) if hl <= hr else (hr, hl)
    if phi(x0 * hmin, vl, hl, vr, hr) >= 0:
        case = 1
        ht = min(x0 * hmin, max(vl - vr + 2 * sql + 2 * sqr, 0) ** 2 / (16 * g))
    elif phi(x0 * hmax, vl, hl, vr, hr) >= 0:
        case = 2
        a = 1 / (2 * math.sqrt(2))
        sm, sM = math.sqrt(hmin), math.sqrt(hmax)
        cc = -hmin * a - sm * sM + sm * (vr - vl) / (2 * math.sqrt(g))
        ht = min(x0 * hmax, ((-sm + math.sqrt(hmin - 4 * a * cc)) / (2 * a)) ** 2)
    else:
        case = 3
        sm, sM = math.sqrt(hmin), math.sqrt(hmax)
        ht = sm * sM * (1 + math.sqrt(2 / g) * (vl - vr) / (sm + sM))
    lbdl = vl - sql * math.sqrt((1 + max((ht - hl) * ovh(hl) / 2, 0)) * (1 + max((ht - hl) * ovh(hl), 0)))
    lbdr = vr + sqr * math.sqrt((1 + max((ht - hr) * ovh(hr) / 2, 0)) * (1 + max((ht - hr) * ovh(hr), 0)))
    return max(abs(lbdl), abs(lbdr)), case


@pytest.mark.parametrize("ul,ur,case", [
    ((1.0, 2.0, 0.0), (1.0, -2.0, 0.0), 1),      # colliding states, h* <= x0 hmin
    ((1.0, -3.0, 0.0), (0.1, 3.0, 0.0), 1),      # rarefactions
    ((1.0, 3.0, 0.0), (0.1, -0.3, 0.0), 2),      # x0 hmin < h* <= x0 hmax
    ((1.0, 0.0, 0.0), (0.0, 0.0, 0.0), 2),       # dry right state (vacuum)
    ((1.0, 8.0, 0.0), (0.5, -4.0, 0.0), 3),      # strong collision, h* > x0 hmax
    ((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 1),       # both dry
])
def test_lambda_known_answers(ul, ur, case):
    """compute_lambda_vacc on the three cases including vacuum: the C oracle
    (through compute_dij on a two-triangle mesh) against an independent Python
    restatement; the two-node edge makes d_12 = |c_12| lambda."""
    g, htiny = 9.81, 1e-4
    lam, cse = _lambda_py(ul, ur, (1.0, 0.0), g, htiny)
    assert cse == case
    rr = np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    jj = np.array([[1, 2, 3]]).T
    o = oracle.Oracle(jj, rr)
    p = C.Params(gravity=g, htiny=htiny, cfl=0.1)
    o.set_params(oracle.Params(*p.fields()))
    mt = o.matrices()
    ia = mt["ia"] - 1
    p12 = [q for q in range(ia[0], ia[1]) if mt["ja"][q] == 2][0]
    cx, cy = mt["cx"][p12], mt["cy"][p12]
    nrm = math.hypot(cx, cy)
    n = (cx / nrm, cy / nrm)
    lam, _ = _lambda_py(ul, ur, n, g, htiny)
    u = np.zeros((3, 3), order="F")
    u[:, 0], u[:, 1], u[:, 2] = ul, ur, ul
    dij, _ = o.compute_dij(u)
    assert dij[p12] == pytest.approx(nrm * lam, rel=1e-14, abs=1e-300)


def test_lake_at_rest_wet_is_preserved():
    """Well-balancing: eta = const over random bathymetry, q = 0, all wet."""
    mesh = M.jittered_mesh(12, 12, 0.0, 1.0, 0.0, 1.0, seed=5)
    rng = np.random.default_rng(0)
    z = 0.2 * rng.random(mesh["rr"].shape[1])
    h = 1.0 - z
    u0 = np.asfortranarray(np.vstack([h, 0 * h, 0 * h]))
    case = C.Case("lake", mesh, C.Params(cfl=0.25, max_water_h=1.0, htiny=1e-4), z, u0, 1.0)
    o = _oracle_for(case)
    u = u0.copy(order="F")
    t = 0.0
    for _ in range(10):
        t = o.rk3_step(u, t)
    assert np.abs(u[0] - h).max() < 1e-13
    assert np.abs(u[1:]).max() < 1e-13


def test_dam_break_positivity_and_walls():
    case = C.dam_break_case(n=21, tfinal=0.1)
    case.u0[0] = np.where(case.mesh["rr"][0] < 0.5, 1.0, 0.0)   # dry downstream bed
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    t, n = o.run(u, 0.0, case.tfinal)
    assert n > 5 and u[0].min() >= 0.0
    for comp, js, vals in case.dirichlet:
        np.testing.assert_array_equal(u[comp, js - 1], vals)


def test_negative_depth_is_reported():
    """check_hmin's STOP becomes an error code (no crash)."""
    case = C.dam_break_case(n=11, tfinal=0.1)
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    u[0, 5] = -0.5
    p = o.get_params(); p.dt = 1e-6; o.set_params(p)
    with pytest.raises(oracle.OracleError) as ei:
        o.euler(u)
    assert ei.value.code == 1


def _fct_generic_py(ia, ja, u, maxn, minn, f, dg):
    """Independent restatement of FCT_generic (SOURCES/SAFE/fct.f90:3-43)."""
    n = len(u)
    rp, rm = np.zeros(n), np.zeros(n)
    for i in range(n):
        pp, pm = 1e-15, -1e-15
        for p in range(ia[i], ia[i + 1]):
            if f[p] >= 0:
                pp += f[p]
            else:
                pm += f[p]
        rp[i] = min(dg[i] * (maxn[i] - u[i]) / pp, 1.0)
        rm[i] = min(dg[i] * (minn[i] - u[i]) / pm, 1.0)
    out = u.copy()
    for i in range(n):
        x = 0.0
        for p in range(ia[i], ia[i + 1]):
            j = ja[p]
            l = min(rp[i], rm[j]) if f[p] >= 0 else min(rm[i], rp[j])
            x += l * f[p]
        out[i] = u[i] + x / dg[i]
    return out


def test_fct_generic_known_answer_and_bounds():
    """FCT_generic against a Python restatement, and Zalesak's property: with
    antisymmetric fluxes and stencil bounds, the limited state stays within
    the bounds of each node's stencil."""
    mesh = M.jittered_mesh(9, 9, 0.0, 1.0, 0.0, 1.0, seed=4)
    o = oracle.Oracle(mesh["jj"], mesh["rr"])
    mt = o.matrices()
    ia, ja = mt["ia"] - 1, mt["ja"] - 1
    n = len(ia) - 1
    rng = np.random.default_rng(5)
    u = rng.random(n)
    maxn = np.array([u[ja[ia[i]:ia[i + 1]]].max() for i in range(n)])
    minn = np.array([u[ja[ia[i]:ia[i + 1]]].min() for i in range(n)])
    f = np.zeros(len(ja))
    pos = {(i, ja[p]): p for i in range(n) for p in range(ia[i], ia[i + 1])}
    for (i, j), p in pos.items():                 # f_ij = -f_ji, f_ii = 0
        if i < j:
            v = rng.normal() * 0.05
            f[p], f[pos[(j, i)]] = v, -v
    dg = mt["lumped"]
    got = o.fct_generic(u, maxn, minn, f, dg)
    ref = _fct_generic_py(ia, ja, u, maxn, minn, f, dg)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-14)
    assert np.all(got <= maxn + 1e-12) and np.all(got >= minn - 1e-12)
    # conservation: sum dg u is unchanged by antisymmetric limited fluxes
    assert abs(np.dot(dg, got) - np.dot(dg, u)) < 1e-13
    # unlimited case: wide bounds pass the fluxes through
    wide = o.fct_generic(u, maxn + 1e3, minn - 1e3, f, dg)
    fsum = np.array([f[ia[i]:ia[i + 1]].sum() for i in range(n)])
    np.testing.assert_allclose(wide, u + fsum / dg, rtol=0, atol=1e-13)


@pytest.mark.parametrize("visc,vtype,roundoff", [
    ("viscous", 1, 1), ("viscous", 2, 1), ("viscous", 2, 0), ("entropy_visc", 2, 1), ("entropy_visc", 2, 0),
    ("fct", 2, 0), ("galerkin", 2, 1)])
def test_viscosity_modes_lake_at_rest_and_mass(visc, vtype, roundoff):
    """Every viscosity mode of euler (update.f90:134-289) in the oracle: the
    wet lake at rest stays at rest (the hydrostatic reconstruction balances
    the topography term in each RHS form), and a dam break stays finite and,
    for the 'type2' viscous modes, non-negative.  (Mass is not an invariant
    of the reference: d_ij is not symmetric on boundary rows.)"""
    mesh = M.jittered_mesh(12, 12, 0.0, 1.0, 0.0, 1.0, seed=5)
    rng = np.random.default_rng(0)
    z = 0.2 * rng.random(mesh["rr"].shape[1])
    h = 1.0 - z
    p = C.Params(cfl=0.25, max_water_h=1.0, htiny=1e-4, viscosity_type=C.VISC[visc], viscous_type=vtype,
                 if_roundoff_fix=roundoff)
    u0 = np.asfortranarray(np.vstack([h, 0 * h, 0 * h]))
    o = _oracle_for(C.Case("lake", mesh, p, z, u0, 1.0))
    u = u0.copy(order="F")
    t = 0.0
    for _ in range(5):
        t = o.rk3_step(u, t)
    tol = 1e-12 if vtype == 2 else 1e-10
    assert np.abs(u[0] - h).max() < tol and np.abs(u[1:]).max() < tol
    base = C.dam_break_case(n=21, tfinal=0.02)
    from dataclasses import replace
    case = replace(base, params=replace(base.params, viscosity_type=C.VISC[visc], viscous_type=vtype,
                                        if_roundoff_fix=roundoff))
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    for _ in range(5):
        o.rk3_step(u, 0.0)
    assert np.isfinite(u).all()
    if vtype == 2 and visc != "galerkin":
        assert u[0].min() >= 0.0

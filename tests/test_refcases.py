"""The reference's test cases (init / sol_anal / bdy of SOURCES/condlim.f90
and SOURCES/main.f90) on the host and the oracle: every case sets up and
steps; the per-call time loop (main.f90:61-91 through euler and bdy) equals
the oracle's own loop bit for bit; the closed-form solutions satisfy the
equations they solve; the reference's data files set up their runs."""
import math

import numpy as np
import pytest

import oracle
from conftest import REF_CASES, GOLDEN, OraclePerCall
from swe import data as D, mesh as M, refcases as R
from swe.update import from_case


def _oracle(case, dirichlet=True):
    o = oracle.Oracle(case.mesh["jj"], case.mesh["rr"])
    o.set_params(oracle.Params(*case.params.fields()))
    o.set_bath(case.bath)
    if dirichlet:
        for comp, js, vals in case.dirichlet:
            o.set_dirichlet(comp, js, vals)
    return o


@pytest.mark.parametrize("tt", sorted(REF_CASES))
def test_reference_case_host_loop_equals_oracle_loop(ref_case, tt):
    """Ten steps of main.f90's loop written on the host over per-call euler
    and bdy equal ten steps of the oracle's loop with fixed Dirichlet data,
    bit for bit; depths stay >= 0 and the boundary values are in place."""
    case = ref_case(tt)
    assert case.bdy_fixed
    o = _oracle(case)
    u = case.u0.copy(order="F")
    t = case.t0
    for _ in range(10):
        t = o.rk3_step(u, t)
    uh, th, n = R.host_time_loop(OraclePerCall(_oracle(case, dirichlet=False)), case.bdy, case.u0, case.t0, 1e30, 10)
    assert n == 10 and th == t
    np.testing.assert_array_equal(uh, u)
    assert np.all(np.isfinite(u)) and u[0].min() >= 0.0
    for comp, js, vals in case.dirichlet:
        np.testing.assert_array_equal(u[comp, js - 1], vals)


def test_init_fields_follow_the_reference():
    """gravity, max_water_h and htiny = 1e-4 max_water_h per init
    (condlim.f90:116-229); type 4 starts at t = 1; types 5 and 11 impose
    their own final time; h0 = 0.32 of type 8 is a single-precision
    literal."""
    rr = np.array([[10.0, 0.0, 15.0], [0.5, 0.0, 13.0]])
    want = {1: (1.0, 0.2), 2: (9.81, 0.2), 3: (9.81, 2.0), 4: (9.81, 0.005), 5: (9.81, 4.0), 6: (9.81, 2.0),
            7: (9.81, 2.0), 8: (9.81, float(np.float32(0.32))), 11: (9.81, 4.0), 12: (9.81, 6.0), 13: (9.81, 0.11)}
    for tt, (g, mwh) in want.items():
        ini = R.init(tt, rr)
        assert (ini["gravity"], ini["max_water_h"]) == (g, mwh)
        assert ini["htiny"] == 1.e-4 * mwh
        assert ini["t0"] == (1.0 if tt == 4 else 0.0)
        assert (ini["tfinal"] is not None) == (tt in (5, 11))
    assert R.H0_ISLAND != 0.32 and R.H0_ISLAND == float(np.float32(0.32))
    assert R.init(2, rr)["bath"][0] == 0.2                       # bump top at x = 10
    assert R.init(8, rr)["bath"][2] == 0.625                     # island top (htop)
    omega = math.sqrt(2 * 9.81 * 0.1)
    assert R.init(5, rr)["tfinal"] == 6.0 * math.acos(-1.0) / omega


def test_subcritical_bump_is_the_bernoulli_root():
    """Type 3 at t > 0: h solves h**3 + b h**2 + d = 0 (the steady
    Bernoulli relation q0**2/(2 g h**2) + h + z = const) on the subcritical
    branch, with q = q0."""
    x = np.linspace(0.0, 25.0, 501)
    rr = np.vstack([x, np.zeros_like(x)])
    g, q0, hL = 9.81, 4.42, 2.0
    h = R.sol_anal(3, 1, rr, 1.0, np.zeros(501), g, 2e-4)
    z = np.maximum(0.0, R._bump(x))
    ber = q0 ** 2 / (2 * g * h ** 2) + h + z
    assert np.allclose(ber, q0 ** 2 / (2 * g * hL ** 2) + hL, rtol=1e-12, atol=0)
    assert np.all(q0 / h < np.sqrt(g * h))                       # subcritical everywhere
    assert np.all(R.sol_anal(3, 2, rr, 1.0, None, g, 2e-4) == q0)
    np.testing.assert_array_equal(R.sol_anal(3, 1, rr, 0.0, None, g, 2e-4), hL - z)


def test_critical_bump_jump_conserves_momentum_flux():
    """Type 7: the pre- and post-shock depths at x = 11.7 conserve
    q0**2/h + g h**2/2 (the hydraulic jump); upstream of the crest the flow
    is subcritical, between crest and shock supercritical."""
    g, q0, xs = 9.81, 0.18, 11.7
    eps = 1e-9
    rr = np.array([[xs - eps, xs + eps, 5.0, 11.0], [0.0, 0.0, 0.0, 0.0]])
    h = R.sol_anal(7, 1, rr, 1.0, None, g, 2e-4)
    M = lambda d: q0 ** 2 / d + g * d ** 2 / 2
    assert M(h[0]) == pytest.approx(M(h[1]), rel=1e-6)
    assert h[0] < (q0 ** 2 / g) ** (1 / 3) < h[1]                # super- then subcritical
    assert q0 / h[2] < math.sqrt(g * h[2]) and q0 / h[3] > math.sqrt(g * h[3])


def test_dam_break_rarefaction_is_continuous():
    """Type 4 (Ritter): h = hL up to x0 - t c, the fan down to 0 at
    x0 + 2 t c, htiny beyond; q is continuous and zero outside the fan."""
    g, hL, t = 9.81, 0.005, 2.0
    c = math.sqrt(g * hL)
    e = 1e-9
    x = 5.0 + np.array([-t * c - e, -t * c + e, 2 * t * c - e, 2 * t * c + e, 0.0])
    rr = np.vstack([x, np.zeros(5)])
    h = R.sol_anal(4, 1, rr, t, None, g, 5e-7)
    q = R.sol_anal(4, 2, rr, t, None, g, 5e-7)
    assert h[0] == hL and h[1] == pytest.approx(hL, rel=1e-8) and h[3] == 5e-7
    assert h[2] == pytest.approx(0.0, abs=1e-15)
    assert h[4] == pytest.approx(4 / (9 * g) * c ** 2, rel=1e-14)
    assert q[0] == 0.0 and q[1] == pytest.approx(0.0, abs=1e-10) and q[3] == 0.0
    assert q[4] == pytest.approx(8 / (27 * g) * c ** 3, rel=1e-14)


def test_paraboloid_cases_keep_a_planar_surface():
    """Types 11 (friction) and 12 (Coriolis): where wet, h + z is a plane in
    x, y at every t, and the velocity q/h is uniform over the wet set."""
    x, y = np.meshgrid(np.linspace(1.0, 3.0, 9), np.linspace(1.0, 3.0, 9))
    for tt, shift in ((11, 0.0), (12, -2.0)):
        rr = np.vstack([x.ravel() + shift, y.ravel() + shift])
        ini = R.init(tt, rr)
        for t in (0.3, 1.7):
            h = R.sol_anal(tt, 1, rr, t, ini["bath"], 9.81, ini["htiny"])
            wet = h > 0
            eta = h[wet] + ini["bath"][wet]
            A = np.c_[rr[0, wet], rr[1, wet], np.ones(wet.sum())]
            coef, res, *_ = np.linalg.lstsq(A, eta, rcond=None)
            assert np.abs(A @ coef - eta).max() < 1e-13
            for k in (2, 3):
                v = R.sol_anal(tt, k, rr, t, ini["bath"], 9.81, ini["htiny"])[wet] / h[wet]
                assert np.ptp(v) < 1e-12 * max(1.0, np.abs(v).max())


def test_sol_anal_reads_bath_by_position():
    """sol_anal of types 1 and 2 indexes the module bath by the position in
    rr: on a subset of n nodes it reads bath of nodes 1..n (the reference's
    own behaviour, kept)."""
    bath = np.array([0.3, 0.0, 0.05, 0.5])
    sub = np.zeros((2, 2))
    np.testing.assert_array_equal(R.sol_anal(1, 1, sub, 1.0, bath, 1.0, 2e-5), [0.0, 0.2])
    np.testing.assert_array_equal(R.sol_anal(2, 1, sub, 1.0, bath, 9.81, 2e-5), [0.0, 0.1])


def test_cases_the_reference_cannot_run_are_refused():
    rr = np.zeros((2, 3))
    with pytest.raises(ValueError, match="Malpasset"):
        R.init(9, rr)
    with pytest.raises(ValueError, match="BUG in init"):
        R.init(10, rr)
    with pytest.raises(ValueError, match="undefined"):
        R.sol_anal(13, 4, rr, 0.5, None, 9.81, 1e-5)
    R.sol_anal(13, 4, rr, 0.0, None, 9.81, 1e-5)                   # defined at t = 0


def test_reference_data_files_set_up_their_runs():
    """SOURCES/data: type 13 ('entropy_visc', CFL 0.08, lambdaSGN 9, h
    imposed on sides 1 and 3 of the SGN channel); the solitary wave moves,
    so the values at the channel ends change with time: the case lists them
    as analytic data, which the device loop evaluates at every stage (or the
    per-call loop imposes on the host).  With qx imposed too, type 13's bdy
    writes its fourth unknown, which sol_anal leaves undefined for t > 0:
    no analytic data, the per-call loop only.  PARABOLOID/data: type 12 on
    the disk with h, qx, qy imposed on its one side; the rim is dry, so the
    values are fixed (zero) and the device loop runs it."""
    d = D.read_my_data(GOLDEN / "ref_data_sources.txt")
    mesh = M.load_mesh_free_format(GOLDEN / "ref_rectangle.1.FEM.gz")
    case = R.case_from_data(d, mesh)
    assert case.params.syst_size == 5 and case.params.viscosity_type == 2 and case.params.lambda_sgn == 9.0
    assert not case.bdy_fixed and case.dirichlet == [] and case.tfinal == 5.0
    ends = M.dirichlet_nodes(mesh["jjs"], mesh["sides"], [1, 3])
    assert len(case.dirichlet_anal) == 1 and case.dirichlet_anal[0][0] == 0
    np.testing.assert_array_equal(np.sort(case.dirichlet_anal[0][1]), np.sort(ends))
    d2 = dict(d, ux_nb_Dir_bdy=1, ux_Dir_list=[1])
    case2 = R.case_from_data(d2, mesh)
    assert not case2.bdy_fixed and case2.dirichlet_anal == []
    with pytest.raises(ValueError, match="per_call"):
        from_case(case2)
    u = case.u0.copy(order="F")
    case.bdy(u, 0.5)
    np.testing.assert_array_equal(u[0, ends - 1], R.sol_anal(13, 1, mesh["rr"][:, ends - 1], 0.5, None, 9.81,
                                                             case.params.htiny))
    o = _oracle(case)
    uh, th, n = R.host_time_loop(OraclePerCall(o), case.bdy, case.u0, 0.0, 1e30, 3)
    assert n == 3 and np.all(np.isfinite(uh)) and uh[0].min() > 0.09

    d = D.read_my_data(GOLDEN / "ref_data_paraboloid.txt")
    mesh = M.load_mesh_free_format(GOLDEN / "ref_cdisk.1_mesh.FEM.gz")
    case = R.case_from_data(d, mesh)
    assert case.bdy_fixed and case.params.type_test == 12 and case.params.viscosity_type == 1
    assert [c for c, _, _ in case.dirichlet] == [0, 1, 2]
    assert all(np.all(v == 0.0) for _, _, v in case.dirichlet)


def test_gzip_mesh_fixture_reads_like_the_plain_file(tmp_path):
    import gzip
    raw = gzip.decompress((GOLDEN / "ref_rectangle.1.FEM.gz").read_bytes())
    (tmp_path / "r.FEM").write_bytes(raw)
    a = M.load_mesh_free_format(tmp_path / "r.FEM")
    b = M.load_mesh_free_format(GOLDEN / "ref_rectangle.1.FEM.gz")
    for k in ("jj", "rr", "jjs", "sides"):
        np.testing.assert_array_equal(a[k], b[k])

"""CUDA path (through the C ABI) against the FP64 oracle and the committed
golden vectors.

FP64 path: bit-exact.  The FP64 kernels keep the reference's evaluation order
and are built without FMA contraction, so setup matrices, d_ij, every stage
intermediate and whole RK3 trajectories must equal the oracle exactly
(Manning friction uses pow() and is held to 1e-12 relative instead).

Mixed path: relative L1 difference of h against the FP64 oracle <= 1e-5
(the target tolerance), h >= 0.
"""
import math
from dataclasses import replace

import numpy as np
import pytest

import oracle
from swe import cases as C, mesh as M
from swe import lib as L
from swe.update import Update, from_case
from conftest import REF_CASES, OraclePerCall

pytestmark = pytest.mark.gpu

MIXED_L1_TOL = 1e-5


def _oracle_for(case):
    o = oracle.Oracle(case.mesh["jj"], case.mesh["rr"])
    o.set_params(oracle.Params(*case.params.fields()))
    o.set_bath(case.bath)
    for comp, js, vals in case.dirichlet:
        o.set_dirichlet(comp, js, vals)
    return o


def _thacker(golden, h="0.2", **kw):
    d = np.load(golden / f"mesh_cav_{h}.npz")
    return C.thacker_case({k: d[k] for k in d.files}, **kw)


def _rel_l1(a, b, w):
    return float(np.sum(w * np.abs(a - b)) / np.sum(w * np.abs(b)))


def test_setup_matrices_bit_exact(golden):
    case = _thacker(golden, "0.1", periods=1.0, cfl=0.3)
    upd = from_case(case)
    o = _oracle_for(case)
    a, b = upd.matrices(), o.matrices()
    for k in ("ia", "ja", "diag", "mass", "lumped", "cx", "cy"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("h", ["0.2", "0.05"])
def test_compute_dij_bit_exact(golden, h):
    case = _thacker(golden, h, periods=1.0, cfl=0.3)
    upd = from_case(case)
    o = _oracle_for(case)
    d_gpu, dt_gpu = upd.compute_dij(case.u0)
    d_orc, dt_orc = o.compute_dij(case.u0)
    np.testing.assert_array_equal(d_gpu, d_orc)
    assert dt_gpu == dt_orc


def test_euler_stage_and_intermediates_bit_exact(golden):
    case = _thacker(golden, "0.2", periods=1.0, cfl=0.3)
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    t = 0.0
    for _ in range(15):                     # a state with wet/dry fronts moving
        t = o.rk3_step(u, t)
    _, dt = o.compute_dij(u)
    p = replace(case.params, dt=dt)
    o.set_params(oracle.Params(*p.fields()))
    upd = from_case(case)
    upd.set_params(p)
    out_o, dump = o.euler(u, dump=True)
    out_g = upd.euler(u)
    inter = upd.euler_intermediates()
    np.testing.assert_array_equal(out_g, out_o)
    for k in ("dij_low", "muij_low", "alpha", "u_low", "res", "fctmat", "rminus", "lij"):
        np.testing.assert_array_equal(inter[k], dump[k], err_msg=k)


MODES = [  # (viscosity_type, viscous_type, if_roundoff_fix)
    ("galerkin", 2, 1), ("viscous", 1, 1), ("viscous", 2, 1), ("viscous", 2, 0),
    ("entropy_visc", 2, 1), ("entropy_visc", 2, 0), ("fct", 2, 0),
]


@pytest.mark.parametrize("visc,vtype,roundoff", MODES)
def test_viscosity_modes_fp64_bit_exact(visc, vtype, roundoff):
    """Every viscosity_type / viscous_type / roundoff combination of euler
    (update.f90:134-289): one stage and three RK3 steps equal the oracle."""
    base = C.dam_break_case(n=21, tfinal=0.05)
    p = replace(base.params, viscosity_type=C.VISC[visc], viscous_type=vtype, if_roundoff_fix=roundoff)
    case = replace(base, params=p)
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    _, dt = o.compute_dij(u)
    pd = replace(p, dt=dt)
    o.set_params(oracle.Params(*pd.fields()))
    upd = from_case(case)
    upd.set_params(pd)
    np.testing.assert_array_equal(upd.euler(u), o.euler(u))
    o.set_params(oracle.Params(*p.fields()))
    upd.set_params(p)
    t = 0.0
    for _ in range(3):
        t = o.rk3_step(u, t)
    upd.upload(case.u0)
    upd.set_time(0.0, 1e30)
    upd.rk3_steps(3)
    np.testing.assert_array_equal(upd.download(), u)


@pytest.mark.parametrize("roundoff", [1, 0])
@pytest.mark.parametrize("prec", [1, 2])
@pytest.mark.parametrize("visc", ["galerkin", "viscous", "entropy_visc"])
def test_viscosity_modes_mixed(visc, prec, roundoff):
    """'galerkin', 'viscous' and 'entropy_visc' ('type2', with and without the
    roundoff fix) in mixed precision and its FP64 split against the FP64
    oracle, on the dam break and on the wet/dry Gaussian-bump basin ('entropy_visc'
    has no positivity limiter: on the wet/dry basin the reference scheme itself
    STOPs with Min h<0, so that mode runs the dam break only)."""
    cases = [(C.dam_break_case(n=41, tfinal=0.05), 5)]
    if visc != "entropy_visc":
        cases.append((C.bump_basin_case(n=40), 10))
    for base, k in cases:
        p = replace(base.params, viscosity_type=C.VISC[visc], precision=prec, if_roundoff_fix=roundoff)
        case = replace(base, params=p)
        u, ug, n, ng, lump = _mixed_vs_oracle(case, nsteps=k, prec=prec)
        assert ug[0].min() >= 0.0
        assert _rel_l1(ug[0], u[0], lump) <= MIXED_L1_TOL, (base.name, _rel_l1(ug[0], u[0], lump))


@pytest.mark.parametrize("prec", [1, 2])
def test_viscous_type1_mixed(prec):
    """'viscous' with 'type1' (smb_1's centred flux and pressure term) in
    mixed precision and its FP64 split against the FP64 oracle."""
    for base, k in ((C.dam_break_case(n=41, tfinal=0.05), 5), (C.bump_basin_case(n=40), 10)):
        p = replace(base.params, viscosity_type=C.VISC["viscous"], viscous_type=1, precision=prec)
        case = replace(base, params=p)
        u, ug, n, ng, lump = _mixed_vs_oracle(case, nsteps=k, prec=prec)
        assert _rel_l1(ug[0], u[0], lump) <= MIXED_L1_TOL, (base.name, _rel_l1(ug[0], u[0], lump))


def test_mode_combinations_the_reference_stops_on():
    base = C.dam_break_case(n=11)
    for visc in ("entropy_visc", "fct"):
        p = replace(base.params, viscosity_type=C.VISC[visc], viscous_type=1)
        with pytest.raises(L.SweError) as ei:
            from_case(replace(base, params=p))
        assert ei.value.code == L.SWE_ERR_ARG
    sgn = C.sgn_case(nx=41, ny=3, nsteps=1)
    p = replace(sgn.params, viscosity_type=C.VISC["viscous"], viscous_type=1, precision=1)
    with pytest.raises(L.SweError):      # mixed 'type1' is built for 3-component systems
        from_case(replace(sgn, params=p))


def test_device_norms_match_oracle(golden):
    """compute_errors' quadrature norms on the device state vs the oracle
    (ns_anal_l1, ns_anal_0; order-independent sums: 1e-13 relative)."""
    case = _thacker(golden, "0.1", periods=1.0, cfl=0.3)
    for prec in (0, 1):
        upd = from_case(case, precision=prec)
        o = _oracle_for(case)
        rj_g, rg_g = upd.gauss_points()
        rj_o, rg_o = o.gauss()
        np.testing.assert_array_equal(rj_g, rj_o)
        np.testing.assert_array_equal(rg_g, rg_o)
        upd.upload(case.u0)
        upd.set_time(0.0, 1e30)
        upd.rk3_steps(10)
        u = upd.download()
        ex = case.exact(1, rg_o, 0.0)
        for field, f_anal in ((0, ex), (0, None), (1, None), (L.FIELD_H32, None)):
            g1, g2 = upd.norms(field, f_anal)
            ff = u[0] * np.sqrt(u[0]) if field == L.FIELD_H32 else u[field]
            o1, o2 = o.norms(ff, np.zeros_like(rj_o) if f_anal is None else f_anal)
            assert g1 == pytest.approx(o1, rel=1e-13, abs=1e-300)
            assert g2 == pytest.approx(o2, rel=1e-13, abs=1e-300)


def test_fct_positivity_operator_bit_exact():
    rng = np.random.default_rng(7)
    mesh = M.jittered_mesh(15, 15, 0, 1, 0, 1, seed=7)
    case = C.Case("x", mesh, C.Params(htiny=1e-3, dt=1e-3), np.zeros(225), np.zeros((3, 225), order="F"), 1.0)
    upd = from_case(case)
    o = _oracle_for(case)
    nnz = upd.sizes()[1]
    hs = rng.random(225) * 2e-3        # straddles the htiny test
    f = rng.normal(size=nnz)
    np.testing.assert_array_equal(upd.fct_positivity(hs, f), o.fct_positivity(hs, f))


def test_fct_generic_operator_bit_exact():
    """FCT_generic (two-sided Zalesak, SAFE/fct.f90:3-43) through the C ABI vs
    the oracle: random bounds that make some R+- < 1 and zero fluxes."""
    rng = np.random.default_rng(8)
    mesh = M.jittered_mesh(17, 13, 0, 1, 0, 1, seed=8)
    n = mesh["rr"].shape[1]
    case = C.Case("x", mesh, C.Params(htiny=1e-3, dt=1e-3), np.zeros(n), np.zeros((3, n), order="F"), 1.0)
    upd = from_case(case)
    o = _oracle_for(case)
    nnz = upd.sizes()[1]
    u = rng.random(n)
    maxn = u + rng.random(n) * 0.02
    minn = u - rng.random(n) * 0.02
    f = rng.normal(size=nnz) * 0.01
    f[rng.random(nnz) < 0.1] = 0.0
    lump = o.matrices()["lumped"]
    np.testing.assert_array_equal(upd.fct_generic(u, maxn, minn, f), o.fct_generic(u, maxn, minn, f, lump))
    dg = rng.random(n) + 0.5
    np.testing.assert_array_equal(upd.fct_generic(u, maxn, minn, f, dg), o.fct_generic(u, maxn, minn, f, dg))


def test_rk3_trajectory_matches_golden(golden):
    """Device-resident graph-captured RK3 loop vs the committed oracle
    trajectory (bit-exact)."""
    g = np.load(golden / "oracle_thacker_cav02.npz")
    case = _thacker(golden, "0.2", periods=1.0, cfl=0.3)
    upd = from_case(case)
    upd.upload(case.u0)
    upd.set_time(0.0, case.tfinal)
    t_all = 0.0
    for k in range(1, len(g["states"])):
        t, dt, n = upd.rk3_steps(int(g["steps_per_state"]))
        assert n == int(g["steps_per_state"])
        np.testing.assert_array_equal(upd.download(), g["states"][k])
        assert t[0] == g["times"][k]
    assert upd.last_launch_count > 0


def test_rk3_run_to_tfinal_matches_oracle(golden):
    """DO WHILE(time < Tfinal) with unclipped dt: same step count, same state."""
    g = np.load(golden / "oracle_dam21.npz")
    case = C.dam_break_case(n=21, tfinal=0.05)
    upd = from_case(case)
    upd.upload(case.u0)
    upd.set_time(0.0, case.tfinal)
    t, dt, n = upd.rk3_steps(int(g["nsteps"]) + 7)     # extra steps are no-ops
    assert n == int(g["nsteps"]) and t[0] == float(g["time"])
    np.testing.assert_array_equal(upd.download(), g["u"])


def test_manning_friction_fp64():
    case = C.bump_basin_case(n=30, nsteps=20)
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    t = 0.0
    for _ in range(20):
        t = o.rk3_step(u, t)
    upd = from_case(case)
    upd.upload(case.u0)
    upd.set_time(0.0, 1e30)
    upd.rk3_steps(20)
    ug = upd.download()
    scale = np.abs(u).max(axis=1, keepdims=True)
    assert np.max(np.abs(ug - u) / scale) < 1e-12


def test_batch_equals_single_instances():
    cases = C.batch_instances(n_inst=3, nmin=200, nmax=2000, seed=11)
    items = [(c.mesh, c.bath, c.params) for c in cases]
    upd = Update(batch=items)
    for b, c in enumerate(cases):
        for comp, js, vals in c.dirichlet:
            upd.set_dirichlet(comp, js, vals, inst=b)
    upd.upload([c.u0 for c in cases])
    upd.set_time(0.0, 1e30)
    upd.rk3_steps(12)
    got = upd.download_split()
    for b, c in enumerate(cases):
        o = _oracle_for(c)
        u = c.u0.copy(order="F")
        t = 0.0
        for _ in range(12):
            t = o.rk3_step(u, t)
        scale = np.abs(u).max(axis=1, keepdims=True) + 1e-300
        assert np.max(np.abs(got[b] - u) / scale) < 1e-12, b


def test_batch_tiled_mixed_equals_single_instances(monkeypatch):
    """Mixed path with every kernel in its shared-memory tile variant and
    64-row tiles, so that tiles straddle instances (row offsets are padded to
    32 only): a batch of three instances against each instance alone.  The
    two may run other launch variants, which perform the same operations:
    bit for bit."""
    monkeypatch.setenv("SWE_TILED", "1")
    monkeypatch.setenv("SWE_TILE", "64")
    cases = C.batch_instances(n_inst=3, nmin=200, nmax=2000, seed=11, precision=1)
    upd = Update(batch=[(c.mesh, c.bath, c.params) for c in cases])
    for b, c in enumerate(cases):
        for comp, js, vals in c.dirichlet:
            upd.set_dirichlet(comp, js, vals, inst=b)
    upd.upload([c.u0 for c in cases])
    upd.set_time(0.0, 1e30)
    upd.rk3_steps(12)
    assert "/tiled" in upd.tuning
    got = upd.download_split()
    upd.close()
    for b, c in enumerate(cases):
        one = from_case(c)
        one.upload(c.u0)
        one.set_time(0.0, 1e30)
        one.rk3_steps(12)
        ref = one.download()
        one.close()
        np.testing.assert_array_equal(got[b], ref, err_msg=str(b))


def test_negative_depth_is_reported_not_trapped():
    case = C.dam_break_case(n=11)
    upd = from_case(case)
    u = case.u0.copy(order="F")
    u[0, 5] = -0.5
    upd.set_params(replace(case.params, dt=1e-6))
    with pytest.raises(L.SweError) as ei:
        upd.euler(u)
    assert ei.value.code == L.SWE_ERR_NEG_H
    # the context stays usable
    u[0, 5] = 1.0
    upd.euler(u)


def _mixed_vs_oracle(case, nsteps=None, prec=1):
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    if nsteps is None:
        t, n = o.run(u, 0.0, case.tfinal)
    else:
        t = 0.0
        for _ in range(nsteps):
            t = o.rk3_step(u, t)
        n = nsteps
    upd = from_case(case, precision=prec)
    upd.upload(case.u0)
    upd.set_time(0.0, case.tfinal if nsteps is None else 1e30)
    tg, _, ng = upd.rk3_steps(n + 50 if nsteps is None else n)
    ug = upd.download()
    return u, ug, n, ng, upd.lumped


@pytest.mark.parametrize("prec", [1, 2])
@pytest.mark.parametrize("which", ["dam", "bump"])
def test_mixed_precision_within_tolerance(which, prec):
    """Well-conditioned workloads: relative L1(h) vs the FP64 oracle <= 1e-5,
    for the mixed path and its FP64 precision split (precision 2)."""
    if which == "dam":
        case, nsteps = C.dam_break_case(n=41, tfinal=0.05), None
    else:
        case, nsteps = C.bump_basin_case(n=60), 60
    u, ug, n, ng, lump = _mixed_vs_oracle(case, nsteps, prec)
    err = _rel_l1(ug[0], u[0], lump)
    assert ug[0].min() >= 0.0
    assert abs(ng - n) <= 1
    assert err <= MIXED_L1_TOL, err


def test_mixed_precision_thacker_within_conditioning(golden):
    """The Thacker case with the reference's +htiny film over the dry box is
    ill-conditioned: the FP64 oracle itself moves by ~4e-3 (relative L1 of h)
    after a quarter period when its initial state is perturbed by 1e-7
    relative.  The mixed path must stay within 3x that sensitivity."""
    case = _thacker(golden, "0.1", periods=0.25, cfl=0.3)
    u, ug, n, ng, lump = _mixed_vs_oracle(case)
    rng = np.random.default_rng(0)
    o = _oracle_for(case)
    up = case.u0.copy(order="F")
    up *= 1 + 1e-7 * rng.uniform(-1, 1, up.shape)
    o.run(up, 0.0, case.tfinal)
    sens = _rel_l1(up[0], u[0], lump)
    err = _rel_l1(ug[0], u[0], lump)
    assert ug[0].min() >= 0.0
    assert err <= 3 * sens + MIXED_L1_TOL, (err, sens)


@pytest.mark.parametrize("prec", [0, 1])
def test_mass_monitor(prec):
    """swe_mass adds in a fixed order: the same bits on every call, equal to
    the host's compensated sum to rounding."""
    case = C.dam_break_case(n=21)
    upd = from_case(case, precision=prec)
    upd.upload(case.u0)
    m = upd.total_mass()[0]
    lump = upd.lumped
    assert m == pytest.approx(math.fsum(lump * case.u0[0]), rel=1e-15)
    upd.set_time(0.0, 1e30)
    upd.rk3_steps(3)
    m3 = upd.total_mass()
    for _ in range(3):
        np.testing.assert_array_equal(upd.total_mass(), m3)
    upd.close()


# Relative mass drift bounds.  In a closed basin whose walls the waves have
# not reached, the reference scheme conserves mass to rounding; the mixed
# path's fluxes are FP32 numbers formed independently by the two rows of an
# edge, so its mass moves by the FP32 rounding of the fluxes.
MASS_DRIFT_TOL = {0: 1e-13, 1: 1e-7}


def _circular_dam(prec):
    mesh = M.lattice_mesh(101, 101)
    x, y = mesh["rr"]
    h = np.where((x - 0.5) ** 2 + (y - 0.5) ** 2 < 0.04, 1.0, 0.1)
    u0 = np.asfortranarray(np.vstack([h, 0 * h, 0 * h]))
    p = C.Params(gravity=9.81, cfl=0.25, max_water_h=1.0, htiny=1e-4, type_test=4, precision=prec)
    return C.Case("circular_dam", mesh, p, np.zeros_like(h), u0, 1e30, C._walls(mesh, 3))


@pytest.mark.parametrize("prec", [0, 1])
def test_mass_conserved_in_a_closed_basin(prec):
    """A circular dam (r = 0.2) in the walled unit square, 101x101 lattice,
    100 SSP-RK3 steps (the wave stays clear of the walls): the total mass
    sum m_i h_i, read on the device, stays within MASS_DRIFT_TOL."""
    case = _circular_dam(prec)
    upd = from_case(case)
    upd.upload(case.u0)
    m0 = upd.total_mass()[0]
    upd.set_time(0.0, 1e30)
    _, _, n = upd.rk3_steps(100)
    u = upd.download()
    m1 = upd.total_mass()[0]
    upd.close()
    assert n == 100
    r2 = (case.mesh["rr"][0] - 0.5) ** 2 + (case.mesh["rr"][1] - 0.5) ** 2
    assert np.abs(u[0][r2 > 0.45 ** 2] - 0.1).max() < 1e-12      # walls still at rest
    drift = abs(m1 - m0) / m0
    print(f"closed basin, relative mass drift over 100 steps, precision {prec}: {drift:.3e}")
    assert drift <= MASS_DRIFT_TOL[prec], drift


def test_mass_change_at_walls_follows_the_reference_scheme():
    """C1 (101x101 dam break, reflective walls) for 200 steps.  The
    reference's d_ij = |c_ij| lambda_max is not symmetric on boundary edges
    (c_ij + c_ji is the boundary integral there), so where the depth varies
    along a wall the scheme itself moves mass (here ~3e-7 relative).  The
    FP64 path follows the oracle bit for bit (its mass change is the
    reference scheme's); the mixed path's mass stays within 5e-8 of it."""
    case = C.dam_break_case(n=101)
    mass = {}
    for prec in (0, 1):
        upd = from_case(case, precision=prec)
        upd.upload(case.u0)
        m0 = upd.total_mass()[0]
        upd.set_time(0.0, 1e30)
        upd.rk3_steps(200)
        mass[prec] = upd.total_mass()[0]
        upd.close()
    print(f"C1 mass change over 200 steps: FP64 {(mass[0] - m0) / m0:.3e}, mixed {(mass[1] - m0) / m0:.3e}")
    assert abs(mass[1] - mass[0]) <= 5e-8 * m0


def test_wetdry_basin_full_size_against_oracle():
    """C3 at its full size: the 4M-node wet/dry basin (2000 x 2000 jittered
    lattice on [0, 10]^2, Gaussian-bump bathymetry, Manning friction, dry
    shores), two SSP-RK3 steps from the workload's own initial state, the
    oracle on every host core beside it.  FP64 equals the oracle to 1e-13
    relative (Manning's pow is the one libm call whose last bit may differ
    from the host's); the mixed path and its precision split are within
    1e-8 relative L1(h) (1.6e-9 after 15 steps in bench.py), with h >= 0
    and the same dt as the oracle to FP32 rounding."""
    case = C.bump_basin_case(n=2000, nsteps=200)
    steps = 2
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    t = 0.0
    for _ in range(steps):
        t = o.rk3_step(u, t)
    del o
    for prec in (0, 1, 2):
        upd = from_case(case, precision=prec)
        upd.set_time(0.0, 1e30)
        ug = upd.rk3_steps_host(case.u0, steps)
        tg = upd.get_time()[0][0]
        lump = upd.lumped
        upd.close()
        if prec == 0:
            assert np.max(np.abs(ug - u)) <= 1e-13 * np.max(np.abs(u)), np.max(np.abs(ug - u))
            assert abs(tg - t) <= 1e-13 * t
        else:
            err = _rel_l1(ug[0], u[0], lump)
            print(f"C3 precision {prec} vs oracle after {steps} steps: relative L1(h) {err:.3e}")
            assert ug[0].min() >= 0.0
            assert err <= 1e-8, err
            assert abs(tg - t) <= 1e-6 * t


def test_sgn_channel_full_size_against_oracle():
    """C5 at its full size: the 10001 x 201 SGN channel (2,010,201 nodes, five
    unknowns, mSGN_RHS source, walls on the long sides), the solitary wave,
    five SSP-RK3 steps at CFL 5e-4, which resolves the relaxation waves (at
    the specified CFL 0.1 the reference's scheme itself collapses on this
    mesh: its dt leaves out their speed, 200 times sqrt(g h) here).  FP64
    equals the oracle bit for bit; the mixed path is within 1e-5 relative
    L1(h) and within 3x the oracle's own sensitivity to a 1e-7 perturbation
    of the initial state, plus 1e-9."""
    case = C.sgn_case(cfl=5e-4)
    steps = 5
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    t = 0.0
    for _ in range(steps):
        t = o.rk3_step(u, t)
    up = case.u0.copy(order="F")
    up *= 1 + 1e-7 * np.random.default_rng(0).uniform(-1, 1, up.shape)
    tp = 0.0
    for _ in range(steps):
        tp = o.rk3_step(up, tp)
    del o
    for prec in (0, 1):
        upd = from_case(case, precision=prec)
        upd.set_time(0.0, 1e30)
        ug = upd.rk3_steps_host(case.u0, steps)
        lump = upd.lumped
        upd.close()
        if prec == 0:
            np.testing.assert_array_equal(ug, u)
        else:
            err = _rel_l1(ug[0], u[0], lump)
            sens = _rel_l1(up[0], u[0], lump)
            print(f"C5 mixed vs oracle after {steps} steps: relative L1(h) {err:.3e} (oracle sensitivity {sens:.3e})")
            assert ug[0].min() >= 0.0
            assert err <= MIXED_L1_TOL, err
            assert err <= 3 * sens + 1e-9, (err, sens)


def test_dam_break_full_size_against_oracle():
    """C1 at its full size: the 101x101 lattice dam break run to t = 0.2 (the
    dt of each step from the CFL condition, unclipped at t_final, as in the
    reference).  FP64 equals the oracle bit for bit; mixed is within the
    relative L1 tolerance of h, with h >= 0."""
    case = C.dam_break_case(n=101, tfinal=0.2)
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    t, n = 0.0, 0
    while t < case.tfinal:
        t = o.rk3_step(u, t)
        n += 1
    for prec in (0, 1, 2):
        upd = from_case(case, precision=prec)
        upd.upload(case.u0)
        upd.set_time(0.0, case.tfinal)
        tg, _, ng = upd.rk3_steps(n + 10)
        ug = upd.download()
        lump = upd.lumped
        upd.close()
        assert ng == n
        if prec == 0:
            np.testing.assert_array_equal(ug, u)
            assert tg[0] == t
        else:
            err = _rel_l1(ug[0], u[0], lump)
            print(f"C1 precision {prec} vs oracle after {n} steps: relative L1(h) {err:.3e}")
            assert ug[0].min() >= 0.0
            assert err <= MIXED_L1_TOL, err


def test_set_bath_after_create_equals_create_with_bath(golden):
    """The Fortran driver builds the matrices before init() sets bath."""
    case = _thacker(golden, "0.2", periods=1.0, cfl=0.3)
    a = from_case(case)
    b = Update(case.mesh, np.zeros_like(case.bath), case.params)
    for comp, js, vals in case.dirichlet:
        b.set_dirichlet(comp, js, vals)
    b.set_bath(case.bath)
    for upd in (a, b):
        upd.upload(case.u0)
        upd.set_time(0.0, 1e30)
        upd.rk3_steps(5)
    np.testing.assert_array_equal(a.download(), b.download())


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_lake_at_rest_is_preserved(prec):
    """Well-balancing: eta = const over random bathymetry, q = 0, all wet.
    (The reference's type2 topography term g h_i (eta_j - eta_i) c_ij is not
    balanced where a dry node borders the lake, so the test is all wet.)"""
    mesh = M.jittered_mesh(40, 40, 0.0, 1.0, 0.0, 1.0, seed=9)
    x, y = mesh["rr"]
    rng = np.random.default_rng(3)
    z = 0.2 * rng.random(x.shape) + 0.3 * np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / 0.02)
    h = 0.8 - z
    u0 = np.asfortranarray(np.vstack([h, 0 * h, 0 * h]))
    p = C.Params(cfl=0.25, max_water_h=0.8, htiny=8e-5, precision=prec)
    case = C.Case("lake", mesh, p, z, u0, 1e30)
    upd = from_case(case)
    upd.upload(u0)
    upd.set_time(0.0, 1e30)
    upd.rk3_steps(20)
    u = upd.download()
    # FP64 balances to rounding.  The mixed path carries eta = h + z rounded
    # once per node, so every flux of a lake at rest is exactly 0: q stays 0
    # and h moves only by the double-float RK combinations (~2^-48 relative)
    tol_h, tol_q = (1e-13, 1e-13) if prec == 0 else (1e-13, 0.0)
    assert np.abs(u[0] - h).max() < tol_h
    assert np.abs(u[1:]).max() <= tol_q


def test_sgn_fp64_bit_exact_and_mixed_close():
    """Hyperbolised SGN (type_test 13, five components, mSGN_RHS source).  The
    stiff relaxation makes the case sensitive: the FP64 oracle moves by
    ~1.6e-5 (relative L1 of h) after 10 steps when its initial state is
    perturbed by 1e-7; the mixed path must stay within 3x that."""
    case = C.sgn_case(nx=81, ny=5, Lx=20.0, Ly=1.0, x0=6.0, lambda_sgn=100.0, cfl=0.1)
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    t = 0.0
    for _ in range(10):
        t = o.rk3_step(u, t)
    up = case.u0.copy(order="F")
    up *= 1 + 1e-7 * np.random.default_rng(0).uniform(-1, 1, up.shape)
    t = 0.0
    for _ in range(10):
        t = o.rk3_step(up, t)
    g = from_case(case)
    g.upload(case.u0)
    g.set_time(0.0, 1e30)
    g.rk3_steps(10)
    np.testing.assert_array_equal(g.download(), u)
    mx = from_case(case, precision=1)
    mx.upload(case.u0)
    mx.set_time(0.0, 1e30)
    mx.rk3_steps(10)
    um = mx.download()
    err = _rel_l1(um[0], u[0], mx.lumped)
    sens = _rel_l1(up[0], u[0], mx.lumped)
    assert err <= 3 * sens + MIXED_L1_TOL, (err, sens)
    assert um[0].min() >= 0.0


@pytest.mark.parametrize("prec", [0, 1])
def test_pinned_buffers_read_directly_match_staged_copies(prec):
    """Uploads from / downloads to page-locked host buffers (the e2e path of
    bench.py) equal those of pageable numpy arrays."""
    torch = pytest.importorskip("torch")
    case = C.dam_break_case(n=41)
    upd = from_case(case, precision=prec)
    pin_in = torch.from_numpy(np.asfortranarray(case.u0).ravel(order="F").copy()).pin_memory()
    pin_out = torch.zeros_like(pin_in).pin_memory()
    outs = []
    for pinned in (False, True):
        if pinned:
            upd.upload_ptr(pin_in.data_ptr())
        else:
            upd.upload(case.u0)
        upd.set_time(0.0, 1e30)
        upd.rk3_steps(5)
        if pinned:
            upd.download_ptr(pin_out.data_ptr())
            outs.append(pin_out.numpy().reshape(case.u0.shape, order="F").copy())
        else:
            outs.append(upd.download())
    np.testing.assert_array_equal(outs[0], outs[1])


@pytest.mark.parametrize("chunks", ["1", "3", "8"])
def test_chunked_transfers_round_trip(monkeypatch, chunks):
    """State transfers split into chunks on their own copy streams (each
    chunk permuted as it lands): an FP64 upload/download round trip returns
    the input bit for bit, from pageable and from page-locked buffers, and a
    step after a chunked upload equals one after an unchunked upload."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("SWE_COPY_CHUNKS", chunks)
    case = C.dam_break_case(n=41)              # 1681 nodes: chunked
    rng = np.random.default_rng(5)
    u = np.asfortranarray(case.u0 + rng.uniform(0.0, 0.01, case.u0.shape))
    upd = from_case(case, precision=0)
    upd.upload(u)
    np.testing.assert_array_equal(upd.download(), u)
    pin_in = torch.from_numpy(u.ravel(order="F").copy()).pin_memory()
    pin_out = torch.zeros_like(pin_in).pin_memory()
    upd.upload_ptr(pin_in.data_ptr())
    upd.download_ptr(pin_out.data_ptr())
    np.testing.assert_array_equal(pin_out.numpy().reshape(u.shape, order="F"), u)
    upd.set_time(0.0, 1e30)
    upd.rk3_steps(3)
    got = upd.download()
    upd.close()
    monkeypatch.setenv("SWE_COPY_CHUNKS", "1")
    ref = from_case(case, precision=0)
    ref.upload(u)
    ref.set_time(0.0, 1e30)
    ref.rk3_steps(3)
    np.testing.assert_array_equal(got, ref.download())
    ref.close()


@pytest.mark.parametrize("prec", [1, 2])
def test_autotuned_variants_agree(monkeypatch, prec):
    """The autotuner only changes launch shapes (block size, entry batch,
    grid, register cap), all of which perform the same operations: the
    autotuned run equals the default one bit for bit."""
    case = C.bump_basin_case(n=60)
    outs = []
    for env in ("0", "1"):
        monkeypatch.setenv("SWE_AUTOTUNE", env)
        upd = from_case(case, precision=prec)
        upd.upload(case.u0)
        upd.set_time(0.0, 1e30)
        upd.rk3_steps(20)
        outs.append(upd.download())
        assert ("autotuned" in upd.tuning) == (env == "1")
    np.testing.assert_array_equal(outs[1], outs[0])


@pytest.mark.parametrize("tile", ["64", "256"])
def test_tiled_kernels_match_global_gathers(golden, monkeypatch, tile):
    """The shared-memory tile variants (node records of a tile of rows and of
    its halo staged in shared memory, neighbours read by tile-local position)
    against the kernels that gather from HBM by column index, bit for bit:
    one Euler stage on a Thacker state with moving wet/dry fronts, and 20
    RK3 steps (dt included) of the bump basin."""
    case = _thacker(golden, "0.1", periods=1.0, cfl=0.3)
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    t = 0.0
    for _ in range(10):                     # wet/dry fronts moving
        t = o.rk3_step(u, t)
    _, dt = o.compute_dij(u)
    p = replace(case.params, dt=dt, precision=1)
    bump = C.bump_basin_case(n=60)
    monkeypatch.setenv("SWE_TILE", tile)
    eul, traj, dts = {}, {}, {}
    for tiled in ("0", "1"):
        monkeypatch.setenv("SWE_TILED", tiled)
        upd = from_case(case, precision=1)
        upd.set_params(p)
        upd.upload(u)
        upd.autotune()
        assert ("/tiled" in upd.tuning) == (tiled == "1"), upd.tuning
        eul[tiled] = upd.euler(u)
        upd.close()
        upd = from_case(bump, precision=1)
        upd.upload(bump.u0)
        upd.set_time(0.0, 1e30)
        _, dts[tiled], _ = upd.rk3_steps(20)
        assert ("/tiled" in upd.tuning) == (tiled == "1"), upd.tuning
        traj[tiled] = upd.download()
        lump = upd.lumped
        upd.close()
    np.testing.assert_array_equal(eul["1"], eul["0"])
    np.testing.assert_array_equal(dts["1"], dts["0"])
    assert traj["1"][0].min() >= 0.0
    np.testing.assert_array_equal(traj["1"], traj["0"])


def test_fixed_tuning_reproduces_autotuned_variants(monkeypatch):
    """SWE_TUNE takes the autotuner's own description and launches exactly
    those variants (profiling runs pin the timed run's choice with it)."""
    case = C.bump_basin_case(n=60)
    monkeypatch.delenv("SWE_TUNE", raising=False)
    upd = from_case(case, precision=1)
    upd.upload(case.u0)
    upd.set_time(0.0, 1e30)
    upd.rk3_steps(10)
    ref = upd.download()
    spec = upd.tuning.split("autotuned ", 1)[1]
    upd.close()
    monkeypatch.setenv("SWE_TUNE", spec)
    upd = from_case(case, precision=1)
    upd.upload(case.u0)
    upd.set_time(0.0, 1e30)
    upd.rk3_steps(10)
    assert upd.tuning.endswith("fixed " + spec)
    np.testing.assert_array_equal(upd.download(), ref)
    upd.close()
    monkeypatch.setenv("SWE_TUNE", "low:block100/batch2")
    upd = from_case(case, precision=1)
    upd.upload(case.u0)
    with pytest.raises(L.SweError, match="SWE_TUNE"):
        upd.rk3_steps(1)
    upd.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_frame_fields_match_oracle(golden, prec):
    """Movie-frame fields computed on the device (main.f90:125-143) equal the
    oracle's restatement on the downloaded state, bit for bit, with wet and
    dry nodes on both sides of 1e-4 hmax0 (the Thacker case without the
    htiny film, whose dry box holds h = 0)."""
    case = _thacker(golden, "0.1", periods=1.0, cfl=0.3, film=False)
    upd = from_case(case, precision=prec)
    upd.upload(case.u0)
    upd.set_time(0.0, 1e30)
    upd.rk3_steps(12)
    hmax0 = float(case.u0[0].max())
    hpz, h = upd.frame_fields(hmax0)
    u = upd.download()
    e_hpz, e_h = oracle.frame_fields(u[0], case.bath, hmax0)
    dry = u[0] <= 1e-4 * hmax0
    assert dry.any() and (~dry).any()
    np.testing.assert_array_equal(hpz, e_hpz)
    np.testing.assert_array_equal(h, e_h)
    upd.close()


def test_async_frames_write_the_reference_text(golden, tmp_path):
    """Frames queued with swe_frame_async between steps (three in a row, so
    one waits for a free buffer) are written by the worker thread as the
    text vtk_2d writes for the state at the time of the call."""
    case = _thacker(golden, "0.1", periods=1.0, cfl=0.3, film=False)
    upd = from_case(case, precision=1)
    upd.upload(case.u0)
    upd.set_time(0.0, 1e30)
    hmax0 = float(case.u0[0].max())
    expect = {}
    for k in range(1, 4):
        upd.rk3_steps(3)
        paths = (tmp_path / f"hpz_{k}.vtk", tmp_path / f"h_{k}.vtk")
        upd.frame_async(paths[0], paths[1], hmax0)
        fields = oracle.frame_fields(upd.download()[0], case.bath, hmax0)
        for p, f in zip(paths, fields):
            expect[p] = oracle.vtk_2d_text(p.name.ljust(200), case.mesh["jj"], case.mesh["rr"], f)
    upd.frames_wait()
    for p, text in expect.items():
        assert p.read_text() == text, p.name
    upd.frame_async(tmp_path / "missing" / "a.vtk", tmp_path / "missing" / "b.vtk", hmax0)
    with pytest.raises(L.SweError, match="cannot write"):
        upd.frames_wait()
    upd.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_gauges_record_every_step(prec):
    """Gauges (main.f90:102-117) placed as the reference does (first element
    where `inside` holds, FE_interpolation weights) and recorded on the
    device after every step, inside the captured step graphs: each row equals
    the oracle's interpolation of the state downloaded after that step, bit
    for bit, and the ring keeps the last 4096 steps."""
    case = C.dam_break_case(n=41)
    jj, rr = case.mesh["jj"], case.mesh["rr"]
    rng = np.random.default_rng(3)
    pts = np.column_stack([rng.uniform(0.05, 0.95, (2, 5)), rr[:, 100], 0.5 * (rr[:, 0] + rr[:, 1])])
    upd = from_case(case, precision=prec)
    elems = upd.set_gauges(pts)
    want = [oracle.gauge_element(jj, rr, pts[:, g]) for g in range(pts.shape[1])]
    np.testing.assert_array_equal(elems, want)
    ff = [oracle.gauge_weights(jj, rr, want[g], pts[:, g]) for g in range(pts.shape[1])]
    upd.upload(case.u0)
    upd.set_time(0.0, 1e30)
    times, states = [], []
    for _ in range(5):
        t, _, _ = upd.rk3_steps(1)
        times.append(t[0]); states.append(upd.download()[0])
    t_rec, h_rec, e_rec, lost = upd.read_gauges()
    assert h_rec.shape == (5, pts.shape[1]) and lost == 0
    for k in range(5):
        assert np.all(t_rec[k] == times[k])
        for g in range(pts.shape[1]):
            sh, se = oracle.gauge_values(jj, want[g], ff[g], states[k], case.bath)
            assert (h_rec[k, g], e_rec[k, g]) == (sh, se), (k, g)
    upd.rk3_steps(4101)                      # graphs of 8 steps plus single steps
    t_rec, h_rec, e_rec, lost = upd.read_gauges()
    assert h_rec.shape[0] == 4096 and lost == 5
    assert np.all(np.diff(t_rec[:, 0]) > 0)
    u = upd.download()[0]
    for g in range(pts.shape[1]):
        assert (h_rec[-1, g], e_rec[-1, g]) == oracle.gauge_values(jj, want[g], ff[g], u, case.bath)
    with pytest.raises(L.SweError, match="no element"):
        upd.set_gauges(np.array([[5.0], [5.0]]))
    upd.set_gauges(np.zeros((2, 0)))
    upd.rk3_steps(2)
    assert upd.read_gauges()[1].shape[0] == 0
    upd.close()


def test_malpasset_time_loop_fixed_dt_and_htiny():
    """Type 9 (Malpasset) runs the time loop with dt = 2.5e-2 and htiny =
    1e-3 instead of COMPUTE_DT (main.f90:67-69), with Manning friction; the
    FP64 path equals the oracle bit for bit.  The reference's Malpasset mesh
    is missing, so a dam break on a 100 m lattice stands in."""
    mesh = M.lattice_mesh(21, 21, 0.0, 100.0, 0.0, 100.0)
    x = mesh["rr"][0]
    u0 = np.asfortranarray(np.vstack([np.where(x < 50.0, 2.0, 0.5), np.zeros_like(x), np.zeros_like(x)]))
    p = C.Params(gravity=9.81, cfl=0.25, max_water_h=2.0, htiny=1e-6, mannings=0.03, type_test=9)
    case = C.Case(name="type9", mesh=mesh, bath=np.zeros_like(x), params=p, u0=u0, dirichlet=[], tfinal=1e30)
    o = _oracle_for(case)
    u = u0.copy(order="F")
    t = 0.0
    for _ in range(10):
        t = o.rk3_step(u, t)
    upd = from_case(case)
    upd.upload(u0)
    upd.set_time(0.0, 1e30)
    tg, dtg, n = upd.rk3_steps(10)
    assert n == 10 and dtg[0] == 2.5e-2 and tg[0] == pytest.approx(0.25, rel=1e-14)
    np.testing.assert_array_equal(upd.download(), u)
    upd.close()


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_checkpoint_resume_is_bit_exact(tmp_path, prec):
    """A run stopped after 5 steps, saved, and resumed in a new context
    continues bit for bit like the uninterrupted run."""
    case = C.dam_break_case(n=31)
    upd = from_case(case, precision=prec)
    upd.upload(case.u0)
    upd.set_time(0.0, 0.2)
    upd.rk3_steps(5)
    upd.save_checkpoint(tmp_path / "ck.npz")
    upd.rk3_steps(7)
    want, (t_want, _, _) = upd.download(), upd.get_time()
    upd.close()
    again = from_case(case, precision=prec)
    again.load_checkpoint(tmp_path / "ck.npz")
    if prec != 0:          # the stored launch configuration, not a new tuning
        assert "fixed " in again.tuning, again.tuning
    again.rk3_steps(7)
    np.testing.assert_array_equal(again.download(), want)
    assert again.get_time()[0][0] == t_want[0]
    other = from_case(C.dam_break_case(n=21), precision=prec)
    with pytest.raises(ValueError):
        other.load_checkpoint(tmp_path / "ck.npz")
    again.close(); other.close()


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_rk3_steps_host_equals_the_three_calls(prec):
    """swe_rk3_steps_host (upload, steps, download in one call) gives the bits
    of swe_upload + swe_rk3_steps + swe_download, also in place (un == unext)
    and with either transfer skipped."""
    case = C.dam_break_case(n=41)
    a = from_case(case, precision=prec)
    b = from_case(case, precision=prec)
    for u in (a, b):
        u.set_time(0.0, 0.2)
    a.upload(case.u0)
    ta, dta, na = a.rk3_steps(3)
    want = a.download()
    got = b.rk3_steps_host(case.u0, 3)
    np.testing.assert_array_equal(got, want)
    tb, _, dtb = b.get_time()
    assert tb[0] == ta[0] and dtb[0] == dta[0]
    # in place: the same buffer in and out, then a run with no upload
    buf = np.asfortranarray(want.copy())
    b.rk3_steps_host_ptr(buf.ctypes.data, buf.ctypes.data, 2)
    a.rk3_steps(2)
    np.testing.assert_array_equal(buf, a.download())
    b.rk3_steps_host_ptr(0, 0, 1)
    a.rk3_steps(1)
    np.testing.assert_array_equal(b.download(), a.download())
    with pytest.raises(ValueError):
        b.rk3_steps_host(case.u0[:, :-1], 1)
    a.close(); b.close()


def _thacker_converging(spacing, prec):
    """Thacker's planar oscillation (type 5), one period, film-free initial
    state, with htiny = 4e-4 (spacing / 0.05)^2: proportional to the lumped
    mass, as the reference's own commented-out choice htiny ~ MINVAL(lumped)
    (SOURCES/main.f90:64-65), and equal to the reference's type-5 value
    1e-4 max_water_h = 4e-4 at spacing 0.05.  With the reference's fixed
    htiny the htiny-regularised shoreline layer keeps the error near 0.02
    under refinement (on any of the meshes tried); a fixed htiny 10x smaller
    makes the scheme itself STOP (Min h<0) on the coarse meshes."""
    mesh = C.thacker_mesh(spacing)
    case = C.thacker_case(mesh, periods=1.0, cfl=0.3, film=False)
    ht = 4e-4 * (spacing / 0.05) ** 2
    rr = mesh["rr"]
    u0 = np.asfortranarray(np.vstack([C.thacker_sol(k, rr, 0.0, ht, 9.81, False) for k in (1, 2, 3)]))
    js = M.dirichlet_nodes(mesh["jjs"], mesh["sides"], [1, 2, 3, 4])
    bc = [(k - 1, js, C.thacker_sol(k, rr[:, js - 1], 0.0, ht, 9.81, False)) for k in (1, 2, 3)]
    case = replace(case, params=replace(case.params, htiny=ht, precision=prec), u0=u0, dirichlet=bc)
    o = oracle.Oracle(mesh["jj"], rr)
    rj, rg = o.gauss()
    upd = from_case(case)
    upd.upload(case.u0)
    upd.set_time(0.0, case.tfinal)
    while True:
        t, _, k = upd.rk3_steps(4000)
        if k < 4000:
            break
    u = upd.download()
    upd.close()
    ex = C.thacker_sol(1, rg, float(t[0]), ht, 9.81, False)
    return o.norms(u[0], ex)[0] / o.norms(np.zeros(o.np), ex)[0]


@pytest.mark.parametrize("prec", [0, 1])
def test_thacker_converges_under_refinement(prec):
    """C2's analytic L1 error of h after one period falls on each halving of
    the mesh spacing (0.1, 0.05, 0.025), in FP64 and in mixed precision
    (measured rates ~1.6 and ~1.4)."""
    errs = [_thacker_converging(hs, prec) for hs in (0.1, 0.05, 0.025)]
    rates = [math.log2(errs[k] / errs[k + 1]) for k in range(2)]
    print(f"Thacker precision {prec}: L1 {errs}, rates {rates}")
    assert all(r > 1.0 for r in rates), (errs, rates)


def _fan(k, closed=True):
    """One centre node (1) in k triangles of a regular fan of radius 1."""
    ang = 2 * np.pi * np.arange(k) / k
    rr = np.vstack([np.r_[0.0, np.cos(ang)], np.r_[0.0, np.sin(ang)]])
    nxt = [(a + 1) % k for a in range(k)] if closed else list(range(1, k))
    jj = np.array([[1, a + 2, b + 2] for a, b in zip(range(len(nxt)), nxt)], np.int32).T
    return {"jj": np.asfortranarray(jj), "rr": np.asfortranarray(rr)}


def _fan_case(k):
    mesh = _fan(k)
    r2 = mesh["rr"][0] ** 2 + mesh["rr"][1] ** 2
    u0 = np.asfortranarray(np.vstack([1.0 + 0.1 * r2, 0.01 * mesh["rr"][0], np.zeros(mesh["rr"].shape[1])]))
    p = C.Params(gravity=9.81, cfl=0.25, max_water_h=1.1, htiny=1e-4, type_test=4)
    return C.Case(name=f"fan{k}", mesh=mesh, bath=np.zeros(u0.shape[1]), params=p, u0=u0, tfinal=1e30)


def test_mesh_edge_cases_match_oracle():
    """A single triangle, and a fan whose centre row has 81 entries (st_csr
    accepts rows up to nparm = 90): matrices, compute_dij and a few RK3 steps
    equal the oracle bit for bit.  A fan whose centre row would need 96
    entries is rejected by both, as the reference STOPs."""
    tri = {"jj": np.asfortranarray(np.array([[1], [2], [3]], np.int32)),
           "rr": np.asfortranarray(np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]))}
    one = C.Case(name="triangle", mesh=tri, bath=np.zeros(3), params=C.Params(type_test=4),
                 u0=np.asfortranarray(np.array([[1.0, 0.5, 0.2], [0.0, 0.1, 0.0], [0.0, 0.0, -0.1]])), tfinal=1e30)
    for case in (one, _fan_case(80)):
        o = _oracle_for(case)
        upd = from_case(case)
        a, b = upd.matrices(), o.matrices()
        for k in ("ia", "ja", "diag", "mass", "lumped", "cx", "cy"):
            np.testing.assert_array_equal(a[k], b[k], err_msg=f"{case.name} {k}")
        dg, dtg = upd.compute_dij(case.u0)
        dr, dtr = o.compute_dij(case.u0)
        np.testing.assert_array_equal(dg, dr)
        assert dtg == dtr
        u = case.u0.copy(order="F")
        t = 0.0
        for _ in range(3):
            t = o.rk3_step(u, t)
        upd.upload(case.u0)
        upd.set_time(0.0, 1e30)
        upd.rk3_steps(3)
        np.testing.assert_array_equal(upd.download(), u, err_msg=case.name)
        upd.close()
    big = _fan_case(95)
    with pytest.raises(L.SweError, match="90 entries"):
        from_case(big)
    with pytest.raises(Exception):
        _oracle_for(big)


@pytest.mark.parametrize("tt", sorted(REF_CASES))
def test_reference_cases_on_the_device_loop(ref_case, tt):
    """The reference's test cases (init, sol_anal and bdy of condlim.f90 and
    main.f90, Dirichlet data fixed over the run): ten FP64 steps of the
    device loop equal the oracle bit for bit.  The mixed path keeps h >= 0
    and stays within 3x the FP64 oracle's own sensitivity to a 1e-7
    perturbation of the initial state (plus 1e-5)."""
    case = ref_case(tt)
    o = _oracle_for(case)
    u = case.u0.copy(order="F")
    t = case.t0
    for _ in range(10):
        t = o.rk3_step(u, t)
    upd = from_case(case)
    upd.upload(case.u0)
    upd.set_time(case.t0, 1e30)
    tg, _, n = upd.rk3_steps(10)
    assert n == 10 and tg[0] == t
    np.testing.assert_array_equal(upd.download(), u)
    upd.close()
    up = case.u0.copy(order="F")
    up *= 1 + 1e-7 * np.random.default_rng(0).uniform(-1, 1, up.shape)
    o2 = _oracle_for(case)
    t = case.t0
    for _ in range(10):
        t = o2.rk3_step(up, t)
    mx = from_case(case, precision=1)
    mx.upload(case.u0)
    mx.set_time(case.t0, 1e30)
    mx.rk3_steps(10)
    um = mx.download()
    err = _rel_l1(um[0], u[0], mx.lumped)
    sens = _rel_l1(up[0], u[0], mx.lumped)
    assert um[0].min() >= 0.0
    assert err <= 3 * sens + MIXED_L1_TOL, (err, sens)
    mx.close()


def test_time_dependent_dirichlet_through_per_call_euler(golden):
    """SOURCES/data (type 13 solitary wave, 'entropy_visc', h imposed at both
    channel ends from sol_anal(t)) on MESHES/SGN_CANAL/rectangle.1: main.f90's
    loop on the host over the C ABI's per-call compute_dij / euler, with bdy
    at the reference's stage times, equals the same loop over the oracle bit
    for bit."""
    from swe import data as D, refcases as R
    d = D.read_my_data(golden / "ref_data_sources.txt")
    mesh = M.load_mesh_free_format(golden / "ref_rectangle.1.FEM.gz")
    case = R.case_from_data(d, mesh)
    assert not case.bdy_fixed
    o = _oracle_for(case)
    want, tw, nw = R.host_time_loop(OraclePerCall(o), case.bdy, case.u0, case.t0, 1e30, 8)
    upd = from_case(case, per_call=True)
    got, tg, ng = R.host_time_loop(R.PerCall(upd), case.bdy, case.u0, case.t0, 1e30, 8)
    assert (ng, tg) == (nw, tw) == (8, tw)
    np.testing.assert_array_equal(got, want)
    upd.close()


def _device_vs_host_anal(case, comps, steps, prec=0):
    """case with analytic Dirichlet data comps [(comp, js)]: the device loop
    (swe_set_dirichlet_anal) against main.f90's loop on the host over the
    per-call euler with bdy = sol_anal at the reference's stage times."""
    from swe import refcases as R

    def bdy(uu, t):
        for comp, js in comps:
            uu[comp, js - 1] = case.exact(comp + 1, case.mesh["rr"][:, js - 1], t)

    host = from_case(replace(case, dirichlet=[], dirichlet_anal=[]), precision=0, per_call=True)
    want, tw, nw = R.host_time_loop(R.PerCall(host), bdy, case.u0, case.t0, 1e30, steps)
    host.close()
    dev = from_case(replace(case, dirichlet=[], dirichlet_anal=comps, bdy_fixed=False), precision=prec)
    dev.upload(case.u0)
    dev.set_time(case.t0, 1e30)
    tg, _, ng = dev.rk3_steps(steps)
    got = dev.download()
    lump = dev.lumped
    dev.close()
    assert ng == nw == steps
    return got, want, lump


def test_time_dependent_dirichlet_on_the_device_loop(golden):
    """SOURCES/data (type 13 solitary wave, 'entropy_visc', h imposed at both
    channel ends from sol_anal(t)) on MESHES/SGN_CANAL/rectangle.1 through
    the device loop, sol_anal evaluated on the device at every stage's bdy
    time, against the host loop over the per-call euler: FP64 within 1e-12
    (CUDA's cosh against the C library's), mixed within the L1 tolerance."""
    from swe import data as D, refcases as R
    d = D.read_my_data(golden / "ref_data_sources.txt")
    mesh = M.load_mesh_free_format(golden / "ref_rectangle.1.FEM.gz")
    case = R.case_from_data(d, mesh)
    assert case.dirichlet_anal and not case.bdy_fixed
    got, want, lump = _device_vs_host_anal(case, case.dirichlet_anal, 8)
    scale = np.abs(want).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(got - want) / scale) < 1e-12
    got1, _, _ = _device_vs_host_anal(case, case.dirichlet_anal, 8, prec=1)
    assert _rel_l1(got1[0], want[0], lump) <= MIXED_L1_TOL


def test_thacker_analytic_dirichlet_on_wet_nodes(golden):
    """Type 5 with h, qx and qy imposed from sol_anal(t) on wet nodes (a disk
    inside the moving water): the device loop against the host loop, FP64
    within 1e-12."""
    case = _thacker(golden, "0.2", periods=1.0, cfl=0.3)
    rr = case.mesh["rr"]
    js = (np.nonzero((rr[0] - 2.0) ** 2 + (rr[1] - 2.0) ** 2 < 0.3 ** 2)[0] + 1).astype(np.int32)
    assert len(js) >= 5
    got, want, _ = _device_vs_host_anal(case, [(0, js), (1, js), (2, js)], 6)
    scale = np.abs(want).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(got - want) / scale) < 1e-12


def test_degenerate_meshes_are_refused():
    """An empty mesh, an element node number out of range, a node that no
    element touches (zero lumped mass, which the reference would divide by)
    and a clockwise triangle are refused with an error status when the
    matrices are built; the device set-up checks every index before it
    reads through it."""
    p = C.Params(type_test=4)
    tri = np.asfortranarray(np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]))
    four = np.asfortranarray(np.array([[0.0, 1.0, 0.0, 2.0], [0.0, 0.0, 1.0, 2.0]]))
    cases = [(np.zeros((3, 0), np.int32), tri, L.SWE_ERR_ARG, "empty mesh"),
             (np.array([[1], [2], [4]], np.int32), tri, L.SWE_ERR_MESH, "out of range"),
             (np.array([[1], [2], [0]], np.int32), tri, L.SWE_ERR_MESH, "out of range"),
             (np.array([[1], [2], [3]], np.int32), four, L.SWE_ERR_MESH, "lumped mass"),
             (np.array([[1], [3], [2]], np.int32), tri, L.SWE_ERR_MESH, "lumped mass")]
    for jj, rr, code, msg in cases:
        mesh = {"jj": np.asfortranarray(jj), "rr": rr}
        with pytest.raises(L.SweError, match=msg) as ei:
            Update(mesh, np.zeros(rr.shape[1]), p)
        assert ei.value.code == code
    ok = Update({"jj": np.asfortranarray(np.array([[1], [2], [3]], np.int32)), "rr": tri}, np.zeros(3), p)
    ok.close()

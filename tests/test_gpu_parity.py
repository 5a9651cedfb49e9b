"""GPU parity: the CUDA path through the C ABI against the oracle.

Reference arithmetic ("reference") must be bit-identical to the oracle (which
is itself bit-identical to the reference sources).  The fast arithmetic must
stay within 1e-12 relative per cell after the stated step counts: for every
cell, max_k |U_k - U_ref_k| / max_k |U_ref_k| over the five conserved fields
(the cell's state error relative to the cell's state).  Per-field ratios are
not used because fields that are zero up to round-off (the momentum of a
radial Sod near its axes) have no scale of their own.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FAST_RTOL = 1e-12


def rel_err(a, b):
    """max over cells of the cell-wise relative error (infinity norm over the 5 fields)."""
    num = np.abs(a - b).max(axis=1)
    den = np.abs(b).max(axis=1)
    return float((num / den).max())


def oracle_mesh(orc, case, cell_order=0):
    lo, hi = case.bcs()
    return orc.OracleMesh(case.problem, case.dim, case.n, case.origin, case.length, bc_lo=lo, bc_hi=hi,
                          cell_order=cell_order)


def oracle_params(orc, case):
    p = case.prm
    return orc.params(vortex_beta=p.vortex_beta, sod_radius=p.sod_radius, sod_rho_in=p.sod_rho_in,
                      sod_p_in=p.sod_p_in, sod_rho_out=p.sod_rho_out, sod_p_out=p.sod_p_out,
                      periodic_exact=int(p.periodic), domain_origin=p.origin, domain_length=p.length)


# ---- unit-level functions ---------------------------------------------------------------

def random_states(n, seed, amp=2.0):
    rng = np.random.default_rng(seed)
    prim = np.column_stack([rng.uniform(0.05, 3, n), rng.uniform(-amp, amp, (n, 3)), rng.uniform(0.05, 3, n)])
    return prim


def test_pointwise_bitwise(orc, mmf):
    from minimmerflow_gb300 import euler
    n = 4096
    prim = random_states(n, 1)
    cons = np.array([orc.prim2cons(p) for p in prim])
    assert np.array_equal(euler.primitive2conservative(prim), cons)
    assert np.array_equal(euler.conservative2primitive(cons), np.array([orc.cons2prim(c) for c in cons]))
    rng = np.random.default_rng(2)
    nrm = rng.normal(size=(n, 3)); nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    p2 = np.array([orc.cons2prim(c) for c in cons])
    assert np.array_equal(euler.evalFluxes(cons, p2, nrm),
                          np.array([orc.eval_fluxes(c, p, q) for c, p, q in zip(cons, p2, nrm)]))
    cr = cons[::-1].copy()
    F, lam = euler.evalSplitting(cons, cr, nrm)
    ref = [orc.eval_splitting(a, b, q) for a, b, q in zip(cons, cr, nrm)]
    assert np.array_equal(F, np.array([r[0] for r in ref]))
    assert np.array_equal(lam, np.array([r[1] for r in ref]))
    for bc in (orc.BC_FREE_FLOW, orc.BC_REFLECTING, orc.BC_WALL):
        g = euler.evalInterfaceBCValues(bc, nrm, cons)
        assert np.array_equal(g, np.array([orc.eval_bc(0, bc, np.zeros(3), q, c) for c, q in zip(cons, nrm)]))
    g = euler.evalInterfaceBCValues(orc.BC_DIRICHLET, nrm, cons, [1.0, 3.0, 0.0, 0.0, 1.0 / 1.4])
    assert np.array_equal(g, np.tile(orc.eval_bc(orc.FFSTEP, orc.BC_DIRICHLET, np.zeros(3), nrm[0], cons[0]),
                                     (n, 1)))


def test_newton_reciprocal_and_sqrt_error_bound(mmf):
    """The fast arithmetic's reciprocal and square root (Newton iterations on the
    hardware approximations) are within 1 ulp of the correctly rounded values."""
    lib = mmf.capi.load()
    rng = np.random.default_rng(5)
    x = np.concatenate([rng.uniform(1e-3, 1e3, 200000), 10.0 ** rng.uniform(-30, 30, 50000),
                        np.array([1.0, 2.0, 0.125, 0.1, 1.4, 7.0])])
    r = np.empty_like(x); q = np.empty_like(x)
    mmf.capi.check(lib.mmf_newton_selftest(x.size, mmf.capi.ptr(x), mmf.capi.ptr(r), mmf.capi.ptr(q)))
    ulp_r = np.abs(r - 1.0 / x) / np.spacing(1.0 / x)
    ulp_q = np.abs(q - np.sqrt(x)) / np.spacing(np.sqrt(x))
    assert ulp_r.max() <= 1.0, ulp_r.max()
    assert ulp_q.max() <= 1.0, ulp_q.max()
    z = np.zeros(1); r0 = np.empty(1); q0 = np.empty(1)
    mmf.capi.check(lib.mmf_newton_selftest(1, mmf.capi.ptr(z), mmf.capi.ptr(r0), mmf.capi.ptr(q0)))
    assert q0[0] == 0.0


def test_fast_2d_with_nonzero_w(orc, mmf):
    """A 2D state with non-zero z-momentum (a passive scalar in 2D) takes the
    five-field kernels; the result still matches the oracle."""
    case = mmf.problem.reference_case("vortex_xy", 2, 32, t_end=0.5)
    m = oracle_mesh(orc, case)
    U0 = m.initial_state()
    U0[:, 3] = 0.05 * U0[:, 0] * np.sin(np.arange(m.ncells))
    U0[:, 4] += 0.5 * U0[:, 3] ** 2 / U0[:, 0]
    U_ref, t_ref, steps_ref = m.run(U0, case.cfl, t_end=0.5)
    with case.solver(arith="fast") as s:
        U, t, steps = s.run(U0, case.cfl, t_end=0.5)
    assert steps == steps_ref
    assert rel_err(U, U_ref) <= FAST_RTOL
    assert np.abs(U[:, 3]).max() > 0.0


# ---- computeRHS -------------------------------------------------------------------------

RHS_CASES = [("vortex_xy", 2, 64), ("radsod", 2, 64), ("vortex_xy", 3, 16), ("vortex_yz", 3, 16),
             ("radsod", 3, 16)]


@pytest.mark.parametrize("pname,dim,n", RHS_CASES)
def test_compute_rhs_bitwise(orc, mmf, pname, dim, n):
    case = mmf.problem.reference_case(pname, dim, n)
    m = oracle_mesh(orc, case)
    rng = np.random.default_rng(7)
    U = m.initial_state() * (1.0 + 0.02 * rng.standard_normal((m.ncells, 1)))
    R_ref, me_ref = m.compute_rhs(U)
    with case.solver(arith="reference") as s:
        R, me = s.compute_rhs(U)
    assert me == me_ref
    assert np.array_equal(R, R_ref)


@pytest.mark.parametrize("dim,n", [(2, (37, 23, 1)), (2, (1, 9, 1)), (2, (9, 1, 1)), (3, (13, 7, 5)),
                                   (3, (31, 1, 3)), (3, (61, 14, 9))])
@pytest.mark.parametrize("periodic", [False, True])
def test_compute_rhs_ragged_bitwise(orc, mmf, dim, n, periodic):
    P = mmf.problem
    case = P.Case("ragged", P.RADSOD, dim, n, (-0.3, -0.2, -0.1), 1.0, 0.5, periodic=periodic,
                  prm=P.Params(sod_radius=0.3))
    m = oracle_mesh(orc, case)
    rng = np.random.default_rng(11)
    U = m.initial_state(oracle_params(orc, case)) * (1.0 + 0.05 * rng.standard_normal((m.ncells, 1)))
    R_ref, me_ref = m.compute_rhs(U)
    with case.solver(arith="reference") as s:
        R, me = s.compute_rhs(U)
    assert me == me_ref
    assert np.array_equal(R, R_ref)


@pytest.mark.parametrize("arith", ["reference", "fast"])
@pytest.mark.parametrize("n,periodic", [((61, 14, 9), False), ((40, 35, 11), True), ((32, 16, 8), True),
                                        ((1, 17, 5), False), ((70, 50, 23), True)])
def test_3d_kernels_give_the_same_bits(orc, mmf, arith, n, periodic):
    """The two 3D order-1 kernels -- row blocks of 30-column segments with
    halo lanes and rows, and 32 x 16 tiles with one-pass halo records, one
    block per tile and chunk or at most one per resident slot -- and every
    plane chunk give the same bits, on grids that the tiles divide and on
    ragged ones; with the reference arithmetic they are the oracle's."""
    P = mmf.problem
    case = P.Case("ragged3d", P.RADSOD, 3, n, (-0.3, -0.2, -0.1), 1.0, 0.5, periodic=periodic,
                  prm=P.Params(sod_radius=0.3))
    m = oracle_mesh(orc, case)
    rng = np.random.default_rng(5)
    U0 = m.initial_state(oracle_params(orc, case)) * (1.0 + 0.05 * rng.standard_normal((m.ncells, 1)))
    steps = 6
    outs = []
    # variant 2 on the 70 x 50 x 23 grid: 12 tile columns x 23 planes on at
    # most one block per slot; 4-plane units all fall in the evenly split
    # last round (shares that start and end inside columns), 1-plane units
    # make one whole round and a partial one
    for variant, chunk in [(0, 4), (1, 4), (1, 3), (1, 64), (2, 4), (2, 1)]:
        with case.solver(arith=arith) as s:
            s.set_shape(chunk, variant)
            U, t, done = s.run(U0, case.cfl, max_steps=steps)
            assert done == steps and s.status() == 0
        outs.append((U, t))
    for U, t in outs[1:]:
        assert t == outs[0][1]
        assert np.array_equal(U, outs[0][0])
    if arith == "reference":
        U_ref, t_ref, _ = m.run(U0, case.cfl, max_steps=steps)
        assert outs[0][1] == t_ref and np.array_equal(outs[0][0], U_ref)


def test_compute_rhs_morton_map(orc, mmf):
    """Raw ids in octree (Morton) order, as bitpit stores VolOctree cells."""
    case = mmf.problem.reference_case("radsod", 3, 16)
    m = oracle_mesh(orc, case, cell_order=1)
    U = m.initial_state()
    R_ref, me_ref = m.compute_rhs(U)
    with case.solver(arith="reference") as s:
        s.set_cell_map(m.grid_of_raw())
        R, me = s.compute_rhs(U)
    assert me == me_ref and np.array_equal(R, R_ref)


# ---- the time loop ----------------------------------------------------------------------

GOLDEN = ["2dIsentropicVortex", "2dRadSod", "3dIsentropicVortexXY", "3dIsentropicVortexYZ", "3dRadSod"]


@pytest.mark.parametrize("name", GOLDEN)
def test_golden_runs(orc, mmf, name):
    """Full reference regression runs on the GPU: bit-identical final state with
    the reference arithmetic, <=1e-12 with the fast one, golden error string."""
    pname, dim, n, cfl, t_end, golden = orc.GOLDEN_CASES[name]
    case = mmf.problem.reference_case(pname, dim, n, cfl=cfl, t_end=t_end)
    m = oracle_mesh(orc, case)
    U0 = m.initial_state()
    U_ref, t_ref, steps_ref = m.run(U0, cfl, t_end=t_end)
    for arith in ("reference", "fast"):
        with case.solver(arith=arith) as s:
            U, t, steps = s.run(U0, cfl, t_end=t_end)
            assert s.status() == 0
        assert steps == steps_ref
        err = m.l1_density_error(U, t_end)
        if arith == "reference":
            assert t == t_ref
            assert np.array_equal(U, U_ref)
            assert "%.12e" % err == golden
        else:
            assert abs(t - t_ref) <= 1e-14 * t_ref
            assert rel_err(U, U_ref) <= FAST_RTOL
            assert abs(err - float(golden)) <= 1e-10 * float(golden)


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_periodic_vortex_2d_64_100_steps(orc, mmf, arith):
    """2D vortex 64^2, periodic borders, CFL 0.5, 100 steps (order 1)."""
    case = mmf.problem.vortex(2, 64, steps=100)
    m = oracle_mesh(orc, case)
    prm = oracle_params(orc, case)
    U0 = m.initial_state(prm)
    U_ref, t_ref, _ = m.run(U0, case.cfl, max_steps=100)
    with case.solver(arith=arith) as s:
        U, t, steps = s.run(U0, case.cfl, max_steps=100)
    assert steps == 100
    if arith == "reference":
        assert np.array_equal(U, U_ref) and t == t_ref
    else:
        assert rel_err(U, U_ref) <= FAST_RTOL
    # periodic borders conserve every field (telescoping face fluxes)
    np.testing.assert_allclose(U.sum(axis=0), U0.sum(axis=0), rtol=1e-12, atol=1e-10)


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_radial_sod_2d_to_end_time(orc, mmf, arith):
    """[-1,1]^2 radial Sod (r < 0.5), transmissive borders, CFL 0.5, to t = 0.25 at 128^2."""
    case = mmf.problem.radial_sod_2d(n=128)
    m = oracle_mesh(orc, case)
    U0 = m.initial_state(oracle_params(orc, case))
    U_ref, t_ref, steps_ref = m.run(U0, case.cfl, t_end=case.t_end)
    with case.solver(arith=arith) as s:
        U, t, steps = s.run(U0, case.cfl, t_end=case.t_end)
    assert steps == steps_ref and abs(t - 0.25) < 1e-15
    if arith == "reference":
        assert np.array_equal(U, U_ref)
    else:
        assert rel_err(U, U_ref) <= FAST_RTOL


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_vortex_3d_both_axes(orc, mmf, arith):
    """3D periodic vortex, axis z and axis x, 24^3, 20 steps."""
    for axis in ("z", "x"):
        case = mmf.problem.vortex(3, 24, axis=axis, steps=20)
        m = oracle_mesh(orc, case)
        U0 = m.initial_state(oracle_params(orc, case))
        U_ref, t_ref, _ = m.run(U0, case.cfl, max_steps=20)
        with case.solver(arith=arith) as s:
            U, t, steps = s.run(U0, case.cfl, max_steps=20)
        assert steps == 20
        if arith == "reference":
            assert np.array_equal(U, U_ref)
        else:
            assert rel_err(U, U_ref) <= FAST_RTOL


def test_full_size_sod_symmetry_and_mass(mmf):
    """The 1024^2 radial Sod of the benchmark, integrated to t = 0.25: the
    solution keeps the x<->y and mirror symmetries of the initial state, and
    mass is conserved (the shock, at r ~ 0.94, is still inside [-1, 1]^2)."""
    case = mmf.problem.radial_sod_2d(n=1024)
    U0 = case.initial_state()
    with case.solver(arith="fast") as s:
        U, t, steps = s.run(U0, case.cfl, t_end=0.25)
        assert s.status() == 0
    assert t == 0.25 and steps > 300
    rho = U[:, 0].reshape(1024, 1024)
    np.testing.assert_allclose(rho, rho.T, rtol=1e-13, atol=0)
    np.testing.assert_allclose(rho, rho[::-1, :], rtol=1e-13, atol=0)
    assert abs(U[:, 0].sum() - U0[:, 0].sum()) <= 1e-12 * U0[:, 0].sum()


def test_end_time_and_step_limit(orc, mmf):
    case = mmf.problem.reference_case("radsod", 2, 32, t_end=0.3)
    U0 = case.initial_state()
    with case.solver(arith="reference") as s:
        s.upload(U0)
        s.time_setup(case.cfl, 0.0, 0.3, -1)
        t, done = s.advance(1000)
        assert t == 0.3
        t2, done2 = s.advance(5)   # past the end time: nothing runs
        assert done2 == 0 and t2 == 0.3
        s.time_setup(case.cfl, 0.0, math.inf, 7)
        t3, done3 = s.advance(100)
        assert done3 == 7


def test_status_reports_negative_pressure(mmf):
    """A non-physical input state (negative pressure) is reported, not trapped."""
    case = mmf.problem.reference_case("radsod", 2, 16)
    U0 = case.initial_state()
    U0[5, 4] = -1.0   # rho E < 0
    with case.solver(arith="fast") as s:
        s.upload(U0)
        s.time_setup(case.cfl, 0.0, math.inf, 1)
        with pytest.raises(mmf.capi.MMFError) as ei:
            s.advance(1)
        assert ei.value.code == mmf.capi.MMF_ERR_STATE
        assert s.status() & 2


@pytest.mark.parametrize("dim,order", [(2, 1), (3, 1), (2, 2)])
def test_autotune_keeps_state_and_bits(mmf, dim, order):
    """mmf_autotune restores the state and the time control, and the chosen
    decomposition gives the same bits as the default one."""
    P = mmf.problem
    case = P.radial_sod_2d(96, t_end=0.05) if dim == 2 else P.radial_sod_ratios(24, 10.0, 4.0, dim=3)
    U0 = case.initial_state()
    outs = []
    for tune in (False, True):
        with case.solver(order=order) as s:
            s.upload(U0)
            s.time_setup(0.4, 0.0, math.inf, 12)
            s.advance(3)
            if tune:
                before = s.download()
                t_before = s.time_info()
                chunk, wpb = s.autotune(trial_steps=2)
                assert chunk > 0 and (wpb > 0) == (dim == 2)
                assert s.time_info() == t_before
                np.testing.assert_array_equal(s.download(), before)
            t, steps = s.advance(100)
            outs.append((s.download(), t, steps))
    assert outs[0][1:] == outs[1][1:] and outs[0][2] == 9
    np.testing.assert_array_equal(outs[0][0], outs[1][0])


@pytest.mark.parametrize("axis", ["z", "x"])
def test_full_size_vortex3d_is_invariant_along_its_axis(mmf, axis):
    """The 256^3 periodic vortex of the benchmark, 50 steps: the initial state
    does not depend on the coordinate along the vortex axis and the borders are
    periodic, so every plane across the axis must stay bit for bit the same
    (the axial faces contribute exactly zero).  The planes also match the 2D
    vortex on 256^2 within the fast-arithmetic bound."""
    P = mmf.problem
    n = 256
    case = P.vortex(3, n, axis=axis, steps=50)
    with case.solver(arith="fast") as s:
        U, t, steps = s.run(case.initial_state(), case.cfl, max_steps=50)
    assert steps == 50
    V = U.reshape(n, n, n, 5)                       # [z][y][x][field]
    planes = V if axis == "z" else np.moveaxis(V, 2, 0)
    assert all(np.array_equal(planes[0], planes[k]) for k in range(1, n))
    if axis == "z":
        c2 = P.vortex(2, n, steps=50)
        with c2.solver(arith="fast") as s2:
            U2, t2, _ = s2.run(c2.initial_state(), c2.cfl, max_steps=50)
        assert abs(t2 - t) <= 1e-13 * t
        assert rel_err(planes[0].reshape(-1, 5), U2) <= FAST_RTOL


def test_full_size_3d_decompositions_agree(mmf):
    """At the benchmark's 256^3, the row-block kernel, the tile kernel with
    one block per tile and 32-plane chunk, and the tile kernel on one block
    per resident slot (128-plane units: a whole round and an evenly split
    last one; 8-plane units: many rounds) give the same bits over five steps
    of a seeded, perturbed radial Sod, which has no symmetry that would hide
    a misplaced plane, row or column."""
    P = mmf.problem
    case = P.radial_sod_ratios(256, 10.0, 4.0, dim=3)
    rng = np.random.default_rng(11)
    U0 = case.initial_state() * (1.0 + 0.01 * rng.standard_normal((256 ** 3, 1)))
    outs = []
    for chunk, variant in [(32, 0), (32, 1), (128, 2), (8, 2)]:
        with case.solver(arith="fast") as s:
            s.set_shape(chunk, variant)
            U, t, steps = s.run(U0, case.cfl, max_steps=5)
            assert steps == 5 and s.status() == 0
        outs.append((U, t))
    for U, t in outs[1:]:
        assert t == outs[0][1]
        assert np.array_equal(U, outs[0][0])


def test_advance_stops_at_the_end_time(mmf):
    """mmf_advance with many more steps than the run needs launches no idle
    graphs: it returns promptly once t_end is reached."""
    import time
    case = mmf.problem.radial_sod_2d(64, t_end=0.05)
    with case.solver() as s:
        s.upload(case.initial_state())
        s.time_setup(case.cfl, 0.0, 0.05)
        t0 = time.perf_counter()
        t, steps = s.advance(1 << 24)
        assert time.perf_counter() - t0 < 5.0
        assert t == 0.05 and steps > 0


@pytest.mark.parametrize("order", [1, 2])
def test_step_log_matches_the_reference_loop(orc, mmf, order):
    """The device step log holds, per step, the values the reference logs
    (main.cpp:399-404): the first stage's maxEig, the dt used (0.9 CFL h /
    maxEig, clamped to the end time) and the time after the step -- bit for
    bit with the reference arithmetic against the oracle's own log of the
    same run.  A ring of 8 keeps the last 8 of 12 steps."""
    case = mmf.problem.reference_case("radsod", 2, 32, t_end=1.0)
    m = oracle_mesh(orc, case)
    U0 = case.initial_state()
    _, _, steps, dtl, mel = m.run(U0, case.cfl, t_end=1.0, max_steps=12, order=order, log=True)
    assert steps == 12
    t_ref = np.cumsum(np.concatenate([[0.0], dtl[:12]]))   # sequential sums, as t += dt
    with case.solver(arith="reference", order=order) as s:
        s.set_step_log(8)
        s.upload(U0)
        s.time_setup(case.cfl, 0.0, 1.0)
        s.advance(12)
        first, log = s.step_log()
    assert first == 4 and log.shape == (8, 3)
    np.testing.assert_array_equal(log[:, 0], mel[4:12])
    np.testing.assert_array_equal(log[:, 1], dtl[4:12])
    np.testing.assert_array_equal(log[:, 2], t_ref[5:13])


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_cartesian_dirichlet_inflow_channel(orc, mmf, arith):
    """A channel with the forward-facing step's Dirichlet inflow on x-lo,
    free flow on x-hi and reflecting walls in y (problem.cpp:404-438) on the
    Cartesian kernels: the Dirichlet ghost state the host precomputes with the
    reference's operation order gives the oracle's bits (reference
    arithmetic) and stays within 1e-12 (fast)."""
    from minimmerflow_gb300.solver import CartesianEuler
    P = mmf.problem
    n, length = (48, 16), 3.0
    lo = [P.BC_DIRICHLET, P.BC_REFLECTING, P.BC_FREE_FLOW]
    hi = [P.BC_FREE_FLOW, P.BC_REFLECTING, P.BC_FREE_FLOW]
    m = orc.OracleMesh(P.FFSTEP, 2, n, (0.0, 0.0, 0.0), length, bc_lo=lo, bc_hi=hi)
    rng = np.random.default_rng(11)
    U0 = m.initial_state()
    U0 *= 1.0 + 0.05 * rng.standard_normal((m.ncells, 1))
    U0[:, 3] = 0.0
    U_ref, t_ref, steps_ref = m.run(U0, 0.5, max_steps=20)
    with CartesianEuler(2, n, (0.0, 0.0, 0.0), length / n[0], lo, hi, arith=arith,
                        dirichlet_prim=(1.0, 3.0, 0.0, 0.0, 1.0 / 1.4)) as s:
        U, t, steps = s.run(U0, 0.5, max_steps=20)
    assert steps == steps_ref == 20
    if arith == "reference":
        assert t == t_ref
        assert np.array_equal(U, U_ref)
    else:
        assert abs(t - t_ref) <= 1e-12 * t_ref
        assert rel_err(U, U_ref) <= FAST_RTOL
    # the inflow enters: the first column moves towards the Dirichlet state
    assert np.abs(U[:, 1] - U0[:, 1]).max() > 0.0

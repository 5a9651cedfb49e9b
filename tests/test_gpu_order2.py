"""GPU parity of the order-2 limited reconstruction (a project extension on
reconstruction::computePolynomials, reconstruction.cpp:47-55) against the
oracle's order-2 restatement: bit-identical with the reference arithmetic,
<= 1e-12 relative per cell with the fast arithmetic (cell-wise norm, as in
test_gpu_parity.py).  Limiter modes: all cells, none, flagged cells."""
import numpy as np
import pytest

from test_gpu_parity import FAST_RTOL, oracle_mesh, oracle_params, rel_err

pytestmark = pytest.mark.gpu


def perturbed(m, prm, seed, amp=0.02):
    rng = np.random.default_rng(seed)
    U = m.initial_state(prm)
    return U * (1.0 + amp * rng.standard_normal((m.ncells, 1)))


CASES = [
    ("sod2d", lambda P: P.radial_sod_2d(n=48)),
    ("vortex2d_periodic", lambda P: P.vortex(2, 40, steps=10)),
    ("radsod2d_reflect", lambda P: P.reference_case("radsod", 2, 32)),
    ("vortex3d_periodic", lambda P: P.vortex(3, 14, steps=5)),
    ("radsod3d_reflect", lambda P: P.reference_case("radsod", 3, 12)),
]


@pytest.mark.parametrize("name,make", CASES)
def test_polynomials_and_rhs_bitwise(orc, mmf, name, make):
    case = make(mmf.problem)
    m = oracle_mesh(orc, case)
    prm = oracle_params(orc, case)
    U = perturbed(m, prm, 1)
    S_ref, act_ref = m.compute_polynomials(U, order=2, want_active=True)
    R_ref, me_ref = m.compute_rhs(U, order=2, slopes=S_ref)
    with case.solver(arith="reference", order=2) as s:
        S, act = s.compute_polynomials(U)
        R, me = s.compute_rhs(U)
    assert np.array_equal(S, S_ref)
    assert np.array_equal(act, act_ref)
    assert act.any() and not act.all()
    assert me == me_ref
    assert np.array_equal(R, R_ref)


@pytest.mark.parametrize("mode", ["none", "flagged"])
def test_limiter_modes_bitwise(orc, mmf, mode):
    """'none' (central slopes everywhere) on the smooth periodic vortex; 'flagged'
    on the radial Sod with the limiter on the ring around the discontinuity
    (central slopes across a discontinuity drive p negative, which the GPU
    reports as MMF_ERR_STATE)."""
    if mode == "none":
        case = mmf.problem.vortex(2, 40, steps=8)
    else:
        case = mmf.problem.radial_sod_2d(n=40)
    m = oracle_mesh(orc, case)
    prm = oracle_params(orc, case)
    U0 = m.initial_state(prm)
    c = m.centroids()
    flags = (np.abs(np.hypot(c[:, 0], c[:, 1]) - 0.5) < 0.25).astype(np.uint8)
    omode = {"none": 1, "flagged": 2}[mode]
    U_ref, t_ref, _ = m.run(U0, case.cfl, max_steps=8, order=2, limiter_mode=omode,
                            limiter_flag=flags if mode == "flagged" else None)
    with case.solver(arith="reference", order=2) as s:
        s.set_limiter(mode, flags if mode == "flagged" else None)
        U, t, steps = s.run(U0, case.cfl, max_steps=8)
    assert steps == 8 and t == t_ref
    assert np.array_equal(U, U_ref)


def test_unlimited_slopes_across_a_shock_are_reported(mmf):
    """Central (unlimited) slopes at the Sod discontinuity produce a negative
    pressure; the context reports it instead of continuing silently."""
    case = mmf.problem.radial_sod_2d(n=40)
    with case.solver(arith="fast", order=2) as s:
        s.set_limiter("none")
        with pytest.raises(mmf.capi.MMFError) as ei:
            s.run(case.initial_state(), case.cfl, max_steps=20)
        assert ei.value.code == mmf.capi.MMF_ERR_STATE


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_vortex_2d_64_order2_100_steps(orc, mmf, arith):
    """2D isentropic vortex 64^2, periodic, beta 5, second-order limited
    reconstruction, CFL 0.5, 100 steps."""
    case = mmf.problem.vortex(2, 64, steps=100)
    m = oracle_mesh(orc, case)
    prm = oracle_params(orc, case)
    U0 = m.initial_state(prm)
    U_ref, t_ref, _ = m.run(U0, case.cfl, max_steps=100, order=2)
    with case.solver(arith=arith, order=2) as s:
        U, t, steps = s.run(U0, case.cfl, max_steps=100)
        act = s.limiter_activity()
    assert steps == 100
    if arith == "reference":
        assert t == t_ref and np.array_equal(U, U_ref)
    else:
        assert rel_err(U, U_ref) <= FAST_RTOL
    # order 2 is more accurate than order 1 on the smooth vortex
    U1, _, _ = m.run(U0, case.cfl, max_steps=100, order=1)
    assert m.l1_density_error(U, t_ref, prm) < 0.5 * m.l1_density_error(U1, t_ref, prm)
    assert act.any()


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_sod_order2_runs(orc, mmf, arith):
    for make, steps in [(lambda P: P.radial_sod_2d(n=96), 40), (lambda P: P.reference_case("radsod", 3, 16), 10),
                        (lambda P: P.vortex(3, 16, axis="x", steps=8), 8)]:
        case = make(mmf.problem)
        m = oracle_mesh(orc, case)
        prm = oracle_params(orc, case)
        U0 = m.initial_state(prm)
        U_ref, t_ref, _ = m.run(U0, case.cfl, max_steps=steps, order=2)
        with case.solver(arith=arith, order=2) as s:
            U, t, n = s.run(U0, case.cfl, max_steps=steps)
            assert s.status() == 0
        assert n == steps
        if arith == "reference":
            assert np.array_equal(U, U_ref)
        else:
            assert rel_err(U, U_ref) <= FAST_RTOL


@pytest.mark.parametrize("arith", ["reference", "fast"])
@pytest.mark.parametrize("n,periodic", [((61, 14, 9), False), ((40, 35, 11), True), ((32, 16, 8), True),
                                        ((1, 17, 5), False)])
def test_3d_order2_chunks_give_the_same_bits(orc, mmf, arith, n, periodic):
    """The 3D order-2 stage kernel (rows of 32 output columns whose x-halo
    face sides the halo warps evaluate one plane ahead) gives the same bits
    for every plane chunk, on ragged grids (a partial last row segment,
    rows past the grid in the last row block, a single column), periodic or
    not; with the reference arithmetic they are the oracle's."""
    P = mmf.problem
    case = P.Case("ragged3d", P.RADSOD, 3, n, (-0.3, -0.2, -0.1), 1.0, 0.4, periodic=periodic,
                  prm=P.Params(sod_radius=0.3))
    m = oracle_mesh(orc, case)
    rng = np.random.default_rng(6)
    U0 = m.initial_state(oracle_params(orc, case)) * (1.0 + 0.05 * rng.standard_normal((m.ncells, 1)))
    steps = 5
    outs = []
    for chunk in (4, 3, 64):
        with case.solver(arith=arith, order=2) as s:
            s.set_shape(chunk, 0)
            U, t, done = s.run(U0, case.cfl, max_steps=steps)
            assert done == steps and s.status() == 0
        outs.append((U, t))
    for U, t in outs[1:]:
        assert t == outs[0][1]
        assert np.array_equal(U, outs[0][0])
    if arith == "reference":
        U_ref, t_ref, _ = m.run(U0, case.cfl, max_steps=steps, order=2)
        assert outs[0][1] == t_ref and np.array_equal(outs[0][0], U_ref)


def screen_samples(rng, n, nv, dim):
    """Cells for the positivity screen: physical states with slopes of random
    size (face states of both signs), face states placed on the boundary
    2 rho E = |m|^2 to within 1e-18 .. 1e-2, densities near zero, magnitudes
    scaled by 2^-300 .. 2^300, momentum at round-off level, exact zeros,
    infinities and NaNs."""
    ie = nv - 1
    nm = nv - 2   # momentum components stored
    rho = np.exp(rng.uniform(np.log(1e-3), np.log(1e3), n))
    vel = rng.normal(0.0, 3.0, (n, nm))
    p = np.exp(rng.uniform(np.log(1e-3), np.log(1e3), n))
    U = np.empty((n, nv))
    U[:, 0] = rho
    U[:, 1:1 + nm] = rho[:, None] * vel
    U[:, ie] = p / 0.4 + 0.5 * rho * (vel ** 2).sum(axis=1)
    S = U[:, None, :] * rng.uniform(-2.5, 2.5, (n, dim, nv))
    kind = rng.integers(0, 8, n)
    # face state on the boundary: pick the +x face f, set uc = f - sigma/2
    b = kind == 1
    f = U[b].copy()
    m2 = (f[:, 1:1 + nm] ** 2).sum(axis=1)
    delta = np.exp(rng.uniform(np.log(1e-18), np.log(1e-2), b.sum())) * rng.choice([-1.0, 1.0], b.sum())
    f[:, ie] = m2 * (1.0 + delta) / (2.0 * f[:, 0])
    U[b] = f - 0.5 * S[b, 0, :]
    # density near zero on a face
    b = kind == 2
    S[b, 0, 0] = -2.0 * U[b, 0] * (1.0 + rng.choice([-1.0, 1.0], b.sum()) * np.exp(rng.uniform(-40, -2, b.sum())))
    # magnitudes
    b = kind == 3
    sc = np.ldexp(1.0, rng.integers(-300, 300, b.sum()))
    U[b] *= sc[:, None]
    S[b] *= sc[:, None, None]
    # momentum at round-off level, small slopes
    b = kind == 4
    U[b, 1:1 + nm] = rng.normal(0.0, 1e-17, (b.sum(), nm))
    S[b] = U[b, None, :] * rng.uniform(-0.1, 0.1, (b.sum(), dim, nv))
    S[b, :, 1:1 + nm] = rng.normal(0.0, 1e-17, (b.sum(), dim, nm))
    # exact zeros
    b = kind == 5
    U[b, 1:1 + nm] = 0.0
    S[b] = 0.0
    # infinities and NaNs here and there
    b = np.flatnonzero(kind == 6)[:50]
    U[b[:25], 0] = np.inf
    S[b[25:], 0, ie] = np.nan
    return np.ascontiguousarray(U), np.ascontiguousarray(S)


@pytest.mark.parametrize("arith,nv,dim", [("reference", 5, 2), ("reference", 5, 3), ("fast", 5, 2), ("fast", 5, 3),
                                          ("fast", 4, 2)])
def test_positivity_screen_matches_fp64(mmf, arith, nv, dim):
    """The FP32 screen of the positivity fallback either defers to FP64 or
    gives the FP64 answer, on 400k adversarial cells; it decides almost all
    physical cells itself."""
    rng = np.random.default_rng(20261204 + 10 * nv + dim)
    n = 400_000
    U, S = screen_samples(rng, n, nv, dim)
    dec = np.empty(n, dtype=np.int32)
    ref = np.empty(n, dtype=np.uint8)
    a = mmf.capi.ARITH_FAST if arith == "fast" else mmf.capi.ARITH_REFERENCE
    mmf.capi.check(mmf.capi.load().mmf_o2_screen_selftest(a, nv, dim, n, mmf.capi.ptr(U), mmf.capi.ptr(S),
                                                          mmf.capi.ptr(dec), mmf.capi.ptr(ref)))
    decided = dec >= 0
    assert np.array_equal(dec[decided], ref[decided].astype(np.int32))
    assert set(np.unique(dec)) <= {-1, 0, 1}
    # both answers occur, and the boundary cases are where the screen defers
    assert (dec == 1).any() and (dec == 0).any() and (dec == -1).any()
    assert np.mean(decided) > 0.8

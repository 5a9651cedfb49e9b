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

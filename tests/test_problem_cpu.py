"""CPU checks of the host problem library against the oracle (initial states,
exact solutions, Morton ordering)."""
import numpy as np


def test_initial_states_match_oracle(orc, mmf):
    P = mmf.problem
    for pname, dim, n in [("vortex_xy", 2, 32), ("radsod", 2, 16), ("vortex_yz", 3, 8), ("radsod", 3, 8)]:
        case = P.reference_case(pname, dim, n)
        m = orc.OracleMesh(case.problem, case.dim, case.n, case.origin, case.length)
        np.testing.assert_allclose(case.initial_state(), m.initial_state(), rtol=2e-15, atol=1e-15)


def test_exact_solution_matches_oracle(orc, mmf):
    P = mmf.problem
    rng = np.random.default_rng(0)
    pts = rng.uniform(-5, 5, (200, 3))
    for prob in (P.VORTEX_XY, P.VORTEX_ZX, P.VORTEX_YZ, P.RADSOD, P.SOD_X, P.FFSTEP):
        ours = P.exact_conservatives(prob, 3, pts, 0.7)
        ref = np.array([orc.exact_conservatives(prob, 3, p, 0.7) for p in pts])
        np.testing.assert_allclose(ours, ref, rtol=2e-15, atol=1e-15)


def test_periodic_vortex_wraps(mmf):
    P = mmf.problem
    case = P.vortex(2, 32, steps=1)
    c = case.centroids()
    # after one period in x and y the exact solution is the initial one
    a = P.exact_conservatives(case.problem, 2, c, 0.0, case.prm)
    b = P.exact_conservatives(case.problem, 2, c, 10.0, case.prm)
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12)


def test_morton_order_matches_oracle(orc, mmf):
    for dim, n in [(2, (8, 8, 1)), (3, (4, 4, 4)), (2, (6, 5, 1))]:
        m = orc.OracleMesh(0, dim, n, (0, 0, 0), 1.0, cell_order=1)
        assert np.array_equal(mmf.problem.morton_order(dim, n), m.grid_of_raw())

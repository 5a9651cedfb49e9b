"""CPU tests of the oracle: the reference goldens, known answers, and (where
the reference tree is present) bit-for-bit agreement with the reference
sources compiled against the bitpit stand-in."""
import os
import subprocess

import numpy as np
import pytest

REF_SRC = os.path.join(os.environ.get("MMF_REFERENCE", "/root/reference"), "src")


@pytest.mark.parametrize("name", ["2dIsentropicVortex", "2dRadSod", "3dIsentropicVortexXY",
                                  "3dIsentropicVortexYZ", "3dRadSod"])
def test_reference_goldens(orc, name):
    """test/<case>/CMakeLists.txt:33 via test/test_driver.py:63 (string compare)."""
    err, s, golden, steps = orc.run_golden(name)
    assert abs(err - float(golden)) <= 1e-10 * float(golden)
    assert s == golden


def test_golden_morton_order(orc):
    """The raw (octree) cell order changes only the error summation order."""
    err0, _, golden, _ = orc.run_golden("2dRadSod")
    err1, _, _, _ = orc.run_golden("2dRadSod", cell_order=1)
    assert abs(err1 - err0) <= 1e-13 * err0


def test_splitting_equal_states_is_physical_flux(orc):
    rng = np.random.default_rng(1)
    for _ in range(20):
        prim = np.array([rng.uniform(0.5, 2), *rng.uniform(-1, 1, 3), rng.uniform(0.5, 2)])
        c = orc.prim2cons(prim)
        n = rng.normal(size=3); n /= np.linalg.norm(n)
        F, lam = orc.eval_splitting(c, c, n)
        f = orc.eval_fluxes(c, orc.cons2prim(c), n)
        np.testing.assert_allclose(F, f, rtol=0, atol=1e-14)
        p = orc.cons2prim(c)
        assert lam == pytest.approx(abs(p[1:4] @ n) + np.sqrt(1.4 * p[4]), rel=1e-14)


def test_splitting_antisymmetry(orc):
    """F(L, R, n) = -F(R, L, -n) exactly: the GPU border faces rely on it."""
    rng = np.random.default_rng(2)
    for _ in range(50):
        cl = orc.prim2cons(np.array([rng.uniform(0.1, 2), *rng.uniform(-2, 2, 3), rng.uniform(0.1, 2)]))
        cr = orc.prim2cons(np.array([rng.uniform(0.1, 2), *rng.uniform(-2, 2, 3), rng.uniform(0.1, 2)]))
        for d in range(3):
            n = np.zeros(3); n[d] = 1.0
            F1, l1 = orc.eval_splitting(cl, cr, n)
            F2, l2 = orc.eval_splitting(cr, cl, -n)
            assert np.array_equal(F1, -F2) and l1 == l2


def test_cons_prim_roundtrip(orc):
    rng = np.random.default_rng(3)
    for _ in range(50):
        prim = np.array([rng.uniform(0.1, 3), *rng.uniform(-3, 3, 3), rng.uniform(0.1, 3)])
        np.testing.assert_allclose(orc.cons2prim(orc.prim2cons(prim)), prim, rtol=1e-14, atol=1e-14)


def test_reflecting_bc_mirrors_normal_velocity(orc):
    rng = np.random.default_rng(4)
    for _ in range(20):
        prim = np.array([rng.uniform(0.1, 3), *rng.uniform(-3, 3, 3), rng.uniform(0.1, 3)])
        c = orc.prim2cons(prim)
        n = np.zeros(3); n[rng.integers(3)] = rng.choice([-1.0, 1.0])
        g = orc.cons2prim(orc.eval_bc(orc.RADSOD, orc.BC_REFLECTING, np.zeros(3), n, c))
        assert g[1:4] @ n == pytest.approx(-(prim[1:4] @ n), abs=1e-13)
        assert g[0] == pytest.approx(prim[0], rel=1e-14)
    c = orc.prim2cons(np.array([1.0, 0.3, 0.2, 0.1, 1.0]))
    assert np.array_equal(orc.eval_bc(0, orc.BC_FREE_FLOW, np.zeros(3), np.array([1.0, 0, 0]), c), c)


def test_dirichlet_bc_is_ffstep_inflow(orc):
    g = orc.eval_bc(orc.FFSTEP, orc.BC_DIRICHLET, np.zeros(3), np.array([-1.0, 0, 0]), np.ones(5))
    np.testing.assert_allclose(orc.cons2prim(g), [1.0, 3.0, 0.0, 0.0, 1.0 / 1.4], rtol=1e-15)


def test_vortex_exact_at_t0_is_initial_state(orc):
    m = orc.golden_mesh("2dIsentropicVortex")
    U0 = m.initial_state()
    assert m.l1_density_error(U0, 0.0) == 0.0


def test_free_stream_preserved(orc):
    m = orc.OracleMesh(orc.VORTEX_XY, 2, (16, 16, 1), (0, 0, 0), 1.0)
    U = np.tile(orc.prim2cons(np.array([1.0, 0.7, -0.3, 0.0, 1.0])), (m.ncells, 1))
    R, me = m.compute_rhs(U)
    assert np.abs(R).max() < 1e-15


def test_rhs_conservation_periodic(orc):
    """With periodic borders the residuals sum to zero (every face flux cancels)."""
    P = orc.BC_PERIODIC
    m = orc.OracleMesh(orc.VORTEX_XY, 2, (24, 16, 1), (-5, -5, 0), 10.0, bc_lo=[P, P, P], bc_hi=[P, P, P])
    rng = np.random.default_rng(5)
    U = m.initial_state() * (1 + 0.01 * rng.standard_normal((m.ncells, 1)))
    R, _ = m.compute_rhs(U)
    assert np.abs(R.sum(axis=0)).max() < 1e-12


def test_order2_limiter_flags_extrema(orc):
    """Order-2 extension: MC limiter is inactive in smooth monotone regions and
    active at extrema and discontinuities."""
    m = orc.OracleMesh(orc.RADSOD, 2, (32, 32, 1), (-1, -1, 0), 2.0, bc_lo=[0, 0, 0], bc_hi=[0, 0, 0])
    U = m.initial_state(orc.params(sod_radius=0.5))
    S, act = m.compute_polynomials(U, order=2, want_active=True)
    c = m.centroids()
    r = np.hypot(c[:, 0], c[:, 1])
    assert act[np.abs(r - 0.5) < 0.05].any()
    assert not act[(r < 0.3)].any()


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference tree not present")
def test_oracle_matches_reference_build(orc, tmp_path):
    """oracle/_ref (reference euler.cpp/utils.cpp/problem.cpp/... + bitpit stand-in)
    and the C restatement give bit-identical final states."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.check_call(["make", "-s", "-f", os.path.join(root, "oracle", "Makefile.ref"),
                           "REF_SRC=" + REF_SRC], cwd=root, timeout=300)
    exe = os.path.join(root, "oracle", "_ref", "mmf_ref")
    for name in ["2dRadSod", "3dIsentropicVortexYZ"]:
        pname, dim, n, cfl, t_end, golden = orc.GOLDEN_CASES[name]
        dump = str(tmp_path / (name + ".bin"))
        out = subprocess.check_output([exe, pname, str(dim), str(n), "1", str(cfl),
                                       "-" if name.startswith("3d") else repr(t_end), "-1", dump],
                                      timeout=300).decode()
        assert ("Final error:  " + golden) in out
        m = orc.golden_mesh(name)
        U, t, steps = m.run(m.initial_state(), cfl, t_end=t_end)
        assert np.array_equal(np.fromfile(dump).reshape(-1, 5), U)


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference tree not present")
@pytest.mark.parametrize("case", ["vortex_body", "ffstep"])
def test_oracle_bodies_match_reference_build(orc, tmp_path, case):
    """Immersed box bodies (reference body.cpp, unsolved cells, BC_WALL faces,
    main.cpp:222-277) and the forward-facing step (problem.cpp:404-477):
    oracle/_ref and the C restatement give bit-identical final states."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.check_call(["make", "-s", "-f", os.path.join(root, "oracle", "Makefile.ref"),
                           "REF_SRC=" + REF_SRC], cwd=root, timeout=300)
    exe = os.path.join(root, "oracle", "_ref", "mmf_ref")
    dump = str(tmp_path / "final.bin")
    if case == "vortex_body":
        box, steps = ((1.0, -1.5, -10.0), (2.5, 1.5, 10.0)), 40
        args = ["vortex_xy", "2", "64", "1", "0.45", "inf", str(steps), dump]
        m = orc.OracleMesh(orc.VORTEX_XY, 2, (64, 64, 1), (-5, -5, 0), 10.0)
    else:
        box, steps = ((0.6, -1.0, -10.0), (4.0, 0.2, 10.0)), 60
        args = ["ffstep", "2", "64", "1", "0.45", "inf", str(steps), dump, "length=3.2"]
        m = orc.OracleMesh(orc.FFSTEP, 2, (64, 64, 1), (0, 0, 0), 3.2)
    args.append("body=" + ",".join(repr(v) for v in box[0] + box[1]))
    subprocess.check_output([exe] + args, timeout=300)
    solid = m.set_bodies([box])
    assert solid.sum() > 50
    U, t, s = m.run(m.initial_state(), 0.45, max_steps=steps)
    assert s == steps
    assert np.array_equal(np.fromfile(dump).reshape(-1, 5), U)


GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLDEN_FILES = sorted(f[:-4] for f in os.listdir(GOLDEN_DIR) if f.endswith(".npz"))


def golden_fixture_mesh(orc, g):
    """The oracle mesh of a fixture written by tests/golden/make_golden.py."""
    prob = orc.PROBLEMS[str(g["problem"])]
    dim, n = int(g["dim"]), int(g["n"])
    origin, length = ((0.0, 0.0, 0.0), float(g["length"])) if prob == orc.FFSTEP else orc.reference_domain(prob)
    m = orc.OracleMesh(prob, dim, (n, n, n if dim == 3 else 1), origin, length)
    b = g["body"]
    if b.size:
        m.set_bodies([(tuple(b[:3]), tuple(b[3:]))])
    return m


@pytest.mark.parametrize("name", GOLDEN_FILES)
def test_oracle_reproduces_reference_fixtures(orc, name):
    """The oracle against the reference's own outputs (fixtures made by the
    reference build): initial state, final state and final time bit for bit,
    and the final-error line of the reference driver."""
    g = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    m = golden_fixture_mesh(orc, g)
    assert np.array_equal(m.initial_state(), g["U0"])
    U, t, steps = m.run(g["U0"], float(g["cfl"]), max_steps=int(g["steps"]))
    assert steps == int(g["steps"]) and t == float(g["t"])
    assert np.array_equal(U, g["U"])
    assert "%.12e" % m.l1_density_error(U, t) == str(g["final_error"])

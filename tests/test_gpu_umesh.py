"""The face-list solver (any MeshGeometricalInfo-like mesh) against the oracle:
bit-identical with the reference arithmetic on the reference goldens, on an
octree (Morton) raw order, with an immersed body (unsolved cells, BC_WALL
faces, main.cpp:222-277) and on the forward-facing step (Dirichlet inflow,
free-flow outflow, reflecting walls, problem.cpp:404-477); <= 1e-12 per cell
with the fast arithmetic."""
import numpy as np
import pytest

from test_gpu_parity import FAST_RTOL, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["2dIsentropicVortex", "2dRadSod", "3dIsentropicVortexYZ", "3dRadSod"])
def test_goldens_on_face_lists(orc, mmf, name):
    from minimmerflow_gb300.umesh import UnstructuredEuler
    pname, dim, n, cfl, t_end, golden = orc.GOLDEN_CASES[name]
    m = orc.golden_mesh(name, cell_order=1)       # octree raw order
    U0 = m.initial_state()
    U_ref, t_ref, s_ref = m.run(U0, cfl, t_end=t_end)
    with UnstructuredEuler.from_oracle_mesh(m) as u:
        R, me = u.compute_rhs(U0)
        U, t, s = u.run(U0, cfl, t_end=t_end)
    R_ref, me_ref = m.compute_rhs(U0)
    assert me == me_ref and np.array_equal(R, R_ref)
    assert s == s_ref and t == t_ref
    assert np.array_equal(U, U_ref)
    assert "%.12e" % m.l1_density_error(U, t_end) == golden
    with UnstructuredEuler.from_oracle_mesh(m, arith="fast") as u:
        U2, _, _ = u.run(U0, cfl, t_end=t_end)
    assert rel_err(U2, U_ref) <= FAST_RTOL


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_immersed_body(orc, mmf, arith):
    from minimmerflow_gb300.umesh import UnstructuredEuler
    m = orc.OracleMesh(orc.VORTEX_XY, 2, (64, 64, 1), (-5, -5, 0), 10.0)
    inside = m.set_bodies([((1.0, -1.5, -10), (2.5, 1.5, 10))])
    assert inside.sum() > 50
    U0 = m.initial_state()
    U_ref, t_ref, _ = m.run(U0, 0.45, max_steps=40)
    with UnstructuredEuler.from_oracle_mesh(m, arith=arith) as u:
        U, t, s = u.run(U0, 0.45, max_steps=40)
    assert s == 40
    if arith == "reference":
        assert np.array_equal(U, U_ref) and t == t_ref
    else:
        assert rel_err(U[~inside], U_ref[~inside]) <= FAST_RTOL
    assert np.array_equal(U[inside], U0[inside])     # solid cells keep their state


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_forward_facing_step(orc, mmf, arith):
    """Mach 3 flow over a step: [0,3.2]^2, step [0.6,3.2] x [0,0.2], 2D."""
    from minimmerflow_gb300.umesh import UnstructuredEuler
    m = orc.OracleMesh(orc.FFSTEP, 2, (64, 64, 1), (0, 0, 0), 3.2)
    bc = m.faces()["bc"]
    assert {orc.BC_DIRICHLET, orc.BC_FREE_FLOW, orc.BC_REFLECTING} <= set(bc.tolist())
    inside = m.set_bodies([((0.6, -1.0, -10), (4.0, 0.2, 10))])
    U0 = m.initial_state()
    U_ref, t_ref, _ = m.run(U0, 0.45, max_steps=60)
    dp = [1.0, 3.0, 0.0, 0.0, 1.0 / 1.4]
    with UnstructuredEuler.from_oracle_mesh(m, arith=arith, dirichlet_prim=dp) as u:
        U, t, s = u.run(U0, 0.45, max_steps=60)
    if arith == "reference":
        assert np.array_equal(U, U_ref)
    else:
        assert rel_err(U[~inside], U_ref[~inside]) <= FAST_RTOL
    # the step reflects the flow: a bow shock raises the density ahead of it
    assert U[~inside, 0].max() > 1.5 * U0[0, 0]


def test_face_list_reports_negative_pressure(orc, mmf):
    """A non-physical input state on the face-list path is reported as
    MMF_ERR_STATE, not trapped (the Cartesian kernels do the same)."""
    from minimmerflow_gb300.umesh import UnstructuredEuler
    m = orc.OracleMesh(orc.RADSOD, 2, (16, 16, 1), (0, 0, 0), 8.0)
    U0 = m.initial_state()
    U0[37, 4] = -1.0
    with UnstructuredEuler.from_oracle_mesh(m, arith="fast") as u:
        with pytest.raises(mmf.capi.MMFError) as ei:
            u.run(U0, 0.45, max_steps=2)
        assert ei.value.code == mmf.capi.MMF_ERR_STATE


def test_face_list_stops_at_the_end_time(orc, mmf):
    """Asking for many more steps than the run needs returns promptly."""
    import time
    from minimmerflow_gb300.umesh import UnstructuredEuler
    m = orc.OracleMesh(orc.RADSOD, 2, (16, 16, 1), (0, 0, 0), 8.0)
    with UnstructuredEuler.from_oracle_mesh(m, arith="fast") as u:
        u.upload(m.initial_state())
        u.time_setup(0.45, 0.0, 0.05)
        t0 = time.perf_counter()
        t, steps = u.advance(1 << 24)
        assert time.perf_counter() - t0 < 5.0
        assert t == 0.05 and steps > 0

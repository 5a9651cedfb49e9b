"""GPU parity at the benchmark sizes: the CUDA path against the oracle on the
full meshes the benchmark measures, not on reduced copies of them.

- 2D radial Sod, 1024^2 cells on [-1,1]^2, rho = p = 1 for r < 0.5 and
  rho = 0.125, p = 0.1 outside, zero velocity, transmissive borders, CFL 0.5:
  the first 128 steps of the run to t = 0.25 (the reference loop,
  src/main.cpp:377-506, restated by the oracle; about 35 s of oracle time),
  on the Cartesian kernels and on the face-list kernels.
- 3D periodic isentropic vortex, beta = 5, on [-5,5]^3 at 64^3, 50 steps,
  vortex axis along z and along x.
- Order 2 (MC limiter on every cell): the 1024^2 radial Sod at CFL 0.4, 10
  steps, and the 3D radial Sod of the learned workload (pressure ratio 10,
  density ratio 8) on 128^3, 3 steps.

The reference arithmetic must give the oracle's bits; the fast arithmetic
must stay within 1e-12 per cell (max_k |U_k - U_ref_k| / max_k |U_ref_k|).
The oracle runs once per case and serves both arithmetics."""
import numpy as np
import pytest

from tests.test_gpu_parity import FAST_RTOL, oracle_mesh, oracle_params, rel_err

pytestmark = pytest.mark.gpu

SOD_STEPS = 128
VORTEX_STEPS = 50
O2_SOD2D_STEPS = 10
O2_SOD3D_STEPS = 3

_cache = {}


def _oracle_run(orc, case, steps, order=1):
    key = (case.name, order, steps)
    if key not in _cache:
        m = oracle_mesh(orc, case)
        U0 = m.initial_state(oracle_params(orc, case))
        U_ref, t_ref, steps_ref = m.run(U0, case.cfl, max_steps=steps, order=order)
        assert steps_ref == steps
        _cache[key] = (U0, U_ref, t_ref)
    return _cache[key]


def _check(U, t, U_ref, t_ref, arith):
    if arith == "reference":
        assert t == t_ref
        assert np.array_equal(U, U_ref)
    else:
        assert abs(t - t_ref) <= 1e-13 * t_ref
        assert rel_err(U, U_ref) <= FAST_RTOL


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_full_size_sod_1024_matches_oracle(orc, mmf, arith):
    case = mmf.problem.radial_sod_2d(n=1024)
    U0, U_ref, t_ref = _oracle_run(orc, case, SOD_STEPS)
    with case.solver(arith=arith) as s:
        U, t, steps = s.run(U0, case.cfl, max_steps=SOD_STEPS)
        assert s.status() == 0
    assert steps == SOD_STEPS
    if arith == "reference":
        assert t == t_ref
        assert np.array_equal(U, U_ref)
    else:
        assert abs(t - t_ref) <= 1e-13 * t_ref
        assert rel_err(U, U_ref) <= FAST_RTOL


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_full_size_sod_1024_face_lists_match_oracle(orc, mmf, arith):
    """The face-list solver (the path for meshes that are not one lattice) on
    the same 1024^2 Sod and 128 steps, against the same oracle run."""
    from minimmerflow_gb300.umesh import UnstructuredEuler
    case = mmf.problem.radial_sod_2d(n=1024)
    U0, U_ref, t_ref = _oracle_run(orc, case, SOD_STEPS)
    m = oracle_mesh(orc, case)
    with UnstructuredEuler.from_oracle_mesh(m, arith=arith) as u:
        U, t, steps = u.run(U0, case.cfl, max_steps=SOD_STEPS)
    assert steps == SOD_STEPS
    _check(U, t, U_ref, t_ref, arith)


@pytest.mark.parametrize("arith", ["reference", "fast"])
@pytest.mark.parametrize("axis", ["z", "x"])
def test_vortex3d_64_matches_oracle(orc, mmf, axis, arith):
    case = mmf.problem.vortex(3, 64, axis=axis, steps=VORTEX_STEPS)
    U0, U_ref, t_ref = _oracle_run(orc, case, VORTEX_STEPS)
    with case.solver(arith=arith) as s:
        U, t, steps = s.run(U0, case.cfl, max_steps=VORTEX_STEPS)
        assert s.status() == 0
    assert steps == VORTEX_STEPS
    if arith == "reference":
        assert t == t_ref
        assert np.array_equal(U, U_ref)
    else:
        assert abs(t - t_ref) <= 1e-13 * t_ref
        assert rel_err(U, U_ref) <= FAST_RTOL


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_full_size_sod_1024_order2_matches_oracle(orc, mmf, arith):
    """The benchmark's 1024^2 radial Sod at order 2 (MC limiter on every cell,
    the `--order 2` line, CFL 0.4), the first 10 steps (about 6 s of oracle
    time)."""
    case = mmf.problem.radial_sod_2d(n=1024, cfl=0.4)
    U0, U_ref, t_ref = _oracle_run(orc, case, O2_SOD2D_STEPS, order=2)
    with case.solver(arith=arith, order=2) as s:
        U, t, steps = s.run(U0, case.cfl, max_steps=O2_SOD2D_STEPS)
        assert s.status() == 0
    assert steps == O2_SOD2D_STEPS
    _check(U, t, U_ref, t_ref, arith)


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_sod3d_128_order2_matches_oracle(orc, mmf, arith):
    """The learned workload's problem -- 3D radial Sod on [-1,1]^3, r < 0.5,
    pressure ratio 10, density ratio 8, transmissive, CFL 0.5 -- at order 2
    with every cell limited, on 128^3 (an eighth of the benchmark's cells: the
    oracle's mesh takes about 600 B per cell), 3 steps (about 6 s of oracle
    time)."""
    case = mmf.problem.radial_sod_ratios(128, 10.0, 8.0, dim=3)
    U0, U_ref, t_ref = _oracle_run(orc, case, O2_SOD3D_STEPS, order=2)
    with case.solver(arith=arith, order=2) as s:
        U, t, steps = s.run(U0, case.cfl, max_steps=O2_SOD3D_STEPS)
        assert s.status() == 0
    assert steps == O2_SOD3D_STEPS
    _check(U, t, U_ref, t_ref, arith)

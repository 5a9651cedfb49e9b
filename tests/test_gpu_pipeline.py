"""GPU: mmf_advance_host with page-locked host buffers runs the banded
pipeline (uploads overlapping stage 1 and, at order 2, its slopes; the last
step's stage 3 band by band, after a banded stage 2 at order 1; downloads
overlapping stage 3).  It must give the same bits as the
unpipelined round trip (pageable buffers: upload, graph-replayed steps,
download), for both arithmetics and orders, periodic and transmissive slow
axes, bands as thin as one marching chunk, one and several steps per call, a 2D state
whose z-momentum is not zero after calls where it was (the stage-1 redo), a
run that reaches its end time, and the per-step log."""
import dataclasses
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def pinned(shape):
    import torch
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


def round_trips(case, arith, states, steps, pin, order=1):
    outs = []
    with case.solver(arith=arith, order=order) as s:
        s.time_setup(case.cfl, 0.0, math.inf, 10 ** 6)
        for U in states:
            h = pinned(U.shape) if pin else np.empty_like(U)
            h[:] = U
            t = s.advance_host(h, steps)
            outs.append((h.copy(), t))
    return outs


def thin(case, n):
    """The case on an n[0] x n[1] strip through the domain's centre line
    (cell edge length / n[0]; 8 rows per band: one marching chunk)."""
    h = case.length / n[0]
    origin = (case.origin[0], -0.5 * n[1] * h, case.origin[2])
    return dataclasses.replace(case, n=n, origin=origin)


CASES = {
    "sod2d_512": lambda P: P.radial_sod_2d(512),
    "sod2d_4096x64": lambda P: thin(P.radial_sod_2d(64), (4096, 64)),
    "vortex2d_4096x64_periodic": lambda P: thin(P.vortex(2, 64), (4096, 64)),
    "vortex2d_512_periodic": lambda P: P.vortex(2, 512),
    "vortex3d_64_periodic": lambda P: P.vortex(3, 64, axis="x"),
    "sod3d_64": lambda P: P.radial_sod_ratios(64, 10.0, 4.0, dim=3),
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("arith", ["reference", "fast"])
@pytest.mark.parametrize("steps", [1, 3])
@pytest.mark.parametrize("order", [1, 2])
def test_pipelined_round_trip_is_bitwise(mmf, name, arith, steps, order):
    case = CASES[name](mmf.problem)
    U0 = case.initial_state()
    states = [U0, U0]
    a = round_trips(case, arith, states, steps, pin=False, order=order)
    b = round_trips(case, arith, states, steps, pin=True, order=order)
    for (ua, ta), (ub, tb) in zip(a, b):
        assert ta == tb
        np.testing.assert_array_equal(ua, ub)


@pytest.mark.parametrize("arith", ["reference", "fast"])
@pytest.mark.parametrize("steps", [1, 2])
@pytest.mark.parametrize("order", [1, 2])
def test_pipelined_z_momentum_switch(mmf, arith, steps, order):
    P = mmf.problem
    case = P.radial_sod_2d(512)
    U0 = case.initial_state()
    Uw = U0.copy()
    rng = np.random.default_rng(3)
    Uw[:, 3] = 1e-3 * rng.standard_normal(len(U0)) * U0[:, 0]
    Uw[:, 4] += 0.5 * Uw[:, 3] ** 2 / Uw[:, 0]
    states = [U0, Uw, U0, Uw]
    a = round_trips(case, arith, states, steps, pin=False, order=order)
    b = round_trips(case, arith, states, steps, pin=True, order=order)
    for (ua, ta), (ub, tb) in zip(a, b):
        assert ta == tb
        np.testing.assert_array_equal(ua, ub)


@pytest.mark.parametrize("pin", [False, True])
def test_pipelined_run_reaches_end_time(mmf, pin):
    """One-step calls up to t_end: the last step is cut to t_end, later calls
    leave the state and the time unchanged (inactive steps)."""
    case = mmf.problem.radial_sod_2d(512)
    U0 = case.initial_state()
    with case.solver() as s:
        s.time_setup(case.cfl, 0.0, 0.01, -1)
        h = pinned(U0.shape) if pin else np.empty_like(U0)
        h[:] = U0
        ts = [s.advance_host(h, 1) for _ in range(40)]
        assert ts[-1] == 0.01 and ts.index(0.01) < 39
        last = h.copy()
        assert s.advance_host(h, 1) == 0.01
        np.testing.assert_array_equal(h, last)
        return_steps = s.time_info()[1]
    with case.solver() as s:
        s.upload(U0)
        s.time_setup(case.cfl, 0.0, 0.01, -1)
        t, steps = s.advance(100)
        assert t == 0.01 and steps == return_steps
        np.testing.assert_array_equal(s.download(), last)


def test_pipelined_step_log(mmf):
    """The per-step log of one-step pinned round trips equals the log of the
    same steps run on the device."""
    case = mmf.problem.radial_sod_2d(512)
    U0 = case.initial_state()
    with case.solver() as s:
        s.set_step_log(16)
        s.time_setup(case.cfl, 0.0, math.inf, 10 ** 6)
        h = pinned(U0.shape)
        h[:] = U0
        for _ in range(5):
            s.advance_host(h, 1)
        first_a, log_a = s.step_log()
    with case.solver() as s:
        s.set_step_log(16)
        s.upload(U0)
        s.time_setup(case.cfl, 0.0, math.inf, 10 ** 6)
        s.advance(5)
        first_b, log_b = s.step_log()
    assert first_a == first_b == 0
    np.testing.assert_array_equal(log_a, log_b)


def test_pipelined_order2_limiter_modes(mmf):
    """Order 2 with the limiter on flagged cells only, and with central slopes
    on a smooth state: the banded round trip keeps the bits."""
    P = mmf.problem
    case = P.vortex(2, 512)
    U0 = case.initial_state()
    flags = (np.arange(case.ncells) % 3 == 0).astype(np.uint8)
    for mode in ("flagged", "none"):
        outs = []
        for pin in (False, True):
            with case.solver(order=2) as s:
                s.set_limiter(mode, flags if mode == "flagged" else None)
                s.time_setup(case.cfl, 0.0, math.inf, 10 ** 6)
                h = pinned(U0.shape) if pin else np.empty_like(U0)
                h[:] = U0
                ts = [s.advance_host(h, 1) for _ in range(3)]
                outs.append((h.copy(), ts, s.limiter_activity()))
        assert outs[0][1] == outs[1][1]
        np.testing.assert_array_equal(outs[0][0], outs[1][0])
        np.testing.assert_array_equal(outs[0][2], outs[1][2])

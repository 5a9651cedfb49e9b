"""GPU: mmf_advance_host with page-locked host buffers runs the banded
pipeline (uploads overlapping stage 1, downloads overlapping stage 3).  It
must give the same bits as the unpipelined round trip (pageable buffers:
upload, graph-replayed steps, download), for both arithmetics, periodic and
transmissive slow axes, several steps per call, and a 2D state whose
z-momentum is not zero after calls where it was (the stage-1 redo)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def pinned(shape):
    import torch
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


def round_trips(case, arith, states, steps, pin):
    outs = []
    with case.solver(arith=arith) as s:
        s.time_setup(case.cfl, 0.0, math.inf, 10 ** 6)
        for U in states:
            h = pinned(U.shape) if pin else np.empty_like(U)
            h[:] = U
            t = s.advance_host(h, steps)
            outs.append((h.copy(), t))
    return outs


CASES = {
    "sod2d_512": lambda P: P.radial_sod_2d(512),
    "vortex2d_512_periodic": lambda P: P.vortex(2, 512),
    "vortex3d_64_periodic": lambda P: P.vortex(3, 64, axis="x"),
    "sod3d_64": lambda P: P.radial_sod_ratios(64, 10.0, 4.0, dim=3),
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("arith", ["reference", "fast"])
@pytest.mark.parametrize("steps", [1, 3])
def test_pipelined_round_trip_is_bitwise(mmf, name, arith, steps):
    case = CASES[name](mmf.problem)
    U0 = case.initial_state()
    states = [U0, U0]
    a = round_trips(case, arith, states, steps, pin=False)
    b = round_trips(case, arith, states, steps, pin=True)
    for (ua, ta), (ub, tb) in zip(a, b):
        assert ta == tb
        np.testing.assert_array_equal(ua, ub)


@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_pipelined_z_momentum_switch(mmf, arith):
    P = mmf.problem
    case = P.radial_sod_2d(512)
    U0 = case.initial_state()
    Uw = U0.copy()
    rng = np.random.default_rng(3)
    Uw[:, 3] = 1e-3 * rng.standard_normal(len(U0)) * U0[:, 0]
    Uw[:, 4] += 0.5 * Uw[:, 3] ** 2 / Uw[:, 0]
    states = [U0, Uw, U0, Uw]
    a = round_trips(case, arith, states, 2, pin=False)
    b = round_trips(case, arith, states, 2, pin=True)
    for (ua, ta), (ub, tb) in zip(a, b):
        assert ta == tb
        np.testing.assert_array_equal(ua, ub)

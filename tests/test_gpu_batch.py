"""Batched persistent solver: each case of a batch gets exactly the state of
its own single-case context (same arithmetic, its own CFL dt); with the
reference arithmetic that is the oracle's state bit for bit.  The autotuner
changes only the decomposition and leaves the state untouched."""
import numpy as np
import pytest

from test_gpu_parity import oracle_mesh, oracle_params

pytestmark = pytest.mark.gpu


def small_sweep(mmf, ncases=10, seed=7):
    return mmf.problem.batched_sweep(ncases=ncases, seed=seed, side_min=5, side_max=70)


@pytest.mark.parametrize("arith", ["fast", "reference"])
def test_batch_equals_single_contexts(mmf, arith):
    from minimmerflow_gb300.batch import BatchEuler
    cases = small_sweep(mmf)
    states = [c.initial_state() for c in cases]
    steps = 12
    with BatchEuler(cases, arith=arith) as b:
        out = b.run(states, steps)
        infos = [b.case_info(i) for i in range(len(cases))]
    for i, (c, U0) in enumerate(zip(cases, states)):
        with c.solver(arith=arith) as s:
            U, t, n = s.run(U0, c.cfl, max_steps=steps)
        assert n == steps and infos[i][1] == steps
        assert infos[i][0] == t
        assert np.array_equal(out[i], U), c.name
    # each case has its own time step
    assert len({round(x[0], 12) for x in infos}) > 1


def test_batch_reference_matches_oracle(orc, mmf):
    from minimmerflow_gb300.batch import BatchEuler
    cases = small_sweep(mmf, ncases=6, seed=11)
    states = []
    refs = []
    for c in cases:
        m = oracle_mesh(orc, c)
        prm = oracle_params(orc, c)
        U0 = m.initial_state(prm)
        states.append(U0)
        refs.append(m.run(U0, c.cfl, max_steps=8)[0])
    with BatchEuler(cases, arith="reference") as b:
        out = b.run(states, 8)
    for o, r in zip(out, refs):
        assert np.array_equal(o, r)


def test_autotune_keeps_state(mmf):
    from minimmerflow_gb300.batch import BatchEuler
    cases = small_sweep(mmf, ncases=16, seed=3)
    states = [c.initial_state() for c in cases]
    with BatchEuler(cases, arith="fast") as b:
        b.upload(states)
        b.time_setup(max_steps=6)
        chunk, bps = b.autotune(trial_steps=2)
        assert chunk in (8, 16, 32, 64) and bps >= 1
        assert b.case_info(0)[1] == 0          # the trials were rolled back
        b.advance_async(6)
        b.synchronize()
        tuned = b.unpack(b.download())
    with BatchEuler(cases, arith="fast") as b:
        b.set_shape(8, 1)
        plain = b.run(states, 6)
    for x, y in zip(tuned, plain):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("arith", ["fast", "reference"])
def test_batch_order2_equals_single_contexts(mmf, arith):
    from minimmerflow_gb300.batch import BatchEuler
    cases = small_sweep(mmf, ncases=8, seed=21)
    for c in cases:
        c.cfl = 0.4
    states = [c.initial_state() for c in cases]
    with BatchEuler(cases, arith=arith, order=2) as b:
        out = b.run(states, 10)
    for i, (c, U0) in enumerate(zip(cases, states)):
        with c.solver(arith=arith, order=2) as s:
            U, t, n = s.run(U0, c.cfl, max_steps=10)
        assert np.array_equal(out[i], U), c.name


def test_batch_order2_with_indicator_equals_single_contexts(mmf):
    """The learned indicator inside the batch gives every case the flags (and so
    the state) of its own single-case run with the same indicator."""
    from minimmerflow_gb300 import indicator
    from minimmerflow_gb300.batch import BatchEuler
    mlp = indicator.TroubledCellMLP(dim=2, seed=4)
    p = mlp.params()
    p[-1] = 0.0   # b3: roughly half the cells flagged by the random network
    mlp.set_params(p)
    # vortices only: a random (untrained) network leaves shock cells unlimited
    cases = [c for c in small_sweep(mmf, ncases=12, seed=22) if c.problem == mmf.problem.VORTEX_XY]
    for c in cases:
        c.cfl = 0.4
    states = [c.initial_state() for c in cases]
    with BatchEuler(cases, arith="fast", order=2) as b:
        b.set_indicator(mlp, 0.5)
        out = b.run(states, 6)
    for i, (c, U0) in enumerate(zip(cases, states)):
        with c.solver(arith="fast", order=2) as s:
            indicator.use_indicator(s, mlp, 0.5)
            U, t, n = s.run(U0, c.cfl, max_steps=6)
        assert np.array_equal(out[i], U), c.name


def test_batch_indicator_every_second_step_equals_single_contexts(mmf):
    """With the indicator run every second step (flags dilated by one cell),
    the batch still gives every case the state of its own single-case run."""
    from minimmerflow_gb300 import indicator
    from minimmerflow_gb300.batch import BatchEuler
    mlp = indicator.TroubledCellMLP(dim=2, seed=4)
    p = mlp.params()
    p[-1] = 0.0
    mlp.set_params(p)
    cases = [c for c in small_sweep(mmf, ncases=12, seed=22) if c.problem == mmf.problem.VORTEX_XY]
    for c in cases:
        c.cfl = 0.4
    states = [c.initial_state() for c in cases]
    with BatchEuler(cases, arith="fast", order=2) as b:
        b.set_indicator(mlp, 0.5, period=2)
        out = b.run(states, 7)
    for i, (c, U0) in enumerate(zip(cases, states)):
        with c.solver(arith="fast", order=2) as s:
            indicator.use_indicator(s, mlp, 0.5, period=2)
            U, t, n = s.run(U0, c.cfl, max_steps=7)
        assert np.array_equal(out[i], U), c.name


def test_full_sweep_every_case_equals_its_own_context(mmf):
    """The benchmark's sweep itself (512 cases, seed 20261203, sides 32..512):
    after 10 steps in one batch, every case holds exactly the state of its own
    single-case run."""
    from minimmerflow_gb300.batch import BatchEuler
    cases = mmf.problem.batched_sweep(ncases=512, seed=20261203)
    states = [c.initial_state() for c in cases]
    steps = 10
    with BatchEuler(cases, arith="fast") as b:
        b.upload(states)
        b.time_setup(max_steps=steps)
        b.autotune(trial_steps=2)
        b.advance_async(steps)
        b.synchronize()
        out = b.unpack(b.download())
        assert all(b.case_info(i)[2] == 0 for i in range(len(cases)))
    for i, (c, U0) in enumerate(zip(cases, states)):
        with c.solver(arith="fast") as s:
            U, t, n = s.run(U0, c.cfl, max_steps=steps)
        assert n == steps
        assert np.array_equal(out[i], U), c.name

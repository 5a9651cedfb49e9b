"""GPU against the reference's own outputs: tests/golden/*.npz hold initial
and final states written by the reference sources (compiled unmodified
against the bitpit stand-in, tests/golden/make_golden.py).  The CUDA path with
the reference arithmetic must reproduce them bit for bit -- the Cartesian
kernels for the plain cases, the face-list kernels for the cases with an
immersed body and the forward-facing step -- and the fast arithmetic within
1e-12 relative per cell."""
import math
import os

import numpy as np
import pytest

from test_gpu_parity import FAST_RTOL, rel_err
from test_oracle import GOLDEN_DIR, GOLDEN_FILES, golden_fixture_mesh

pytestmark = pytest.mark.gpu


def cartesian_case(mmf, g):
    P = mmf.problem
    prob = P.PROBLEMS[str(g["problem"])]
    case = P.reference_case(prob, int(g["dim"]), int(g["n"]), cfl=float(g["cfl"]))
    case.t_end = math.inf
    return case


@pytest.mark.parametrize("name", GOLDEN_FILES)
@pytest.mark.parametrize("arith", ["reference", "fast"])
def test_cuda_reproduces_reference_fixtures(orc, mmf, name, arith):
    g = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    steps, cfl = int(g["steps"]), float(g["cfl"])
    if g["body"].size:
        from minimmerflow_gb300.umesh import UnstructuredEuler
        m = golden_fixture_mesh(orc, g)
        dp = [1.0, 3.0, 0.0, 0.0, 1.0 / 1.4] if str(g["problem"]) == "ffstep" else [0.0] * 5
        with UnstructuredEuler.from_oracle_mesh(m, arith=arith, dirichlet_prim=dp) as u:
            U, t, s = u.run(g["U0"], cfl, max_steps=steps)
    else:
        case = cartesian_case(mmf, g)
        with case.solver(arith=arith) as sv:
            sv.upload(g["U0"])
            sv.time_setup(cfl, 0.0, math.inf, steps)
            t, s = sv.advance(steps + 5)
            U = sv.download()
            if arith == "reference":
                # the device initial state (CUDA exp/pow) against the reference's (glibc)
                sv.init_state(case)
                assert rel_err(sv.download(), g["U0"]) <= 1e-14
    assert s == steps
    if arith == "reference":
        assert t == float(g["t"])
        assert np.array_equal(U, g["U"])
    else:
        assert abs(t - float(g["t"])) <= 1e-12 * float(g["t"])
        assert rel_err(U, g["U"]) <= FAST_RTOL

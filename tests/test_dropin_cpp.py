"""The C++ adapter as a drop-in: the reference's own time loop written against
mmf_gb300::euler::computeRHS (tests/cpp/test_dropin.cpp) and the device-resident
Stepper reproduce the oracle bit for bit."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_dropin(tmpdir):
    import minimmerflow_gb300 as mmf
    import oracle
    lib = mmf.build_library()
    olib = oracle.build()
    exe = os.path.join(str(tmpdir), "test_dropin")
    subprocess.check_call(["g++", "-std=c++11", "-O2", "-ffp-contract=off",
                           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"),
                           "-I", os.path.join(ROOT, "oracle", "ref_shim"),
                           os.path.join(ROOT, "tests", "cpp", "test_dropin.cpp"), lib, olib,
                           "-Wl,-rpath," + os.path.dirname(lib), "-Wl,-rpath," + os.path.dirname(olib),
                           "-lm", "-o", exe])
    return exe


def test_dropin_builds(tmp_path):
    """The adapter compiles against bitpit-like types (no GPU needed)."""
    assert os.path.exists(build_dropin(tmp_path))


@pytest.mark.gpu
@pytest.mark.parametrize("problem,dim,n,steps,body", [("radsod", 2, 64, 12, False), ("vortex_xy", 3, 16, 6, False),
                                                      ("vortex_xy", 2, 64, 20, True), ("ffstep", 2, 64, 40, True)])
def test_dropin_loop_matches_oracle(orc, tmp_path, problem, dim, n, steps, body):
    exe = build_dropin(tmp_path)
    a, b = str(tmp_path / "loop.bin"), str(tmp_path / "stepper.bin")
    cmd = [exe, problem, str(dim), str(n), str(steps), a, b] + (["body"] if body else [])
    out = subprocess.check_output(cmd, timeout=300).decode()
    assert out.startswith("steps")
    prob = orc.PROBLEMS[problem]
    origin, length = ((0.0, 0.0, 0.0), 3.2) if prob == orc.FFSTEP else orc.reference_domain(prob)
    m = orc.OracleMesh(prob, dim, (n, n, n if dim == 3 else 1), origin, length)
    if body and prob == orc.FFSTEP:
        m.set_bodies([((0.6, -1.0, -10), (4.0, 0.2, 10))])
    elif body:
        m.set_bodies([((1.0, -1.5, -10), (2.5, 1.5, 10))])
    U_ref, t, s = m.run(m.initial_state(), 0.45, max_steps=steps)
    assert np.array_equal(np.fromfile(a).reshape(-1, 5), U_ref)
    assert np.array_equal(np.fromfile(b).reshape(-1, 5), U_ref)

"""GPU: initial states and the L1 density error computed on the device
(problem.cpp:247-392, main.cpp:335-344 and 550-567), the VTK output of the
cell fields (solver_writer.cpp:56-119) and checkpoint/restart.

The initial states are compared with the numpy restatement cell by cell:
the prim2cons arithmetic is the reference's (no contraction), and exp/pow of
the vortex may differ from numpy's in the last bit, so the bound is 1e-14
relative per cell.  The L1 error sums in a different order and its exact
solution carries the same last-bit differences: 1e-12 relative.
"""
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

IC_RTOL = 1e-14


def rel_err(a, b):
    num = np.abs(a - b).max(axis=1)
    den = np.abs(b).max(axis=1)
    return float((num / den).max())


def cases(P):
    ff = P.Case("ffstep", P.FFSTEP, 2, (48, 16, 1), (0.0, 0.0, 0.0), 3.0, 0.5, t_end=0.1, border_bc=P.BC_FREE_FLOW)
    sod_y = P.reference_case("sod3d_y", 3, 16)
    return [P.vortex(2, 64), P.vortex(3, 24, axis="x"), P.reference_case("vortex_zx", 3, 20),
            P.radial_sod_2d(64), P.radial_sod_ratios(24, 10.0, 4.0, dim=3), P.reference_case("radsod", 2, 40),
            P.reference_case("sod3d_x", 2, 40), sod_y, ff]


@pytest.mark.parametrize("idx", range(9))
def test_init_state_matches_restatement(mmf, idx):
    case = cases(mmf.problem)[idx]
    with case.solver() as s:
        s.init_state(case)
        U = s.download()
    assert rel_err(U, case.initial_state()) <= IC_RTOL


@pytest.mark.parametrize("which", ["vortex2d", "vortex3d", "sod"])
def test_l1_density_error(mmf, which):
    P = mmf.problem
    case = {"vortex2d": P.vortex(2, 64, steps=30), "vortex3d": P.vortex(3, 24, axis="x", steps=10),
            "sod": P.radial_sod_2d(96, t_end=0.05)}[which]
    with case.solver() as s:
        s.init_state(case)
        assert s.l1_density_error(case, 0.0) <= 1e-13
        U, t, steps = s.run(s.download(), case.cfl, t_end=case.t_end, max_steps=case.max_steps)
        s.upload(U)
        e_dev = s.l1_density_error(case, t)
    e_ref = case.l1_density_error(U, t)
    assert e_ref > 0
    assert abs(e_dev - e_ref) <= 1e-12 * e_ref


def read_vtk(path):
    raw = open(path, "rb").read()
    head, _, rest = raw.partition(b'<AppendedData encoding="raw">\n_')
    text = head.decode()
    arrays = {}
    for line in text.splitlines():
        if "<DataArray" in line:
            name = line.split('Name="')[1].split('"')[0]
            off = int(line.split('offset="')[1].split('"')[0])
            typ = line.split('type="')[1].split('"')[0]
            nbytes = struct.unpack_from("<Q", rest, off)[0]
            dt = np.int32 if typ == "Int32" else np.float64
            arrays[name] = np.frombuffer(rest, dtype=dt, count=nbytes // np.dtype(dt).itemsize, offset=off + 8)
    extent = text.split('WholeExtent="')[1].split('"')[0]
    return text, [int(v) for v in extent.split()], arrays


@pytest.mark.parametrize("dim,order", [(2, 1), (3, 1), (2, 2)])
def test_vtk_fields(mmf, tmp_path, dim, order):
    P = mmf.problem
    case = P.vortex(2, 48, steps=5) if dim == 2 else P.radial_sod_ratios(20, 10.0, 4.0, dim=3, max_steps=5)
    with case.solver(order=order) as s:
        U, t, _ = s.run(case.initial_state(), case.cfl, max_steps=case.max_steps)
        s.upload(U)
        s.write_vtk(tmp_path / "out.vti")
        R, _ = s.compute_rhs(U)
    text, ext, a = read_vtk(tmp_path / "out.vti")
    n = case.n
    assert ext == [0, n[0], 0, n[1], 0, n[2] if dim == 3 else 0]
    assert list(a) == ["solved", "velocity", "pressure", "temperature", "density", "residualC", "residualMX",
                       "residualMY", "residualMZ", "residualE"]
    assert np.all(a["solved"] == 1)
    for k, name in enumerate(["residualC", "residualMX", "residualMY", "residualMZ", "residualE"]):
        np.testing.assert_array_equal(a[name], R[:, k])
    rho = U[:, 0]
    vel = U[:, 1:4] / rho[:, None]
    p = (P.GAMMA - 1.0) * (U[:, 4] - 0.5 * rho * (vel * vel).sum(axis=1))
    np.testing.assert_array_equal(a["density"], rho)
    np.testing.assert_allclose(a["velocity"].reshape(-1, 3), vel, rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(a["pressure"], p, rtol=1e-12)
    np.testing.assert_allclose(a["temperature"], p / rho, rtol=1e-12)


@pytest.mark.parametrize("order", [1, 2])
def test_checkpoint_restart_is_bitwise(mmf, tmp_path, order):
    P = mmf.problem
    case = P.radial_sod_2d(64, t_end=0.1)
    ck = tmp_path / "state.ckpt"
    with case.solver(order=order) as s:
        s.init_state(case)
        s.time_setup(case.cfl, 0.0, case.t_end)
        s.advance(7)
        s.save_checkpoint(ck)
        t_a, steps_a = s.advance(1 << 20)
        U_a = s.download()
    with case.solver(order=order) as s:
        s.load_checkpoint(ck)
        t_b, steps_b = s.advance(1 << 20)
        U_b = s.download()
    assert t_a == t_b and steps_a == steps_b
    np.testing.assert_array_equal(U_a, U_b)


def test_checkpoint_rejects_other_grid(mmf, tmp_path):
    P = mmf.problem
    a, b = P.radial_sod_2d(32), P.radial_sod_2d(48)
    ck = tmp_path / "a.ckpt"
    with a.solver() as s:
        s.init_state(a)
        s.time_setup(a.cfl, 0.0, a.t_end)
        s.save_checkpoint(ck)
    with b.solver() as s:
        with pytest.raises(mmf.capi.MMFError):
            s.load_checkpoint(ck)

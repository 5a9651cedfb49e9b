"""mmf_compute_rhs_noalloc: the residual for callers that cannot allocate device
memory (code running under another library's graph capture, real-time loops,
pool-managed device memory).  Called through the C ABI with device buffers the
test owns, twice in a row on different states, it must give exactly what the
context-based mmf_compute_rhs gives (the reference arithmetic is bit-exact, so
the tolerance of these tests is equality).

This file is collected last so that a run stopping at the first failure has
already run every other test; it passes alone and after the other tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pname,dim,n,morton", [("radsod", 2, 64, False), ("vortex_xy", 3, 16, False),
                                                ("radsod", 3, 16, True), ("vortex_xy", 2, 256, False)])
def test_noalloc_rhs_matches_context_rhs(mmf, pname, dim, n, morton):
    import torch
    lib = mmf.capi.load()
    case = mmf.problem.reference_case(pname, dim, n)
    rng = np.random.default_rng(3)
    U0 = case.initial_state()
    states = [U0 * (1.0 + 0.02 * rng.standard_normal((case.ncells, 1))),
              U0 * (1.0 + 0.05 * rng.standard_normal((case.ncells, 1)))]
    raw_to_cell = mmf.problem.morton_order(dim, case.n) if morton else None
    with case.solver(arith="reference") as s:
        if morton:
            s.set_cell_map(raw_to_cell)
        expected = [s.compute_rhs(U) for U in states]
        grid = s.grid
    dev = torch.device("cuda", 0)
    d_map = torch.from_numpy(raw_to_cell).to(dev) if morton else None
    d_rhs = torch.full((case.ncells, 5), float("nan"), dtype=torch.float64, device=dev)
    d_me = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    for U, (R_ref, me_ref) in zip(states, expected):
        d_u = torch.from_numpy(U).to(dev)
        torch.cuda.synchronize()
        rc = lib.mmf_compute_rhs_noalloc(C.byref(grid), mmf.capi.ptr(d_u), mmf.capi.ptr(d_rhs),
                                         mmf.capi.ptr(d_me), mmf.capi.ptr(d_map), None)
        assert rc == 0, lib.mmf_last_error()
        torch.cuda.synchronize()
        assert np.array_equal(d_rhs.cpu().numpy(), R_ref)
        assert d_me.item() == me_ref


def test_noalloc_rejects_meshes_above_the_maximum(mmf):
    lib = mmf.capi.load()
    case = mmf.problem.reference_case("radsod", 2, 512)   # 262144 cells > 65536
    g = mmf.capi.Grid()
    g.dim, g.h, g.order, g.arith = 2, case.h, 1, 0
    g.n[0], g.n[1], g.n[2] = 512, 512, 1
    buf = (C.c_double * 8)()
    rc = lib.mmf_compute_rhs_noalloc(C.byref(g), buf, buf, buf, None, None)
    assert rc == mmf.capi.MMF_ERR_ARG
    assert b"65536" in lib.mmf_last_error()

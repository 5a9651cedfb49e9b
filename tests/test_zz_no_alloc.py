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


def _grid(mmf, n, h=0.1):
    g = mmf.capi.Grid()
    g.dim, g.h, g.order, g.arith = 2, h, 1, 0
    g.n[0], g.n[1], g.n[2] = n, n, 1
    return g


def test_noalloc_rejects_meshes_above_the_maximum(mmf):
    """Sizes beyond the static array, and what the entry point does not
    support, are refused before any GPU work is queued (the buffers here are
    host memory that no kernel ever sees)."""
    lib = mmf.capi.load()
    buf = (C.c_double * 8)()
    g = _grid(mmf, 512)   # 262144 cells > 65536
    rc = lib.mmf_compute_rhs_noalloc(C.byref(g), buf, buf, buf, None, None)
    assert rc == mmf.capi.MMF_ERR_ARG
    assert b"65536" in lib.mmf_last_error()
    g = _grid(mmf, 2**31 - 1)   # extents whose product overflows 64 bits
    g.dim, g.n[2] = 3, 2**31 - 1
    assert lib.mmf_compute_rhs_noalloc(C.byref(g), buf, buf, buf, None, None) == mmf.capi.MMF_ERR_ARG
    assert b"65536" in lib.mmf_last_error()
    g = _grid(mmf, 16)
    g.arith = mmf.capi.ARITH_FAST
    assert lib.mmf_compute_rhs_noalloc(C.byref(g), buf, buf, buf, None, None) == mmf.capi.MMF_ERR_UNSUPPORTED
    g.arith = 7
    assert lib.mmf_compute_rhs_noalloc(C.byref(g), buf, buf, buf, None, None) == mmf.capi.MMF_ERR_ARG
    g = _grid(mmf, 16)
    g.order = 2
    assert lib.mmf_compute_rhs_noalloc(C.byref(g), buf, buf, buf, None, None) == mmf.capi.MMF_ERR_UNSUPPORTED
    g = _grid(mmf, 16)
    g.bc_lo[1] = 9   # no such border condition
    assert lib.mmf_compute_rhs_noalloc(C.byref(g), buf, buf, buf, None, None) == mmf.capi.MMF_ERR_ARG
    assert b"border" in lib.mmf_last_error()
    g = _grid(mmf, 16, h=0.0)
    assert lib.mmf_compute_rhs_noalloc(C.byref(g), buf, buf, buf, None, None) == mmf.capi.MMF_ERR_ARG


@pytest.mark.parametrize("fault", ["duplicate", "out_of_range"])
def test_noalloc_map_that_is_not_a_permutation_gives_nan(mmf, fault):
    """A cell map with a repeated entry leaves a cell that no raw row fills,
    whose state would be the previous call's; one with an entry outside
    [0, n) is skipped by the kernels' bounds checks.  Either way the call
    writes NaN everywhere instead of a residual.  A good call right after
    gives the exact residual again."""
    import torch
    lib = mmf.capi.load()
    case = mmf.problem.reference_case("radsod", 2, 32)
    U = case.initial_state()
    with case.solver(arith="reference") as s:
        R_ref, me_ref = s.compute_rhs(U)
        grid = s.grid
    dev = torch.device("cuda", 0)
    bad = np.arange(case.ncells, dtype=np.int64)
    if fault == "duplicate":
        bad[5] = 6
    else:
        bad[5] = case.ncells + 3
        bad[9] = -1
    d_u = torch.from_numpy(U).to(dev)
    d_rhs = torch.zeros((case.ncells, 5), dtype=torch.float64, device=dev)
    d_me = torch.zeros((1,), dtype=torch.float64, device=dev)
    for m, expect_nan in [(bad, True), (np.arange(case.ncells, dtype=np.int64), False)]:
        d_map = torch.from_numpy(m).to(dev)
        torch.cuda.synchronize()
        rc = lib.mmf_compute_rhs_noalloc(C.byref(grid), mmf.capi.ptr(d_u), mmf.capi.ptr(d_rhs),
                                         mmf.capi.ptr(d_me), mmf.capi.ptr(d_map), None)
        assert rc == 0, lib.mmf_last_error()
        torch.cuda.synchronize()
        R = d_rhs.cpu().numpy()
        if expect_nan:
            assert np.isnan(R).all() and np.isnan(d_me.item())
        else:
            assert np.array_equal(R, R_ref) and d_me.item() == me_ref

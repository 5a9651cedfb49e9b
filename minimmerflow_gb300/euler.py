"""Reference-named entry points of src/euler.cpp and src/utils.cpp, batched on the GPU.

Each function takes numpy arrays of n items (AoS) and returns numpy arrays;
all arithmetic runs in the CUDA library with the reference operation order.
"""
import numpy as np

from . import capi


def _a(x, cols):
    a = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, cols)
    return a


def conservative2primitive(cons):
    """utils::conservative2primitive (utils.cpp:48-63)."""
    c = _a(cons, 5); p = np.empty_like(c)
    capi.check(capi.load().mmf_cons2prim(c.shape[0], capi.ptr(c), capi.ptr(p)))
    return p


def primitive2conservative(prim):
    """utils::primitive2conservative (utils.cpp:71-83)."""
    p = _a(prim, 5); c = np.empty_like(p)
    capi.check(capi.load().mmf_prim2cons(p.shape[0], capi.ptr(p), capi.ptr(c)))
    return c


def evalFluxes(cons, prim, normal):
    """euler::evalFluxes (euler.cpp:83-113)."""
    c, p, n = _a(cons, 5), _a(prim, 5), _a(normal, 3)
    f = np.empty_like(c)
    capi.check(capi.load().mmf_eval_fluxes(c.shape[0], capi.ptr(c), capi.ptr(p), capi.ptr(n), capi.ptr(f)))
    return f


def evalSplitting(cons_l, cons_r, normal):
    """euler::evalSplitting (euler.cpp:42-73): returns (fluxes, lambda)."""
    cl, cr, n = _a(cons_l, 5), _a(cons_r, 5), _a(normal, 3)
    f = np.empty_like(cl); lam = np.empty(cl.shape[0])
    capi.check(capi.load().mmf_eval_splitting(cl.shape[0], capi.ptr(cl), capi.ptr(cr), capi.ptr(n),
                                              capi.ptr(f), capi.ptr(lam)))
    return f, lam


def evalInterfaceBCValues(bc_type, normal, cons, dirichlet_prim=None):
    """euler::evalInterfaceBCValues (euler.cpp:261-288)."""
    c, n = _a(cons, 5), _a(normal, 3)
    out = np.empty_like(c)
    dp = None if dirichlet_prim is None else np.ascontiguousarray(dirichlet_prim, dtype=np.float64)
    capi.check(capi.load().mmf_eval_bc_values(c.shape[0], int(bc_type), capi.ptr(n), capi.ptr(c),
                                              capi.ptr(dp), capi.ptr(out)))
    return out


def computeRHS(solver, cons):
    """euler::computeRHS (euler.cpp:127-249) on a solver context: (rhs, maxEig)."""
    return solver.compute_rhs(cons)

"""Host side of the GB300 Euler step: one CUDA context per Cartesian mesh.

`CartesianEuler` owns a device context created through the C ABI
(include/mmf_gb300.h).  State crosses the boundary in the reference's
PiercedStorage raw layout, AoS float64 [n_raw][5] with fields
(rho, rho u, rho v, rho w, rho E) (constants.hpp:43-47).
"""
import ctypes as C
import math

import numpy as np

from . import capi

_BC_NAMES = {"free_flow": capi.BC_FREE_FLOW, "reflecting": capi.BC_REFLECTING, "wall": capi.BC_WALL,
             "dirichlet": capi.BC_DIRICHLET, "periodic": capi.BC_PERIODIC}


def _bc(v):
    return _BC_NAMES[v] if isinstance(v, str) else int(v)


def problem_struct(case):
    p = case.prm
    s = capi.Problem()
    s.problem = case.problem
    s.vortex_beta, s.sod_radius = p.vortex_beta, p.sod_radius
    s.sod_rho_in, s.sod_p_in, s.sod_rho_out, s.sod_p_out = p.sod_rho_in, p.sod_p_in, p.sod_rho_out, p.sod_p_out
    s.periodic_exact = int(p.periodic)
    return s


class CartesianEuler:
    """Uniform Cartesian FV Euler solver context on one GPU.

    Parameters mirror the reference setup: ``dim`` and cells per direction
    ``n`` (main.cpp:98-107, 146-150), ``origin`` and cell edge ``h`` (the
    VolOctree constructor), border conditions per side (problem.cpp:404-438,
    plus periodic), reconstruction ``order`` (reconstruction.cpp:67-79) and
    the arithmetic: "reference" (bit-identical to the reference) or "fast".
    """

    def __init__(self, dim, n, origin, h, bc_lo, bc_hi, order=1, arith="fast", device=0,
                 dirichlet_prim=(0.0,) * 5, chunk=0):
        self._lib = capi.load()
        g = capi.Grid()
        g.dim = dim
        n = list(n) + [1] * (3 - len(n))
        for d in range(3):
            g.n[d] = int(n[d])
            g.origin[d] = float(origin[d])
            g.bc_lo[d] = _bc(bc_lo[d]) if d < dim else capi.BC_FREE_FLOW
            g.bc_hi[d] = _bc(bc_hi[d]) if d < dim else capi.BC_FREE_FLOW
        g.h = float(h)
        for k in range(5):
            g.dirichlet_prim[k] = float(dirichlet_prim[k])
        g.order = order
        g.arith = {"reference": capi.ARITH_REFERENCE, "fast": capi.ARITH_FAST}[arith] if isinstance(arith, str) else arith
        g.chunk = chunk
        self.grid = g
        self.dim = dim
        self.n = tuple(n[:3])
        self.ncells = n[0] * n[1] * (n[2] if dim == 3 else 1)
        self._ctx = C.c_void_p()
        capi.check(self._lib.mmf_create(C.byref(g), device, C.byref(self._ctx)))

    # -- lifetime ----------------------------------------------------------------------
    def close(self):
        if getattr(self, "_ctx", None) is not None and self._ctx.value:
            self._lib.mmf_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- layout ------------------------------------------------------------------------
    def set_cell_map(self, raw_to_cell):
        """Raw id -> grid index (i + n0 (j + n1 k)) for a non-row-major raw order."""
        if raw_to_cell is None:
            capi.check(self._lib.mmf_set_cell_map(self._ctx, self.ncells, None))
            return
        m = np.ascontiguousarray(raw_to_cell, dtype=np.int64)
        capi.check(self._lib.mmf_set_cell_map(self._ctx, m.size, m.ctypes.data_as(C.POINTER(C.c_int64))))

    def upload(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        capi.check(self._lib.mmf_upload_state(self._ctx, capi.ptr(U), self.ncells))

    def download(self, out=None):
        out = np.empty((self.ncells, 5)) if out is None else out
        capi.check(self._lib.mmf_download_state(self._ctx, capi.ptr(out), self.ncells))
        return out

    def upload_device(self, t):
        """Upload from a device tensor/pointer holding AoS [n_raw][5] float64."""
        capi.check(self._lib.mmf_upload_state_device(self._ctx, capi.ptr(t), self.ncells))

    def download_device(self, t):
        capi.check(self._lib.mmf_download_state_device(self._ctx, capi.ptr(t), self.ncells))

    # -- reference entry points --------------------------------------------------------
    def compute_rhs(self, U):
        """euler::computeRHS (euler.cpp:127-249): residual (not divided by V) and maxEig."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        R = np.empty((self.ncells, 5))
        me = C.c_double()
        capi.check(self._lib.mmf_compute_rhs(self._ctx, capi.ptr(U), capi.ptr(R), C.byref(me), self.ncells))
        return R, me.value

    def compute_polynomials(self, U=None, want_slopes=True, want_active=True):
        """reconstruction::computePolynomials (reconstruction.cpp:47-55) of state U.

        Order 1: nothing to compute (returns None).  Order 2: returns
        (slopes [n_raw, 3, 5], limiter_active [n_raw] uint8)."""
        if self.grid.order == 1:
            capi.check(self._lib.mmf_compute_polynomials(self._ctx, None, None, None, self.ncells))
            return None
        U = np.ascontiguousarray(U, dtype=np.float64)
        S = np.empty((self.ncells, 3, 5)) if want_slopes else None
        A = np.empty(self.ncells, dtype=np.uint8) if want_active else None
        capi.check(self._lib.mmf_compute_polynomials(self._ctx, capi.ptr(U), capi.ptr(S), capi.ptr(A), self.ncells))
        return S, A

    def set_limiter(self, mode, flags=None):
        """Order-2 limiter: 'all', 'none' or 'flagged' (flags: one byte per raw id)."""
        m = {"all": capi.LIMIT_ALL, "none": capi.LIMIT_NONE, "flagged": capi.LIMIT_FLAGGED}.get(mode, mode)
        f = None if flags is None else np.ascontiguousarray(flags, dtype=np.uint8)
        capi.check(self._lib.mmf_set_limiter(self._ctx, m, capi.ptr(f), self.ncells))

    def set_limiter_flags_device(self, d_flags_grid):
        capi.check(self._lib.mmf_set_limiter_flags_device(self._ctx, capi.ptr(d_flags_grid)))

    def limiter_activity(self):
        a = np.empty(self.ncells, dtype=np.uint8)
        capi.check(self._lib.mmf_get_limiter_activity(self._ctx, capi.ptr(a), self.ncells))
        return a

    def time_setup(self, cfl, t=0.0, t_end=math.inf, max_steps=-1):
        capi.check(self._lib.mmf_time_setup(self._ctx, cfl, t, t_end, max_steps))

    def advance(self, n_steps):
        """Up to n_steps SSP-RK3 steps (main.cpp:377-506); returns (t, steps_done)."""
        t = C.c_double()
        done = C.c_int64()
        capi.check(self._lib.mmf_advance(self._ctx, n_steps, C.byref(t), C.byref(done)))
        return t.value, done.value

    def advance_async(self, n_steps):
        """Enqueue n_steps steps on the context stream without waiting."""
        capi.check(self._lib.mmf_advance_async(self._ctx, n_steps))

    def time_info(self):
        t, st = C.c_double(), C.c_int64()
        capi.check(self._lib.mmf_time_info(self._ctx, C.byref(t), C.byref(st)))
        return t.value, st.value

    @property
    def stream_handle(self):
        """cudaStream_t of the context (for events recorded on its stream)."""
        return self._lib.mmf_get_stream(self._ctx)

    def advance_host(self, U, n_steps):
        """Upload U (host AoS), advance, download into U; returns t."""
        t = C.c_double()
        capi.check(self._lib.mmf_advance_host(self._ctx, capi.ptr(U), self.ncells, n_steps, C.byref(t)))
        return t.value

    def rk_stage(self, stage):
        capi.check(self._lib.mmf_rk_stage(self._ctx, stage))

    def last_step_info(self):
        dt, me = C.c_double(), C.c_double()
        capi.check(self._lib.mmf_last_step_info(self._ctx, C.byref(dt), C.byref(me)))
        return dt.value, me.value

    def status(self):
        s = C.c_uint()
        capi.check(self._lib.mmf_get_status(self._ctx, C.byref(s)))
        return s.value

    def synchronize(self):
        capi.check(self._lib.mmf_synchronize(self._ctx))

    @property
    def launch_count(self):
        return self._lib.mmf_launch_count(self._ctx)

    def set_shape(self, chunk, variant):
        """Pin the decomposition: rows / planes per chunk, and warps per block
        (2D) or the 3D kernel (0 = row blocks, 1 = tiles with one block per
        tile and chunk, 2 = tiles with one block per resident slot)."""
        capi.check(self._lib.mmf_set_shape(self._ctx, chunk, variant))

    def autotune(self, trial_steps=4):
        """Pick the stage kernels' decomposition by timing (state restored);
        returns (chunk, warps_per_block)."""
        ch, w = C.c_int(), C.c_int()
        capi.check(self._lib.mmf_autotune(self._ctx, trial_steps, C.byref(ch), C.byref(w)))
        return ch.value, w.value

    def set_step_log(self, capacity):
        """Keep (maxEig, dt, t) of the last 'capacity' steps on the device."""
        capi.check(self._lib.mmf_set_step_log(self._ctx, capacity))

    def step_log(self, max_entries=1 << 20):
        """(first step index, array [n, 3] of maxEig, dt, t after the step)."""
        out = np.empty((max_entries, 3))
        first, n = C.c_int64(), C.c_int64()
        capi.check(self._lib.mmf_get_step_log(self._ctx, capi.ptr(out), max_entries, C.byref(first), C.byref(n)))
        return first.value, out[:n.value].copy()

    def init_state(self, case):
        """Initial state of a problem case computed on the device (problem.cpp:247-392)."""
        capi.check(self._lib.mmf_init_state(self._ctx, C.byref(problem_struct(case))))

    def l1_density_error(self, case, t):
        """sum |rho - rho_exact(t)| V on the device (main.cpp:550-567)."""
        e = C.c_double()
        capi.check(self._lib.mmf_l1_density_error(self._ctx, C.byref(problem_struct(case)), t, C.byref(e)))
        return e.value

    def write_vtk(self, path):
        capi.check(self._lib.mmf_write_vtk(self._ctx, str(path).encode()))

    def save_checkpoint(self, path):
        capi.check(self._lib.mmf_save_checkpoint(self._ctx, str(path).encode()))

    def load_checkpoint(self, path):
        capi.check(self._lib.mmf_load_checkpoint(self._ctx, str(path).encode()))

    def run(self, U0, cfl, t_end=math.inf, max_steps=-1, t_start=0.0, batch=1 << 30):
        """Reference loop (main.cpp:377-506) from U0 to t_end / max_steps; returns (U, t, steps)."""
        self.upload(U0)
        self.time_setup(cfl, t_start, t_end, max_steps)
        steps = 0
        t = t_start
        while True:
            want = max_steps - steps if max_steps >= 0 else 4096
            want = min(want, batch)
            if want <= 0:
                break
            t, done = self.advance(want)
            steps += done
            if done < want:
                break
        return self.download(), t, steps

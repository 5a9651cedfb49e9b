"""Batched solver: many independent 2D cases of uneven size in one persistent
launch per RK stage (C ABI mmf_batch_*), each case with its own CFL time step."""
import ctypes as C

import numpy as np

from . import capi
from .solver import _bc


class BatchEuler:
    """Context over a list of 2D problem cases (minimmerflow_gb300.problem.Case)."""

    def __init__(self, cases, arith="fast", device=0, order=1):
        self._lib = capi.load()
        self.cases = list(cases)
        grids = (capi.Grid * len(self.cases))()
        for g, case in zip(grids, self.cases):
            if case.dim != 2:
                raise ValueError("batched cases are 2D")
            lo, hi = case.bcs()
            g.dim = 2
            for d in range(3):
                g.n[d] = int(case.n[d]) if d < 2 else 1
                g.origin[d] = float(case.origin[d])
                g.bc_lo[d] = _bc(lo[d]) if d < 2 else 0
                g.bc_hi[d] = _bc(hi[d]) if d < 2 else 0
            g.h = case.h
            g.order = order
            g.arith = {"reference": capi.ARITH_REFERENCE, "fast": capi.ARITH_FAST}[arith]
        self._b = C.c_void_p()
        capi.check(self._lib.mmf_batch_create(len(self.cases), grids, device, C.byref(self._b)))
        self.sizes = np.array([c.ncells for c in self.cases], dtype=np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)[:-1]])
        self.total = int(self.sizes.sum())

    def close(self):
        if getattr(self, "_b", None) is not None and self._b.value:
            self._lib.mmf_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def pack(self, states):
        return np.ascontiguousarray(np.concatenate([np.asarray(s).reshape(-1, 5) for s in states]), dtype=np.float64)

    def unpack(self, U):
        return [U[o:o + n] for o, n in zip(self.offsets, self.sizes)]

    def upload(self, states):
        U = self.pack(states) if isinstance(states, (list, tuple)) else np.ascontiguousarray(states, dtype=np.float64)
        capi.check(self._lib.mmf_batch_upload(self._b, capi.ptr(U), self.total))

    def download(self):
        U = np.empty((self.total, 5))
        capi.check(self._lib.mmf_batch_download(self._b, capi.ptr(U), self.total))
        return U

    def time_setup(self, cfl=None, t_end=None, max_steps=-1):
        cf = np.array([c.cfl for c in self.cases] if cfl is None else cfl, dtype=np.float64)
        te = None if t_end is None else np.ascontiguousarray(t_end, dtype=np.float64)
        capi.check(self._lib.mmf_batch_time_setup(self._b, capi.ptr(cf), capi.ptr(te), max_steps))

    def advance_async(self, n_steps):
        capi.check(self._lib.mmf_batch_advance_async(self._b, n_steps))

    def synchronize(self):
        capi.check(self._lib.mmf_batch_synchronize(self._b))

    def case_info(self, c):
        t, s, st = C.c_double(), C.c_int64(), C.c_uint()
        capi.check(self._lib.mmf_batch_case_info(self._b, c, C.byref(t), C.byref(s), C.byref(st)))
        return t.value, s.value, st.value

    def set_shape(self, chunk, blocks_per_sm=0):
        capi.check(self._lib.mmf_batch_set_shape(self._b, chunk, blocks_per_sm))

    def shape(self):
        a, b = C.c_int(), C.c_int()
        capi.check(self._lib.mmf_batch_get_shape(self._b, C.byref(a), C.byref(b)))
        return a.value, b.value

    def autotune(self, trial_steps=4):
        a, b = C.c_int(), C.c_int()
        capi.check(self._lib.mmf_batch_autotune(self._b, trial_steps, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_limiter(self, mode):
        m = {"all": capi.LIMIT_ALL, "none": capi.LIMIT_NONE, "flagged": capi.LIMIT_FLAGGED}.get(mode, mode)
        capi.check(self._lib.mmf_batch_set_limiter(self._b, m))

    def set_indicator(self, mlp, threshold, period=1):
        """Order-2 batches: the learned indicator (2D) gates the limiter of every
        case, every step or every second step (period 2, flags dilated by one cell)."""
        capi.check(self._lib.mmf_batch_set_indicator(self._b, mlp.handle if mlp is not None else None, threshold))
        if mlp is not None:
            capi.check(self._lib.mmf_batch_set_indicator_period(self._b, period))

    @property
    def stream_handle(self):
        return self._lib.mmf_batch_get_stream(self._b)

    @property
    def launch_count(self):
        return self._lib.mmf_batch_launch_count(self._b)

    def run(self, states, steps):
        """Advance every case 'steps' steps (no end time); returns the per-case states."""
        self.upload(states)
        self.time_setup(max_steps=steps)
        self.advance_async(steps)
        self.synchronize()
        return self.unpack(self.download())

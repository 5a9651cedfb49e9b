"""Face-list solver context (C ABI mmf_umesh_*): the Euler step on any mesh given
as MeshGeometricalInfo-like arrays -- refined meshes, immersed bodies (unsolved
cells, BC_WALL faces), per-face border conditions (the forward-facing step)."""
import ctypes as C
import math

import numpy as np

from . import capi


class UnstructuredEuler:
    """Arrays: cell_volume, cell_size [n]; solved [n] (uint8, optional);
    owner, neigh [nf] (int64, neigh -1 on a border); area [nf]; normal [nf, 3];
    bc [nf] (int32, -1 inside)."""

    def __init__(self, dim, cell_volume, cell_size, owner, neigh, area, normal, bc, solved=None, arith="reference",
                 dirichlet_prim=(0.0,) * 5, device=0):
        self._lib = capi.load()
        self._keep = [np.ascontiguousarray(cell_volume, dtype=np.float64),
                      np.ascontiguousarray(cell_size, dtype=np.float64),
                      None if solved is None else np.ascontiguousarray(solved, dtype=np.uint8),
                      np.ascontiguousarray(owner, dtype=np.int64), np.ascontiguousarray(neigh, dtype=np.int64),
                      np.ascontiguousarray(area, dtype=np.float64),
                      np.ascontiguousarray(normal, dtype=np.float64).reshape(-1, 3),
                      np.ascontiguousarray(bc, dtype=np.int32)]
        vol, size, sol, own, nei, ar, nrm, b = self._keep
        d = capi.UMeshDesc()
        d.dim = dim
        d.n_cells = vol.size
        d.n_faces = own.size
        d.cell_volume, d.cell_size = vol.ctypes.data, size.ctypes.data
        d.solved = sol.ctypes.data if sol is not None else None
        d.owner, d.neigh, d.area, d.normal, d.bc = own.ctypes.data, nei.ctypes.data, ar.ctypes.data, nrm.ctypes.data, b.ctypes.data
        for k in range(5):
            d.dirichlet_prim[k] = float(dirichlet_prim[k])
        d.arith = {"reference": capi.ARITH_REFERENCE, "fast": capi.ARITH_FAST}[arith]
        self.ncells = int(vol.size)
        self._u = C.c_void_p()
        capi.check(self._lib.mmf_umesh_create(C.byref(d), device, C.byref(self._u)))

    @classmethod
    def from_oracle_mesh(cls, m, arith="reference", dirichlet_prim=(0.0,) * 5):
        """From the oracle's face-list mesh (test infrastructure)."""
        f = m.faces()
        n = m.ncells
        vol = np.ctypeslib.as_array(m.m.cell_volume, shape=(n,)).copy()
        size = np.ctypeslib.as_array(m.m.cell_size, shape=(n,)).copy()
        solved = np.ctypeslib.as_array(m.m.solved, shape=(n,)).copy()
        return cls(m.dim, vol, size, f["owner"], f["neigh"], f["area"], f["normal"], f["bc"], solved=solved,
                   arith=arith, dirichlet_prim=dirichlet_prim)

    def close(self):
        if getattr(self, "_u", None) is not None and self._u.value:
            self._lib.mmf_umesh_destroy(self._u)
            self._u = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def compute_rhs(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        R = np.empty((self.ncells, 5))
        me = C.c_double()
        capi.check(self._lib.mmf_umesh_compute_rhs(self._u, capi.ptr(U), capi.ptr(R), C.byref(me), self.ncells))
        return R, me.value

    def run(self, U0, cfl, t_end=math.inf, max_steps=-1):
        U = np.ascontiguousarray(U0, dtype=np.float64)
        capi.check(self._lib.mmf_umesh_upload(self._u, capi.ptr(U), self.ncells))
        capi.check(self._lib.mmf_umesh_time_setup(self._u, cfl, 0.0, t_end, max_steps))
        steps, t = 0, 0.0
        while True:
            want = max_steps - steps if max_steps >= 0 else 4096
            if want <= 0:
                break
            tt, done = C.c_double(), C.c_int64()
            capi.check(self._lib.mmf_umesh_advance(self._u, want, C.byref(tt), C.byref(done)))
            steps += done.value
            t = tt.value
            if done.value < want:
                break
        out = np.empty((self.ncells, 5))
        capi.check(self._lib.mmf_umesh_download(self._u, capi.ptr(out), self.ncells))
        return out, t, steps

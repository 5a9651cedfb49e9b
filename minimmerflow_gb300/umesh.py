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

    @classmethod
    def cartesian(cls, case, arith="fast", device=0):
        """The face list of a uniform grid (grid order, x faces then y then z,
        the border and periodic faces included), as MeshGeometricalInfo would
        describe it: the normal points from owner to neighbour, a border face
        has its owner inside (euler.cpp:166-178)."""
        f = cartesian_faces(case)
        return cls(case.dim, f["volume"], f["size"], f["owner"], f["neigh"], f["area"], f["normal"], f["bc"],
                   arith=arith, device=device)

    def upload(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        capi.check(self._lib.mmf_umesh_upload(self._u, capi.ptr(U), self.ncells))

    def download(self):
        out = np.empty((self.ncells, 5))
        capi.check(self._lib.mmf_umesh_download(self._u, capi.ptr(out), self.ncells))
        return out

    def time_setup(self, cfl, t=0.0, t_end=math.inf, max_steps=-1):
        capi.check(self._lib.mmf_umesh_time_setup(self._u, cfl, t, t_end, max_steps))

    def advance(self, n_steps):
        tt, done = C.c_double(), C.c_int64()
        capi.check(self._lib.mmf_umesh_advance(self._u, n_steps, C.byref(tt), C.byref(done)))
        return tt.value, done.value

    @property
    def launch_count(self):
        return int(self._lib.mmf_umesh_launch_count(self._u))

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


def cartesian_faces(case):
    """Face arrays of the uniform grid of a problem case (see UnstructuredEuler.cartesian)."""
    dim = case.dim
    nx, ny, nz = case.n[0], case.n[1], case.n[2] if dim == 3 else 1
    h = case.h
    lo, hi = case.bcs()
    periodic = lo[0] == 16
    owners, neighs, normals, bcs = [], [], [], []
    cell = np.arange(nx * ny * nz, dtype=np.int64).reshape(nz, ny, nx)
    for d in range(dim):
        c = np.moveaxis(cell, 2 - d, 2)            # direction d last
        m = c.shape[2]
        e = np.zeros(3)
        e[d] = 1.0
        if periodic:
            own = np.concatenate([c[:, :, -1:], c[:, :, :-1]], axis=2)
            nei = c
            owners.append(own.reshape(-1))
            neighs.append(nei.reshape(-1))
            normals.append(np.tile(e, (own.size, 1)))
            bcs.append(np.full(own.size, -1, dtype=np.int32))
            continue
        # faces 0..m along d: 0 and m are borders
        own = np.concatenate([c[:, :, :1], c[:, :, :-1], c[:, :, -1:]], axis=2)
        nei = np.concatenate([np.full(c[:, :, :1].shape, -1), c[:, :, 1:], np.full(c[:, :, :1].shape, -1)], axis=2)
        nrm = np.tile(e, own.shape + (1,))
        nrm[:, :, 0] = -e
        b = np.full(own.shape, -1, dtype=np.int32)
        b[:, :, 0] = lo[d]
        b[:, :, m] = hi[d]
        owners.append(own.reshape(-1))
        neighs.append(nei.reshape(-1))
        normals.append(nrm.reshape(-1, 3))
        bcs.append(b.reshape(-1))
    n = nx * ny * nz
    return dict(volume=np.full(n, h ** dim), size=np.full(n, h), owner=np.concatenate(owners),
                neigh=np.concatenate(neighs), area=np.full(sum(o.size for o in owners), h ** (dim - 1)),
                normal=np.concatenate(normals), bc=np.concatenate(bcs))

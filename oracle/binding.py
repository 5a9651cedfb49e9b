"""ctypes binding of the C oracle (test infrastructure only; see mmf_oracle.h).

The shared library is built by :func:`build` (gcc -O2 -ffp-contract=off) into
``oracle/_build``.  Arrays cross the boundary as contiguous numpy buffers.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libmmf_oracle.so")

N_FIELDS = 5
BC_NONE, BC_FREE_FLOW, BC_REFLECTING, BC_WALL, BC_DIRICHLET = -1, 0, 1, 2, 3
BC_PERIODIC = 16
(VORTEX_XY, VORTEX_ZX, VORTEX_YZ, RADSOD, SOD_X, SOD_Y, SOD_Z, FFSTEP) = range(8)
PROBLEMS = {"vortex_xy": VORTEX_XY, "vortex_zx": VORTEX_ZX, "vortex_yz": VORTEX_YZ,
            "radsod": RADSOD, "sod3d_x": SOD_X, "sod3d_y": SOD_Y, "sod3d_z": SOD_Z,
            "ffstep": FFSTEP}


def build(force=False):
    """Compile the oracle restatement (plain C) into oracle/_build."""
    src = os.path.join(HERE, "mmf_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "mmf_oracle.h"))):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                           "-o", tmp, src, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Params(C.Structure):
    _fields_ = [("vortex_beta", C.c_double), ("sod_radius", C.c_double),
                ("sod_rho_in", C.c_double), ("sod_p_in", C.c_double),
                ("sod_rho_out", C.c_double), ("sod_p_out", C.c_double),
                ("periodic_exact", C.c_int), ("domain_origin", C.c_double * 3),
                ("domain_length", C.c_double)]


class Mesh(C.Structure):
    _fields_ = [("dim", C.c_int), ("n", C.c_int64 * 3), ("origin", C.c_double * 3), ("h", C.c_double),
                ("bc_lo", C.c_int * 3), ("bc_hi", C.c_int * 3), ("cell_order", C.c_int),
                ("ncells", C.c_int64), ("raw_of_grid", C.POINTER(C.c_int64)),
                ("grid_of_raw", C.POINTER(C.c_int64)), ("cell_volume", C.POINTER(C.c_double)),
                ("cell_size", C.POINTER(C.c_double)), ("cell_centroid", C.POINTER(C.c_double)),
                ("solved", C.POINTER(C.c_ubyte)), ("nfaces", C.c_int64),
                ("owner", C.POINTER(C.c_int64)), ("neigh", C.POINTER(C.c_int64)),
                ("area", C.POINTER(C.c_double)), ("normal", C.POINTER(C.c_double)),
                ("fcentroid", C.POINTER(C.c_double)), ("bc", C.POINTER(C.c_int)),
                ("fdir", C.POINTER(C.c_int))]


class RunCfg(C.Structure):
    _fields_ = [("problem", C.c_int), ("order", C.c_int), ("cfl", C.c_double),
                ("t_start", C.c_double), ("t_end", C.c_double), ("max_steps", C.c_int64),
                ("limiter_mode", C.c_int), ("limiter_flag", C.POINTER(C.c_ubyte)),
                ("dt_log", C.POINTER(C.c_double)), ("maxeig_log", C.POINTER(C.c_double))]


_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_params_default.argtypes = [C.POINTER(Params)]
        L.orc_cons2prim.argtypes = [_dp, _dp]
        L.orc_prim2cons.argtypes = [_dp, _dp]
        L.orc_normal_velocity.argtypes = [_dp, _dp]
        L.orc_normal_velocity.restype = C.c_double
        L.orc_eval_fluxes.argtypes = [_dp, _dp, _dp, _dp]
        L.orc_eval_splitting.argtypes = [_dp, _dp, _dp, _dp, C.POINTER(C.c_double)]
        L.orc_eval_bc.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_exact_conservatives.argtypes = [C.c_int, C.c_int, C.POINTER(Params), _dp, C.c_double, _dp]
        L.orc_border_bc_type.argtypes = [C.c_int, _dp]
        L.orc_border_bc_type.restype = C.c_int
        L.orc_mesh_build.argtypes = [C.POINTER(Mesh), C.c_int, C.c_int, C.POINTER(C.c_int64),
                                     C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_int),
                                     C.POINTER(C.c_int), C.c_int]
        L.orc_mesh_free.argtypes = [C.POINTER(Mesh)]
        L.orc_compute_polynomials.argtypes = [C.POINTER(Mesh), C.c_int, C.c_int, _dp, C.c_void_p,
                                              C.c_int, C.c_void_p, C.c_void_p]
        L.orc_compute_rhs.argtypes = [C.POINTER(Mesh), C.c_int, C.c_int, _dp, C.c_void_p, _dp,
                                      C.POINTER(C.c_double)]
        L.orc_run.argtypes = [C.POINTER(Mesh), C.POINTER(RunCfg), _dp, C.POINTER(C.c_double)]
        L.orc_run.restype = C.c_int64
        L.orc_initial_state.argtypes = [C.POINTER(Mesh), C.c_int, C.POINTER(Params), _dp]
        L.orc_l1_density_error.argtypes = [C.POINTER(Mesh), C.c_int, C.POINTER(Params), _dp, C.c_double]
        L.orc_l1_density_error.restype = C.c_double
        L.orc_now.restype = C.c_double
        _lib = L
    return _lib


def params(**kw):
    p = Params()
    lib().orc_params_default(C.byref(p))
    for k, v in kw.items():
        if k == "domain_origin":
            for i in range(3):
                p.domain_origin[i] = v[i]
        else:
            setattr(p, k, v)
    return p


# ---- pointwise physics (utils.cpp / euler.cpp) -------------------------------------------

def cons2prim(c):
    c = np.ascontiguousarray(c, dtype=np.float64); p = np.empty(5)
    lib().orc_cons2prim(c, p); return p


def prim2cons(p):
    p = np.ascontiguousarray(p, dtype=np.float64); c = np.empty(5)
    lib().orc_prim2cons(p, c); return c


def eval_fluxes(c, p, n):
    f = np.empty(5)
    lib().orc_eval_fluxes(np.ascontiguousarray(c, dtype=np.float64), np.ascontiguousarray(p, dtype=np.float64),
                          np.ascontiguousarray(n, dtype=np.float64), f)
    return f


def eval_splitting(cl, cr, n):
    f = np.empty(5); lam = C.c_double()
    lib().orc_eval_splitting(np.ascontiguousarray(cl, dtype=np.float64), np.ascontiguousarray(cr, dtype=np.float64),
                             np.ascontiguousarray(n, dtype=np.float64), f, C.byref(lam))
    return f, lam.value


def eval_bc(problem, bc, point, n, c):
    out = np.empty(5)
    lib().orc_eval_bc(problem, bc, np.ascontiguousarray(point, dtype=np.float64),
                      np.ascontiguousarray(n, dtype=np.float64), np.ascontiguousarray(c, dtype=np.float64), out)
    return out


def exact_conservatives(problem, dim, point, t, prm=None):
    prm = prm or params(); out = np.empty(5)
    lib().orc_exact_conservatives(problem, dim, C.byref(prm), np.ascontiguousarray(point, dtype=np.float64), t, out)
    return out


# ---- mesh + solver ------------------------------------------------------------------------

class OracleMesh:
    """Uniform Cartesian mesh with the MeshGeometricalInfo arrays the path reads."""

    def __init__(self, problem, dim, n, origin, length, bc_lo=None, bc_hi=None, cell_order=0):
        self.m = Mesh()
        nn = (C.c_int64 * 3)(*(list(n) + [1] * (3 - len(n))))
        oo = (C.c_double * 3)(*origin)
        lo = (C.c_int * 3)(*bc_lo) if bc_lo is not None else None
        hi = (C.c_int * 3)(*bc_hi) if bc_hi is not None else None
        lib().orc_mesh_build(C.byref(self.m), problem, dim, nn, oo, float(length), lo, hi, cell_order)
        self.problem = problem
        self.dim = dim

    def __del__(self):
        if getattr(self, "m", None) is not None and _lib is not None:
            _lib.orc_mesh_free(C.byref(self.m))
            self.m = None

    @property
    def ncells(self):
        return self.m.ncells

    @property
    def nfaces(self):
        return self.m.nfaces

    def _arr(self, ptr, n, dtype):
        return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)

    def grid_of_raw(self):
        return self._arr(self.m.grid_of_raw, self.ncells, np.int64)

    def raw_of_grid(self):
        return self._arr(self.m.raw_of_grid, self.ncells, np.int64)

    def centroids(self):
        return self._arr(self.m.cell_centroid, 3 * self.ncells, np.float64).reshape(-1, 3)

    def faces(self):
        nf = self.nfaces
        return dict(owner=self._arr(self.m.owner, nf, np.int64), neigh=self._arr(self.m.neigh, nf, np.int64),
                    area=self._arr(self.m.area, nf, np.float64),
                    normal=self._arr(self.m.normal, 3 * nf, np.float64).reshape(-1, 3),
                    centroid=self._arr(self.m.fcentroid, 3 * nf, np.float64).reshape(-1, 3),
                    bc=self._arr(self.m.bc, nf, np.int32), fdir=self._arr(self.m.fdir, nf, np.int32))

    def set_bodies(self, boxes):
        """Box bodies: a cell is solid when its centroid lies in a box, bounds
        included (body.cpp:80-95); solid cells are not solved and interior
        faces between a fluid and a solid cell become BC_WALL
        (main.cpp:222-277).  boxes = [((xmin, ymin, zmin), (xmax, ymax, zmax)), ...].
        Returns the solid-cell mask (raw order)."""
        n, nf = self.ncells, self.nfaces
        c = self.centroids()
        solid = np.zeros(n, dtype=bool)
        for lo, hi in boxes:
            solid |= np.all((c >= np.asarray(lo, dtype=np.float64)) & (c <= np.asarray(hi, dtype=np.float64)), axis=1)
        solved = np.ctypeslib.as_array(self.m.solved, shape=(n,))
        solved[:] = ~solid
        bc = np.ctypeslib.as_array(self.m.bc, shape=(nf,))
        owner = np.ctypeslib.as_array(self.m.owner, shape=(nf,))
        neigh = np.ctypeslib.as_array(self.m.neigh, shape=(nf,))
        interior = neigh >= 0
        wall = interior & (solid[owner] != solid[np.where(interior, neigh, 0)])
        bc[wall] = BC_WALL
        return solid

    def initial_state(self, prm=None):
        prm = prm or params()
        U = np.empty(self.ncells * 5)
        lib().orc_initial_state(C.byref(self.m), self.problem, C.byref(prm), U)
        return U.reshape(-1, 5)

    def compute_polynomials(self, U, order=2, limiter_mode=0, flag=None, want_active=False):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        S = np.zeros(self.ncells * 15)
        act = np.zeros(self.ncells, dtype=np.uint8) if want_active else None
        fl = np.ascontiguousarray(flag, dtype=np.uint8) if flag is not None else None
        lib().orc_compute_polynomials(C.byref(self.m), self.problem, order, U, S.ctypes.data, limiter_mode,
                                      fl.ctypes.data if fl is not None else None,
                                      act.ctypes.data if act is not None else None)
        return (S.reshape(-1, 3, 5), act) if want_active else S.reshape(-1, 3, 5)

    def compute_rhs(self, U, order=1, slopes=None):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        R = np.empty_like(U); me = C.c_double()
        S = np.ascontiguousarray(slopes, dtype=np.float64).reshape(-1) if slopes is not None else None
        lib().orc_compute_rhs(C.byref(self.m), self.problem, order, U, S.ctypes.data if S is not None else None,
                              R, C.byref(me))
        return R.reshape(-1, 5), me.value

    def run(self, U, cfl, t_end=float("inf"), max_steps=-1, order=1, t_start=0.0, limiter_mode=0,
            limiter_flag=None, log=False):
        """SSP-RK3 loop (main.cpp:377-506). Returns (U_final, t, steps[, dt_log, maxeig_log])."""
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1).copy()
        cfg = RunCfg()
        cfg.problem, cfg.order, cfg.cfl = self.problem, order, cfl
        cfg.t_start, cfg.t_end, cfg.max_steps, cfg.limiter_mode = t_start, t_end, max_steps, limiter_mode
        fl = None
        if limiter_flag is not None:
            fl = np.ascontiguousarray(limiter_flag, dtype=np.uint8)
            cfg.limiter_flag = fl.ctypes.data_as(C.POINTER(C.c_ubyte))
        cap = max_steps if max_steps >= 0 else 1 << 16
        dtl = np.zeros(cap) if log else None
        mel = np.zeros(cap) if log else None
        if log:
            cfg.dt_log = dtl.ctypes.data_as(C.POINTER(C.c_double))
            cfg.maxeig_log = mel.ctypes.data_as(C.POINTER(C.c_double))
        t = C.c_double()
        steps = lib().orc_run(C.byref(self.m), C.byref(cfg), U, C.byref(t))
        if log:
            return U.reshape(-1, 5), t.value, steps, dtl[:steps], mel[:steps]
        return U.reshape(-1, 5), t.value, steps

    def l1_density_error(self, U, t, prm=None):
        prm = prm or params()
        return lib().orc_l1_density_error(C.byref(self.m), self.problem, C.byref(prm),
                                          np.ascontiguousarray(U, dtype=np.float64).reshape(-1), t)


# ---- the reference regression cases (test/<case>/settings.xml + CMakeLists.txt:33) --------

GOLDEN_CASES = {
    # name: (problem, dim, nCells, CFL, t_end, golden "Final error")
    "2dIsentropicVortex": ("vortex_xy", 2, 64, 0.45, 2.0, "1.388164788184e+00"),
    "2dRadSod": ("radsod", 2, 64, 0.45, 1.0, "1.091296206337e+00"),
    "3dIsentropicVortexXY": ("vortex_xy", 3, 32, 0.45, 2.0, "1.843404549197e+01"),
    "3dIsentropicVortexYZ": ("vortex_yz", 3, 32, 0.45, 1.0, "1.182056784168e+01"),
    "3dRadSod": ("radsod", 3, 32, 0.45, 4.0, "1.557229341641e+00"),
}


def reference_domain(problem):
    """problem.cpp:70-149 default origin and length."""
    if problem in (VORTEX_XY, VORTEX_ZX, VORTEX_YZ):
        return (-5.0, -5.0, -5.0), 10.0
    if problem in (SOD_X, SOD_Y, SOD_Z):
        return (-1.0, -1.0, -1.0), 2.0
    if problem == RADSOD:
        return (0.0, 0.0, 0.0), 8.0
    raise ValueError("domain length is mandatory for this problem")


def golden_mesh(name, cell_order=0):
    pname, dim, n, cfl, t_end, golden = GOLDEN_CASES[name]
    prob = PROBLEMS[pname]
    origin, length = reference_domain(prob)
    return OracleMesh(prob, dim, (n, n, n if dim == 3 else 1), origin, length, cell_order=cell_order)


def run_golden(name, cell_order=0):
    """Run one reference regression case; returns (error, formatted, golden, steps)."""
    pname, dim, n, cfl, t_end, golden = GOLDEN_CASES[name]
    m = golden_mesh(name, cell_order)
    U0 = m.initial_state()
    U, t, steps = m.run(U0, cfl, t_end=t_end)
    err = m.l1_density_error(U, t_end)
    return err, "%.12e" % err, golden, steps

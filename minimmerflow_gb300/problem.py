"""Problem library of the Euler step: initial/exact states, border conditions
and the standard workloads, vectorised on the host (numpy).

Restates src/problem.cpp: problem types (problem.hpp:33-42), default domains
(problem.cpp:70-149), end times (problem.cpp:175-211), the exact solutions
(problem.cpp:247-392) and border BC types (problem.cpp:404-438).  Parameters
that the reference hard-codes (vortex strength, Sod radius and states) are
arguments here so the benchmark workloads (a [-1,1]^2 radial Sod with r<0.5,
periodic vortices, uneven batched cases) can be expressed; their defaults
are the reference constants.
"""
import math
from dataclasses import dataclass, field

import numpy as np

GAMMA = 1.4
VORTEX_XY, VORTEX_ZX, VORTEX_YZ, RADSOD, SOD_X, SOD_Y, SOD_Z, FFSTEP = range(8)
PROBLEMS = {"vortex_xy": VORTEX_XY, "vortex_zx": VORTEX_ZX, "vortex_yz": VORTEX_YZ, "radsod": RADSOD,
            "sod3d_x": SOD_X, "sod3d_y": SOD_Y, "sod3d_z": SOD_Z, "ffstep": FFSTEP}
BC_FREE_FLOW, BC_REFLECTING, BC_WALL, BC_DIRICHLET, BC_PERIODIC = 0, 1, 2, 3, 16


@dataclass
class Params:
    vortex_beta: float = 5.0
    sod_radius: float = 1.0
    sod_rho_in: float = 1.0
    sod_p_in: float = 1.0
    sod_rho_out: float = 0.125
    sod_p_out: float = 0.1
    periodic: bool = False
    origin: tuple = (0.0, 0.0, 0.0)
    length: float = 0.0


def default_domain(problem):
    """problem.cpp:86-148."""
    if problem in (VORTEX_XY, VORTEX_ZX, VORTEX_YZ):
        return (-5.0, -5.0, -5.0), 10.0
    if problem in (SOD_X, SOD_Y, SOD_Z):
        return (-1.0, -1.0, -1.0), 2.0
    if problem == RADSOD:
        return (0.0, 0.0, 0.0), 8.0
    raise ValueError("the length of the domain is mandatory for this problem")


def default_end_time(problem, dim):
    """problem.cpp:185-207."""
    if problem in (VORTEX_XY, VORTEX_ZX, VORTEX_YZ):
        return 2.0 if dim == 2 else 1.0
    if problem in (SOD_X, SOD_Y, SOD_Z):
        return 0.3
    return 4.0


def prim2cons(p):
    """utils.cpp:71-83 over arrays [..., 5] (p, u, v, w, T)."""
    c = np.empty_like(p)
    rho = p[..., 0] / p[..., 4]
    c[..., 0] = rho
    c[..., 1] = rho * p[..., 1]
    c[..., 2] = rho * p[..., 2]
    c[..., 3] = rho * p[..., 3]
    c[..., 4] = rho * p[..., 4] / (GAMMA - 1.0) + 0.5 * rho * (p[..., 1] * p[..., 1] + p[..., 2] * p[..., 2]
                                                               + p[..., 3] * p[..., 3])
    return c


def exact_conservatives(problem, dim, points, t, prm=None):
    """problem.cpp:247-392 at points [N, 3]; returns conservatives [N, 5]."""
    prm = prm or Params()
    pts = np.array(points, dtype=np.float64, copy=True).reshape(-1, 3)
    prim = np.zeros((pts.shape[0], 5))
    if problem in (VORTEX_XY, VORTEX_ZX, VORTEX_YZ):
        uinf = [1.0, 1.0, 1.0]
        if problem == VORTEX_XY:
            uinf[2] = 0.0
        elif problem == VORTEX_ZX:
            uinf[1] = 0.0
        else:
            uinf[0] = 0.0
        for d in range(3):
            pts[:, d] -= t * uinf[d]
        if prm.periodic:
            for d in range(dim):
                o, L = prm.origin[d], prm.length
                x = pts[:, d]
                while np.any(x < o):
                    x[x < o] += L
                while np.any(x >= o + L):
                    x[x >= o + L] -= L
        if problem == VORTEX_XY:
            csi, eta = pts[:, 0], pts[:, 1]
        elif problem == VORTEX_ZX:
            csi, eta = pts[:, 2], pts[:, 0]
        else:
            csi, eta = pts[:, 1], pts[:, 2]
        r = np.sqrt(csi * csi + eta * eta)
        shape = prm.vortex_beta / (2 * math.pi) * np.exp(0.5 * (1 - r * r))
        zero = np.zeros_like(shape)
        if problem == VORTEX_XY:
            du, dv, dw = -eta * shape, csi * shape, zero
        elif problem == VORTEX_ZX:
            dw, du, dv = -eta * shape, csi * shape, zero
        else:
            dv, dw, du = -eta * shape, csi * shape, zero
        dT = -(GAMMA - 1.0) / (2 * GAMMA) * shape * shape
        dp = np.power(1.0 + dT, GAMMA / (GAMMA - 1.0)) - 1.0
        prim[:, 0] = 1.0 + dp
        prim[:, 1] = uinf[0] + du
        prim[:, 2] = uinf[1] + dv
        prim[:, 3] = (uinf[2] + dw) if dim == 3 else 0.0
        prim[:, 4] = 1.0 + dT
    elif problem == RADSOD:
        r = np.sqrt(pts[:, 0] * pts[:, 0] + pts[:, 1] * pts[:, 1] + pts[:, 2] * pts[:, 2])
        inside = r < prm.sod_radius
        prim[:, 0] = np.where(inside, prm.sod_p_in, prm.sod_p_out)
        prim[:, 4] = np.where(inside, prm.sod_p_in / prm.sod_rho_in, prm.sod_p_out / prm.sod_rho_out)
    elif problem in (SOD_X, SOD_Y, SOD_Z):
        r = pts[:, {SOD_X: 0, SOD_Y: 1, SOD_Z: 2}[problem]]
        prim[:, 0] = np.where(r < 0.0, 1.0, 0.1)
        prim[:, 4] = np.where(r < 0.0, 1.0 / 1.0, 0.1 / 0.125)
    elif problem == FFSTEP:
        prim[:, 0], prim[:, 1], prim[:, 4] = 1.0, 3.0, 1.0 / 1.4
    else:
        raise ValueError("unknown problem %r" % problem)
    return prim2cons(prim)


def border_bc_type(problem):
    """problem.cpp:404-420 (FFSTEP borders depend on the face, see dirichlet_prim)."""
    if problem == RADSOD:
        return BC_REFLECTING
    return BC_FREE_FLOW


def cell_centroids(dim, n, origin, h):
    """Centroids of a uniform grid in grid order (x fastest)."""
    nz = n[2] if dim == 3 else 1
    k, j, i = np.meshgrid(np.arange(nz), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    c = np.empty((i.size, 3))
    c[:, 0] = origin[0] + (i.reshape(-1) + 0.5) * h
    c[:, 1] = origin[1] + (j.reshape(-1) + 0.5) * h
    c[:, 2] = origin[2] + (k.reshape(-1) + 0.5) * h if dim == 3 else origin[2]
    return c


def morton_order(dim, n):
    """raw -> grid map of an octree (Z-order) cell numbering."""
    nz = n[2] if dim == 3 else 1
    k, j, i = np.meshgrid(np.arange(nz), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    i, j, k = i.reshape(-1).astype(np.uint64), j.reshape(-1).astype(np.uint64), k.reshape(-1).astype(np.uint64)

    def spread(x):
        r = np.zeros_like(x)
        for b in range(21):
            r |= ((x >> np.uint64(b)) & np.uint64(1)) << np.uint64(b * dim)
        return r
    key = spread(i) | (spread(j) << np.uint64(1))
    if dim == 3:
        key |= spread(k) << np.uint64(2)
    return np.argsort(key, kind="stable").astype(np.int64)


@dataclass
class Case:
    """A workload: mesh, borders, physics parameters and time control."""
    name: str
    problem: int
    dim: int
    n: tuple
    origin: tuple
    length: float
    cfl: float
    t_end: float = math.inf
    max_steps: int = -1
    periodic: bool = False
    prm: Params = field(default_factory=Params)
    border_bc: int = None     # overrides the problem's border condition (problem.cpp:404-420)

    @property
    def h(self):
        return self.length / self.n[0]

    @property
    def ncells(self):
        return int(np.prod(self.n[:self.dim]))

    def bcs(self):
        if self.periodic:
            return [BC_PERIODIC] * 3, [BC_PERIODIC] * 3
        b = border_bc_type(self.problem) if self.border_bc is None else self.border_bc
        return [b] * 3, [b] * 3

    def centroids(self):
        return cell_centroids(self.dim, self.n, self.origin, self.h)

    def initial_state(self):
        return exact_conservatives(self.problem, self.dim, self.centroids(), 0.0, self.prm)

    def solver(self, arith="fast", device=0, chunk=0, order=1):
        from .solver import CartesianEuler
        lo, hi = self.bcs()
        return CartesianEuler(self.dim, self.n, self.origin, self.h, lo, hi, order=order, arith=arith,
                              device=device, chunk=chunk)

    def l1_density_error(self, U, t):
        """main.cpp:550-561: sum |rho - rho_exact(t)| V over the cells."""
        ex = exact_conservatives(self.problem, self.dim, self.centroids(), t, self.prm)
        vol = self.h ** 2 if self.dim == 2 else self.h * self.h * self.h
        return float(np.sum(np.abs(U[:, 0] - ex[:, 0]) * vol))


def reference_case(problem, dim, ncells, cfl=0.45, t_end=None):
    """A reference regression setup (test/<case>/settings.xml)."""
    p = PROBLEMS[problem] if isinstance(problem, str) else problem
    if p in (VORTEX_ZX, VORTEX_YZ):
        dim = 3
    origin, length = default_domain(p)
    n = (ncells, ncells, ncells if dim == 3 else 1)
    te = default_end_time(p, dim) if t_end is None else t_end
    return Case("reference", p, dim, n, origin, length, cfl, t_end=te)


def radial_sod_2d(n=1024, t_end=0.25, cfl=0.5, max_steps=-1):
    """Radial Sod on [-1,1]^2: rho=p=1 for r<0.5, rho=0.125, p=0.1 outside, transmissive borders."""
    prm = Params(sod_radius=0.5)
    return Case("radial_sod_2d_%d" % n, RADSOD, 2, (n, n, 1), (-1.0, -1.0, 0.0), 2.0, cfl, t_end=t_end,
                max_steps=max_steps, prm=prm, border_bc=BC_FREE_FLOW)


def vortex(dim=2, n=64, axis="z", steps=100, cfl=0.5, beta=5.0, periodic=True):
    """Isentropic vortex on [-5,5]^dim, periodic borders, `steps` steps."""
    prob = VORTEX_XY if axis == "z" else VORTEX_YZ
    origin = (-5.0, -5.0, -5.0) if dim == 3 else (-5.0, -5.0, 0.0)
    prm = Params(vortex_beta=beta, periodic=periodic, origin=origin, length=10.0)
    return Case("vortex_%dd_%d_%s" % (dim, n, axis), prob, dim, (n, n, n if dim == 3 else 1), origin, 10.0,
                cfl, max_steps=steps, periodic=periodic, prm=prm)


def radial_sod_ratios(n, p_ratio, rho_ratio, cfl=0.5, max_steps=-1, dim=2):
    """[-1,1]^2 radial Sod, r < 0.5: rho = p = 1 inside, p = 1/p_ratio and
    rho = 1/rho_ratio outside, transmissive borders."""
    prm = Params(sod_radius=0.5, sod_rho_in=1.0, sod_p_in=1.0, sod_rho_out=1.0 / rho_ratio,
                 sod_p_out=1.0 / p_ratio)
    return Case("sod_p%.3g_r%.3g_%d" % (p_ratio, rho_ratio, n), RADSOD, dim, (n, n, n if dim == 3 else 1),
                (-1.0, -1.0, -1.0 if dim == 3 else 0.0), 2.0, cfl, max_steps=max_steps, prm=prm,
                border_bc=BC_FREE_FLOW)


def batched_sweep(ncases=512, seed=20261203, side_min=32, side_max=512, steps=-1):
    """Independent 2D cases of uneven size from a seed: mesh side uniform in
    [side_min, side_max]; even-indexed cases are isentropic vortices with beta
    ~ U[1, 8] ([-5,5]^2, periodic), odd-indexed ones radial Sods with pressure
    ratio ~ log-U[2, 100] and density ratio ~ U[2, 10]; CFL 0.5."""
    rng = np.random.default_rng(seed)
    cases = []
    for i in range(ncases):
        n = int(rng.integers(side_min, side_max + 1))
        if i % 2 == 0:
            beta = float(rng.uniform(1.0, 8.0))
            c = vortex(2, n, steps=steps, beta=beta)
            c.name = "vortex_b%.3g_%d" % (beta, n)
        else:
            pr = float(np.exp(rng.uniform(np.log(2.0), np.log(100.0))))
            rr = float(rng.uniform(2.0, 10.0))
            c = radial_sod_ratios(n, pr, rr, max_steps=steps)
        c.t_end = math.inf
        cases.append(c)
    return cases

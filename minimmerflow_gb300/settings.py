"""The reference's configuration file, settings.xml (root <minimmerflow
version="1">, main.cpp:73-74), read into a problem case.

Keys, with the reference's defaults:
  problem/type                       vortex_xy | vortex_zx | vortex_yz | radsod |
                                     sod3d_x | sod3d_y | sod3d_z | ffstep
                                     (problem.cpp:37-59; others are an error)
  problem/dimensions                 2; vortex_zx and vortex_yz are 3D (problem.cpp:70-83)
  problem/domain/origin/{x,y,z}      per problem: -5 (vortices), -1 (Sods), 0 (problem.cpp:86-115)
  problem/domain/length              10 (vortices), 2 (Sods), 8 (radsod); mandatory
                                     otherwise (problem.cpp:117-148)
  problem/start                      0, read as an integer as the reference does
                                     (problem.cpp:164)
  problem/time/end                   2 (2D vortices), 1 (3D vortices), 0.3 (Sods),
                                     4 (radsod, ffstep) (problem.cpp:175-211)
  discretization/space/order, nCells (main.cpp:98-111; nCells may be overridden
                                     like argv[1])
  discretization/time/CFL            (main.cpp:100)
  bodies/<any>/{type=box, xMin..zMax} (body.cpp:49-72)
"""
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

from . import problem as P


@dataclass
class Settings:
    case: P.Case
    order: int
    t_start: float
    bodies: list = field(default_factory=list)   # [((xmin, ymin, zmin), (xmax, ymax, zmax)), ...]

    @property
    def needs_face_list(self):
        """Immersed bodies and the forward-facing step's per-face borders need
        the face-list solver; the rest runs on the Cartesian kernels."""
        return bool(self.bodies) or self.case.problem == P.FFSTEP


def _node(root, path):
    n = root
    for part in path.split("/"):
        n = None if n is None else n.find(part)
    return n


def _text(root, path, default=None):
    n = _node(root, path)
    if n is None or n.text is None or not n.text.strip():
        if default is None:
            raise ValueError("settings.xml: missing %s" % path)
        return default
    return n.text.strip()


def _leading_int(s):
    """istream >> int of the reference's config reader: the leading integer."""
    s = s.strip()
    i = 1 if s[:1] in "+-" else 0
    while i < len(s) and s[i].isdigit():
        i += 1
    return int(s[:i]) if i > (1 if s[:1] in "+-" else 0) else 0


def load(source, n_cells=None):
    """Parse settings.xml (a path or the XML text); n_cells overrides
    discretization/space/nCells (the reference's argv[1])."""
    text = source
    if "<" not in source:
        with open(source) as f:
            text = f.read()
    root = ET.fromstring(text)
    if root.tag != "minimmerflow":
        raise ValueError("settings.xml: the root element is not <minimmerflow>")
    key = _text(root, "problem/type")
    if key not in P.PROBLEMS:
        raise ValueError("Problem %s is not supported." % key)
    prob = P.PROBLEMS[key]
    dim = 3 if prob in (P.VORTEX_ZX, P.VORTEX_YZ) else int(_text(root, "problem/dimensions", "2"))
    if _node(root, "problem/domain/origin") is not None:
        origin = tuple(float(_text(root, "problem/domain/origin/" + a, "0")) for a in "xyz")
    elif prob in (P.VORTEX_XY, P.VORTEX_ZX, P.VORTEX_YZ):
        origin = (-5.0, -5.0, -5.0)
    elif prob in (P.SOD_X, P.SOD_Y, P.SOD_Z):
        origin = (-1.0, -1.0, -1.0)
    else:
        origin = (0.0, 0.0, 0.0)
    if _node(root, "problem/domain/length") is not None:
        length = float(_text(root, "problem/domain/length"))
    else:
        length = P.default_domain(prob)[1]
    t_start = float(_leading_int(_text(root, "problem/start", "0")))
    t_end = float(_text(root, "problem/time/end")) if _node(root, "problem/time/end") is not None \
        else P.default_end_time(prob, dim)
    order = int(_text(root, "discretization/space/order"))
    cfl = float(_text(root, "discretization/time/CFL"))
    n = int(n_cells) if n_cells is not None else _leading_int(_text(root, "discretization/space/nCells"))
    bodies = []
    for b in (list(_node(root, "bodies")) if _node(root, "bodies") is not None else []):
        shape = (b.findtext("type") or "").strip()
        if shape != "box":
            raise ValueError('Body shape "%s" is not supported.' % shape)
        lo = tuple(float(b.findtext(k)) for k in ("xMin", "yMin", "zMin"))
        hi = tuple(float(b.findtext(k)) for k in ("xMax", "yMax", "zMax"))
        bodies.append((lo, hi))
    case = P.Case("settings_%s_%dd_%d" % (key, dim, n), prob, dim, (n, n, n if dim == 3 else 1), origin, length, cfl,
                  t_end=t_end)
    return Settings(case=case, order=order, t_start=t_start, bodies=bodies)

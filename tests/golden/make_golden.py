"""Golden fixtures from the reference itself (test infrastructure).

Builds oracle/_ref/mmf_ref -- the reference's own physics sources (euler.cpp,
utils.cpp, reconstruction.cpp, problem.cpp, mesh_info.cpp, body.cpp), compiled
unmodified from the reference tree against the bitpit stand-in in
oracle/ref_shim -- runs it on small cases and stores, per case, the initial
state the reference computed, its final state after a fixed number of steps,
the final time and the "Final error" line, as tests/golden/<case>.npz.  Raw
order is the stand-in's row-major cell order (x fastest), i.e. grid order.

  python tests/golden/make_golden.py [REF_SRC]

The reference tree is only needed here; the fixtures travel with the tests.
"""
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# name: (problem, dim, nCells, CFL, steps, extra options)
CASES = {
    "radsod2d_24": ("radsod", 2, 24, 0.45, 20, []),
    "vortex_xy2d_24": ("vortex_xy", 2, 24, 0.45, 20, []),
    "vortex_yz3d_8": ("vortex_yz", 3, 8, 0.45, 10, []),
    "radsod3d_10": ("radsod", 3, 10, 0.45, 10, []),
    "vortex_body2d_32": ("vortex_xy", 2, 32, 0.45, 20, ["body=1.0,-1.5,-10.0,2.5,1.5,10.0"]),
    "ffstep_body2d_32": ("ffstep", 2, 32, 0.45, 30, ["length=3.2", "body=0.6,-1.0,-10.0,4.0,0.2,10.0"]),
}


def main(ref_src):
    subprocess.check_call(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile.ref"), "REF_SRC=" + ref_src],
                          cwd=ROOT)
    exe = os.path.join(ROOT, "oracle", "_ref", "mmf_ref")
    with tempfile.TemporaryDirectory() as tmp:
        for name, (prob, dim, n, cfl, steps, extra) in CASES.items():
            fin, ini = os.path.join(tmp, "final.bin"), os.path.join(tmp, "init.bin")
            out = subprocess.check_output([exe, prob, str(dim), str(n), "1", str(cfl), "inf", str(steps), fin,
                                           "init=" + ini] + extra, timeout=600).decode()
            err = re.search(r"Final error:\s+(\S+)", out).group(1)
            t = float(re.search(r"Final time:\s+(\S+)", out).group(1))
            got = int(re.search(r"Steps:\s+(\d+)", out).group(1))
            assert got == steps
            body = [b.split("=", 1)[1] for b in extra if b.startswith("body=")]
            length = [float(b.split("=", 1)[1]) for b in extra if b.startswith("length=")]
            np.savez_compressed(os.path.join(HERE, name + ".npz"),
                                U0=np.fromfile(ini).reshape(-1, 5), U=np.fromfile(fin).reshape(-1, 5),
                                t=t, steps=steps, cfl=cfl, problem=prob, dim=dim, n=n,
                                body=np.array([float(v) for v in body[0].split(",")]) if body else np.zeros(0),
                                length=length[0] if length else 0.0, final_error=err)
            print(name, err, t)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1
         else os.path.join(os.environ.get("MMF_REFERENCE", "/root/reference"), "src"))

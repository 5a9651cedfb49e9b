"""In-tree build of the CUDA library (libmmf_gb300.so) for sm_103a.

The three translation units compile in parallel with nvcc; the reference-
arithmetic unit (mmf_exact.cu) is built with -fmad=false so that no
multiply-add is contracted (bit-identical to the reference's CPU results).
"""
import os
import shutil
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libmmf_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = [("mmf_exact.cu", ["-fmad=false"]), ("mmf_fast.cu", ["-fmad=false"]), ("mmf_capi.cu", []), ("mmf_noalloc.cu", []), ("mmf_batch.cu", []), ("mmf_mlp.cu", []), ("mmf_umesh.cu", ["-fmad=false"]), ("mmf_io.cu", ["-fmad=false"]), ("mmf_rate.cu", ["-fmad=false"])]


def nvcc():
    path = shutil.which("nvcc")
    if path is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        path = "/usr/local/cuda/bin/nvcc"
    if path is None:
        raise RuntimeError("nvcc not found: the CUDA library cannot be built")
    return path


def _sources():
    out = []
    for d in (CSRC, os.path.join(os.path.dirname(HERE), "include")):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h")):
                out.append(os.path.join(d, f))
    return out


def up_to_date():
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False):
    """Compile every CUDA translation unit and link libmmf_gb300.so (in-tree)."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(LIB_DIR, exist_ok=True)
    cc = nvcc()
    tmp = tempfile.mkdtemp(prefix="mmf_build_", dir=LIB_DIR)
    try:
        common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-O3"] + ARCH
        procs = []
        objs = []
        for src, extra in UNITS:
            obj = os.path.join(tmp, src.replace(".cu", ".o"))
            objs.append(obj)
            cmd = [cc] + common + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        for cmd, p in procs:
            out, _ = p.communicate()
            if p.returncode != 0:
                raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), out.decode(errors="replace")))
            if verbose and out:
                print(out.decode(errors="replace"))
        tmp_lib = os.path.join(tmp, "libmmf_gb300.so")
        subprocess.check_call([cc, "-shared"] + ARCH + objs + ["-o", tmp_lib, "-lcudart"])
        os.replace(tmp_lib, LIB_PATH)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return LIB_PATH

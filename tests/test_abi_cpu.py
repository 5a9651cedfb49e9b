"""CPU checks of the C ABI: the library builds for sm_103a, loads, exports every
symbol include/mmf_gb300.h declares, validates arguments before touching a
device, and fails loudly (no CPU fallback) when no GPU is present."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "mmf_gb300.h")).read()
    return sorted(set(re.findall(r"\b(mmf_[a-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported(mmf):
    lib = mmf.capi.load()
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(mmf.capi.EXPORTS) == syms


def test_abi_version(mmf):
    assert mmf.capi.load().mmf_abi_version() == 1


def _grid(mmf, **kw):
    g = mmf.capi.Grid()
    g.dim, g.h, g.order, g.arith = 2, 1.0, 1, 1
    g.n[0] = g.n[1] = 8
    for k, v in kw.items():
        if k in ("n", "bc_lo", "bc_hi"):
            for i, x in enumerate(v):
                getattr(g, k)[i] = x
        else:
            setattr(g, k, v)
    return g


@pytest.mark.parametrize("kw,code", [
    (dict(dim=4), -1), (dict(h=0.0), -1), (dict(n=[0, 8, 1]), -1), (dict(order=3), -4),
    (dict(bc_lo=[16, 0, 0], bc_hi=[0, 0, 0]), -1), (dict(bc_lo=[7, 0, 0]), -1), (dict(arith=5), -1)])
def test_create_rejects_bad_arguments(mmf, kw, code):
    lib = mmf.capi.load()
    ctx = C.c_void_p()
    assert lib.mmf_create(C.byref(_grid(mmf, **kw)), 0, C.byref(ctx)) == code
    assert not ctx.value
    assert lib.mmf_last_error()


def test_null_context_is_an_error(mmf):
    lib = mmf.capi.load()
    assert lib.mmf_synchronize(None) == -1
    assert lib.mmf_destroy(None) == 0


def test_no_cpu_fallback_without_gpu(mmf):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = mmf.capi.load()
    ctx = C.c_void_p()
    assert lib.mmf_create(C.byref(_grid(mmf)), 0, C.byref(ctx)) == -2
    with pytest.raises(mmf.capi.MMFError):
        from minimmerflow_gb300 import euler
        euler.conservative2primitive([[1.0, 0, 0, 0, 2.5]])


def test_null_handles_are_argument_errors(mmf):
    """Every entry point that takes a context, a batch, a face-list context or
    an MLP rejects a null handle with MMF_ERR_ARG before touching a device."""
    lib = mmf.capi.load()
    d = C.c_double()
    i64 = C.c_int64()
    ci = C.c_int()
    prob = mmf.capi.Problem()
    calls = {
        "mmf_upload_state": (None, None, 0), "mmf_download_state": (None, None, 0),
        "mmf_compute_rhs": (None, None, None, None, 0), "mmf_time_setup": (None, 0.5, 0.0, 1.0, -1),
        "mmf_advance": (None, 1, C.byref(d), C.byref(i64)), "mmf_advance_async": (None, 1),
        "mmf_advance_host": (None, None, 0, 1, C.byref(d)), "mmf_rk_stage": (None, 1),
        "mmf_autotune": (None, 2, C.byref(ci), C.byref(ci)),
        "mmf_init_state": (None, C.byref(prob)), "mmf_l1_density_error": (None, C.byref(prob), 0.0, C.byref(d)),
        "mmf_write_vtk": (None, b"x.vti"), "mmf_save_checkpoint": (None, b"x.ckpt"),
        "mmf_load_checkpoint": (None, b"x.ckpt"),
        "mmf_umesh_advance": (None, 1, C.byref(d), C.byref(i64)),
        "mmf_batch_advance_async": (None, 1), "mmf_batch_synchronize": (None,),
    }
    for name, args in calls.items():
        rc = getattr(lib, name)(*args)
        assert rc == mmf.capi.MMF_ERR_ARG, (name, rc)

"""The C-ABI library loads and exports every entry point include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "taichi_lbm3d_gb300", "liblbm_gb300.so")


def declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"^\s*(?:int|void|int32_t|int64_t)\s+(lbm_\w+)\s*\(", txt, flags=re.M))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        from taichi_lbm3d_gb300 import build
        build.build()
    return ctypes.CDLL(LIB)


def test_header_declares_entry_points():
    names = declared()
    assert "lbm_create" in names and "lbm_step" in names and len(names) >= 20


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_exports_are_plain_c(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True, text=True).stdout
    for n in declared():
        assert re.search(r" T %s$" % n, out, flags=re.M), n


def test_abi_version_and_struct_sizes(lib):
    from taichi_lbm3d_gb300 import _native
    assert lib.lbm_abi_version() == 1
    # LbmParams layout: 3 + 6 ints, 6 + 18 + 1 + 3 doubles, ... (checked by offsets of the last fields)
    P = _native.LbmParams
    assert P.block_size.offset + 4 <= ctypes.sizeof(P)
    assert P.rho_bc.offset % 8 == 0 and P.niu_l.offset % 8 == 0


def test_create_without_gpu_fails_loudly(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    from taichi_lbm3d_gb300 import _native
    with pytest.raises(_native.LbmError) as ei:
        _native.Lattice(_native.make_params((8, 8, 8)))
    assert ei.value.code == _native.LBM_ENODEV


def test_null_handles_are_rejected_without_a_gpu(lib):
    """Host-side failure paths: every handle call given NULL returns LBM_EINVAL
    (and records a message) before touching CUDA; the NVTX ranges around the
    calls are inert without a profiler."""
    P = ctypes.c_void_p
    lib.lbm_step_async.argtypes = [P, ctypes.c_int32]
    lib.lbm_step.argtypes = [P, ctypes.c_int32]
    lib.lbm_init.argtypes = [P, P, P]
    lib.lbm_get_macros.argtypes = [P, P, P]
    lib.lbm_reductions.argtypes = [P, P]
    lib.lbm_set_geometry_strided.argtypes = [P, P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]
    lib.lbm_run_to_convergence.argtypes = [P, ctypes.c_double, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                                           P, P, P]
    lib.lbm_last_error.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
    calls = [lambda: lib.lbm_step_async(None, 1), lambda: lib.lbm_step(None, 1),
             lambda: lib.lbm_init(None, None, None), lambda: lib.lbm_get_macros(None, None, None),
             lambda: lib.lbm_reductions(None, None), lambda: lib.lbm_set_geometry_strided(None, None, 1, 1, 1),
             lambda: lib.lbm_run_to_convergence(None, 1e-6, 10, 10, 0, None, None, None)]
    for c in calls:
        assert c() == -1
    buf = ctypes.create_string_buffer(256)
    lib.lbm_last_error(None, buf, 256)
    assert b"NULL" in buf.value

"""The -DLBM_DEBUG build (index checks in the single-phase step, read back by
lbm_synchronize) compiles for sm_103a; the default build carries none of it.
Compile-only: no GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "taichi_lbm3d_gb300", "csrc")


def test_debug_build_compiles(tmp_path):
    import concurrent.futures as cf
    from taichi_lbm3d_gb300 import build
    nvcc = build._nvcc()
    if shutil.which(nvcc) is None and not os.path.exists(nvcc):
        pytest.skip("nvcc not available")

    def compile_one(src):
        cmd = [nvcc] + build.NVCC_FLAGS + ["-DLBM_DEBUG", "-c", os.path.join(CSRC, src),
                                           "-o", str(tmp_path / (src + ".o"))]
        return src, subprocess.run(cmd, capture_output=True, text=True)

    with cf.ThreadPoolExecutor(3) as ex:
        for src, r in ex.map(compile_one, ["lbm_sp.cu", "lbm_capi.cu", "lbm_tp.cu"]):
            assert r.returncode == 0, (src, r.stderr[-2000:])


def test_default_build_has_no_debug_checks():
    txt = open(os.path.join(CSRC, "lbm_kernels.cuh")).read() + open(os.path.join(CSRC, "lbm_sp.cu")).read()
    # every use of the debug flag sits inside #ifdef LBM_DEBUG
    depth, inside = 0, []
    for line in txt.splitlines():
        t = line.strip()
        if t.startswith("#ifdef LBM_DEBUG"):
            depth += 1
        elif depth and t.startswith("#if"):
            depth += 1
        elif depth and t.startswith("#endif"):
            depth -= 1
        elif "g_lbm_debug" in t or "lbm_debug_fail" in t:
            inside.append(depth > 0)
    assert inside and all(inside)

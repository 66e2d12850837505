"""The -DLBM_DEBUG library on the GPU: the single-phase step with its index
checks compiled in (node coordinates inside the lattice, every gathered map
entry below the fluid-node count) runs the small parity cases bit for bit
against the oracle, and neither lbm_synchronize nor lbm_run_to_convergence
reports a failed check.

The debug library is built into a temporary directory and driven from a child
process, so the default library loaded by the other tests is untouched.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[2])
from taichi_lbm3d_gb300 import _native
_native.load(sys.argv[1])
from oracle.oracle import Oracle, make_params as op
from taichi_lbm3d_gb300.geometry import cavity_shell, sphere_pack

def native(p):
    return _native.make_params((p.nx, p.ny, p.nz), niu=p.niu, force=tuple(p.force), bc=tuple(p.bc),
                               rho_bc=tuple(p.rho_bc), vel_bc=[tuple(v) for v in p.vel_bc],
                               visc_convention=p.visc_convention, guo_convention=p.guo_convention)

vel = ((0, 0, 0),) * 5 + ((0.1, 0.0, 0.0),)
cases = [(op((16, 16, 16), niu=0.1, bc=(0, 0, 0, 0, 0, 2), vel_bc=vel), cavity_shell(16), 50),
         (op((40, 32, 24), niu=0.1, bc=(1, 1, 0, 0, 0, 0), rho_bc=(1.0005, 1.0, 1, 1, 1, 1)),
          sphere_pack((40, 32, 24), 3, 6, 0.45, seed=5), 200),
         (op((33, 20, 17), niu=0.1, force=(1e-5, 0, 0), visc_convention=1, guo_convention=2),
          sphere_pack((33, 20, 17), 2, 4, 0.45, seed=6), 100)]
for p, solid, n in cases:
    lat = _native.Lattice(native(p))
    lat.set_geometry(solid)
    lat.init()
    lat.step(n)                         # lbm_step ends in lbm_synchronize: raises on a failed check
    rho, v = lat.macros()
    o = Oracle(p, solid)
    o.step(n)
    fl = solid == 0
    assert np.array_equal(rho[fl], o.field("rho").astype(np.float32)[fl])
    assert np.array_equal(v[fl], o.field("v").astype(np.float32)[fl])
    r = lat.run_to_convergence(tol=0.0, check_every=25, max_steps=50)
    assert r is not None
    lat.close()
print("debug build ok")
"""


def test_debug_library_runs_parity_cases(tmp_path):
    from taichi_lbm3d_gb300 import build
    nvcc = build._nvcc()
    srcs = build.sources()

    def compile_one(src):
        obj = str(tmp_path / (os.path.basename(src)[:-3] + ".o"))
        r = subprocess.run([nvcc] + build.NVCC_FLAGS + ["-DLBM_DEBUG", "-c", src, "-o", obj],
                           capture_output=True, text=True)
        assert r.returncode == 0, (src, r.stderr[-2000:])
        return obj

    with cf.ThreadPoolExecutor(min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    lib = str(tmp_path / "liblbm_gb300_debug.so")
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", lib] + objs +
                       ["-lcudart"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([sys.executable, "-c", CHILD, lib, ROOT], capture_output=True, text=True, cwd=ROOT,
                       timeout=600)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert "debug build ok" in r.stdout

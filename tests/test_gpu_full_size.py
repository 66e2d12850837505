"""Parity at the benchmark workloads' own sizes, through the C ABI.

The other GPU tests pin the kernels on lattices of 64^3 and smaller.  These run
the full workloads against the FP32 CPU oracle:

* the 256^3 sphere pack (seed 2, radii U[4,10], porosity 0.35, percolating
  cluster; 5,866,274 fluid nodes) with fixed pressure 1.0005 / 1.0 on the x
  faces, periodic y/z, niu 0.1 and the class conventions, 100 steps of
  ``LB3D_Solver_Single_Phase.step`` (Single_phase/LBM_3D_SinglePhase_Solver.py:477-481):
  rho, v and max|v| bit for bit.  At this size the packed 11/11/10-bit node
  coordinates, more than 2^16 CTAs and every face row are exercised;
* the 131^3 two-phase drainage (seed 3, radii U[3,8], porosity 0.40, psi slab,
  CapA 0.005), 50 steps of the script's loop
  (2phase/lbm_solver_3d_2phase_sparse.py:626-632): rho, v, psi, rho_r and rho_b
  bit for bit in the direction-ordered colour sum.  131 is odd, so fluid rows
  never line up with the 32-node population chunks;
* subvolumes of the batched workload (edges 160, 48, 96, 64 drawn from its
  seeded distribution) advanced together in one batch: each subvolume's rho and
  v against its own oracle lattice, bit for bit in FP32 and within the 16-bit
  tolerance in FP16 deviation storage.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from oracle.oracle import make_params as oracle_params
from taichi_lbm3d_gb300 import _native
from taichi_lbm3d_gb300.geometry import sphere_pack
from tests import goldens as G

pytestmark = pytest.mark.gpu


def _fp32_norm_max(v, fl):
    """cal_max_v (SP:394-402): FP32 norm per cell, max over the lattice."""
    w = v[fl].astype(np.float32)
    n2 = (w[:, 0] * w[:, 0] + w[:, 1] * w[:, 1]) + w[:, 2] * w[:, 2]
    return float(np.sqrt(n2.astype(np.float32)).max())


def test_porous256_pressure_100_steps_bit_exact():
    shape = (256, 256, 256)
    solid = sphere_pack(shape, 4.0, 10.0, 0.35, 2)
    fl = solid == 0
    assert int(fl.sum()) == 5866274
    p = oracle_params(shape, niu=0.1, bc=(1, 1, 0, 0, 0, 0), rho_bc=(1.0005, 1.0, 1, 1, 1, 1))
    lat = _native.Lattice(_native.make_params(shape, niu=0.1, bc=(1, 1, 0, 0, 0, 0),
                                              rho_bc=(1.0005, 1.0, 1, 1, 1, 1)))
    lat.set_geometry(solid)
    lat.init()
    lat.step(100)
    rho, v = lat.macros()
    max_v = lat.max_v()
    lat.close()
    o = Oracle(p, solid)
    o.step(100)
    rho_o = o.field("rho").astype(np.float32)
    v_o = o.field("v").astype(np.float32)
    o.close()
    assert np.array_equal(rho[fl], rho_o[fl])
    assert np.array_equal(v[fl], v_o[fl])
    assert max_v == _fp32_norm_max(v_o, fl)
    assert max_v > 0.0


def test_drainage131_50_steps_bit_exact():
    shape = (131, 131, 131)
    solid = sphere_pack(shape, 3.0, 8.0, 0.40, seed=3)
    psi0 = -np.ones(shape, np.float32)
    psi0[:5] = 1.0
    op = oracle_params(shape, bc=(1, 1, 0, 0, 0, 0), rho_bc=(1.001, 1.0, 1, 1, 1, 1), visc_convention=1,
                       guo_convention=1, bc_form=1, two_phase=True, niu_l=0.05, niu_g=0.2, psi_solid=0.7,
                       cap_a=0.005, psi_bc=(1, 1, 0, 0, 0, 0), psi_val=(1.0, -1.0, 1, 1, 1, 1))
    lat = _native.Lattice(_native.make_params(shape, niu=0.1, bc=(1, 1, 0, 0, 0, 0),
                                              rho_bc=(1.001, 1.0, 1, 1, 1, 1), visc_convention=1,
                                              guo_convention=1, bc_form=1, two_phase=True, niu_l=0.05,
                                              niu_g=0.2, psi_solid=0.7, cap_a=0.005,
                                              psi_bc=(1, 1, 0, 0, 0, 0), psi_val=(1.0, -1.0, 1, 1, 1, 1)))
    lat.set_geometry(solid)
    lat.set_psi(psi0)
    lat.init()
    lat.step(50)
    rho, v = lat.macros()
    psi, rr, rb = lat.phase()
    lat.close()
    gpu = {"rho": rho, "v": v, "psi": psi, "rho_r": rr, "rho_b": rb}
    o = Oracle(op, solid, psi0)
    o.step(50)
    fl = solid == 0
    for f, a in gpu.items():
        assert np.array_equal(a[fl], o.field(f).astype(np.float32)[fl]), f
    o.close()
    # the drainage front has entered the pack: some fluid nodes changed phase
    assert 0 < int((psi[fl] > 0).sum()) < int(fl.sum())


BATCH_SEEDS = (4000, 4002, 4010, 4020)     # edges 160, 48, 96, 64 of the batched workload
BATCH_STEPS = 200


@pytest.fixture(scope="module")
def batch_solids():
    from taichi_lbm3d_gb300.batch import subvolume_sample
    return [subvolume_sample(s) for s in BATCH_SEEDS]


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_batched_subvolumes_fieldwise_vs_oracle(batch_solids, storage):
    from taichi_lbm3d_gb300.batch import Batch
    S = batch_solids
    assert [s.shape[0] for s in S] == [160, 48, 96, 64]
    force = (1e-6, 0.0, 0.0)
    b = Batch(S, niu=0.1, force=force, storage=storage, visc_convention=1, guo_convention=2)
    b.configure([1024] * len(S), 256)
    b.init()
    b.step(BATCH_STEPS, chunk=50, use_graph=True)
    for q, s in enumerate(S):
        rho, v = b.macros(q)
        fl = s == 0
        p = oracle_params(s.shape, niu=0.1, force=force, visc_convention=1, guo_convention=2)
        o = Oracle(p, s, precision=32 if storage == "f32" else 64)
        # the batch's readback streams its current (post-collision) populations
        # once more: the macros of the next step, BATCH_STEPS + 1
        o.step(BATCH_STEPS + 1)
        if storage == "f32":
            assert np.array_equal(rho[fl], o.field("rho").astype(np.float32)[fl]), q
            assert np.array_equal(v[fl], o.field("v").astype(np.float32)[fl]), q
        else:
            # FP16 deviation storage against FP64: the 16-bit tolerance of the
            # single-lattice storage tests (normwise v, rho deviation from rest)
            e_v = G.normwise_rel(v, o.field("v"), fl)
            r64 = o.field("rho")
            e_rho = np.abs(rho[fl] - r64[fl]).max() / max(np.abs(r64[fl] - 1.0).max(), 1e-30)
            assert e_v < 2e-2 and e_rho < 2e-2, (q, e_v, e_rho)
        o.close()
    b.close()

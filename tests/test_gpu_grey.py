"""GPU parity of the grey-scale (partial bounce-back) step.

* through the drop-in class against the fixtures made from the reference
  script's own source: bit-exact;
* against the CPU oracle on larger random grey fields (x-inside fast path,
  fixed-velocity faces whose upstream cells are solid): bit-exact in FP32,
  to round-off in FP64;
* deviation-form storage variants against the FP64 oracle, normwise.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle, make_params
from taichi_lbm3d_gb300 import LB3D_Solver_Grey_Scale, _native
from tests import goldens as G

pytestmark = pytest.mark.gpu


def grey_lattice(op, ns, storage="f32"):
    lat = _native.Lattice(_native.make_params((op.nx, op.ny, op.nz), niu=op.niu, force=tuple(op.force),
                                              bc=tuple(op.bc), rho_bc=tuple(op.rho_bc),
                                              vel_bc=[tuple(v) for v in op.vel_bc], visc_convention=1,
                                              guo_convention=1, bc_form=1, storage=storage))
    lat.set_geometry(G.grey_solid(ns))
    lat.set_grey(ns)
    lat.init()
    return lat


def grey_oracle(op, ns, precision=32):
    o = Oracle(op, G.grey_solid(ns), precision=precision)
    o.set_field("ns", ns)
    return o


def random_ns(shape, seed, walls=False):
    rng = np.random.default_rng(seed)
    ns = rng.choice([0.0, 0.0, 0.0, 0.05, 0.2, 0.5, 0.9, 1.0], size=shape)
    if walls:
        ns[:, 0, :] = ns[:, -1, :] = 1.0
    return ns


@pytest.mark.parametrize("name", G.GREY_CASES)
def test_grey_golden_cases_bit_exact_through_class(name):
    d = G.load(name)
    P = G.params_of(d)
    shape = tuple(int(x) for x in d["shape"])
    lb = LB3D_Solver_Grey_Scale(*shape)
    lb.fx, lb.fy, lb.fz = P["force"]
    lb.niu = P["niu"]
    lb.bc_x_left, lb.bc_x_right = P["bc"][0], P["bc"][1]
    lb.rho_bcxl, lb.rho_bcxr = P["rho_bc"][0], P["rho_bc"][1]
    lb.vx_bcxl, lb.vy_bcxl, lb.vz_bcxl = P["vel_bc"][0]
    lb.vx_bcxr, lb.vy_bcxr, lb.vz_bcxr = P["vel_bc"][1]
    lb.ns.from_numpy(d["ns"])
    lb.solid.from_numpy(d["ns"].astype(int))
    lb.init_simulation()
    done = 0
    for st in d["steps"]:
        lb.run(int(st) - done)
        done = int(st)
        assert np.array_equal(lb.rho.to_numpy(), d["rho_%d" % st]), (name, st)
        assert np.array_equal(lb.v.to_numpy(), d["v_%d" % st]), (name, st)
    lb.close()


def random_force_case():
    shape = (72, 20, 12)
    ns = random_ns(shape, 41)
    op = make_params(shape, niu=0.08, force=(3e-5, -1e-5, 2e-5), visc_convention=1, guo_convention=1, bc_form=1,
                     grey=True)
    return shape, ns, op


def test_grey_random_field_with_force_bit_exact():
    shape, ns, op = random_force_case()
    o = grey_oracle(op, ns)
    o.step(150)
    lat = grey_lattice(op, ns)
    lat.step(150)
    rho, v = lat.macros()
    fl = G.grey_solid(ns) == 0
    assert np.array_equal(rho[fl], o.field("rho").astype(np.float32)[fl])
    assert np.array_equal(v[fl], o.field("v").astype(np.float32)[fl])


def test_grey_fp64_agrees_with_fp64_oracle_to_round_off():
    shape, ns, op = random_force_case()
    o = grey_oracle(op, ns, 64)
    o.step(150)
    lat = grey_lattice(op, ns, "f64")
    lat.step(150)
    rho, v = lat.macros_f64()
    fl = G.grey_solid(ns) == 0
    e_rho = np.abs(rho[fl] - o.field("rho")[fl]).max() / np.abs(o.field("rho")[fl] - 1.0).max()
    e_v = G.normwise_rel(v, o.field("v"), fl)
    assert e_rho < 1e-9 and e_v < 1e-9, (e_rho, e_v)


@pytest.mark.parametrize("bc", [(2, 1), (1, 2), (2, 2), (1, 1)])
def test_grey_x_faces_bit_exact(bc):
    """Velocity faces read the slots that no fluid cell pushes into (walls at
    y = 0 / ny-1 reach the faces); pressure faces use the previous step's v."""
    shape = (40, 14, 9)
    ns = random_ns(shape, 42, walls=True)
    op = make_params(shape, niu=0.1, bc=(bc[0], bc[1], 0, 0, 0, 0), rho_bc=(1.003, 0.999, 1, 1, 1, 1),
                     vel_bc=((0.01, 0.002, 0.0), (0.004, 0.0, -0.001), (0, 0, 0), (0, 0, 0), (0, 0, 0), (0, 0, 0)),
                     visc_convention=1, guo_convention=1, bc_form=1, grey=True)
    o = grey_oracle(op, ns)
    o.step(120)
    lat = grey_lattice(op, ns)
    lat.step(120)
    rho, v = lat.macros()
    fl = G.grey_solid(ns) == 0
    assert np.array_equal(rho[fl], o.field("rho").astype(np.float32)[fl])
    assert np.array_equal(v[fl], o.field("v").astype(np.float32)[fl])


# Deviation-form storage after 300 steps from rest, normwise against FP64
@pytest.mark.parametrize("storage,tol", [("f32dev", 1e-4), ("f16", 2e-2), ("bf16", 1e-1)])
def test_grey_storage_variants_close_to_fp64_oracle(storage, tol):
    shape = (48, 16, 12)
    ns = random_ns(shape, 43, walls=True)
    op = make_params(shape, niu=0.1, force=(2e-5, 0, 0), bc=(1, 1, 0, 0, 0, 0), rho_bc=(1.002, 1.0, 1, 1, 1, 1),
                     visc_convention=1, guo_convention=1, bc_form=1, grey=True)
    o = grey_oracle(op, ns, 64)
    o.step(300)
    lat = grey_lattice(op, ns, storage)
    lat.step(300)
    rho, v = lat.macros_f64()
    fl = G.grey_solid(ns) == 0
    e_rho = np.abs(rho[fl] - o.field("rho")[fl]).max() / np.abs(o.field("rho")[fl] - 1.0).max()
    e_v = G.normwise_rel(v, o.field("v"), fl)
    print("grey storage %s: e_rho %.3e e_v %.3e" % (storage, e_rho, e_v))
    assert e_rho < tol and e_v < tol, (storage, e_rho, e_v)


def test_grey_rejects_y_z_faces():
    shape = (8, 8, 8)
    ns = np.zeros(shape)
    lat = _native.Lattice(_native.make_params(shape, bc=(0, 0, 1, 0, 0, 0), visc_convention=1, guo_convention=1))
    lat.set_geometry(G.grey_solid(ns))
    with pytest.raises(_native.LbmError):
        lat.set_grey(ns)
    lat.close()


def test_grey_zero_ns_equals_open_push_without_bounce_back():
    """ns = 0 everywhere and no solid: the grey step is plain periodic
    streaming, the same as the single-phase step on an all-fluid lattice."""
    shape = (24, 12, 10)
    ns = np.zeros(shape)
    op = make_params(shape, niu=0.1, force=(1e-5, 0, 0), visc_convention=1, guo_convention=1, bc_form=1, grey=True)
    lat = grey_lattice(op, ns)
    lat.step(50)
    ref = _native.Lattice(_native.make_params(shape, niu=0.1, force=(1e-5, 0, 0), visc_convention=1,
                                              guo_convention=1, bc_form=1))
    ref.set_geometry(np.zeros(shape, np.int8))
    ref.init()
    ref.step(50)
    a, b = lat.macros(), ref.macros()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])

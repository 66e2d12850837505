"""Degenerate and ragged lattices: no fluid node at all, a single fluid cell,
and boxes one cell thin in x, y or z.  The reference runs all of these (its
loops simply have nothing or little to do); here an all-solid lattice steps
as a no-op, and the thin and single-cell boxes agree bit for bit with the CPU
oracle (periodic wrap onto the node itself, bounce-back on every side)."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from oracle.oracle import make_params as oracle_params
from taichi_lbm3d_gb300 import _native

pytestmark = pytest.mark.gpu


def native(p, storage="f32", **kw):
    return _native.make_params((p.nx, p.ny, p.nz), niu=p.niu, force=tuple(p.force), bc=tuple(p.bc),
                               rho_bc=tuple(p.rho_bc), vel_bc=[tuple(v) for v in p.vel_bc],
                               visc_convention=p.visc_convention, guo_convention=p.guo_convention,
                               bc_form=p.bc_form, storage=storage, **kw)


@pytest.mark.parametrize("storage", ["f32", "f16", "f64"])
def test_all_solid_lattice_steps_as_a_no_op(storage):
    shape = (6, 5, 4)
    p = oracle_params(shape, niu=0.1, force=(1e-5, 0.0, 0.0))
    lat = _native.Lattice(native(p, storage))
    lat.set_geometry(np.ones(shape, np.int8))
    lat.init()
    lat.step(7)
    assert lat.info().n_fluid == 0
    rho, v = lat.macros()
    assert np.all(rho == 1.0) and np.all(v == 0.0)
    st = lat.stats()
    assert st.mass == 0.0 and st.n_fluid == 0 and st.n_nonfinite == 0
    darcy_v, steps, converged = lat.run_to_convergence(tol=1e-6, check_every=10, max_steps=100)
    assert converged and darcy_v == 0.0 and steps == 20
    lat.close()


def test_all_solid_grey_and_two_phase_lattices():
    shape = (5, 4, 3)
    g = _native.Lattice(_native.make_params(shape, niu=0.1, visc_convention=1, guo_convention=1, bc_form=1))
    g.set_geometry(np.ones(shape, np.int8))
    g.set_grey(np.ones(shape))
    g.init()
    g.step(3)
    rho, v = g.macros()
    assert np.all(rho == 1.0) and np.all(v == 0.0)
    g.close()
    t = _native.Lattice(_native.make_params(shape, niu=0.1, two_phase=True))
    t.set_geometry(np.ones(shape, np.int8))
    psi0 = np.where(np.arange(shape[0])[:, None, None] < 2, 1.0, -1.0) * np.ones(shape)
    t.set_psi(psi0.astype(np.float32))
    t.init()
    t.step(3)
    psi, _, _ = t.phase()
    assert np.array_equal(psi, psi0.astype(np.float32))   # solid cells keep the input psi
    t.close()


@pytest.mark.parametrize("shape", [(1, 7, 5), (6, 1, 4), (5, 6, 1), (1, 1, 9), (1, 1, 1)])
def test_thin_boxes_match_oracle_bit_exact(shape):
    rng = np.random.default_rng(sum(shape))
    solid = (rng.random(shape) < 0.25).astype(np.int8)
    solid.flat[0] = 0                                     # at least one fluid cell
    p = oracle_params(shape, niu=0.08, force=(2e-5, -1e-5, 3e-5), visc_convention=1, guo_convention=2)
    o = Oracle(p, solid)
    o.step(25)
    lat = _native.Lattice(native(p))
    lat.set_geometry(solid)
    lat.init()
    lat.step(25)
    rho, v = lat.macros()
    lat.close()
    fl = solid == 0
    assert np.array_equal(rho[fl], o.field("rho").astype(np.float32)[fl])
    assert np.array_equal(v[fl], o.field("v").astype(np.float32)[fl])


def test_single_fluid_cell_in_a_solid_box():
    shape = (3, 3, 3)
    solid = np.ones(shape, np.int8)
    solid[1, 1, 1] = 0
    p = oracle_params(shape, niu=0.1, force=(1e-5, 0.0, 0.0), visc_convention=1, guo_convention=2)
    o = Oracle(p, solid)
    o.step(40)
    lat = _native.Lattice(native(p))
    lat.set_geometry(solid)
    lat.init()
    lat.step(40)
    rho, v = lat.macros()
    lat.close()
    assert rho[1, 1, 1] == np.float32(o.field("rho")[1, 1, 1])
    assert np.array_equal(v[1, 1, 1], o.field("v").astype(np.float32)[1, 1, 1])

"""Consecutive step launches overlap: a step's CTAs may become resident while
the previous launch drains (programmatic dependent launch) and wait for it
before touching any state.  The results must not depend on how the steps are
issued: K steps in one call, K one-step calls, and one-step calls interleaved
with readbacks and reductions (other kernels and copies between the steps)
give bit-identical fields.  The lattices are large enough that every launch
runs many waves of CTAs, so the overlap does happen."""
import numpy as np
import pytest

from taichi_lbm3d_gb300 import _native
from taichi_lbm3d_gb300.geometry import sphere_pack

pytestmark = pytest.mark.gpu

K = 30


def issue(lat, how):
    if how == "one_call":
        lat.step(K)
    elif how == "single_steps":
        for _ in range(K):
            lat.step(1)
    else:   # single steps with readbacks and reductions in between
        for i in range(K):
            lat.step(1)
            if i % 4 == 1:
                lat.macros()
            if i % 5 == 2:
                lat.stats()


def fields(lat, two_phase=False):
    rho, v = lat.macros()
    out = [rho, v]
    if two_phase:
        out += list(lat.phase())
    return out


def same(a, b):
    return all(np.array_equal(x, y, equal_nan=True) for x, y in zip(a, b))


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_single_phase_results_do_not_depend_on_launch_grouping(storage):
    shape = (128, 128, 128)
    solid = sphere_pack(shape, 3.0, 8.0, 0.40, seed=5)
    p = _native.make_params(shape, niu=0.1, bc=(1, 1, 0, 0, 0, 0), rho_bc=(1.001, 1.0, 1, 1, 1, 1),
                            force=(1e-6, 0.0, 0.0), storage=storage)
    res = {}
    for how in ("one_call", "single_steps", "interleaved"):
        lat = _native.Lattice(p)
        lat.set_geometry(solid)
        lat.init()
        issue(lat, how)
        res[how] = fields(lat)
        lat.close()
    assert np.abs(res["one_call"][1]).max() > 0
    assert same(res["one_call"], res["single_steps"])
    assert same(res["one_call"], res["interleaved"])


def test_grey_results_do_not_depend_on_launch_grouping():
    shape = (96, 96, 96)
    rng = np.random.default_rng(7)
    ns = rng.choice([0.0, 0.0, 0.0, 0.1, 0.5, 1.0], size=shape)
    p = _native.make_params(shape, niu=0.1, force=(2e-5, 0.0, 0.0), visc_convention=1, guo_convention=1,
                            bc_form=1)
    res = {}
    for how in ("one_call", "single_steps", "interleaved"):
        lat = _native.Lattice(p)
        lat.set_geometry((ns >= 1.0).astype(np.int8))
        lat.set_grey(ns)
        lat.init()
        issue(lat, how)
        res[how] = fields(lat)
        lat.close()
    assert np.abs(res["one_call"][1]).max() > 0
    assert same(res["one_call"], res["single_steps"])
    assert same(res["one_call"], res["interleaved"])


def test_two_phase_results_do_not_depend_on_launch_grouping():
    shape = (96, 64, 64)
    solid = sphere_pack(shape, 3.0, 6.0, 0.45, seed=9)
    psi0 = -np.ones(shape, np.float32)
    psi0[:6] = 1.0
    p = _native.make_params(shape, niu=0.1, bc=(1, 1, 0, 0, 0, 0), rho_bc=(1.001, 1.0, 1, 1, 1, 1),
                            visc_convention=1, guo_convention=1, bc_form=1, two_phase=True, niu_l=0.05, niu_g=0.2,
                            psi_solid=0.7, cap_a=0.005, psi_bc=(1, 1, 0, 0, 0, 0), psi_val=(1.0, -1.0, 1, 1, 1, 1))
    res = {}
    for how in ("one_call", "single_steps", "interleaved"):
        lat = _native.Lattice(p)
        lat.set_geometry(solid)
        lat.set_psi(psi0)
        lat.init()
        issue(lat, how)
        res[how] = fields(lat, two_phase=True)
        lat.close()
    assert np.abs(res["one_call"][1]).max() > 0
    assert same(res["one_call"], res["single_steps"])
    assert same(res["one_call"], res["interleaved"])

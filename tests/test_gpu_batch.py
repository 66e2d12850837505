"""Batched persistent launch (K5) and its autotuner."""
import json

import numpy as np
import pytest

from taichi_lbm3d_gb300 import _native
from taichi_lbm3d_gb300.geometry import sphere_pack

pytestmark = pytest.mark.gpu


def solids():
    return [sphere_pack((24, 24, 24), 2, 4, 0.45, seed=51), sphere_pack((32, 32, 32), 2.5, 5, 0.40, seed=52),
            sphere_pack((16, 16, 16), 1.5, 3, 0.50, seed=53)]


@pytest.mark.parametrize("storage", ["f32", "f16"])
@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_matches_single_lattices(storage, use_graph):
    from taichi_lbm3d_gb300.batch import Batch
    S = solids()
    b = Batch(S, niu=0.1, force=(1e-5, 0, 0), storage=storage)
    b.configure([64, 128, 32], 128)
    b.init()
    darcy, steps, conv = b.run_to_convergence(tol=0.0, check_every=50, max_steps=100, use_graph=use_graph)
    assert list(steps) == [100, 100, 100] and not conv.any()
    for q, s in enumerate(S):
        lat = _native.Lattice(_native.make_params(s.shape, niu=0.1, force=(1e-5, 0, 0), visc_convention=1,
                                                  guo_convention=2, storage=storage))
        lat.set_geometry(s)
        lat.init()
        lat.step(100)
        ref = lat.stats().mom[0] / s.size
        assert abs(darcy[q] - ref) <= 1e-12 * abs(ref), (q, darcy[q], ref)
    b.close()


def test_batch_converges_and_drops_subvolumes():
    from taichi_lbm3d_gb300.batch import Batch
    S = solids()
    b = Batch(S, niu=0.1, force=(1e-5, 0, 0), storage="f32dev")
    b.configure([256] * 3, 256)
    b.init()
    darcy, steps, conv = b.run_to_convergence(tol=1e-4, check_every=100, max_steps=20000)
    assert conv.all() and (steps > 0).all()
    k = b.permeability(darcy)
    assert (k > 0).all() and np.isfinite(k).all()


def test_autotuner_caches(tmp_path):
    from taichi_lbm3d_gb300 import autotune
    path = str(tmp_path / "tune.json")
    S = solids()
    res = autotune.tune({24: [S[0]], 16: [S[2]]}, storage="f32", path=path)
    assert set(res) == {16, 24} and all(r["tile"] in autotune.TILES for r in res.values())
    data = json.load(open(path))
    assert len(data) == 2
    res2 = autotune.tune({24: [S[0]], 16: [S[2]]}, storage="f32", path=path)
    assert res2[24]["when"] == res[24]["when"]          # served from the cache
    tiles, block = autotune.plan([24, 16, 24], res)
    assert len(tiles) == 3 and block in autotune.BLOCKS


def test_batch_beyond_int32_population_offsets():
    """A batch whose populations span more than 2^31 elements: three
    384x384x300 all-fluid subvolumes (132,710,400 nodes, 2.52e9 elements) ahead
    of a porous one.  The last subvolume's state must match its own single
    lattice bit for bit, and the uniform ones must stay uniform up to the
    FP16 encoder's stochastic rounding, which rounds each node with its own
    random bits (spread of rho below 1e-5, of v_x below 1% of its mean)."""
    from taichi_lbm3d_gb300.batch import Batch
    big = np.zeros((384, 384, 300), np.int8)
    small = sphere_pack((32, 32, 32), 2.5, 5, 0.40, seed=52)
    b = Batch([big, big, big, small], niu=0.1, force=(1e-5, 0, 0), storage="f16")
    assert b.info()["nodes"] * 19 > 2 ** 31
    b.configure([4096, 4096, 4096, 256], 256)
    b.init()
    b.step(20, chunk=10)
    rho_s, v_s = b.macros(3)
    rho_b, v_b = b.macros(2)
    b.close()
    lat = _native.Lattice(_native.make_params(small.shape, niu=0.1, force=(1e-5, 0, 0), visc_convention=1,
                                              guo_convention=2, storage="f16"))
    lat.set_geometry(small)
    lat.init()
    lat.step(21)            # the macros of step 21 are those of the state the batch holds after 20
    rho_r, v_r = lat.macros()
    lat.close()
    assert np.array_equal(rho_s, rho_r) and np.array_equal(v_s, v_r)
    vx = v_b[..., 0].astype(np.float64)
    assert np.ptp(rho_b) < 1e-5 and vx.mean() > 0 and np.ptp(vx) < 1e-2 * vx.mean()
    assert np.abs(v_b[..., 1:]).max() < 1e-2 * vx.mean()


def test_batch_with_an_all_solid_subvolume():
    """A subvolume without fluid rides along: zero Darcy velocity, converged at
    its second check, rho = 1 / v = 0 everywhere; the others are unaffected."""
    from taichi_lbm3d_gb300.batch import Batch
    S = solids()
    S.insert(1, np.ones((12, 10, 8), np.int8))
    b = Batch(S, niu=0.1, force=(1e-5, 0, 0), storage="f32")
    b.configure([64, 64, 128, 32], 128)
    b.init()
    darcy, steps, conv = b.run_to_convergence(tol=0.0, check_every=50, max_steps=100)
    assert darcy[1] == 0.0 and conv[1] and steps[1] == 100
    rho, v = b.macros(1)
    assert np.all(rho == 1.0) and np.all(v == 0.0)
    ref = Batch([S[0]], niu=0.1, force=(1e-5, 0, 0), storage="f32")
    ref.configure([64], 128)
    ref.init()
    d0, _, _ = ref.run_to_convergence(tol=0.0, check_every=50, max_steps=100)
    assert abs(darcy[0] - d0[0]) <= 1e-12 * abs(d0[0])
    ref.close()
    b.close()

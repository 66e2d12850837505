"""GPU parity of the fused single-phase kernel (K1) through the C ABI.

Checks, in order of strictness:
  * sparse index, neighbour table and pure streaming permutation: bit-exact
    against the reference's own periodic_index / streaming1 (golden fixtures);
  * rho / v after N steps: bit-exact against the golden fixtures and the CPU
    oracle (FP32), and within the 1e-6 normwise relative tolerance of the spec
    after 1000 steps of the 64^3 lid-driven cavity;
  * storage variants (FP16/BF16 deviation, FP64) against the FP64 oracle.
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from oracle.oracle import make_params as oracle_params
from taichi_lbm3d_gb300 import _native
from taichi_lbm3d_gb300.geometry import cavity_shell, sphere_pack
from tests import goldens as G

pytestmark = pytest.mark.gpu

TOL = 1e-6  # normwise relative rho / v tolerance after 1000 FP32 steps


def native_from_oracle_params(p, storage="f32"):
    return _native.make_params((p.nx, p.ny, p.nz), niu=p.niu, force=tuple(p.force), bc=tuple(p.bc),
                               rho_bc=tuple(p.rho_bc), vel_bc=[tuple(v) for v in p.vel_bc],
                               visc_convention=p.visc_convention, guo_convention=p.guo_convention,
                               bc_form=p.bc_form, storage=storage)


def lattice(p, solid, storage="f32"):
    lat = _native.Lattice(native_from_oracle_params(p, storage))
    lat.set_geometry(solid)
    lat.init()
    return lat


def test_fluid_index_and_neighbours_match_reference():
    d = G.load("sp_stream")
    shape = tuple(int(x) for x in d["shape"])
    solid = d["solid"]
    lat = lattice(oracle_params(shape), solid)
    idx = lat.fluid_index()
    exp = np.nonzero(solid.ravel(order="F") == 0)[0]
    assert np.array_equal(idx, exp)
    node_of_cell = -np.ones(solid.size, np.int64)
    node_of_cell[exp] = np.arange(exp.size)
    nbr = lat.neighbors()                       # [18][n_fluid] pull sources
    ref = d["nbr"]                              # periodic_index(x + e_s) of every cell
    nx, ny, nz = shape
    for n, c in enumerate(exp):
        i, j, k = c % nx, (c // nx) % ny, c // (nx * ny)
        for s in range(1, 19):
            ip = ref[i, j, k, s]
            cip = ip[0] + nx * (ip[1] + ny * ip[2])
            lr = [0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17][s]
            if solid[tuple(ip)] == 0:
                assert nbr[s - 1, node_of_cell[cip]] == n        # target pulls from x
            else:
                assert nbr[lr - 1, n] == -1 - n                  # bounce into own LR slot


def test_streaming_permutation_bit_exact():
    d = G.load("sp_stream")
    shape = tuple(int(x) for x in d["shape"])
    solid = d["solid"]
    lat = lattice(oracle_params(shape), solid)
    idx = lat.fluid_index()
    f_in = d["f_in"].reshape((-1, 19), order="F")[idx].T           # [19][n_fluid]
    out = lat.debug_stream(f_in)
    exp = d["F_out"].reshape((-1, 19), order="F")[idx].T
    assert np.array_equal(out, exp)


@pytest.mark.parametrize("name", G.SP_CASES)
def test_golden_cases_bit_exact(name):
    d = G.load(name)
    p = G.oracle_params(d)
    lat = lattice(p, d["solid"])
    fluid = d["solid"] == 0
    done = 0
    for st in d["steps"]:
        lat.step(int(st) - done)
        done = int(st)
        rho, v = lat.macros()
        assert np.array_equal(rho[fluid], d["rho_%d" % st][fluid]), (name, st)
        assert np.array_equal(v[fluid], d["v_%d" % st][fluid]), (name, st)
        assert lat.max_v() == d["maxv_%d" % st]


def test_cavity50_fixture_first_step():
    d = G.load("sp_cavity50")
    solid = G.cavity_solid_50()
    P = G.params_of(d)
    lat = lattice(oracle_params((50, 50, 50), niu=P["niu"], bc=P["bc"], rho_bc=P["rho_bc"], vel_bc=P["vel_bc"]),
                  solid)
    lat.step(1)
    rho, v = lat.macros()
    fl = solid == 0
    assert np.array_equal(rho[fl], d["rho_1"][fl]) and np.array_equal(v[fl], d["v_1"][fl])


def cavity64_params():
    # the 64^3 lid-driven cavity: shell on 5 faces, z-top moving with vx = 0.1, niu = 0.1
    return oracle_params((64, 64, 64), niu=0.1, bc=(0, 0, 0, 0, 0, 2),
                         vel_bc=((0, 0, 0),) * 5 + ((0.1, 0.0, 0.0),))


@pytest.fixture(scope="module")
def cavity64_1000():
    p = cavity64_params()
    solid = cavity_shell(64)
    o = Oracle(p, solid)
    o.step(1000)
    lat = lattice(p, solid)
    lat.step(1000)
    return solid, o, lat


def test_cavity64_1000_steps_within_tolerance(cavity64_1000):
    solid, o, lat = cavity64_1000
    rho, v = lat.macros()
    fl = solid == 0
    e_rho = G.normwise_rel(rho, o.field("rho"), fl)
    e_v = G.normwise_rel(v, o.field("v"), fl)
    assert e_rho <= TOL and e_v <= TOL, (e_rho, e_v)


def test_cavity64_1000_steps_bit_exact(cavity64_1000):
    solid, o, lat = cavity64_1000
    rho, v = lat.macros()
    fl = solid == 0
    assert np.array_equal(rho[fl], o.field("rho").astype(np.float32)[fl])
    assert np.array_equal(v[fl], o.field("v").astype(np.float32)[fl])


def test_porous_pressure_and_force_bit_exact():
    solid = sphere_pack((40, 32, 24), 3, 6, 0.45, seed=5)
    for p in (oracle_params((40, 32, 24), niu=0.1, bc=(1, 1, 0, 0, 0, 0), rho_bc=(1.0005, 1.0, 1, 1, 1, 1)),
              oracle_params((40, 32, 24), niu=0.1, force=(1e-5, 0, 0), visc_convention=1, guo_convention=2)):
        o = Oracle(p, solid)
        o.step(200)
        lat = lattice(p, solid)
        lat.step(200)
        rho, v = lat.macros()
        fl = solid == 0
        assert np.array_equal(rho[fl], o.field("rho").astype(np.float32)[fl])
        assert np.array_equal(v[fl], o.field("v").astype(np.float32)[fl])


def test_rest_state_is_invariant_and_mass_conserved():
    solid = sphere_pack((24, 24, 24), 2, 4, 0.5, seed=3)
    p = oracle_params((24, 24, 24), niu=0.1)
    lat = lattice(p, solid)
    lat.step(50)
    # at rest the state stays at rest up to FP32 round-off of the M / M^-1 round
    # trip, and the kernel rounds exactly as the reference arithmetic does
    rho, v = lat.macros()
    fl = solid == 0
    assert np.abs(rho[fl] - 1.0).max() < 1e-5 and lat.stats().max_v < 1e-6
    o = Oracle(p, solid)
    o.step(50)
    assert np.array_equal(rho[fl], o.field("rho").astype(np.float32)[fl])
    assert lat.stats().n_nonfinite == 0
    # periodic, forced: mass is conserved to FP32 round-off
    lat2 = lattice(oracle_params((24, 24, 24), niu=0.1, force=(1e-5, 2e-6, 0)), solid)
    lat2.step(1)
    m0 = lat2.stats().mass
    lat2.step(300)
    assert abs(lat2.stats().mass - m0) / m0 < 1e-5


def test_reductions_match_host_sums():
    d = G.load("sp_mixed")
    lat = lattice(G.oracle_params(d), d["solid"])
    lat.step(10)
    rho, v = lat.macros()
    fl = d["solid"] == 0
    st = lat.stats()
    assert st.n_fluid == fl.sum()
    assert abs(st.mass - rho[fl].astype(np.float64).sum()) < 1e-9 * fl.sum()
    for c in range(3):
        assert abs(st.mom[c] - v[..., c][fl].astype(np.float64).sum()) < 1e-12 * fl.sum() + 1e-15
    norms = np.sqrt((v[fl] * v[fl]).sum(axis=1, dtype=np.float32)).astype(np.float32)
    assert np.float32(st.max_v) == norms.max()


# Transient (300 steps from rest) error of the deviation-storage variants,
# normwise against the FP64 oracle: FP16 keeps 11 significant bits of f - w,
# BF16 8; FP64 must agree to round-off.
@pytest.mark.parametrize("storage,tol", [("f32dev", 1e-4), ("f16", 2e-2), ("bf16", 1e-1)])
@pytest.mark.parametrize("guo", [0, 1, 2])
def test_forced_storage_variants_close_to_fp64_oracle(storage, tol, guo):
    """Body-force runs: the deviation-form kernels add the Guo moments in
    closed form; every convention stays within the storage's tolerance of the
    FP64 oracle's dense form."""
    solid = sphere_pack((32, 24, 24), 2.5, 5, 0.45, seed=19)
    p = oracle_params((32, 24, 24), niu=0.1, force=(2e-5, -1e-5, 5e-6), visc_convention=1, guo_convention=guo)
    o = Oracle(p, solid, precision=64)
    o.step(300)
    lat = lattice(p, solid, storage=storage)
    lat.step(300)
    rho, v = lat.macros_f64()
    fl = solid == 0
    e_rho = np.abs(rho[fl] - o.field("rho")[fl]).max() / max(np.abs(o.field("rho")[fl] - 1.0).max(), 1e-30)
    e_v = G.normwise_rel(v, o.field("v"), fl)
    print("forced storage %s guo %d: e_rho %.3e e_v %.3e" % (storage, guo, e_rho, e_v))
    assert e_v < tol and e_rho < max(tol, 1e-3), (storage, guo, e_rho, e_v)


@pytest.mark.parametrize("storage,tol", [("f64", 1e-9), ("f32dev", 1e-4), ("f16", 2e-2), ("bf16", 1e-1)])
def test_storage_variants_close_to_fp64_oracle(storage, tol):
    solid = sphere_pack((32, 24, 24), 2.5, 5, 0.45, seed=9)
    p = oracle_params((32, 24, 24), niu=0.1, bc=(1, 1, 0, 0, 0, 0), rho_bc=(1.002, 1.0, 1, 1, 1, 1),
                      visc_convention=1)
    o = Oracle(p, solid, precision=64)
    o.step(300)
    lat = lattice(p, solid, storage=storage)
    lat.step(300)
    rho, v = lat.macros_f64()
    fl = solid == 0
    # velocities are ~1e-4: compare the deviation from rest of rho, and v normwise
    e_rho = np.abs(rho[fl] - o.field("rho")[fl]).max() / np.abs(o.field("rho")[fl] - 1.0).max()
    e_v = G.normwise_rel(v, o.field("v"), fl)
    print("storage %s: e_rho %.3e e_v %.3e" % (storage, e_rho, e_v))
    assert e_rho < tol and e_v < tol, (storage, e_rho, e_v)


def test_checkpoint_roundtrip_and_init_from_fields():
    solid = sphere_pack((20, 16, 16), 2, 3, 0.5, seed=4)
    p = oracle_params((20, 16, 16), niu=0.1, force=(1e-5, 0, 0))
    a = lattice(p, solid)
    a.step(30)
    f = a.populations()
    b = lattice(p, solid)
    b.set_populations(f)
    a.step(20)
    b.step(20)
    assert np.array_equal(a.populations(), b.populations())
    rho, v = a.macros()
    c = _native.Lattice(native_from_oracle_params(p))
    c.set_geometry(solid)
    c.init(rho, v)
    c.step(1)
    r2, _ = c.macros()
    assert np.isfinite(r2).all()


def test_errors_are_reported():
    p = _native.make_params((8, 8, 8), bc=(5, 0, 0, 0, 0, 0))
    with pytest.raises(_native.LbmError) as ei:
        _native.Lattice(p)
    assert "bc[0]" in str(ei.value)
    lat = _native.Lattice(_native.make_params((8, 8, 8)))
    with pytest.raises(_native.LbmError):
        lat.step(1)          # before geometry / init


def test_strided_geometry_gives_the_same_index():
    """The device-built index does not depend on the mask's memory layout
    (C order, Fortran order, a bool view, a non-contiguous slice)."""
    solid = sphere_pack((30, 22, 17), 2.0, 4.0, 0.45, seed=12)
    ref = None
    big = np.zeros((60, 22, 17), np.int8)
    big[::2] = solid
    for arr in (solid, np.asfortranarray(solid), solid.astype(bool), big[::2], solid.astype(np.int32)):
        lat = _native.Lattice(_native.make_params(solid.shape))
        lat.set_geometry(arr)
        idx = lat.fluid_index()
        nb = lat.neighbors()
        lat.close()
        if ref is None:
            ref = (idx, nb)
            cells = np.nonzero(solid.ravel(order="F") == 0)[0]
            assert np.array_equal(idx, cells)
        else:
            assert np.array_equal(idx, ref[0]) and np.array_equal(nb, ref[1])


def test_too_many_fluid_nodes_for_one_lattice_is_an_error():
    # 512 x 512 x 440 all fluid = 115,343,360 nodes > 2^31 / 19
    lat = _native.Lattice(_native.make_params((512, 512, 440)))
    with pytest.raises(_native.LbmError) as ei:
        lat.set_geometry(np.zeros((512, 512, 440), np.int8))
    assert "fluid nodes" in str(ei.value)
    lat.close()


@pytest.mark.parametrize("mode", ["1", "2"])
def test_staged_step_kernels_bit_exact(mode, monkeypatch):
    """The opt-in staged step kernels (LBM_SP_TILED=1: persistent, tiles claimed
    from a counter; 2: one tile per CTA) stage coordinates and map rows in
    shared memory with bulk copies; results equal the oracle's bit for bit, on a
    pack where most 256-node tiles are staged (131-cell rows) and on a forced
    all-periodic case whose tiles span y faces and z planes."""
    monkeypatch.setenv("LBM_SP_TILED", mode)
    cases = [(sphere_pack((131, 40, 30), 3, 8, 0.40, seed=3),
              oracle_params((131, 40, 30), niu=0.1, bc=(1, 1, 0, 0, 0, 0), rho_bc=(1.0005, 1.0, 1, 1, 1, 1)), 150),
             (sphere_pack((33, 20, 17), 2, 4, 0.45, seed=6),
              oracle_params((33, 20, 17), niu=0.1, force=(1e-5, 0, 0), visc_convention=1, guo_convention=2), 120)]
    for solid, p, n in cases:
        lat = lattice(p, solid)
        lat.step(n // 2)
        lat.step_async(n - n // 2)          # consecutive launches share the claim counter
        lat.synchronize()
        rho, v = lat.macros()
        o = Oracle(p, solid)
        o.step(n)
        fl = solid == 0
        assert np.array_equal(rho[fl], o.field("rho").astype(np.float32)[fl])
        assert np.array_equal(v[fl], o.field("v").astype(np.float32)[fl])
        lat.close()

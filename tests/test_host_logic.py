"""Host-side logic that needs no GPU: I/O formats, synthetic geometry,
autotuner planning, multi-rank timing reduction (gloo, world size 2)."""
import os
import socket

import numpy as np
import pytest

from taichi_lbm3d_gb300 import autotune, geometry, vtk


def test_vtk_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    shape = (5, 4, 3)
    solid = (rng.random(shape) > 0.7).astype(np.int8)
    rho = rng.random(shape).astype(np.float32)
    v = rng.random(shape + (3,)).astype(np.float32)
    f = vtk.grid_to_vtk(str(tmp_path / "out"), np.arange(5.0), np.arange(4.0), np.arange(3.0),
                        {"Solid": solid, "rho": rho, "velocity": (v[..., 0], v[..., 1], v[..., 2])})
    d = vtk.read_vtr(f)
    assert np.array_equal(d["Solid"], solid) and np.array_equal(d["rho"], rho)
    assert np.array_equal(d["velocity"], v)


def test_ascii_geometry_roundtrip(tmp_path):
    s = geometry.cavity_shell(6)
    path = str(tmp_path / "geo.dat")
    geometry.write_ascii_geometry(path, s)
    assert np.array_equal(geometry.read_ascii_geometry(path, s.shape), s)
    lines = open(path).read().split()
    assert len(lines) == s.size and lines[0] == "1"          # x fastest, first cell is the shell


def test_ascii_geometry_rejects_wrong_size(tmp_path):
    path = str(tmp_path / "g.dat")
    np.savetxt(path, np.zeros(10), fmt="%d")
    with pytest.raises(ValueError):
        geometry.read_ascii_geometry(path, (3, 3, 3))


def test_sphere_pack_porosity_and_percolation():
    from scipy import ndimage
    s = geometry.sphere_pack((48, 40, 40), 3, 6, 0.4, seed=7)
    s2 = geometry.sphere_pack((48, 40, 40), 3, 6, 0.4, seed=7)
    assert np.array_equal(s, s2)                                # seeded, deterministic
    raw = geometry.sphere_pack((48, 40, 40), 3, 6, 0.4, seed=7, percolate=False)
    assert 1.0 - raw.mean() <= 0.4 + 1e-9                       # stopped at the target porosity
    assert np.all(s >= raw)                                     # percolation only adds solid
    fluid = s == 0
    lab, _ = ndimage.label(np.concatenate([fluid, fluid], axis=1))   # y wrap by tiling
    assert fluid[0].any() and fluid[-1].any()


def test_distance_to_solid():
    s = np.zeros((9, 9, 9), np.int8)
    s[4, 4, 4] = 1
    d = geometry.distance_to_solid(s)
    assert d[4, 4, 4] == 0 and d[4, 4, 7] == 3 and abs(d[5, 5, 5] - np.sqrt(3)) < 1e-6


def test_autotune_plan_uses_tuned_tiles():
    tuned = {48: {"tile": 256, "block": 128}, 160: {"tile": 1024, "block": 256}}
    tiles, block = autotune.plan([48, 48, 160], tuned)
    assert tiles == [256, 256, 1024] and block == 256          # the 160^3 class holds most cells


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    q.put((rank, bench.max_over_ranks(1.0 + rank)))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    import multiprocessing as mp
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert got == {0: 2.0, 1: 2.0}


def test_grey_class_parameters_and_geometry_file(tmp_path):
    """The grey-scale class maps the script's globals onto the C parameters:
    tau = 3 niu + 1/2 and the script's Guo form, in-place velocity faces, and
    x faces only (the script's y/z settings have no effect)."""
    from taichi_lbm3d_gb300 import LB3D_Solver_Grey_Scale
    lb = LB3D_Solver_Grey_Scale(6, 5, 4)
    assert (lb.fx, lb.niu, lb.bc_x_left, lb.rho_bcxr) == (1.0e-6, 0.1, 0, 0.995)   # script defaults
    lb.bc_x_left, lb.rho_bcxl = 1, 1.002
    lb.bc_x_right, lb.vx_bcxr = 2, 0.01
    lb.bc_y_left = 1                                     # ignored, as in the script
    p = lb._params()
    assert list(p.bc) == [1, 2, 0, 0, 0, 0]
    assert p.rho_bc[0] == 1.002 and p.vel_bc[1][0] == 0.01
    assert (p.visc_convention, p.guo_convention, p.bc_form) == (1, 1, 1)
    assert tuple(p.force) == (1.0e-6, 0.0, 0.0)
    # geometry file: x fastest, float64 like np.loadtxt; solid = ns.astype(int)
    ns = np.zeros((6, 5, 4))
    ns[:, 0, :] = 1.0
    ns[2:4, 2, 1] = 0.2
    path = tmp_path / "BC.dat"
    np.savetxt(path, ns.ravel(order="F"))
    got = lb.load_geo(str(path))
    assert got.dtype == np.float64 and np.array_equal(got, ns)
    assert np.array_equal(lb.solid.to_numpy(), ns.astype(int)) and np.array_equal(lb.ns.to_numpy(), ns)


def test_voxelize_cli_rejects_missing_file(tmp_path):
    from taichi_lbm3d_gb300 import voxelize as vx
    with pytest.raises(OSError):
        vx.main([str(tmp_path / "absent.stl")])
    bad = tmp_path / "bad.stl"
    bad.write_text("not a mesh")
    with pytest.raises(ValueError):
        vx.read_stl(str(bad))


def test_unet_rejects_unknown_activation():
    pytest.importorskip("torch")
    from taichi_lbm3d_gb300.unet import ACTIVATIONS, UNet3D
    assert ACTIVATIONS == {"relu": 0, "gelu": 1}
    with pytest.raises(ValueError):
        UNet3D(seed=0, activation="tanh")


def test_two_phase_saturation_and_interface_position():
    """Host-side diagnostics of the two-phase class on a synthetic psi field:
    saturation = share of fluid cells with psi > 0, interface = mean x of the
    sign changes along x between fluid cells (cell faces at x + 1/2)."""
    from taichi_lbm3d_gb300 import LB3D_Solver_Two_Phase
    s = LB3D_Solver_Two_Phase(8, 3, 2)
    solid = np.zeros((8, 3, 2), np.int8)
    solid[:, 0, :] = 1                                   # one solid row: 8 x 2 x 2 = 32 fluid cells
    s.solid.from_numpy(solid)
    psi = -np.ones((8, 3, 2), np.float32)
    psi[:3] = 1.0                                        # invading phase in x = 0, 1, 2
    psi[:5, 2, 1] = 1.0                                  # one row reaches x = 4
    s._phase = lambda: (psi, None, None)
    assert s.saturation() == (3 * 4 + 2) / 32
    assert s.interface_position() == (3 * 2.5 + 4.5) / 4
    psi[:] = -1.0
    assert s.saturation() == 0.0 and np.isnan(s.interface_position())


def test_warmstart_summary():
    from taichi_lbm3d_gb300.warmstart import summarize
    rows = []
    for q, (rest_s, warm_s, rest_st, warm_st, r16_st) in enumerate(
            [(10.0, 2.0, 10000, 3000, 3500), (4.0, 1.0, 4000, 2000, 2000), (6.0, 3.0, 6000, 2500, 2000)]):
        rows.append({"rest_f32_seconds": rest_s, "warm_f16_seconds": warm_s, "rest_f32_steps": rest_st,
                     "warm_f16_steps": warm_st, "rest_f16_steps": r16_st, "warm_v_f16_steps": warm_st,
                     "speedup_warm_f16_vs_rest_f32": rest_s / warm_s,
                     "step_ratio_warm_vs_rest_f16": r16_st / warm_st, "step_ratio_warm_v_vs_rest_f16": r16_st / warm_st})
    rows[0]["warm_f16_k_err"] = 1e-5
    sm = summarize(rows)
    assert sm["n"] == 3 and sm["speedup_total"] == 20.0 / 6.0 and sm["speedup_median"] == 4.0
    assert (sm["warm_fewer_steps"], sm["warm_more_steps"]) == (1, 1)
    assert sm["k_err_warm_f16_vs_f64_max"] == 1e-5 and sm["k_err_rest_f32_vs_f64_max"] is None


def test_run_to_convergence_jsonl_log(tmp_path):
    """The logged convergence loop (host side) on a stand-in lattice whose Darcy
    velocity approaches 1e-3 geometrically: one JSON line per check, the stop
    rule of lbm_run_to_convergence (|dv| <= tol |v| between checks), and the
    same permeability formula."""
    import json
    from types import SimpleNamespace
    from taichi_lbm3d_gb300 import LB3D_Solver_Single_Phase

    class FakeLattice:
        def __init__(self):
            self.steps = 0

        def step(self, n):
            self.steps += n

        def stats(self):
            vm = 1e-3 * (1 - 0.5 ** (self.steps / 100))
            return SimpleNamespace(mom=(vm * 64, 0.0, 0.0), mass=40.0, max_v=2 * vm, n_nonfinite=0)

        def info(self):
            return SimpleNamespace(n_fluid=40)

    lb = LB3D_Solver_Single_Phase(4, 4, 4, viscosity_convention="standard", guo_convention="standard")
    lb.niu, lb.fx, lb.tau_f = 0.1, 1e-5, 0.8
    lb._lat = FakeLattice()
    path = tmp_path / "conv.jsonl"
    r = lb.run_to_convergence(tol=1e-3, check_every=100, max_steps=10_000, log=str(path))
    rows = [json.loads(x) for x in path.read_text().splitlines()]
    # rel change between checks n and n+1 is 0.5^(n+1) / (1 - 0.5^(n+1)) <= 1e-3 first at n + 1 = 10
    assert r["converged"] and r["steps"] == 1000 and len(rows) == 10
    assert rows[0]["rel_change"] is None and rows[-1]["rel_change"] <= 1e-3 < rows[-2]["rel_change"]
    assert abs(r["k"] - 0.1 * r["darcy_v"] / 1e-5) <= 1e-12 * r["k"]
    assert rows[-1]["steps"] == 1000 and rows[-1]["mass"] == 40.0

"""Generate golden fixtures by running the reference solver's own source.

Run where a checkout of the reference (taichi_LBM3D) is available, read-only,
giving its root with ``--ref`` or the ``TAICHI_LBM3D_REF`` environment variable:

    python tests/golden/make_golden.py --ref PATH [--only NAME ...]

Taichi is not installable offline, so ``taichi_numpy_shim`` stands in for it:
the reference's kernel bodies (``Single_phase/LBM_3D_SinglePhase_Solver.py``,
``2phase/lbm_solver_3d_2phase_sparse.py`` and
``Grey_Scale/lbm_solver_3d_Macro_Sukop.py``) execute unmodified as Python over
FP32 numpy fields.  The two scripts are module-level programs; their
parameter lines (lattice size, BC codes, physical constants) are edited the way
its README tells a user to edit them, and the file is cut before its main loop
(``time_init = time.time()``); kernel bodies are not touched.

Outputs ``tests/golden/*.npz``; each holds the case's inputs (solid mask,
parameters) and the reference's outputs.  Nothing on the GPU test path reads
the reference checkout; only these fixtures.
"""
import argparse
import importlib.util
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import taichi_numpy_shim  # noqa: E402

taichi_numpy_shim.install()


# ---------------------------------------------------------------- geometry
def spheres_mask(shape, n_spheres, rmin, rmax, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = shape
    solid = np.zeros(shape, dtype=np.int8)
    X, Y, Z = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    for _ in range(n_spheres):
        c = rng.uniform([0, 0, 0], [nx, ny, nz])
        r = rng.uniform(rmin, rmax)
        solid[(X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 <= r * r] = 1
    return solid


def cavity_shell(n, open_face="z1"):
    s = np.zeros((n, n, n), dtype=np.int8)
    s[0, :, :] = 1
    s[-1, :, :] = 1
    s[:, 0, :] = 1
    s[:, -1, :] = 1
    s[:, :, 0] = 1
    if open_face != "z1":
        raise ValueError(open_face)
    return s


# ------------------------------------------------------- single-phase class
def load_class(ref):
    path = os.path.join(ref, "Single_phase", "LBM_3D_SinglePhase_Solver.py")
    spec = importlib.util.spec_from_file_location("ref_lbm_sp", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.LB3D_Solver_Single_Phase


def run_class(cls, shape, solid, setup, steps_list):
    nx, ny, nz = shape
    lb = cls(nx, ny, nz, False)
    lb.solid.from_numpy(solid)
    setup(lb)
    lb.init_simulation()
    out = {}
    done = 0
    for st in steps_list:
        while done < st:
            lb.step()
            done += 1
        out["rho_%d" % st] = lb.rho.to_numpy().astype(np.float32)
        out["v_%d" % st] = lb.v.to_numpy().astype(np.float32)
        out["maxv_%d" % st] = np.float32(lb.get_max_v())
    params = dict(niu=lb.niu, fx=lb.fx, fy=lb.fy, fz=lb.fz,
                  bc=[lb.bc_x_left, lb.bc_x_right, lb.bc_y_left, lb.bc_y_right, lb.bc_z_left, lb.bc_z_right],
                  rho_bc=[lb.rho_bcxl, lb.rho_bcxr, lb.rho_bcyl, lb.rho_bcyr, lb.rho_bczl, lb.rho_bczr],
                  vel_bc=[[lb.vx_bcxl, lb.vy_bcxl, lb.vz_bcxl], [lb.vx_bcxr, lb.vy_bcxr, lb.vz_bcxr],
                          [lb.vx_bcyl, lb.vy_bcyl, lb.vz_bcyl], [lb.vx_bcyr, lb.vy_bcyr, lb.vz_bcyr],
                          [lb.vx_bczl, lb.vy_bczl, lb.vz_bczl], [lb.vx_bczr, lb.vy_bczr, lb.vz_bczr]])
    return out, params


def case_sp(cls, name, shape, solid, setup, steps_list):
    t0 = time.time()
    out, params = run_class(cls, shape, solid, setup, steps_list)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), solid=solid.astype(np.int8),
                        shape=np.array(shape), steps=np.array(steps_list),
                        params=json.dumps(params), kind="single_phase_class", **out)
    print("%-22s %6.1fs  %s" % (name, time.time() - t0, params["bc"]))


def gen_single_phase(ref, only):
    cls = load_class(ref)

    def want(n):
        return not only or n in only

    if want("sp_cavity8"):
        def s(lb):
            lb.set_viscosity(0.1)
            lb.set_bc_vel_z1([0.1, 0.0, 0.0])
        case_sp(cls, "sp_cavity8", (8, 8, 8), cavity_shell(8), s, [1, 5, 20])

    if want("sp_poiseuille"):
        g = np.zeros((4, 10, 8), dtype=np.int8)
        g[:, :, 0] = 1
        g[:, :, -1] = 1

        def s(lb):
            lb.set_force([0.0, 1e-4, 0.0])
            lb.set_viscosity(0.1667)
        case_sp(cls, "sp_poiseuille", (4, 10, 8), g, s, [1, 20])

    if want("sp_pressure"):
        g = spheres_mask((10, 8, 8), 4, 1.5, 3.0, seed=11)

        def s(lb):
            lb.set_viscosity(0.1)
            lb.set_bc_rho_x0(1.005)
            lb.set_bc_rho_x1(1.0)
        case_sp(cls, "sp_pressure", (10, 8, 8), g, s, [1, 20])

    if want("sp_mixed"):
        g = spheres_mask((8, 7, 6), 3, 1.0, 2.2, seed=12)

        def s(lb):
            lb.set_viscosity(0.05)
            lb.set_force([2e-5, -1e-5, 3e-5])
            lb.set_bc_rho_x0(1.002)
            lb.set_bc_vel_x1([0.01, 0.0, 0.005])
            lb.set_bc_vel_y0([0.0, 0.02, 0.01])
            lb.set_bc_rho_y1(0.998)
            lb.set_bc_vel_z0([0.015, -0.01, 0.0])
            lb.set_bc_rho_z1(1.001)
        case_sp(cls, "sp_mixed", (8, 7, 6), g, s, [1, 10])

    if want("sp_stream"):
        # pure streaming permutation: one streaming1() sweep on random f
        shape = (7, 6, 5)
        g = spheres_mask(shape, 3, 1.0, 2.0, seed=13)
        lb = cls(*shape, False)
        lb.solid.from_numpy(g)
        lb.init_simulation()
        rng = np.random.default_rng(14)
        f0 = rng.standard_normal(shape + (19,)).astype(np.float32)
        lb.f.from_numpy(f0)
        lb.F.from_numpy(np.full(shape + (19,), np.nan, dtype=np.float32))
        lb.streaming1()
        Fo = lb.F.to_numpy()
        # neighbour table exactly as periodic_index computes it (all cells, 19 dirs)
        e = lb.e.to_numpy()
        nbr = np.zeros(shape + (19, 3), dtype=np.int32)
        for i in range(shape[0]):
            for j in range(shape[1]):
                for k in range(shape[2]):
                    for q in range(19):
                        ip = lb.periodic_index(taichi_numpy_shim._make_vec([i, j, k], np.int32) + lb.e[q])
                        nbr[i, j, k, q] = np.asarray(ip)
        np.savez_compressed(os.path.join(HERE, "sp_stream.npz"), solid=g, shape=np.array(shape),
                            f_in=f0, F_out=Fo, nbr=nbr, e=e, kind="stream")
        print("sp_stream done")

    if want("sp_cavity50"):
        path = os.path.join(ref, "Single_phase", "geo_cavity.dat")
        lb = cls(50, 50, 50, False)
        lb.init_geo(path)
        solid = lb.solid.to_numpy().astype(np.int8)

        def s(lb2):
            lb2.set_bc_vel_x1([0.0, 0.0, 0.1])
        t0 = time.time()
        out, params = run_class(cls, (50, 50, 50), solid, s, [1])
        np.savez_compressed(os.path.join(HERE, "sp_cavity50.npz"),
                            solid_bits=np.packbits(solid.ravel(order="F")),
                            n_solid=np.int64(solid.sum()), shape=np.array((50, 50, 50)),
                            steps=np.array([1]), params=json.dumps(params),
                            kind="single_phase_class", **out)
        print("sp_cavity50 %.1fs" % (time.time() - t0))


# --------------------------------------------------------- two-phase script
TP_FILE = os.path.join("2phase", "lbm_solver_3d_2phase_sparse.py")


def load_two_phase(ref, p):
    src = open(os.path.join(ref, TP_FILE)).read()
    src = src.split("time_init = time.time()")[0]
    sub = {
        "nx,ny,nz = 131,131,131\n": "nx,ny,nz = %d,%d,%d\n" % tuple(p["shape"]),
        "fx,fy,fz = 5.0e-5,0.0,0.0\n": "fx,fy,fz = %r,%r,%r\n" % tuple(p["force"]),
        "niu_l = 0.1         #psi>0\n": "niu_l = %r\n" % p["niu_l"],
        "niu_g = 0.1         #psi<0\n": "niu_g = %r\n" % p["niu_g"],
        "psi_solid = 0.7\n": "psi_solid = %r\n" % p["psi_solid"],
        "CapA = 0.005\n": "CapA = %r\n" % p["CapA"],
    }
    faces = ["x_left", "x_right", "y_left", "y_right", "z_left", "z_right"]
    short = ["xl", "xr", "yl", "yr", "zl", "zr"]
    for line in src.splitlines(keepends=True):
        for fi, (fc, sh) in enumerate(zip(faces, short)):
            if line.startswith("bc_%s, rho_bc%s" % (fc, sh)):
                v = p["vel_bc"][fi]
                sub[line] = "bc_%s, rho_bc%s, vx_bc%s, vy_bc%s, vz_bc%s = %d, %r, %r, %r, %r\n" % (
                    fc, sh, sh, sh, sh, p["bc"][fi], p["rho_bc"][fi], v[0], v[1], v[2])
            if line.startswith("bc_psi_%s, psi_%s" % (fc, fc)):
                sub[line] = "bc_psi_%s, psi_%s = %d, %r\n" % (fc, fc, p["psi_bc"][fi], p["psi_val"][fi])
    lines = src.splitlines(keepends=True)
    for a, b in sub.items():
        hits = [n for n, ln in enumerate(lines) if ln == a]
        assert len(hits) == 1, a
        lines[hits[0]] = b
    src = "".join(lines)
    g = {"__name__": "ref_lbm_2phase"}
    exec(compile(src, os.path.join(ref, TP_FILE), "exec"), g)
    return g


def case_tp(ref, name, p, solid, psi0, steps_list):
    t0 = time.time()
    g = load_two_phase(ref, p)
    g["solid"].from_numpy(solid)
    g["psi"].from_numpy(psi0)
    g["static_init"]()
    g["init"]()
    out = {}
    done = 0
    nx, ny, nz = p["shape"]
    for st in steps_list:
        while done < st:
            g["colission"]()
            g["streaming1"]()
            g["Boundary_condition"]()
            g["streaming3"]()
            g["Boundary_condition_psi"]()
            done += 1
        out["rho_%d" % st] = g["rho"].to_numpy()[:nx, :ny, :nz].astype(np.float32)
        out["v_%d" % st] = g["v"].to_numpy()[:nx, :ny, :nz].astype(np.float32)
        out["psi_%d" % st] = g["psi"].to_numpy()[:nx, :ny, :nz].astype(np.float32)
        out["rho_r_%d" % st] = g["rho_r"].to_numpy()[:nx, :ny, :nz].astype(np.float32)
        out["rho_b_%d" % st] = g["rho_b"].to_numpy()[:nx, :ny, :nz].astype(np.float32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), solid=solid.astype(np.int8),
                        psi0=psi0.astype(np.float32), shape=np.array(p["shape"]),
                        steps=np.array(steps_list), params=json.dumps(p), kind="two_phase_script", **out)
    print("%-22s %6.1fs" % (name, time.time() - t0))


def tp_params(shape, **kw):
    p = dict(shape=list(shape), force=[0.0, 0.0, 0.0], niu_l=0.05, niu_g=0.2, psi_solid=0.7, CapA=0.005,
             bc=[0] * 6, rho_bc=[1.0] * 6, vel_bc=[[0.0, 0.0, 0.0]] * 6, psi_bc=[0] * 6, psi_val=[1.0] * 6)
    p.update(kw)
    return p


def gen_two_phase(ref, only):
    def want(n):
        return not only or n in only

    if want("tp_drain"):
        shape = (12, 8, 8)
        solid = spheres_mask(shape, 4, 1.2, 2.5, seed=21)
        psi0 = -np.ones(shape, dtype=np.float32)
        psi0[:3] = 1.0
        p = tp_params(shape, bc=[1, 1, 0, 0, 0, 0], rho_bc=[1.001, 1.0, 1.0, 1.0, 1.0, 1.0],
                      psi_bc=[1, 1, 0, 0, 0, 0], psi_val=[1.0, -1.0, 1.0, 1.0, 1.0, 1.0])
        case_tp(ref, "tp_drain", p, solid, psi0, [1, 8])

    if want("tp_periodic"):
        shape = (10, 8, 8)
        solid = spheres_mask(shape, 3, 1.0, 2.0, seed=22)
        X, Y, Z = np.meshgrid(np.arange(10), np.arange(8), np.arange(8), indexing="ij")
        psi0 = np.where((X - 5) ** 2 + (Y - 4) ** 2 + (Z - 4) ** 2 < 7, 1.0, -1.0).astype(np.float32)
        p = tp_params(shape, force=[5e-5, -2e-5, 0.0], niu_l=0.1, niu_g=0.1)
        case_tp(ref, "tp_periodic", p, solid, psi0, [1, 8])

    if want("tp_velbc"):
        shape = (8, 6, 7)
        solid = spheres_mask(shape, 2, 1.0, 1.8, seed=23)
        psi0 = np.where(np.arange(8)[:, None, None] < 4, 1.0, -1.0) * np.ones(shape)
        p = tp_params(shape, bc=[1, 2, 2, 0, 2, 1], rho_bc=[1.002, 1.0, 1.0, 1.0, 1.0, 0.999],
                      psi_bc=[1, 0, 0, 0, 1, 0], psi_val=[1.0, 1.0, 1.0, 1.0, -1.0, 1.0])
        case_tp(ref, "tp_velbc", p, solid, psi0.astype(np.float32), [1, 6])


# ------------------------------------------------------- grey-scale script
GREY_FILE = os.path.join("Grey_Scale", "lbm_solver_3d_Macro_Sukop.py")


def load_grey(ref, p):
    """The grey-scale script with its parameter lines set to ``p`` and cut
    before its main loop (``time_init = time.time()``)."""
    src = open(os.path.join(ref, GREY_FILE)).read()
    src = src.split("time_init = time.time()")[0]
    sub = {
        "nx,ny,nz = 60,50,5\n": "nx,ny,nz = %d,%d,%d\n" % tuple(p["shape"]),
        "fx,fy,fz = 1.0e-6,0.0,0.0\n": "fx,fy,fz = %r,%r,%r\n" % tuple(p["force"]),
        "niu = 0.1\n": "niu = %r\n" % p["niu"],
    }
    faces = ["x_left", "x_right", "y_left", "y_right", "z_left", "z_right"]
    short = ["xl", "xr", "yl", "yr", "zl", "zr"]
    lines = src.splitlines(keepends=True)
    for line in lines:
        for fi, (fc, sh) in enumerate(zip(faces, short)):
            if line.startswith("bc_%s, rho_bc%s" % (fc, sh)):
                v = p["vel_bc"][fi]
                sub[line] = "bc_%s, rho_bc%s, vx_bc%s, vy_bc%s, vz_bc%s = %d, %r, %r, %r, %r\n" % (
                    fc, sh, sh, sh, sh, p["bc"][fi], p["rho_bc"][fi], v[0], v[1], v[2])
    for a, b in sub.items():
        hits = [n for n, ln in enumerate(lines) if ln == a]
        assert len(hits) == 1, a
        lines[hits[0]] = b
    g = {"__name__": "ref_lbm_grey"}
    exec(compile("".join(lines), os.path.join(ref, GREY_FILE), "exec"), g)
    return g


def case_grey(ref, name, p, ns, steps_list):
    """Run the script's main-loop body (:330-336) and store rho, v after each
    listed step count.  solid = ns.astype(int) as the script does (:321)."""
    t0 = time.time()
    g = load_grey(ref, p)
    g["solid"].from_numpy(ns.astype(int))
    g["ns"].from_numpy(ns)
    g["static_init"]()
    g["init"]()
    out = {}
    done = 0
    for st in steps_list:
        while done < st:
            g["colission"]()
            g["streaming0"]()
            g["streaming1"]()
            g["Boundary_condition"]()
            g["streaming3"]()
            done += 1
        out["rho_%d" % st] = g["rho"].to_numpy().astype(np.float32)
        out["v_%d" % st] = g["v"].to_numpy().astype(np.float32)
        out["F_%d" % st] = g["F"].to_numpy().astype(np.float32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), ns=ns.astype(np.float64), shape=np.array(p["shape"]),
                        steps=np.array(steps_list), params=json.dumps(p), kind="grey_script", **out)
    print("%-22s %6.1fs" % (name, time.time() - t0))


def grey_params(shape, **kw):
    p = dict(shape=list(shape), force=[0.0, 0.0, 0.0], niu=0.1, bc=[0] * 6, rho_bc=[1.0] * 6,
             vel_bc=[[0.0, 0.0, 0.0]] * 6)
    p.update(kw)
    return p


def gen_grey(ref, only):
    def want(n):
        return not only or n in only

    if want("grey_channel"):
        # channel: ns = 1 walls at y = 0 and y = ny-1, a grey (ns = 0.2) layer
        # along the lower wall, open fluid above; body force along x
        shape = (12, 10, 4)
        ns = np.zeros(shape)
        ns[:, 0, :] = ns[:, -1, :] = 1.0
        ns[:, 1:4, :] = 0.2
        case_grey(ref, "grey_channel", grey_params(shape, force=[1e-4, 0.0, 0.0]), ns, [1, 10])

    if want("grey_mixed"):
        # seeded random ns in {0, 0.1, 0.2, 0.5, 1}, oblique body force
        shape = (9, 8, 6)
        rng = np.random.default_rng(31)
        ns = rng.choice([0.0, 0.0, 0.0, 0.1, 0.2, 0.5, 1.0], size=shape)
        case_grey(ref, "grey_mixed", grey_params(shape, force=[2e-5, -1e-5, 5e-6]), ns, [1, 8])

    if want("grey_faces"):
        # x faces: velocity (in-place form) on the left, pressure on the right;
        # walls at y = 0 / y = ny-1 reach the faces, so face cells have solid
        # upstream neighbours
        shape = (10, 7, 5)
        rng = np.random.default_rng(32)
        ns = rng.choice([0.0, 0.0, 0.3, 1.0], size=shape, p=[0.5, 0.2, 0.2, 0.1])
        ns[:, 0, :] = ns[:, -1, :] = 1.0
        p = grey_params(shape, bc=[2, 1, 0, 0, 0, 0], rho_bc=[1.0, 0.998, 1.0, 1.0, 1.0, 1.0])
        case_grey(ref, "grey_faces", p, ns, [1, 6])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("TAICHI_LBM3D_REF"),
                    help="root of the reference checkout (or set TAICHI_LBM3D_REF)")
    ap.add_argument("--only", nargs="*", default=[])
    a = ap.parse_args()
    if not a.ref:
        ap.error("give the reference checkout with --ref PATH or TAICHI_LBM3D_REF")
    gen_single_phase(a.ref, a.only)
    gen_two_phase(a.ref, a.only)
    gen_grey(a.ref, a.only)


if __name__ == "__main__":
    main()

"""STL surface mesh -> voxel solid geometry on the GPU.

Replaces the reference's only native tool, Single_phase/Convert_stl_to_binary.cpp:
it reads an STL, forms the grid points (x0 + dx i, y0 + dx j, z0 + dx k) of the
box [x0, x1) x [y0, y1) x [z0, z1) with n = ceil((x1 - x0) / dx) points per axis
(:43-60, :86-93), flags each point solid when it is inside the surface or on it
(:117-123), and writes the flags as a legacy VTK STRUCTURED_POINTS file
(:127-150) and the mesh as OBJ (:80).  The classification runs in
csrc/vox.cu (exact generalized winding number, one GPU thread per point); the
reference's libigl dependency is not needed.

    python -m taichi_lbm3d_gb300.voxelize mesh.stl --lo -10 -5 -15 --hi 50 5 15 --dx 0.5 \\
        --vtk binary_geometry_check.vtk --geo geo.dat

The defaults of ``--lo/--hi/--dx`` are the reference's hard-coded box.  ``--geo``
also writes the flags as the 0/1 ASCII file ``init_geo`` reads (x fastest).
"""
import argparse
import ctypes
import math
import os
import struct
import sys

import numpy as np

from . import _native

REF_LO = (-10.0, -5.0, -15.0)
REF_HI = (50.0, 5.0, 15.0)
REF_DX = 0.5

_bound = False


def _lib():
    global _bound
    L = _native.load()
    if not _bound:
        L.lbm_voxelize.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_float, ctypes.c_int32,
                                   ctypes.c_int32, ctypes.c_int32, ctypes.c_float, ctypes.c_int32, ctypes.c_void_p,
                                   ctypes.c_void_p]
        L.lbm_voxelize.restype = ctypes.c_int
        _bound = True
    return L


# ------------------------------------------------------------------ STL I/O
def read_stl(filename):
    """Triangles (n, 3, 3) float32 from a binary or ASCII STL file."""
    with open(filename, "rb") as fh:
        data = fh.read()
    if len(data) >= 84:
        n = struct.unpack_from("<I", data, 80)[0]
        if len(data) == 84 + 50 * n:
            rec = np.frombuffer(data, dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", 9), ("a", "<u2")]), count=n,
                                offset=84)
            return np.ascontiguousarray(rec["v"].reshape(n, 3, 3))
    words = data.split()
    verts = [i for i, w in enumerate(words) if w == b"vertex"]
    if not verts or len(verts) % 3:
        raise ValueError("%s: not a binary STL and no ASCII facets found" % filename)
    idx = np.array(verts)[:, None] + np.arange(1, 4)[None, :]
    v = np.array([float(words[i]) for i in idx.ravel()], dtype=np.float32)
    return v.reshape(-1, 3, 3)


def write_stl(filename, tris, ascii=False):
    tris = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
    n = np.cross(b - a, c - a)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    if ascii:
        with open(filename, "w") as fh:
            fh.write("solid mesh\n")
            for t, nn in zip(tris, n):
                fh.write("  facet normal %.9g %.9g %.9g\n    outer loop\n" % tuple(nn))
                for v in t:
                    fh.write("      vertex %.9g %.9g %.9g\n" % tuple(v))
                fh.write("    endloop\n  endfacet\n")
            fh.write("endsolid mesh\n")
        return
    rec = np.zeros(len(tris), dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", 9), ("a", "<u2")]))
    rec["n"] = n
    rec["v"] = tris.reshape(-1, 9)
    with open(filename, "wb") as fh:
        fh.write(b"taichi_lbm3d_gb300 binary STL".ljust(80, b" "))
        fh.write(struct.pack("<I", len(tris)))
        fh.write(rec.tobytes())


def write_obj(filename, tris):
    """Mesh as OBJ (shared vertices merged), like the reference's check file (:80)."""
    tris = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    uniq, inv = np.unique(tris.reshape(-1, 3), axis=0, return_inverse=True)
    with open(filename, "w") as fh:
        for v in uniq:
            fh.write("v %.9g %.9g %.9g\n" % tuple(v))
        for f in inv.reshape(-1, 3) + 1:
            fh.write("f %d %d %d\n" % tuple(f))


# ------------------------------------------------------------ voxelisation
def grid_dims(lo, hi, dx):
    """Points per axis, ceil((hi - lo) / dx) in FP32 as the reference computes it (:57-60)."""
    f = np.float32
    return tuple(int(math.ceil(f(f(h) - f(l)) / f(dx))) for l, h in zip(lo, hi))


def voxelize(tris, lo=REF_LO, hi=REF_HI, dx=REF_DX, surf_eps=-1.0, device=0, dims=None, with_winding=False):
    """Solid flags (nx, ny, nz) int8 of the box's grid points (1 inside or on
    the surface); with ``with_winding`` also the winding numbers."""
    t = np.ascontiguousarray(np.asarray(tris, np.float32).reshape(-1, 9))
    nx, ny, nz = dims if dims is not None else grid_dims(lo, hi, dx)
    origin = np.ascontiguousarray(np.asarray(lo, np.float32))
    solid = np.empty(nx * ny * nz, np.int8)
    w = np.empty(nx * ny * nz, np.float64) if with_winding else None
    rc = _lib().lbm_voxelize(t.ctypes.data if t.size else None, t.shape[0], origin.ctypes.data, float(dx), nx, ny, nz,
                             float(surf_eps), int(device), solid.ctypes.data, w.ctypes.data if w is not None else None)
    _native.check(rc)
    solid = solid.reshape((nx, ny, nz), order="F")
    if with_winding:
        return solid, w.reshape((nx, ny, nz), order="F")
    return solid


def write_vtk_structured_points(filename, flags, title="taichi_lbm3d_gb300 voxelised solid geometry"):
    """Legacy ASCII VTK STRUCTURED_POINTS of the flags, x fastest (the
    reference's output layout, :127-150)."""
    nx, ny, nz = flags.shape
    with open(filename, "w") as fh:
        fh.write("# vtk DataFile Version 2.0\n%s\nASCII\nDATASET STRUCTURED_POINTS\n" % title)
        fh.write("DIMENSIONS %d %d %d\nORIGIN 0 0 0\nSPACING 1 1 1\n" % (nx, ny, nz))
        fh.write("POINT_DATA %d\nSCALARS sample_scalars float\nLOOKUP_TABLE default\n" % (nx * ny * nz))
        vals = np.asarray(flags).ravel(order="F").astype(np.int64)
        fh.write(" ".join(map(str, vals.tolist())))
        fh.write(" \n")


def read_vtk_structured_points(filename):
    with open(filename) as fh:
        lines = fh.read().split("\n")
    dims = None
    for n, ln in enumerate(lines):
        if ln.startswith("DIMENSIONS"):
            dims = tuple(int(x) for x in ln.split()[1:4])
        if ln.startswith("LOOKUP_TABLE"):
            vals = np.array(" ".join(lines[n + 1:]).split(), dtype=np.float64)
            return vals.reshape(dims, order="F")
    raise ValueError("%s: no point data" % filename)


# ------------------------------------------------------------ test meshes
def _orient_outward(tris):
    """Flip all triangles if the enclosed signed volume is negative."""
    a, b, c = tris[:, 0].astype(np.float64), tris[:, 1].astype(np.float64), tris[:, 2].astype(np.float64)
    vol = np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0
    return tris if vol >= 0 else tris[:, ::-1].copy()


def box_mesh(lo, hi):
    """Closed axis-aligned box, 12 triangles."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    P = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float64)
    quads = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5), (0, 4, 7, 3)]
    tris = []
    for a, b, c, d in quads:
        tris += [(P[a], P[b], P[c]), (P[a], P[c], P[d])]
    return _orient_outward(np.array(tris, np.float32))


def icosphere(center, radius, subdiv=3):
    """Subdivided icosahedron projected on the sphere (20 * 4^subdiv triangles)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    V = [np.array(v, np.float64) / np.linalg.norm(v) for v in V]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                cache[key] = len(V) - 1
            return cache[key]

        F2 = []
        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            F2 += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = F2
    Vs = np.array(V) * radius + np.asarray(center, np.float64)
    return _orient_outward(Vs[np.array(F)].astype(np.float32))


def torus(center, R, r, nu=48, nv=24):
    """Torus around the z axis (major radius R, minor r)."""
    u = np.linspace(0, 2 * np.pi, nu, endpoint=False)
    v = np.linspace(0, 2 * np.pi, nv, endpoint=False)

    def P(i, j):
        uu, vv = u[i % nu], v[j % nv]
        return np.array([(R + r * np.cos(vv)) * np.cos(uu), (R + r * np.cos(vv)) * np.sin(uu), r * np.sin(vv)])

    tris = []
    for i in range(nu):
        for j in range(nv):
            a, b, c, d = P(i, j), P(i + 1, j), P(i + 1, j + 1), P(i, j + 1)
            tris += [(a, b, c), (a, c, d)]
    return _orient_outward((np.array(tris) + np.asarray(center, np.float64)).astype(np.float32))


def naca4_wing(code="0012", chord=40.0, span=20.0, n=80, x0=0.0, z0=-10.0):
    """Closed extruded NACA 4-digit wing: section in x-y (leading edge at x0),
    span along z from z0.  Published NACA 4-digit thickness and camber
    equations, closed trailing edge (last coefficient -0.1036), cosine spacing."""
    m, p, t = int(code[0]) / 100.0, int(code[1]) / 10.0, int(code[2:]) / 100.0
    beta = np.linspace(0, np.pi, n)
    x = 0.5 * (1 - np.cos(beta))
    yt = 5 * t * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x ** 2 + 0.2843 * x ** 3 - 0.1036 * x ** 4)
    if m > 0 and p > 0:
        yc = np.where(x < p, m / p ** 2 * (2 * p * x - x ** 2), m / (1 - p) ** 2 * ((1 - 2 * p) + 2 * p * x - x ** 2))
        dyc = np.where(x < p, 2 * m / p ** 2 * (p - x), 2 * m / (1 - p) ** 2 * (p - x))
    else:
        yc = np.zeros_like(x)
        dyc = np.zeros_like(x)
    th = np.arctan(dyc)
    xu, yu = x - yt * np.sin(th), yc + yt * np.cos(th)
    xl, yl = x + yt * np.sin(th), yc - yt * np.cos(th)
    up = np.stack([x0 + chord * xu, chord * yu], 1)
    lo = np.stack([x0 + chord * xl, chord * yl], 1)
    lo[0] = up[0]
    lo[-1] = up[-1]
    z1 = z0 + span
    tris = []
    # outline: upper from LE to TE, lower back from TE to LE
    ring = np.concatenate([up, lo[-2:0:-1]])
    for a in range(len(ring)):
        p0, p1 = ring[a], ring[(a + 1) % len(ring)]
        A, B = np.array([p0[0], p0[1], z0]), np.array([p1[0], p1[1], z0])
        C, D = np.array([p1[0], p1[1], z1]), np.array([p0[0], p0[1], z1])
        tris += [(A, B, C), (A, C, D)]
    # end caps: strips between upper and lower surface at matching stations
    for zc, flip in ((z0, False), (z1, True)):
        for a in range(n - 1):
            U0, U1 = np.array([*up[a], zc]), np.array([*up[a + 1], zc])
            L0, L1 = np.array([*lo[a], zc]), np.array([*lo[a + 1], zc])
            for tri in ((U0, L0, U1), (L0, L1, U1)):
                if np.linalg.norm(np.cross(tri[1] - tri[0], tri[2] - tri[0])) == 0:
                    continue
                tris.append(tri[::-1] if flip else tri)
    tris = np.array(tris, np.float64)
    # the side strip and the caps are built with a fixed winding; make the caps agree with the sides
    return _fix_orientation(tris).astype(np.float32)


def _fix_orientation(tris):
    """Orient every triangle consistently with its neighbours (edge-sharing
    propagation), then outward."""
    key = lambda p: tuple(np.round(p, 9))
    edges = {}
    for t, tri in enumerate(tris):
        for e in range(3):
            a, b = key(tri[e]), key(tri[(e + 1) % 3])
            edges.setdefault((min(a, b), max(a, b)), []).append(t)
    flip = np.full(len(tris), -1)
    for seed in range(len(tris)):
        if flip[seed] >= 0:
            continue
        flip[seed] = 0
        stack = [seed]
        while stack:
            t = stack.pop()
            tri = tris[t] if not flip[t] else tris[t][::-1]
            for e in range(3):
                a, b = key(tri[e]), key(tri[(e + 1) % 3])
                for u in edges[(min(a, b), max(a, b))]:
                    if u == t or flip[u] >= 0:
                        continue
                    tu = tris[u]
                    same = any(key(tu[f]) == a and key(tu[(f + 1) % 3]) == b for f in range(3))
                    flip[u] = 1 if same else 0
                    stack.append(u)
    out = np.array([tr[::-1] if f else tr for tr, f in zip(tris, flip)])
    return _orient_outward(out)


def is_closed(tris):
    """Every edge shared by exactly two triangles with opposite directions."""
    key = lambda p: tuple(np.round(np.asarray(p, np.float64), 6))
    count = {}
    for tri in np.asarray(tris):
        for e in range(3):
            a, b = key(tri[e]), key(tri[(e + 1) % 3])
            count[(a, b)] = count.get((a, b), 0) + 1
    return all(count.get((b, a), 0) == c == 1 for (a, b), c in count.items())


# -------------------------------------------------------------------- CLI
def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("stl")
    ap.add_argument("--lo", type=float, nargs=3, default=list(REF_LO))
    ap.add_argument("--hi", type=float, nargs=3, default=list(REF_HI))
    ap.add_argument("--dx", type=float, default=REF_DX)
    ap.add_argument("--vtk", default="binary_geometry_check.vtk")
    ap.add_argument("--obj", default=None, help="also write the mesh as OBJ")
    ap.add_argument("--geo", default=None, help="also write the 0/1 ASCII geometry file (x fastest)")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    tris = read_stl(a.stl)
    if a.obj:
        write_obj(a.obj, tris)
    dims = grid_dims(a.lo, a.hi, a.dx)
    print("Mesh size: %d X %d X %d (%d triangles)" % (dims + (len(tris),)))
    solid = voxelize(tris, a.lo, a.hi, a.dx, device=a.device)
    write_vtk_structured_points(a.vtk, solid)
    if a.geo:
        from .geometry import write_ascii_geometry
        write_ascii_geometry(a.geo, solid)
    print("solid fraction %.4f -> %s" % (solid.mean(), os.path.abspath(a.vtk)))
    return 0


if __name__ == "__main__":
    sys.exit(main())

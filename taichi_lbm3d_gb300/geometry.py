"""Geometry input/output and the seeded synthetic porous media.

* ``read_ascii_geometry`` / ``read_ascii_field``: the reference's ASCII voxel
  format (one value per line, x fastest; ``init_geo``,
  Single_phase/LBM_3D_SinglePhase_Solver.py:173-177; psi files,
  2phase/lbm_solver_3d_2phase_sparse.py:195-203).  Values > 0 are solid.
* ``sphere_pack``: overlapping spheres, centres uniform over the (periodic) box,
  radii uniform in [rmin, rmax], added one at a time until the fluid fraction
  is <= the target porosity; then fluid not connected to both x faces is made
  solid (6-connected; periodic in y and z).  numpy.random.default_rng(seed)
  drives it, so a seed always gives the same mask.
* ``distance_to_solid``: exact Euclidean distance of each fluid cell to the
  nearest solid cell (input channel of the warm-start network).
"""
import numpy as np


def read_ascii_geometry(filename, shape):
    """Solid mask (int8, shape (nx,ny,nz)) from an ASCII 0/1 file, x fastest."""
    n = int(np.prod(shape))
    vals = _read_numbers(filename, n)
    if vals.size != n:
        raise ValueError("%s holds %d values, lattice %s needs %d" % (filename, vals.size, shape, n))
    solid = (vals > 0).astype(np.int8)
    return solid.reshape(shape, order="F")


def read_ascii_field(filename, shape, dtype=np.float32):
    """Field of the lattice shape from an ASCII file, x fastest (float32 unless
    ``dtype`` says otherwise; np.loadtxt's float64 for the grey-scale ns)."""
    n = int(np.prod(shape))
    vals = _read_numbers(filename, n)
    if vals.size != n:
        raise ValueError("%s holds %d values, lattice %s needs %d" % (filename, vals.size, shape, n))
    return vals.astype(dtype).reshape(shape, order="F")


def write_ascii_geometry(filename, solid, fmt="%d"):
    a = np.asarray(solid).ravel(order="F")
    np.savetxt(filename, a, fmt=fmt)


def _read_numbers(filename, n=None):
    """All numbers of the file, as np.loadtxt would read them (float64): the
    library's parallel parser (lbm_read_ascii) when it is built, else numpy.
    Reading is host work; no GPU is involved either way.  With n given, a file
    holding another count raises ValueError."""
    from . import _native
    try:
        return _native.read_ascii(filename, n)
    except _native.LbmError as e:
        if e.code != _native.LBM_ENODEV:      # the file itself is bad
            raise ValueError(str(e)) from None
    except OSError:                           # library present but not loadable here
        pass
    with open(filename, "rb") as fh:
        data = fh.read()
    return np.array(data.split(), dtype=np.float64)


def sphere_pack(shape, rmin, rmax, porosity, seed, percolate=True, max_spheres=10_000_000):
    """Seeded overlapping-sphere pack; returns int8 solid mask (1 = solid)."""
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    solid = np.zeros(shape, dtype=np.int8)
    ncell = nx * ny * nz
    n_solid = 0
    target_solid = int(np.ceil((1.0 - porosity) * ncell))
    for _ in range(max_spheres):
        if n_solid >= target_solid:
            break
        c = rng.uniform(0.0, 1.0, 3) * np.array([nx, ny, nz])
        r = rng.uniform(rmin, rmax)
        lo = np.floor(c - r).astype(int)
        hi = np.ceil(c + r).astype(int)
        xs = np.arange(lo[0], hi[0] + 1)
        ys = np.arange(lo[1], hi[1] + 1)
        zs = np.arange(lo[2], hi[2] + 1)
        dx2 = (xs - c[0]) ** 2
        dy2 = (ys - c[1]) ** 2
        dz2 = (zs - c[2]) ** 2
        inside = (dx2[:, None, None] + dy2[None, :, None] + dz2[None, None, :]) <= r * r
        ix = np.mod(xs, nx)[:, None, None]
        iy = np.mod(ys, ny)[None, :, None]
        iz = np.mod(zs, nz)[None, None, :]
        ixb, iyb, izb = np.broadcast_arrays(ix, iy, iz)
        sel = (ixb[inside], iyb[inside], izb[inside])
        if np.all(hi - lo + 1 <= np.array(shape)):
            n_solid += int(sel[0].size - solid[sel].sum())   # wrapped indices are distinct
            solid[sel] = 1
        else:                                                  # sphere wider than the box
            solid[sel] = 1
            n_solid = int(solid.sum())
    if percolate:
        solid = percolating(solid)
    return solid


def percolating(solid):
    """Make solid every fluid cell not 6-connected to both x faces
    (connectivity wraps in y and z)."""
    from scipy import ndimage
    fluid = solid == 0
    lab, n = ndimage.label(fluid)
    if n == 0:
        return solid.copy()
    parent = np.arange(n + 1)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    def union_faces(a, b):
        m = (a > 0) & (b > 0)
        for p, q in set(zip(a[m].tolist(), b[m].tolist())):
            rp, rq = find(p), find(q)
            if rp != rq:
                parent[max(rp, rq)] = min(rp, rq)

    union_faces(lab[:, 0, :], lab[:, -1, :])   # periodic y
    union_faces(lab[:, :, 0], lab[:, :, -1])   # periodic z
    roots = np.array([find(a) for a in range(n + 1)])
    rl = roots[lab]
    left = set(np.unique(rl[0][fluid[0]]).tolist())
    right = set(np.unique(rl[-1][fluid[-1]]).tolist())
    keep = left & right
    keep.discard(0)
    keep_mask = np.isin(rl, np.array(sorted(keep), dtype=rl.dtype)) & fluid
    out = np.ones_like(solid)
    out[keep_mask] = 0
    return out


def distance_to_solid(solid):
    """Exact Euclidean distance (in cells) from each cell to the nearest solid
    cell; 0 at solid cells."""
    from scipy import ndimage
    return ndimage.distance_transform_edt(np.asarray(solid) == 0).astype(np.float32)


def cavity_shell(n, moving="z1"):
    """Lid-driven cavity: one-node solid shell on five faces, the ``moving``
    face left fluid for the velocity boundary condition."""
    s = np.ones((n, n, n), dtype=np.int8)
    s[1:-1, 1:-1, 1:-1] = 0
    ax = {"x": 0, "y": 1, "z": 2}[moving[0]]
    idx = [slice(1, -1)] * 3
    idx[ax] = -1 if moving[1] == "1" else 0
    s[tuple(idx)] = 0
    return s

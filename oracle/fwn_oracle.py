"""Fast winding number of a triangle soup (FP64, numpy): the approximation the
reference's voxeliser classifies with.

TEST INFRASTRUCTURE ONLY: tests/ are its callers.  Single_phase/Convert_stl_to_binary.cpp:117-123
(taichi_LBM3D tree) calls libigl's ``signed_distance_fast_winding_number`` (libigl is
not vendored in the reference and not installed here), which marks a point solid when
1 - 2|w| <= 0 with w the *fast* winding number of Barill, Dickson, Schmidt, Levin and
Jacobson, "Fast Winding Numbers for Soups and Clouds" (ACM TOG 37(4), 2018).  This
module restates that published algorithm; the tree it builds is its own (an octree of
triangle centroids), so its far-field errors follow the same bound as libigl's, not
libigl's exact values:

* a tree over the triangles; every node keeps its area-weighted centre p, its radius r
  (largest distance from p to a vertex of its triangles) and the first three moments of
  its area-weighted normals about p:  sum a n,  sum a (c - p) (x) n  and
  sum [a (c - p)(c - p)^T + (a/12) sum_i (v_i - c)(v_i - c)^T] (x) n  (c the centroid,
  v_i the vertices; the last term is the triangle's exact second moment);
* at a query q a node with |q - p| > beta r contributes the order-2 Taylor expansion of
  the dipole integral  w = int grad G(x) . n dA,  G(x) = -1 / (4 pi |x - q|),  about p;
  a nearer leaf contributes its triangles' exact solid angles (Van Oosterom & Strackee);
  a nearer inner node recurses.  beta = 2 is libigl's default accuracy scale.
"""
import numpy as np

FOUR_PI = 4.0 * np.pi


def solid_angles(tris, q):
    """Exact winding-number contributions of triangles (T,3,3) at points q (Q,3): (Q, T)."""
    a = tris[None, :, 0, :] - q[:, None, :]
    b = tris[None, :, 1, :] - q[:, None, :]
    c = tris[None, :, 2, :] - q[:, None, :]
    la, lb, lc = (np.linalg.norm(x, axis=-1) for x in (a, b, c))
    det = np.einsum("qti,qti->qt", a, np.cross(b, c))
    den = la * lb * lc + np.einsum("qti,qti->qt", a, b) * lc + np.einsum("qti,qti->qt", a, c) * lb + \
        np.einsum("qti,qti->qt", b, c) * la
    return 2.0 * np.arctan2(det, den) / FOUR_PI


class _Node:
    __slots__ = ("idx", "children", "p", "r", "m0", "m1", "m2")


def _build(tris, idx, lo, hi, leaf, depth):
    node = _Node()
    node.idx = idx
    t = tris[idx]
    cen = t.mean(axis=1)
    an = 0.5 * np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])         # area times unit normal
    area = np.linalg.norm(an, axis=1)
    w = area / area.sum() if area.sum() > 0 else np.full(len(idx), 1.0 / len(idx))
    p = (w[:, None] * cen).sum(axis=0)
    node.p = p
    node.r = float(np.linalg.norm(t - p, axis=2).max())
    d = cen - p
    node.m0 = an.sum(axis=0)
    node.m1 = np.einsum("tj,ti->ij", d, an)                            # [i][j] = sum n_i d_j
    cov = np.einsum("t,tj,tk->tjk", area, d, d)
    dv = t - cen[:, None, :]
    cov += (area / 12.0)[:, None, None] * np.einsum("tvj,tvk->tjk", dv, dv)
    node.m2 = np.einsum("tjk,ti->ijk", cov / np.maximum(area, 1e-300)[:, None, None], an)
    node.children = []
    if len(idx) > leaf and depth < 20:
        mid = 0.5 * (lo + hi)
        octant = ((cen[:, 0] > mid[0]).astype(int) | ((cen[:, 1] > mid[1]).astype(int) << 1) |
                  ((cen[:, 2] > mid[2]).astype(int) << 2))
        if len(np.unique(octant)) > 1:
            for o in range(8):
                sel = idx[octant == o]
                if len(sel):
                    clo = np.where([(o >> a) & 1 for a in range(3)], mid, lo)
                    chi = np.where([(o >> a) & 1 for a in range(3)], hi, mid)
                    node.children.append(_build(tris, sel, clo, chi, leaf, depth + 1))
    return node


def build_tree(tris, leaf=8):
    tris = np.asarray(tris, np.float64).reshape(-1, 3, 3)
    cen = tris.mean(axis=1)
    lo, hi = cen.min(axis=0) - 1e-9, cen.max(axis=0) + 1e-9
    return tris, _build(tris, np.arange(len(tris)), lo, hi, leaf, 0)


def _taylor(node, q):
    """Order-2 far-field contribution of a node at points q (Q,3)."""
    r = node.p[None, :] - q                                              # x - q at the expansion centre
    R2 = (r * r).sum(axis=1)
    R = np.sqrt(R2)
    inv3 = 1.0 / (R2 * R)
    inv5 = inv3 / R2
    inv7 = inv5 / R2
    # grad G, Hessian and third derivative of G(x) = -1/(4 pi |x - q|) at x = p
    g = r * inv3[:, None] / FOUR_PI
    w = g @ node.m0
    tr1 = np.trace(node.m1)
    rm1r = np.einsum("qi,ij,qj->q", r, node.m1, r)
    w += (tr1 * inv3 - 3.0 * rm1r * inv5) / FOUR_PI
    # T_ijk = [-3 (d_ij r_k + d_ik r_j + d_jk r_i) / R^5 + 15 r_i r_j r_k / R^7] / 4 pi, contracted with m2 / 2
    m2 = node.m2
    t1 = np.einsum("iik,qk->q", m2, r) + np.einsum("iji,qj->q", m2, r) + np.einsum("ijj,qi->q", m2, r)
    t2 = np.einsum("ijk,qi,qj,qk->q", m2, r, r, r)
    w += 0.5 * (-3.0 * t1 * inv5 + 15.0 * t2 * inv7) / FOUR_PI
    return w


def fast_winding_number(tree, q, beta=2.0):
    """Fast winding number of the soup at points q (Q,3)."""
    tris, root = tree
    q = np.asarray(q, np.float64).reshape(-1, 3)
    out = np.zeros(len(q))
    stack = [(root, np.arange(len(q)))]
    while stack:
        node, sel = stack.pop()
        if not len(sel):
            continue
        d = np.linalg.norm(q[sel] - node.p, axis=1)
        far = d > beta * node.r
        if far.any():
            out[sel[far]] += _taylor(node, q[sel[far]])
        near = sel[~far]
        if not len(near):
            continue
        if node.children:
            for ch in node.children:
                stack.append((ch, near))
        else:
            for a in range(0, len(near), 4096):
                part = near[a:a + 4096]
                out[part] += solid_angles(tris[node.idx], q[part]).sum(axis=1)
    return out


def grid_points(origin, dx, dims):
    """Grid points (x fastest), formed in FP32 as the reference does (:86-93)."""
    nx, ny, nz = dims
    o = np.asarray(origin, np.float32)
    i, j, k = np.meshgrid(np.arange(nx, dtype=np.float32), np.arange(ny, dtype=np.float32),
                          np.arange(nz, dtype=np.float32), indexing="ij")
    pts = np.stack([o[0] + np.float32(dx) * i, o[1] + np.float32(dx) * j, o[2] + np.float32(dx) * k], axis=-1)
    return pts.astype(np.float64)      # (nx, ny, nz, 3)

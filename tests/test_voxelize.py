"""Host side of the STL voxeliser: STL/VTK I/O, test meshes, and the FP64
oracle's classification on meshes with known insides (no GPU)."""
import numpy as np
import pytest

from oracle import oracle
from taichi_lbm3d_gb300 import voxelize as vx


@pytest.mark.parametrize("ascii", [False, True])
def test_stl_roundtrip(tmp_path, ascii):
    tris = vx.icosphere((1.0, -2.0, 0.5), 3.0, subdiv=1)
    path = str(tmp_path / "m.stl")
    vx.write_stl(path, tris, ascii=ascii)
    back = vx.read_stl(path)
    assert back.shape == tris.shape and back.dtype == np.float32
    assert np.array_equal(back, tris)


@pytest.mark.parametrize("mesh", ["box", "sphere", "torus", "naca0012", "naca2412"])
def test_meshes_closed_and_outward(mesh):
    tris = {"box": lambda: vx.box_mesh((0, 0, 0), (3, 2, 1)),
            "sphere": lambda: vx.icosphere((0, 0, 0), 5.0, 2),
            "torus": lambda: vx.torus((0, 0, 0), 6.0, 2.0),
            "naca0012": lambda: vx.naca4_wing("0012"),
            "naca2412": lambda: vx.naca4_wing("2412")}[mesh]()
    assert vx.is_closed(tris)
    a, b, c = (tris[:, q].astype(np.float64) for q in range(3))
    assert np.einsum("ij,ij->i", a, np.cross(b, c)).sum() > 0


def test_reference_box_dimensions():
    # Convert_stl_to_binary.cpp's box (-10..50, -5..5, -15..15) at dx = 0.5
    assert vx.grid_dims(vx.REF_LO, vx.REF_HI, vx.REF_DX) == (120, 20, 60)


def test_oracle_sphere_inside_outside():
    tris = vx.icosphere((0.1, -0.2, 0.3), 7.0, subdiv=3)
    origin, dx, dims = (-9.5, -9.5, -9.5), 1.0, (20, 20, 20)
    solid, w = oracle.voxelize(tris, origin, dx, dims)
    g = [origin[c] + dx * np.arange(dims[c]) for c in range(3)]
    X, Y, Z = np.meshgrid(*g, indexing="ij")
    r = np.sqrt((X - 0.1) ** 2 + (Y + 0.2) ** 2 + (Z - 0.3) ** 2)
    inner, outer = r < 6.8, r > 7.05          # the icosphere lies between 0.99 r and r
    assert np.all(solid[inner] == 1) and np.all(solid[outer] == 0)
    assert np.allclose(w[inner], 1.0, atol=1e-9) and np.allclose(w[outer], 0.0, atol=1e-9)


def test_oracle_points_on_faces_are_solid():
    # box faces on grid planes: face, edge and corner points count as solid
    tris = vx.box_mesh((2.0, 2.0, 2.0), (6.0, 5.0, 4.0))
    solid, w = oracle.voxelize(tris, (0.0, 0.0, 0.0), 1.0, (9, 8, 7))
    exp = np.zeros((9, 8, 7), np.int8)
    exp[2:7, 2:6, 2:5] = 1
    assert np.array_equal(solid, exp)


def test_oracle_torus_hole_is_fluid():
    tris = vx.torus((0, 0, 0), 6.0, 2.0, nu=64, nv=32)
    solid, _ = oracle.voxelize(tris, (-9.0, -9.0, -3.0), 1.0, (19, 19, 7))
    assert solid[9, 9, 3] == 0                      # centre of the hole
    assert solid[9 + 6, 9, 3] == 1                  # on the core circle
    assert solid[0, 0, 3] == 0


def test_vtk_structured_points_roundtrip(tmp_path):
    rng = np.random.default_rng(1)
    f = (rng.random((5, 4, 3)) < 0.4).astype(np.int8)
    path = str(tmp_path / "g.vtk")
    vx.write_vtk_structured_points(path, f)
    txt = open(path).read().split("\n")
    assert txt[0] == "# vtk DataFile Version 2.0" and txt[3] == "DATASET STRUCTURED_POINTS"
    assert "DIMENSIONS 5 4 3" in txt and "POINT_DATA 60" in txt
    assert np.array_equal(vx.read_vtk_structured_points(path), f)


def _fwn_vs_exact(tris, origin, dx, dims):
    from oracle import fwn_oracle as F
    tree = F.build_tree(tris)
    pts = F.grid_points(origin, dx, dims).reshape(-1, 3)
    wf = F.fast_winding_number(tree, pts).reshape(dims).ravel(order="F")
    _, w = oracle.voxelize(tris, origin, dx, dims)
    d = oracle.mesh_distance(tris, origin, dx, dims).reshape(-1, order="F")
    return wf, w.reshape(-1, order="F"), d


@pytest.mark.parametrize("mesh", ["sphere", "torus", "naca0012_reference_box"])
def test_fast_winding_number_matches_exact_classification(mesh):
    """The reference tool classifies with libigl's fast winding number (order-2
    far field, accuracy 2); restated in oracle/fwn_oracle.py it stays within a
    few 1e-3 of the exact winding number off the surface, and on these closed
    meshes, where the exact number is 0 or 1 off the surface, both rules mark the
    same grid points solid (points on a triangle are solid by the distance rule)."""
    tris, origin, dx, dims = {
        "sphere": (vx.icosphere((0.1, -0.2, 0.3), 7.0, subdiv=3), (-9.5, -9.5, -9.5), 1.0, (20, 20, 20)),
        "torus": (vx.torus((0, 0, 0), 6.0, 2.0), (-9.25, -9.25, -4.25), 0.5, (38, 38, 18)),
        "naca0012_reference_box": (vx.naca4_wing("0012"), vx.REF_LO, vx.REF_DX,
                                   vx.grid_dims(vx.REF_LO, vx.REF_HI, vx.REF_DX)),
    }[mesh]
    wf, w, d = _fwn_vs_exact(tris, origin, dx, dims)
    off = d > 1e-5 * dx
    err = np.abs(wf - w)[off]
    print("%s: max |w_fast - w| off the surface %.2e" % (mesh, err.max()))
    assert err.max() < 1e-2
    assert np.array_equal(np.abs(wf[off]) >= 0.5, np.abs(w[off]) >= 0.5)


def test_fast_winding_number_band_on_an_open_mesh():
    """A sphere with 4 triangles removed: the winding number is fractional near
    the hole, and the fast and exact classifications may differ only where the
    exact |w| lies within the fast method's error of 1/2 (the unpinned band)."""
    tris = vx.icosphere((0.1, -0.2, 0.3), 7.0, subdiv=3)
    top = np.argsort(tris[:, :, 2].mean(axis=1))[-4:]
    tris = np.delete(tris, top, axis=0)
    origin, dx, dims = (-9.5, -9.5, -9.5), 1.0, (20, 20, 20)
    wf, w, d = _fwn_vs_exact(tris, origin, dx, dims)
    off = d > 1e-5 * dx
    err = np.abs(wf - w)[off].max()
    differ = (np.abs(wf) >= 0.5) != (np.abs(w) >= 0.5)
    band = np.abs(np.abs(w) - 0.5) <= err
    assert ((w[off] > 0.02) & (w[off] < 0.98)).any()        # fractional winding numbers exist
    assert not (differ & off & ~band).any()

"""D3Q19 tables used by the product, checked against the reference's definitions
(LBM_3D_SinglePhase_Solver.py:64-85, :183-197)."""
import numpy as np

M_REF = np.array([
    [1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1],
    [-1, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1],
    [1, -2, -2, -2, -2, -2, -2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1],
    [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
    [0, -2, 2, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
    [0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1],
    [0, 0, 0, -2, 2, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1],
    [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1],
    [0, 0, 0, 0, 0, -2, 2, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1],
    [0, 2, 2, -1, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2],
    [0, -2, -2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2],
    [0, 0, 0, 1, 1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0],
    [0, 0, 0, -1, -1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, -1, 1, -1, 1, 0, 0, 0, 0],
    [0, 0, 0, 0, 0, 0, 0, -1, 1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1],
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, -1, 1, 1, -1]])


def test_moment_matrix_is_invertible():
    assert abs(np.linalg.det(M_REF)) > 1


def test_closed_form_guo_moments_match_the_dense_transform():
    """The deviation-form kernels add the Guo term's moments M (w o g) in
    closed form (csrc/lbm_kernels.cuh); they equal the dense product for any
    u, F and convention (gc, gd)."""
    from fractions import Fraction as Fr
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "taichi_lbm3d_gb300", "csrc"))
    import gen_mrt
    M = gen_mrt.M
    E = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (1, 1, 0), (-1, -1, 0),
         (1, -1, 0), (-1, 1, 0), (1, 0, 1), (-1, 0, -1), (1, 0, -1), (-1, 0, 1), (0, 1, 1), (0, -1, -1), (0, 1, -1),
         (0, -1, 1)]
    W = [Fr(1, 3)] + [Fr(1, 18)] * 6 + [Fr(1, 36)] * 12
    rng = np.random.default_rng(4)
    for gc, gd in ((Fr(1, 3), Fr(1, 9)), (Fr(1), Fr(1)), (Fr(3), Fr(9))):
        for _ in range(4):
            u = [Fr(int(x), 1000) for x in rng.integers(-50, 50, 3)]
            F = [Fr(int(x), 10 ** 6) for x in rng.integers(-9, 9, 3)]
            dot = lambda a, b: sum(x * y for x, y in zip(a, b))
            g = [gc * dot([e - v for e, v in zip(E[l], u)], F) + gd * dot(E[l], u) * dot(E[l], F) for l in range(19)]
            dense = [sum(M[r][l] * W[l] * g[l] for l in range(19)) for r in range(19)]
            uf = dot(u, F)
            closed = [Fr(0)] * 19
            closed[0] = (gd / 3 - gc) * uf
            closed[1] = Fr(2, 9) * gd * uf
            closed[3], closed[5], closed[7] = gc * F[0] / 3, gc * F[1] / 3, gc * F[2] / 3
            closed[9] = gd * (4 * u[0] * F[0] - 2 * u[1] * F[1] - 2 * u[2] * F[2]) / 9
            closed[11] = Fr(2, 9) * gd * (u[1] * F[1] - u[2] * F[2])
            closed[13] = gd * (u[0] * F[1] + u[1] * F[0]) / 9
            closed[14] = gd * (u[1] * F[2] + u[2] * F[1]) / 9
            closed[15] = gd * (u[0] * F[2] + u[2] * F[0]) / 9
            assert dense == closed


def test_class_exposes_the_reference_moment_matrices():
    """LB3D_Solver_Single_Phase.M / inv_M as the reference holds them: M in FP32
    and inv(M) computed in FP64, stored in FP32 (SP:61-110)."""
    from taichi_lbm3d_gb300 import LB3D_Solver_Single_Phase
    lb = LB3D_Solver_Single_Phase(4, 4, 4)
    assert lb.M.dtype == np.float32 and np.array_equal(lb.M, M_REF.astype(np.float32))
    assert lb.inv_M.dtype == np.float32
    assert np.array_equal(lb.inv_M, np.linalg.inv(M_REF.astype(np.float64)).astype(np.float32))

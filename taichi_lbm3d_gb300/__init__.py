"""GB300-native (sm_103a) D3Q19 MRT lattice Boltzmann hot path with the
solver-class API of taichi_LBM3D.

    from taichi_lbm3d_gb300 import LB3D_Solver_Single_Phase
    lb3d = LB3D_Solver_Single_Phase(64, 64, 64)
    lb3d.init_geo("geo.dat"); lb3d.set_bc_vel_z1([0.1, 0, 0])
    lb3d.init_simulation()
    for it in range(1000): lb3d.step()

All compute runs in liblbm_gb300.so (hand-written CUDA for sm_103a, called
through ctypes); there is no CPU fallback.
"""
from .solver import LB3D_Solver_Single_Phase  # noqa: F401
from .two_phase import LB3D_Solver_Two_Phase  # noqa: F401
from .grey import LB3D_Solver_Grey_Scale  # noqa: F401

__all__ = ["LB3D_Solver_Single_Phase", "LB3D_Solver_Two_Phase", "LB3D_Solver_Grey_Scale"]

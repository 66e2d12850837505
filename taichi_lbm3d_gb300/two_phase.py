"""Two-phase colour-gradient solver with the parameters of the reference's script
(2phase/lbm_solver_3d_2phase_sparse.py) as attributes.

The reference has no class for this solver: its parameters are module globals
(:17-40) that users edit, and its main loop is colission / streaming1 /
Boundary_condition / streaming3 / Boundary_condition_psi (:626-632).  This
class keeps those names and defaults (niu_l, niu_g, psi_solid, CapA, fx/fy/fz,
bc_* / rho_bc* / v*_bc*, bc_psi_* / psi_*) and runs the step on the GPU
through liblbm_gb300.so (two launches per step, see csrc/lbm_tp.cu).

Conventions of the script kept: tau = 3 niu + 0.5 via wl, wg (:104-105), Guo
term without the /3, /9 factors (:242-248), velocity faces in the in-place form
(:502-506), psi update rho_r - rho_b/(rho_r + rho_b) (:606).  One deliberate
difference: the script's static_init assigns its BC velocities to local
variables, so its velocity faces always use u = 0 (:224-229); this class uses
the v*_bc* values it is given.
"""
import numpy as np

from . import _native
from .fields import DeviceField, HostField
from .geometry import read_ascii_field, read_ascii_geometry
from .vtk import grid_to_vtk


class LB3D_Solver_Two_Phase:
    def __init__(self, nx, ny, nz, storage="f32", device=0, block_size=0):
        self.nx, self.ny, self.nz = nx, ny, nz
        # physical parameters (defaults of the script, :18-40)
        self.fx, self.fy, self.fz = 5.0e-5, 0.0, 0.0
        self.niu_l = 0.1
        self.niu_g = 0.1
        self.psi_solid = 0.7
        self.CapA = 0.005
        self.bc_x_left, self.rho_bcxl, self.vx_bcxl, self.vy_bcxl, self.vz_bcxl = 0, 1.0, 0.0e-5, 0.0, 0.0
        self.bc_x_right, self.rho_bcxr, self.vx_bcxr, self.vy_bcxr, self.vz_bcxr = 0, 1.0, 0.0, 0.0, 0.0
        self.bc_y_left, self.rho_bcyl, self.vx_bcyl, self.vy_bcyl, self.vz_bcyl = 0, 1.0, 0.0, 0.0, 0.0
        self.bc_y_right, self.rho_bcyr, self.vx_bcyr, self.vy_bcyr, self.vz_bcyr = 0, 1.0, 0.0, 0.0, 0.0
        self.bc_z_left, self.rho_bczl, self.vx_bczl, self.vy_bczl, self.vz_bczl = 0, 1.0, 0.0, 0.0, 0.0
        self.bc_z_right, self.rho_bczr, self.vx_bczr, self.vy_bczr, self.vz_bczr = 0, 1.0, 0.0, 0.0, 0.0
        self.bc_psi_x_left, self.psi_x_left = 1, -1.0
        self.bc_psi_x_right, self.psi_x_right = 0, 1.0
        self.bc_psi_y_left, self.psi_y_left = 0, 1.0
        self.bc_psi_y_right, self.psi_y_right = 0, 1.0
        self.bc_psi_z_left, self.psi_z_left = 0, 1.0
        self.bc_psi_z_right, self.psi_z_right = 0, 1.0
        self.storage = storage
        self.device = device
        self.block_size = block_size

        shape = (nx, ny, nz)
        self.solid = HostField(shape, np.int8)
        self.psi = HostField(shape, np.float32)
        self.rho = DeviceField(lambda: self._macros()[0], shape)
        self.v = DeviceField(lambda: self._macros()[1], shape + (3,))
        self.phase = DeviceField(lambda: self._phase()[0], shape)
        self.rho_r = DeviceField(lambda: self._phase()[1], shape)
        self.rho_b = DeviceField(lambda: self._phase()[2], shape)
        self.x = np.linspace(0, nx, nx)
        self.y = np.linspace(0, ny, ny)
        self.z = np.linspace(0, nz, nz)
        self._lat = None
        self._mcache = None
        self._pcache = None

    # ------------------------------------------------------------ setup
    def init_geo(self, filename, filename2):
        """Solid (0/1) and phase (-1/1) ASCII files, x fastest (:195-203)."""
        shape = (self.nx, self.ny, self.nz)
        self.solid.from_numpy(read_ascii_geometry(filename, shape))
        self.psi.from_numpy(read_ascii_field(filename2, shape))

    def _params(self):
        return _native.make_params(
            (self.nx, self.ny, self.nz), niu=0.1, force=(self.fx, self.fy, self.fz),
            bc=[self.bc_x_left, self.bc_x_right, self.bc_y_left, self.bc_y_right, self.bc_z_left, self.bc_z_right],
            rho_bc=[self.rho_bcxl, self.rho_bcxr, self.rho_bcyl, self.rho_bcyr, self.rho_bczl, self.rho_bczr],
            vel_bc=[[self.vx_bcxl, self.vy_bcxl, self.vz_bcxl], [self.vx_bcxr, self.vy_bcxr, self.vz_bcxr],
                    [self.vx_bcyl, self.vy_bcyl, self.vz_bcyl], [self.vx_bcyr, self.vy_bcyr, self.vz_bcyr],
                    [self.vx_bczl, self.vy_bczl, self.vz_bczl], [self.vx_bczr, self.vy_bczr, self.vz_bczr]],
            visc_convention=1, guo_convention=1, bc_form=1, storage=self.storage, two_phase=True,
            niu_l=self.niu_l, niu_g=self.niu_g, psi_solid=self.psi_solid, cap_a=self.CapA,
            psi_bc=[self.bc_psi_x_left, self.bc_psi_x_right, self.bc_psi_y_left, self.bc_psi_y_right,
                    self.bc_psi_z_left, self.bc_psi_z_right],
            psi_val=[self.psi_x_left, self.psi_x_right, self.psi_y_left, self.psi_y_right, self.psi_z_left,
                     self.psi_z_right],
            device=self.device, block_size=self.block_size)

    def init_simulation(self):
        """static_init + init (:205-229, :174-187): rho = 1, v = 0, f = feq,
        rho_r = (psi + 1)/2, rho_b = 1 - rho_r."""
        if self._lat is not None:
            self._lat.close()
        self._lat = _native.Lattice(self._params())
        self._lat.set_geometry(self.solid.array)
        self._lat.set_psi(self.psi.array)
        self._lat.init()
        self._mcache = self._pcache = None

    # ------------------------------------------------------------ stepping
    def _need(self):
        if self._lat is None:
            raise RuntimeError("call init_simulation() first")
        return self._lat

    def step(self):
        self._need().step(1)
        self._mcache = self._pcache = None

    def run(self, nsteps):
        self._need().step(int(nsteps))
        self._mcache = self._pcache = None

    # ------------------------------------------------------------ outputs
    def _macros(self):
        if self._mcache is None:
            self._mcache = self._need().macros()
        return self._mcache

    def _phase(self):
        if self._pcache is None:
            self._pcache = self._need().phase()
        return self._pcache

    def get_max_v(self):
        return self._need().max_v()

    def stats(self):
        return self._need().stats()

    def saturation(self):
        """Fraction of fluid cells with psi > 0 (the non-wetting phase)."""
        psi = self._phase()[0]
        fl = self.solid.array == 0
        return float((psi[fl] > 0).sum()) / max(1, int(fl.sum()))

    def interface_position(self):
        """Mean x of the fluid cells where psi changes sign along x."""
        psi = self._phase()[0]
        fl = self.solid.array == 0
        a, b = psi[:-1], psi[1:]
        both = fl[:-1] & fl[1:]
        hit = both & (np.sign(a) != np.sign(b))
        if not hit.any():
            return float("nan")
        xs = np.nonzero(hit)[0] + 0.5
        return float(xs.mean())

    def export_VTK(self, n):
        rho, v = self._macros()
        psi = self._phase()[0]
        return grid_to_vtk("./structured" + str(n), self.x, self.y, self.z,
                           {"Solid": np.ascontiguousarray(self.solid.to_numpy()), "rho": np.ascontiguousarray(rho),
                            "phase": np.ascontiguousarray(psi),
                            "velocity": (np.ascontiguousarray(v[..., 0]), np.ascontiguousarray(v[..., 1]),
                                         np.ascontiguousarray(v[..., 2]))})

    def close(self):
        if self._lat is not None:
            self._lat.close()
            self._lat = None

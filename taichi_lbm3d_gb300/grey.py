"""Grey-scale (partial bounce-back) single-phase solver with the parameters of
the reference's script (Grey_Scale/lbm_solver_3d_Macro_Sukop.py) as attributes.

The reference has no class for this solver: its parameters are module globals
(:8-27) and its main loop is colission / streaming0 / streaming1 /
Boundary_condition / streaming3 (:330-336).  This class keeps those names and
defaults and runs the step on the GPU through liblbm_gb300.so
(csrc/lbm_grey.cu, one launch per step).

Conventions of the script kept: tau = 3 niu + 0.5 (:57), Guo term without the
/3, /9 factors (:184-189), solid = ns.astype(int) (:321), the partial
bounce-back rule f2 = f + ns (f[x+e_s, LR s] - f) of streaming0 (:234-240),
fixed faces on x only, velocity faces in the in-place form (:263-293).  The
script's y/z face settings have no effect there; here too they are kept as
attributes and ignored.  One deliberate difference: the script's static_init
assigns its BC velocities to local variables, so its velocity faces always
use u = 0 (:166-171); this class uses the v*_bc* values it is given (the
defaults are 0).
"""
import numpy as np

from . import _native
from .fields import DeviceField, HostField
from .geometry import read_ascii_field
from .vtk import grid_to_vtk


class LB3D_Solver_Grey_Scale:
    def __init__(self, nx, ny, nz, storage="f32", device=0, block_size=0):
        self.nx, self.ny, self.nz = nx, ny, nz
        # physical parameters (defaults of the script, :8-27)
        self.fx, self.fy, self.fz = 1.0e-6, 0.0, 0.0
        self.niu = 0.1
        self.bc_x_left, self.rho_bcxl, self.vx_bcxl, self.vy_bcxl, self.vz_bcxl = 0, 1.0, 0.0e-5, 0.0, 0.0
        self.bc_x_right, self.rho_bcxr, self.vx_bcxr, self.vy_bcxr, self.vz_bcxr = 0, 0.995, 0.0, 0.0, 0.0
        self.bc_y_left, self.rho_bcyl, self.vx_bcyl, self.vy_bcyl, self.vz_bcyl = 0, 1.0, 0.0, 0.0, 0.0
        self.bc_y_right, self.rho_bcyr, self.vx_bcyr, self.vy_bcyr, self.vz_bcyr = 0, 1.0, 0.0, 0.0, 0.0
        self.bc_z_left, self.rho_bczl, self.vx_bczl, self.vy_bczl, self.vz_bczl = 0, 1.0, 0.0, 0.0, 0.0
        self.bc_z_right, self.rho_bczr, self.vx_bczr, self.vy_bczr, self.vz_bczr = 0, 1.0, 0.0, 0.0, 0.0
        self.storage = storage
        self.device = device
        self.block_size = block_size

        shape = (nx, ny, nz)
        self.ns = HostField(shape, np.float64)
        self.solid = HostField(shape, np.int32)
        self.rho = DeviceField(lambda: self._macros()[0], shape)
        self.v = DeviceField(lambda: self._macros()[1], shape + (3,))
        self.x = np.linspace(0, nx, nx)
        self.y = np.linspace(0, ny, ny)
        self.z = np.linspace(0, nz, nz)
        self._lat = None
        self._mcache = None

    # ------------------------------------------------------------ setup
    def init_geo(self, filename):
        """The ns field from an ASCII file, x fastest, as float64 (:142-145)."""
        return read_ascii_field(filename, (self.nx, self.ny, self.nz), dtype=np.float64)

    def load_geo(self, filename):
        """ns from the file and solid = ns.astype(int), as the script's main
        program does (:320-324)."""
        ns = self.init_geo(filename)
        self.solid.from_numpy(ns.astype(int))
        self.ns.from_numpy(ns)
        return ns

    def _params(self):
        return _native.make_params(
            (self.nx, self.ny, self.nz), niu=self.niu, force=(self.fx, self.fy, self.fz),
            bc=[self.bc_x_left, self.bc_x_right, 0, 0, 0, 0],
            rho_bc=[self.rho_bcxl, self.rho_bcxr, 1.0, 1.0, 1.0, 1.0],
            vel_bc=[[self.vx_bcxl, self.vy_bcxl, self.vz_bcxl], [self.vx_bcxr, self.vy_bcxr, self.vz_bcxr],
                    [0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]],
            visc_convention=1, guo_convention=1, bc_form=1, storage=self.storage, device=self.device,
            block_size=self.block_size)

    def init_simulation(self):
        """static_init + init (:148-173, :120-127): rho = 1, v = 0, f = F = feq."""
        if self._lat is not None:
            self._lat.close()
        self._lat = _native.Lattice(self._params())
        self._lat.set_geometry((self.solid.array != 0).astype(np.int8))
        self._lat.set_grey(self.ns.array)
        self._lat.init()
        self._mcache = None

    # ------------------------------------------------------------ stepping
    def _need(self):
        if self._lat is None:
            raise RuntimeError("call init_simulation() first")
        return self._lat

    def step(self):
        """One pass of the script's main loop (:330-336)."""
        self._need().step(1)
        self._mcache = None

    def run(self, nsteps):
        self._need().step(int(nsteps))
        self._mcache = None

    # ------------------------------------------------------------ outputs
    def _macros(self):
        if self._mcache is None:
            self._mcache = self._need().macros()
        return self._mcache

    def get_max_v(self):
        return self._need().max_v()

    def stats(self):
        return self._need().stats()

    def export_VTK(self, n):
        """The script's output fields Solid, rho, velocity (:352-363)."""
        rho, v = self._macros()
        return grid_to_vtk("./structured" + str(n), self.x, self.y, self.z,
                           {"Solid": np.ascontiguousarray(self.solid.to_numpy()), "rho": np.ascontiguousarray(rho),
                            "velocity": (np.ascontiguousarray(v[..., 0]), np.ascontiguousarray(v[..., 1]),
                                         np.ascontiguousarray(v[..., 2]))})

    def close(self):
        if self._lat is not None:
            self._lat.close()
            self._lat = None

"""Drop-in for ``LB3D_Solver_Single_Phase`` (Single_phase/LBM_3D_SinglePhase_Solver.py).

Same constructor, public attributes, setters and methods as the reference
class; the Taichi kernels behind ``init_simulation``/``step``/``get_max_v`` are
replaced by the fused sm_103a kernels of liblbm_gb300.so (ctypes, no CPU path).

Behaviour kept from the reference (line numbers in that file):
  * BC codes 0 periodic / 1 pressure / 2 velocity per face (:22-28), setters
    switch the code and store the value (:405-451);
  * ``init_simulation`` captures the BC velocities, tau = niu/3 + 0.5, the
    S_dig rates and the force flag (:118-149); changes made afterwards take
    effect at the next ``init_simulation`` (the reference bakes BC types and the
    force flag into the kernels on the first step, :230, :274);
  * ``get_max_v`` returns max |v| over all cells (:394-402);
  * ``export_VTK(n)`` writes ./LB_SingelPhase_<n>.vtr (:462-475).
Additions: ``run(n)`` (n steps in one call), ``storage`` ('f32', 'f16', 'bf16',
'f64'), ``viscosity_convention`` / ``guo_convention`` ('class' reproduces the
reference class, 'standard'/'script' the other files' formulas), ``stats()``
(FP64 reductions), ``permeability()``, ``run_to_convergence()``, checkpoints.
"""
import numpy as np

from . import _native
from .fields import DeviceField, HostField
from .geometry import read_ascii_geometry
from .vtk import grid_to_vtk

VISC = {"class": 0, "standard": 1}
GUO = {"class": 0, "script": 1, "standard": 2}

# D3Q19 tables as the reference defines them (:64-85, :183-197)
E = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [1, 1, 0],
              [-1, -1, 0], [1, -1, 0], [-1, 1, 0], [1, 0, 1], [-1, 0, -1], [1, 0, -1], [-1, 0, 1], [0, 1, 1],
              [0, -1, -1], [0, 1, -1], [0, -1, 1]], dtype=np.int32)
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, dtype=np.float32)
LR = [0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17]
_MOMENTS = None


def moment_matrices():
    """M and inv_M as the reference's class holds them (SP:61-110): M of the
    kernels' generator (csrc/gen_mrt.py) in FP32, and inv(M) taken in FP64 and
    stored as FP32 (Q14)."""
    global _MOMENTS
    if _MOMENTS is None:
        import importlib.util
        import os
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "gen_mrt.py")
        spec = importlib.util.spec_from_file_location("_lbm_gen_mrt", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        m = np.array(mod.M, dtype=np.float64)
        _MOMENTS = (m.astype(np.float32), np.linalg.inv(m).astype(np.float32))
    return _MOMENTS[0].copy(), _MOMENTS[1].copy()


class LB3D_Solver_Single_Phase:
    def __init__(self, nx, ny, nz, sparse_storage=False, storage="f32", device=0,
                 viscosity_convention="class", guo_convention="class", block_size=0):
        self.enable_projection = True
        # The fused kernels always store the compacted fluid list (memory ~ fluid
        # nodes), which is what the reference's pointer-block sparse storage is for.
        self.sparse_storage = sparse_storage
        self.nx, self.ny, self.nz = nx, ny, nz
        self.fx, self.fy, self.fz = 0.0e-6, 0.0, 0.0
        self.niu = 0.16667
        self.bc_x_left, self.rho_bcxl, self.vx_bcxl, self.vy_bcxl, self.vz_bcxl = 0, 1.0, 0.0e-5, 0.0, 0.0
        self.bc_x_right, self.rho_bcxr, self.vx_bcxr, self.vy_bcxr, self.vz_bcxr = 0, 1.0, 0.0, 0.0, 0.0
        self.bc_y_left, self.rho_bcyl, self.vx_bcyl, self.vy_bcyl, self.vz_bcyl = 0, 1.0, 0.0, 0.0, 0.0
        self.bc_y_right, self.rho_bcyr, self.vx_bcyr, self.vy_bcyr, self.vz_bcyr = 0, 1.0, 0.0, 0.0, 0.0
        self.bc_z_left, self.rho_bczl, self.vx_bczl, self.vy_bczl, self.vz_bczl = 0, 1.0, 0.0, 0.0, 0.0
        self.bc_z_right, self.rho_bczr, self.vx_bczr, self.vy_bczr, self.vz_bczr = 0, 1.0, 0.0, 0.0, 0.0
        self.storage = storage
        self.device = device
        self.viscosity_convention = viscosity_convention
        self.guo_convention = guo_convention
        self.block_size = block_size
        self.bc_form = 0

        self.solid = HostField((nx, ny, nz), np.int8)
        self.rho = DeviceField(lambda: self._macros()[0], (nx, ny, nz))
        self.v = DeviceField(lambda: self._macros()[1], (nx, ny, nz, 3))
        self.e = E.copy()
        self.e_f = E.astype(np.float32)
        self.w = W.copy()
        self.LR = list(LR)
        self.M, self.inv_M = moment_matrices()
        self.x = np.linspace(0, nx, nx)
        self.y = np.linspace(0, ny, ny)
        self.z = np.linspace(0, nz, nz)
        self._lat = None
        self._geo_version = -1
        self._cache = None

    # ------------------------------------------------------------ setup
    def init_geo(self, filename):
        """ASCII 0/1 voxel file, x fastest; values > 0 are solid (:173-177)."""
        self.solid.from_numpy(read_ascii_geometry(filename, (self.nx, self.ny, self.nz)))

    def _params(self):
        bc = [self.bc_x_left, self.bc_x_right, self.bc_y_left, self.bc_y_right, self.bc_z_left, self.bc_z_right]
        rho_bc = [self.rho_bcxl, self.rho_bcxr, self.rho_bcyl, self.rho_bcyr, self.rho_bczl, self.rho_bczr]
        return _native.make_params(
            (self.nx, self.ny, self.nz), niu=self.niu, force=(self.fx, self.fy, self.fz), bc=bc, rho_bc=rho_bc,
            vel_bc=[self.bc_vel_x_left, self.bc_vel_x_right, self.bc_vel_y_left, self.bc_vel_y_right,
                    self.bc_vel_z_left, self.bc_vel_z_right],
            visc_convention=VISC[self.viscosity_convention], guo_convention=GUO[self.guo_convention],
            bc_form=self.bc_form, storage=self.storage, device=self.device, block_size=self.block_size)

    def init_simulation(self, rho=None, v=None):
        """Capture parameters (:118-149) and initialise f = feq(rho, v), by
        default rho = 1, v = 0 (init, :160-170).  ``rho``/``v`` (dense arrays)
        start from a given macroscopic field instead (warm start)."""
        self.bc_vel_x_left = [self.vx_bcxl, self.vy_bcxl, self.vz_bcxl]
        self.bc_vel_x_right = [self.vx_bcxr, self.vy_bcxr, self.vz_bcxr]
        self.bc_vel_y_left = [self.vx_bcyl, self.vy_bcyl, self.vz_bcyl]
        self.bc_vel_y_right = [self.vx_bcyr, self.vy_bcyr, self.vz_bcyr]
        self.bc_vel_z_left = [self.vx_bczl, self.vy_bczl, self.vz_bczl]
        self.bc_vel_z_right = [self.vx_bczr, self.vy_bczr, self.vz_bczr]
        if self.viscosity_convention == "class":
            self.tau_f = self.niu / 3.0 + 0.5
        else:
            self.tau_f = 3.0 * self.niu + 0.5
        self.s_v = 1.0 / self.tau_f
        self.s_other = 8.0 * (2.0 - self.s_v) / (8.0 - self.s_v)
        self.S_dig = np.array([0, self.s_v, self.s_v, 0, self.s_other, 0, self.s_other, 0, self.s_other,
                               self.s_v, self.s_v, self.s_v, self.s_v, self.s_v, self.s_v, self.s_v,
                               self.s_other, self.s_other, self.s_other], dtype=np.float32)
        self.ext_f = np.array([self.fx, self.fy, self.fz], dtype=np.float32)
        self.force_flag = 1 if (abs(self.fx) > 0 or abs(self.fy) > 0 or abs(self.fz) > 0) else 0
        if self._lat is not None:
            self._lat.close()
        self._lat = _native.Lattice(self._params())
        self._lat.set_geometry(self.solid.array)
        self._geo_version = self.solid.version
        self._lat.init(rho, v)
        self._cache = None

    # ------------------------------------------------------------ stepping
    def _need(self):
        if self._lat is None:
            raise RuntimeError("call init_simulation() first")
        return self._lat

    def step(self):
        """One time step (:477-481)."""
        self._need().step(1)
        self._cache = None

    def run(self, nsteps):
        """nsteps time steps in one native call (one kernel launch per step)."""
        self._need().step(int(nsteps))
        self._cache = None

    # ------------------------------------------------------------ outputs
    def _macros(self):
        if self._cache is None:
            self._cache = self._need().macros()
        return self._cache

    def get_max_v(self):
        """max |v| over all cells (:394-402)."""
        return self._need().max_v()

    def stats(self):
        """FP64 reductions over fluid nodes: mass, momentum, max |v|, non-finite count."""
        return self._need().stats()

    @property
    def n_fluid(self):
        return int(self._need().info().n_fluid)

    def nu_eff(self):
        """Kinematic viscosity the relaxation rate implies: (tau - 1/2)/3."""
        return (self.tau_f - 0.5) / 3.0

    def permeability(self, axis=0):
        """Permeability along ``axis`` from the Darcy velocity (mean v over all
        cells, solid cells count as 0):  k = nu_eff <v> / F_eff  for a body force
        (F_eff = the momentum the Guo term injects per step: F/9 in the class
        form, :236; F/3 in the script form; F in the standard form),
        k = nu_eff <v> (L-1) / ((rho_in - rho_out)/3)  for a pressure drop."""
        st = self.stats()
        return self._k_from_darcy(st.mom[axis] / (self.nx * self.ny * self.nz), axis)

    def _k_from_darcy(self, vmean, axis):
        f = (self.fx, self.fy, self.fz)[axis]
        if f != 0:
            f_eff = f * {"class": 1.0 / 9.0, "script": 1.0 / 3.0, "standard": 1.0}[self.guo_convention]
            return self.nu_eff() * vmean / f_eff
        rin = (self.rho_bcxl, self.rho_bcyl, self.rho_bczl)[axis]
        rout = (self.rho_bcxr, self.rho_bcyr, self.rho_bczr)[axis]
        L = (self.nx, self.ny, self.nz)[axis]
        return self.nu_eff() * vmean * (L - 1) / ((rin - rout) / 3.0)

    def run_to_convergence(self, tol=1e-6, check_every=500, max_steps=1_000_000, axis=0, log=None):
        """Step until the permeability changes by <= tol (relative) over
        ``check_every`` steps; returns dict(k, darcy_v, steps, converged).

        ``log`` (a path or a writable text file) records one JSON line per check:
        steps, Darcy velocity, k, its relative change, FP64 mass, max |v|,
        non-finite count, MLUPS since the start.  Without it the whole loop runs
        in the library (lbm_run_to_convergence); with it the same loop runs here,
        one lbm_step + lbm_reductions per check."""
        if log is None:
            dv, steps, conv = self._need().run_to_convergence(tol, check_every, max_steps, axis)
            self._cache = None
            return {"k": self._k_from_darcy(dv, axis), "darcy_v": dv, "steps": steps, "converged": conv}
        import json
        import os
        import time
        lat = self._need()
        if check_every < 1 or max_steps < 1 or axis not in (0, 1, 2) or not tol >= 0:
            raise ValueError("bad tol / check_every / max_steps / axis")
        own = isinstance(log, (str, os.PathLike))
        fh = open(log, "a") if own else log
        ncell = self.nx * self.ny * self.nz
        nf = self.n_fluid
        prev, done, conv, vm = None, 0, False, 0.0
        t0 = time.perf_counter()
        try:
            while done < max_steps:
                n = min(check_every, max_steps - done)
                lat.step(n)
                done += n
                self._cache = None
                st = lat.stats()
                if st.n_nonfinite:
                    raise _native.LbmError(_native.LBM_EDIVERGED, "run_to_convergence: non-finite rho or v")
                vm = st.mom[axis] / ncell
                rel = abs(vm - prev) / abs(vm) if prev is not None and vm != 0 else None
                fh.write(json.dumps({"steps": done, "darcy_v": vm, "k": self._k_from_darcy(vm, axis),
                                     "rel_change": rel, "mass": st.mass, "max_v": st.max_v,
                                     "n_nonfinite": int(st.n_nonfinite),
                                     "mlups": nf * done / max(time.perf_counter() - t0, 1e-12) / 1e6}) + "\n")
                if prev is not None and abs(vm - prev) <= tol * abs(vm):
                    conv = True
                    break
                prev = vm
        finally:
            if own:
                fh.close()
        return {"k": self._k_from_darcy(vm, axis), "darcy_v": vm, "steps": done, "converged": conv}

    def export_VTK(self, n):
        rho, v = self._macros()
        return grid_to_vtk("./LB_SingelPhase_" + str(n), self.x, self.y, self.z,
                           {"Solid": np.ascontiguousarray(self.solid.to_numpy()),
                            "rho": np.ascontiguousarray(rho),
                            "velocity": (np.ascontiguousarray(v[..., 0]), np.ascontiguousarray(v[..., 1]),
                                         np.ascontiguousarray(v[..., 2]))})

    # ------------------------------------------------------------ checkpoint
    def save_checkpoint(self, path):
        lat = self._need()
        np.savez(path, f=lat.populations(), steps=lat.info().steps_done, solid=self.solid.to_numpy())

    def load_checkpoint(self, path):
        d = np.load(path)
        if not np.array_equal(d["solid"], self.solid.to_numpy()):
            raise ValueError("checkpoint geometry differs from the solver's")
        self._need().set_populations(d["f"])
        self._cache = None

    # ------------------------------------------------------------ setters (:405-458)
    def set_bc_vel_x1(self, vel):
        self.bc_x_right = 2
        self.vx_bcxr, self.vy_bcxr, self.vz_bcxr = vel[0], vel[1], vel[2]

    def set_bc_vel_x0(self, vel):
        self.bc_x_left = 2
        self.vx_bcxl, self.vy_bcxl, self.vz_bcxl = vel[0], vel[1], vel[2]

    def set_bc_vel_y1(self, vel):
        self.bc_y_right = 2
        self.vx_bcyr, self.vy_bcyr, self.vz_bcyr = vel[0], vel[1], vel[2]

    def set_bc_vel_y0(self, vel):
        self.bc_y_left = 2
        self.vx_bcyl, self.vy_bcyl, self.vz_bcyl = vel[0], vel[1], vel[2]

    def set_bc_vel_z1(self, vel):
        self.bc_z_right = 2
        self.vx_bczr, self.vy_bczr, self.vz_bczr = vel[0], vel[1], vel[2]

    def set_bc_vel_z0(self, vel):
        self.bc_z_left = 2
        self.vx_bczl, self.vy_bczl, self.vz_bczl = vel[0], vel[1], vel[2]

    def set_bc_rho_x0(self, rho):
        self.bc_x_left = 1
        self.rho_bcxl = rho

    def set_bc_rho_x1(self, rho):
        self.bc_x_right = 1
        self.rho_bcxr = rho

    def set_bc_rho_y0(self, rho):
        self.bc_y_left = 1
        self.rho_bcyl = rho

    def set_bc_rho_y1(self, rho):
        self.bc_y_right = 1
        self.rho_bcyr = rho

    def set_bc_rho_z0(self, rho):
        self.bc_z_left = 1
        self.rho_bczl = rho

    def set_bc_rho_z1(self, rho):
        self.bc_z_right = 1
        self.rho_bczr = rho

    def set_viscosity(self, niu):
        self.niu = niu

    def set_force(self, force):
        self.fx, self.fy, self.fz = force[0], force[1], force[2]

    def close(self):
        if self._lat is not None:
            self._lat.close()
            self._lat = None

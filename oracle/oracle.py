"""ctypes wrapper of the CPU oracle (liblbm_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of bench.py, never by the product package.  Arrays cross the
boundary in the lattice order of the reference's geometry files: x fastest,
cell id = i + nx*(j + ny*k) (``init_geo``, LBM_3D_SinglePhase_Solver.py:173-177).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbm_oracle.so")


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("bc", ctypes.c_int32 * 6),
        ("rho_bc", ctypes.c_double * 6),
        ("vel_bc", (ctypes.c_double * 3) * 6),
        ("niu", ctypes.c_double),
        ("force", ctypes.c_double * 3),
        ("visc_convention", ctypes.c_int32),
        ("guo_convention", ctypes.c_int32),
        ("bc_form", ctypes.c_int32),
        ("two_phase", ctypes.c_int32),
        ("niu_l", ctypes.c_double), ("niu_g", ctypes.c_double),
        ("psi_solid", ctypes.c_double), ("cap_a", ctypes.c_double),
        ("psi_bc", ctypes.c_int32 * 6),
        ("psi_val", ctypes.c_double * 6),
        ("ref_emulation", ctypes.c_int32),
        ("grey", ctypes.c_int32),
    ]


def build(force=False):
    """Compile the oracle with gcc (OpenMP, no FP contraction)."""
    srcs = [os.path.join(HERE, f) for f in ("lbm_oracle.c", "vox_oracle.c")]
    body = os.path.join(HERE, "lbm_oracle_body.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(f) for f in srcs + [body])):
        return LIB_PATH
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB_PATH] + srcs + ["-lm"]
    subprocess.check_call(cmd, cwd=HERE)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.lbm_oracle_create.restype = ctypes.c_void_p
        L.lbm_oracle_create.argtypes = [ctypes.POINTER(OracleParams), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.lbm_oracle_destroy.argtypes = [ctypes.c_void_p]
        L.lbm_oracle_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.lbm_oracle_stream_only.argtypes = [ctypes.c_void_p]
        L.lbm_oracle_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.lbm_oracle_set.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        assert L.lbm_oracle_sizeof_params() == ctypes.sizeof(OracleParams)
        L.lbm_oracle_voxelize.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_float,
                                          ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
                                          ctypes.c_void_p, ctypes.c_void_p]
        L.lbm_oracle_mesh_distance.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_float,
                                               ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]
        _lib = L
    return _lib


def make_params(shape, niu=0.16667, force=(0.0, 0.0, 0.0), bc=(0,) * 6, rho_bc=(1.0,) * 6,
                vel_bc=((0.0, 0.0, 0.0),) * 6, visc_convention=0, guo_convention=0, bc_form=0,
                two_phase=False, niu_l=0.1, niu_g=0.1, psi_solid=0.7, cap_a=0.005,
                psi_bc=(0,) * 6, psi_val=(1.0,) * 6, ref_emulation=0, grey=False):
    p = OracleParams()
    p.nx, p.ny, p.nz = shape
    for f in range(6):
        p.bc[f] = bc[f]
        p.rho_bc[f] = rho_bc[f]
        for c in range(3):
            p.vel_bc[f][c] = vel_bc[f][c]
        p.psi_bc[f] = psi_bc[f]
        p.psi_val[f] = psi_val[f]
    p.niu = niu
    for c in range(3):
        p.force[c] = force[c]
    p.visc_convention = visc_convention
    p.guo_convention = guo_convention
    p.bc_form = bc_form
    p.two_phase = 1 if two_phase else 0
    p.niu_l, p.niu_g, p.psi_solid, p.cap_a = niu_l, niu_g, psi_solid, cap_a
    p.ref_emulation = ref_emulation
    p.grey = 1 if grey else 0
    return p


class Oracle:
    """One lattice of the CPU oracle.  ``solid`` and ``psi`` are (nx,ny,nz) arrays."""

    def __init__(self, params, solid, psi=None, precision=32):
        self.p = params
        self.shape = (params.nx, params.ny, params.nz)
        self.ncell = params.nx * params.ny * params.nz
        s = np.ascontiguousarray(np.asarray(solid).ravel(order="F"), dtype=np.int8)
        ps = None
        if psi is not None:
            ps = np.ascontiguousarray(np.asarray(psi).ravel(order="F"), dtype=np.float32)
        self._keep = (s, ps)
        self.h = lib().lbm_oracle_create(ctypes.byref(params), s.ctypes.data,
                                         ps.ctypes.data if ps is not None else None, precision)
        if not self.h:
            raise RuntimeError("lbm_oracle_create failed")

    def close(self):
        if self.h:
            lib().lbm_oracle_destroy(self.h)
            self.h = None

    __del__ = close

    def step(self, n=1):
        if lib().lbm_oracle_step(self.h, int(n)) != 0:
            raise RuntimeError("oracle step failed")

    def stream_only(self):
        lib().lbm_oracle_stream_only(self.h)

    def _get(self, what, comps):
        out = np.empty(self.ncell * comps if what != 7 else 361, dtype=np.float64)
        if lib().lbm_oracle_get(self.h, what, out.ctypes.data) != 0:
            raise RuntimeError("oracle get failed")
        return out

    def field(self, name):
        """Return a field as an (nx,ny,nz[,c]) array (Fortran cell order undone)."""
        what, comps = {"rho": (0, 1), "v": (1, 3), "f": (2, 19), "F": (3, 19), "psi": (4, 1),
                       "rho_r": (5, 1), "rho_b": (6, 1), "ns": (8, 1)}[name]
        a = self._get(what, comps)
        if comps == 1:
            return a.reshape(self.shape, order="F")
        return a.reshape((self.ncell, comps)).reshape(self.shape + (comps,), order="F")

    def inv_m(self):
        return self._get(7, 1).reshape(19, 19)

    def set_field(self, name, arr):
        what, comps = {"f": (2, 19), "F": (3, 19), "ns": (8, 1)}[name]
        a = np.asarray(arr, dtype=np.float64).reshape(self.shape + (comps,))
        flat = np.ascontiguousarray(a.reshape((self.ncell, comps), order="F"))
        if lib().lbm_oracle_set(self.h, what, flat.ctypes.data) != 0:
            raise RuntimeError("oracle set failed")


def voxelize(tris, origin, dx, dims, surf_eps=-1.0):
    """FP64 oracle of the voxeliser: (solid int8 (nx,ny,nz), winding (nx,ny,nz))."""
    t = np.ascontiguousarray(np.asarray(tris, np.float32).reshape(-1, 9))
    o = np.ascontiguousarray(np.asarray(origin, np.float32))
    nx, ny, nz = (int(x) for x in dims)
    solid = np.empty(nx * ny * nz, np.int8)
    w = np.empty(nx * ny * nz, np.float64)
    if lib().lbm_oracle_voxelize(t.ctypes.data, t.shape[0], o.ctypes.data, float(dx), nx, ny, nz, float(surf_eps),
                                 solid.ctypes.data, w.ctypes.data) != 0:
        raise RuntimeError("oracle voxelize failed")
    return solid.reshape((nx, ny, nz), order="F"), w.reshape((nx, ny, nz), order="F")


def mesh_distance(tris, origin, dx, dims):
    t = np.ascontiguousarray(np.asarray(tris, np.float32).reshape(-1, 9))
    o = np.ascontiguousarray(np.asarray(origin, np.float32))
    nx, ny, nz = (int(x) for x in dims)
    d = np.empty(nx * ny * nz, np.float64)
    lib().lbm_oracle_mesh_distance(t.ctypes.data, t.shape[0], o.ctypes.data, float(dx), nx, ny, nz, d.ctypes.data)
    return d.reshape((nx, ny, nz), order="F")

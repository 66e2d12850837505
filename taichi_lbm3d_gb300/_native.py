"""ctypes binding of liblbm_gb300.so (the C ABI in include/lbm_gb300.h).

The library is loaded from this package directory; there is no fallback: if it
is missing or no sm_103 device is present, the calls raise.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "liblbm_gb300.so")

LBM_OK, LBM_EINVAL, LBM_ENODEV, LBM_ENOMEM, LBM_ECUDA, LBM_ESTATE, LBM_EDIVERGED = 0, -1, -2, -3, -4, -5, -6
STORE = {"f32": 0, "f16": 1, "bf16": 2, "f64": 3, "f32dev": 4}
STORE_NAME = {v: k for k, v in STORE.items()}


class LbmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


class LbmParams(ctypes.Structure):
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
        ("storage", ctypes.c_int32),
        ("two_phase", ctypes.c_int32),
        ("niu_l", ctypes.c_double), ("niu_g", ctypes.c_double),
        ("psi_solid", ctypes.c_double), ("cap_a", ctypes.c_double),
        ("psi_bc", ctypes.c_int32 * 6),
        ("psi_val", ctypes.c_double * 6),
        ("device", ctypes.c_int32),
        ("block_size", ctypes.c_int32),
    ]


class LbmInfo(ctypes.Structure):
    _fields_ = [("n_cells", ctypes.c_int64), ("n_fluid", ctypes.c_int64), ("steps_done", ctypes.c_int64),
                ("device_bytes", ctypes.c_int64), ("storage", ctypes.c_int32), ("two_phase", ctypes.c_int32),
                ("sm_count", ctypes.c_int32), ("abi_version", ctypes.c_int32)]


class LbmStats(ctypes.Structure):
    _fields_ = [("mass", ctypes.c_double), ("mom", ctypes.c_double * 3), ("max_v", ctypes.c_double),
                ("n_nonfinite", ctypes.c_int64), ("n_fluid", ctypes.c_int64)]


_P = ctypes.c_void_p
# name -> argtypes (restype int unless noted)
SIGNATURES = {
    "lbm_abi_version": [],
    "lbm_create": [ctypes.POINTER(LbmParams), ctypes.POINTER(_P)],
    "lbm_destroy": [_P],
    "lbm_set_geometry": [_P, _P],
    "lbm_set_geometry_strided": [_P, _P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64],
    "lbm_set_psi": [_P, _P],
    "lbm_set_grey": [_P, _P],
    "lbm_init": [_P, _P, _P],
    "lbm_step": [_P, ctypes.c_int32],
    "lbm_step_async": [_P, ctypes.c_int32],
    "lbm_synchronize": [_P],
    "lbm_get_stream": [_P, ctypes.POINTER(_P)],
    "lbm_get_macros": [_P, _P, _P],
    "lbm_get_macros_f64": [_P, _P, _P],
    "lbm_get_phase": [_P, _P, _P, _P],
    "lbm_get_max_v": [_P, ctypes.POINTER(ctypes.c_float)],
    "lbm_reductions": [_P, ctypes.POINTER(LbmStats)],
    "lbm_get_info": [_P, ctypes.POINTER(LbmInfo)],
    "lbm_run_to_convergence": [_P, ctypes.c_double, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                               ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64),
                               ctypes.POINTER(ctypes.c_int32)],
    "lbm_get_fluid_index": [_P, _P],
    "lbm_get_neighbors": [_P, _P],
    "lbm_get_populations": [_P, _P],
    "lbm_set_populations": [_P, _P],
    "lbm_debug_stream": [_P, _P, _P],
    "lbm_last_error": [_P, ctypes.c_char_p, ctypes.c_size_t],
    "lbm_read_ascii": [ctypes.c_char_p, _P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)],
    "lbm_get_psi": [_P, _P],
}

_lib = None


def load(path=LIB_PATH):
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise LbmError(LBM_ENODEV, "liblbm_gb300.so not built: run `python -m taichi_lbm3d_gb300.build` "
                                       "(there is no CPU fallback)")
        L = ctypes.CDLL(path)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        if L.lbm_abi_version() != 1:
            raise LbmError(LBM_EINVAL, "ABI version mismatch")
        _lib = L
    return _lib


def read_ascii(path, n=None):
    """Whitespace-separated numbers of an ASCII file as float64, parsed by the
    library on the host (lbm_read_ascii); n, when given, is the count the file
    must hold."""
    L = load()
    cnt = ctypes.c_int64(0)
    p = os.fsencode(path)
    if n is None:
        check(L.lbm_read_ascii(p, None, 0, ctypes.byref(cnt)))
        n = cnt.value
    out = np.empty(int(n), np.float64)
    check(L.lbm_read_ascii(p, ptr(out), int(n), ctypes.byref(cnt)))
    return out


def last_error(h=None):
    buf = ctypes.create_string_buffer(1024)
    load().lbm_last_error(h, buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc, h=None):
    if rc != LBM_OK:
        raise LbmError(rc, last_error(h))
    return rc


def ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class Lattice:
    """Owner of one native handle (one lattice on one GPU)."""

    def __init__(self, params):
        L = load()
        self.params = params
        h = _P()
        check(L.lbm_create(ctypes.byref(params), ctypes.byref(h)))
        self.h = h
        self.shape = (params.nx, params.ny, params.nz)
        self.ncell = params.nx * params.ny * params.nz

    def close(self):
        if getattr(self, "h", None):
            load().lbm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, rc):
        return check(rc, self.h)

    # --- setup
    def set_geometry(self, solid):
        """solid: (nx, ny, nz) array, > 0 solid.  Passed with its own strides
        (no transposing copy) when it is int8 or bool."""
        a = np.asarray(solid)
        if a.shape != self.shape:
            if a.size != self.ncell:
                raise ValueError("solid has %d cells, lattice has %d" % (a.size, self.ncell))
            a = a.reshape(self.shape, order="F")
        if a.dtype == np.bool_:
            a = a.view(np.int8)
        elif a.dtype != np.int8:
            a = (a > 0).astype(np.int8)
        if any(st < 0 for st in a.strides):
            a = np.array(a, order="F")
        self._c(load().lbm_set_geometry_strided(self.h, ptr(a), *(int(st) for st in a.strides)))

    def set_psi(self, psi):
        a = np.ascontiguousarray(np.asarray(psi, dtype=np.float32).ravel(order="F"))
        self._c(load().lbm_set_psi(self.h, ptr(a)))

    def set_grey(self, ns):
        """Partial bounce-back fraction per cell (call after set_geometry)."""
        a = np.ascontiguousarray(np.asarray(ns, dtype=np.float64).ravel(order="F"))
        if a.size != self.ncell:
            raise ValueError("ns has %d cells, lattice has %d" % (a.size, self.ncell))
        self._c(load().lbm_set_grey(self.h, ptr(a)))

    def init(self, rho=None, v=None):
        if rho is None:
            self._c(load().lbm_init(self.h, None, None))
        else:
            r = np.ascontiguousarray(np.asarray(rho, np.float32).ravel(order="F"))
            vv = np.ascontiguousarray(np.asarray(v, np.float32).reshape(self.shape + (3,)).reshape((-1, 3), order="F"))
            self._c(load().lbm_init(self.h, ptr(r), ptr(vv)))

    # --- stepping
    def step(self, n=1):
        self._c(load().lbm_step(self.h, int(n)))

    def step_async(self, n=1):
        self._c(load().lbm_step_async(self.h, int(n)))

    def synchronize(self):
        self._c(load().lbm_synchronize(self.h))

    def stream(self):
        s = _P()
        self._c(load().lbm_get_stream(self.h, ctypes.byref(s)))
        return s.value

    # --- readback
    def macros(self):
        rho = np.empty(self.ncell, np.float32)
        v = np.empty(self.ncell * 3, np.float32)
        self._c(load().lbm_get_macros(self.h, ptr(rho), ptr(v)))
        return rho.reshape(self.shape, order="F"), v.reshape((self.ncell, 3)).reshape(self.shape + (3,), order="F")

    def macros_f64(self):
        rho = np.empty(self.ncell, np.float64)
        v = np.empty(self.ncell * 3, np.float64)
        self._c(load().lbm_get_macros_f64(self.h, ptr(rho), ptr(v)))
        return rho.reshape(self.shape, order="F"), v.reshape((self.ncell, 3)).reshape(self.shape + (3,), order="F")

    def phase(self):
        out = [np.empty(self.ncell, np.float32) for _ in range(3)]
        self._c(load().lbm_get_phase(self.h, *[ptr(a) for a in out]))
        return tuple(a.reshape(self.shape, order="F") for a in out)

    def psi(self):
        out = np.empty(self.ncell, np.float32)
        self._c(load().lbm_get_psi(self.h, ptr(out)))
        return out.reshape(self.shape, order="F")

    def max_v(self):
        f = ctypes.c_float()
        self._c(load().lbm_get_max_v(self.h, ctypes.byref(f)))
        return f.value

    def stats(self):
        st = LbmStats()
        self._c(load().lbm_reductions(self.h, ctypes.byref(st)))
        return st

    def run_to_convergence(self, tol=1e-6, check_every=500, max_steps=1_000_000, axis=0):
        """Step until the FP64 Darcy velocity changes by <= tol between checks."""
        dv, st, cv = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int32()
        self._c(load().lbm_run_to_convergence(self.h, float(tol), int(check_every), int(max_steps), int(axis),
                                              ctypes.byref(dv), ctypes.byref(st), ctypes.byref(cv)))
        return dv.value, st.value, bool(cv.value)

    def info(self):
        inf = LbmInfo()
        self._c(load().lbm_get_info(self.h, ctypes.byref(inf)))
        return inf

    def fluid_index(self):
        n = self.info().n_fluid
        a = np.empty(n, np.int32)
        self._c(load().lbm_get_fluid_index(self.h, ptr(a)))
        return a

    def neighbors(self):
        n = self.info().n_fluid
        a = np.empty((18, n), np.int32)
        self._c(load().lbm_get_neighbors(self.h, ptr(a)))
        return a

    def populations(self):
        n = self.info().n_fluid
        a = np.empty((19, n), np.float64)
        self._c(load().lbm_get_populations(self.h, ptr(a)))
        return a

    def set_populations(self, f):
        a = np.ascontiguousarray(f, dtype=np.float64)
        self._c(load().lbm_set_populations(self.h, ptr(a)))

    def debug_stream(self, f_in):
        a = np.ascontiguousarray(f_in, dtype=np.float32)
        out = np.empty_like(a)
        self._c(load().lbm_debug_stream(self.h, ptr(a), ptr(out)))
        return out


def make_params(shape, niu=0.16667, force=(0.0, 0.0, 0.0), bc=(0,) * 6, rho_bc=(1.0,) * 6,
                vel_bc=((0.0, 0.0, 0.0),) * 6, visc_convention=0, guo_convention=0, bc_form=0, storage="f32",
                two_phase=False, niu_l=0.1, niu_g=0.1, psi_solid=0.7, cap_a=0.005, psi_bc=(0,) * 6,
                psi_val=(1.0,) * 6, device=0, block_size=0):
    p = LbmParams()
    p.nx, p.ny, p.nz = (int(x) for x in shape)
    for f in range(6):
        p.bc[f] = int(bc[f])
        p.rho_bc[f] = float(rho_bc[f])
        for c in range(3):
            p.vel_bc[f][c] = float(vel_bc[f][c])
        p.psi_bc[f] = int(psi_bc[f])
        p.psi_val[f] = float(psi_val[f])
    p.niu = float(niu)
    for c in range(3):
        p.force[c] = float(force[c])
    p.visc_convention = int(visc_convention)
    p.guo_convention = int(guo_convention)
    p.bc_form = int(bc_form)
    p.storage = STORE[storage] if isinstance(storage, str) else int(storage)
    p.two_phase = 1 if two_phase else 0
    p.niu_l, p.niu_g, p.psi_solid, p.cap_a = float(niu_l), float(niu_g), float(psi_solid), float(cap_a)
    p.device = int(device)
    p.block_size = int(block_size)
    return p

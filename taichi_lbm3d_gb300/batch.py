"""Batched permeability of many independent porous subvolumes on one GPU.

One persistent kernel per time step advances every active subvolume (work
tiles claimed from an atomic counter), ``check_every`` steps are captured into
one CUDA graph, converged subvolumes leave the work list (csrc/lbm_batch.cu).
Tile lengths and the CTA size come from the project's autotuner
(``autotune.py``), cached in a JSON file.

The reference has no batched mode (one lattice per process); the single-lattice
update is the same step as ``LB3D_Solver_Single_Phase`` with all faces periodic.
"""
import ctypes

import numpy as np

from . import _native

_P = ctypes.c_void_p
_SIGS = {
    "lbm_batch_create": [ctypes.POINTER(_native.LbmParams), ctypes.c_int32, _P, _P, ctypes.POINTER(_P)],
    "lbm_batch_destroy": [_P],
    "lbm_batch_configure": [_P, _P, ctypes.c_int32],
    "lbm_batch_init": [_P],
    "lbm_batch_step": [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32],
    "lbm_batch_run_to_convergence": [_P, ctypes.c_double, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, _P, _P,
                                     _P],
    "lbm_batch_get_stream": [_P, ctypes.POINTER(_P)],
    "lbm_batch_get_macros": [_P, ctypes.c_int32, _P, _P],
    "lbm_batch_info": [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                       ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)],
}


def _lib():
    L = _native.load()
    if not getattr(L, "_batch_bound", False):
        for n, a in _SIGS.items():
            f = getattr(L, n)
            f.argtypes = a
            f.restype = ctypes.c_int
        L._batch_bound = True
    return L


class Batch:
    """Subvolumes (list of int8 solid masks, any shapes) advanced together."""

    def __init__(self, solids, niu=0.1, force=(1e-6, 0.0, 0.0), storage="f16", visc_convention=1,
                 guo_convention=2, device=0):
        self.shapes = [tuple(int(x) for x in s.shape) for s in solids]
        self.n = len(solids)
        dims = np.ascontiguousarray(np.array(self.shapes, dtype=np.int32).ravel())
        flat = np.ascontiguousarray(np.concatenate([np.asarray(s, np.int8).ravel(order="F") for s in solids]))
        self.params = _native.make_params((1, 1, 1), niu=niu, force=force, visc_convention=visc_convention,
                                          guo_convention=guo_convention, storage=storage, device=device)
        self.niu, self.force, self.storage = niu, force, storage
        self.visc_convention, self.guo_convention = visc_convention, guo_convention
        h = _P()
        _native.check(_lib().lbm_batch_create(ctypes.byref(self.params), self.n, _native.ptr(dims),
                                              _native.ptr(flat), ctypes.byref(h)))
        self.h = h
        self.edges = [s[0] for s in self.shapes]

    def close(self):
        if getattr(self, "h", None):
            _lib().lbm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, rc):
        if rc != 0:
            raise _native.LbmError(rc, _native.last_error(self.h))

    def configure(self, tile_len, block):
        t = np.ascontiguousarray(np.asarray(tile_len, np.int32))
        assert t.size == self.n
        self._c(_lib().lbm_batch_configure(self.h, _native.ptr(t), int(block)))

    def init(self):
        self._c(_lib().lbm_batch_init(self.h))

    def step(self, nsteps, chunk=None, use_graph=True):
        chunk = chunk or nsteps
        self._c(_lib().lbm_batch_step(self.h, int(nsteps), int(chunk), 1 if use_graph else 0))

    def run_to_convergence(self, tol=1e-6, check_every=500, max_steps=200_000, use_graph=True):
        d = np.zeros(self.n, np.float64)
        st = np.zeros(self.n, np.int64)
        cv = np.zeros(self.n, np.int32)
        self._c(_lib().lbm_batch_run_to_convergence(self.h, float(tol), int(check_every), int(max_steps),
                                                    1 if use_graph else 0, _native.ptr(d), _native.ptr(st),
                                                    _native.ptr(cv)))
        return d, st, cv.astype(bool)

    def macros(self, q):
        """Dense rho (nx,ny,nz) and v (nx,ny,nz,3) of subvolume q from its current state."""
        shape = self.shapes[q]
        nc = int(np.prod(shape))
        rho = np.empty(nc, np.float32)
        v = np.empty(nc * 3, np.float32)
        self._c(_lib().lbm_batch_get_macros(self.h, int(q), _native.ptr(rho), _native.ptr(v)))
        return rho.reshape(shape, order="F"), v.reshape((nc, 3)).reshape(shape + (3,), order="F")

    def stream(self):
        s = _P()
        self._c(_lib().lbm_batch_get_stream(self.h, ctypes.byref(s)))
        return s.value

    def info(self):
        a, b, c, d = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()
        self._c(_lib().lbm_batch_info(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d)))
        return {"nodes": a.value, "n_fluid": b.value, "grid": c.value, "tiles": d.value}

    def permeability(self, darcy):
        """k = nu_eff <v> / F_eff per subvolume (body force along x)."""
        tau = 3 * self.niu + 0.5 if self.visc_convention == 1 else self.niu / 3 + 0.5
        nu = (tau - 0.5) / 3.0
        f_eff = self.force[0] * {0: 1.0 / 9.0, 1: 1.0 / 3.0, 2: 1.0}[self.guo_convention]
        return nu * np.asarray(darcy) / f_eff


def subvolume_sample(seed, edges=(48, 64, 96, 128, 160)):
    """One subvolume of the batched-permeability workload: edge uniform from
    ``edges``, porosity U[0.25, 0.50], sphere radii U[3, 8], percolating."""
    from .geometry import sphere_pack
    rng = np.random.default_rng(seed)
    edge = int(rng.choice(edges))
    phi = float(rng.uniform(0.25, 0.50))
    return sphere_pack((edge, edge, edge), 3.0, 8.0, phi, seed)


def subvolume_solids(seeds, workers=None):
    """Generate the subvolumes in parallel (spawned processes: call this before
    the first CUDA call of the process)."""
    import multiprocessing as mp
    import os
    workers = workers or max(1, min(16, len(os.sched_getaffinity(0))))
    if workers == 1:
        return [subvolume_sample(s) for s in seeds]
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(subvolume_sample, list(seeds), chunksize=1)

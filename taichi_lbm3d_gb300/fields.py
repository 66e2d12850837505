"""Field-like views that keep the reference's ``field.from_numpy`` /
``field.to_numpy`` idiom working on top of the native lattice.

The reference exposes Taichi fields (``solid``, ``rho``, ``v``, ``psi``) and its
drivers call ``lb3d.solid.from_numpy(geometry)`` (Single_phase/
example_poiseuille_flow.py:24) and ``self.rho.to_numpy()`` (LBM_3D_SinglePhase_Solver.py:470).
"""
import numpy as np


class HostField:
    """A host-resident lattice field (numpy array of the lattice shape)."""

    def __init__(self, shape, dtype):
        self.shape = tuple(shape)
        self.dtype = np.dtype(dtype)
        self._a = np.zeros(self.shape, dtype=self.dtype)
        self.version = 0

    def from_numpy(self, arr):
        arr = np.asarray(arr)
        if arr.shape != self.shape:
            raise ValueError("expected shape %s, got %s" % (self.shape, arr.shape))
        self._a[...] = arr.astype(self.dtype)
        self.version += 1

    def to_numpy(self):
        return self._a.copy()

    def fill(self, val):
        self._a[...] = val
        self.version += 1

    def __getitem__(self, idx):
        return self._a[idx]

    def __setitem__(self, idx, val):
        self._a[idx] = val
        self.version += 1

    @property
    def array(self):
        return self._a


class DeviceField:
    """A read-only view of a field that lives on the GPU (fetched on demand)."""

    def __init__(self, fetch, shape):
        self._fetch = fetch
        self.shape = tuple(shape)

    def to_numpy(self):
        return self._fetch()

    def __getitem__(self, idx):
        return self._fetch()[idx]

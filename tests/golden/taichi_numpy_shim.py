"""A minimal numpy stand-in for the ``taichi`` module, used ONLY to execute the
reference solver's own Python source (Single_phase/LBM_3D_SinglePhase_Solver.py
and 2phase/lbm_solver_3d_2phase_sparse.py) on tiny lattices, so that golden
fixtures can be generated in a container where Taichi itself is not installed.

Semantics emulated (Taichi >= 1.0, default_fp = f32):

* fields are dense numpy arrays (f32 / i32 / i8); a ``pointer``/``dense``
  SNode tree is flattened to a dense array of the padded shape.  Reads of cells
  that Taichi would leave inactive return 0, which is what a zero-initialised
  dense array gives;
* ``@ti.kernel`` / ``@ti.func`` run as plain Python; parallel struct-fors run
  sequentially in C order (i slowest).  The only order-dependent kernel in the
  reference is the two-phase colour push (``+=`` under Taichi's implicit
  atomics), whose FP32 summation order is therefore one valid order of many;
* vector arithmetic is FP32: int (op) float promotes to f32 (not f64 as numpy
  would), Python float literals are weak (cast to f32), ``dot``/``sum``/``@``
  accumulate sequentially, left to right.  Taichi's LLVM back end may contract
  or reassociate under fast-math, so goldens are compared with a tolerance.

This module is test infrastructure; nothing in the product imports it.
"""
import itertools
import math
import sys
import types

import numpy as np

f32 = np.float32
f64 = np.float64
i32 = np.int32
i8 = np.int8
u8 = np.uint8
ijk = "ijk"
ijkl = "ijkl"
cpu = "cpu"
gpu = "gpu"
cuda = "cuda"


def _is_floaty(a):
    if isinstance(a, np.ndarray):
        return a.dtype.kind == "f"
    return isinstance(a, (float, np.floating))


class Vec(np.ndarray):
    """Small Taichi vector/matrix value (a numpy view or a fresh array)."""

    def __array_ufunc__(self, ufunc, method, *inputs, **kw):
        floaty = any(_is_floaty(a) for a in inputs)
        args = []
        for a in inputs:
            if isinstance(a, Vec):
                a = a.view(np.ndarray)
            if floaty and isinstance(a, np.ndarray) and a.dtype.kind != "f":
                a = a.astype(f32)
            elif floaty and isinstance(a, np.ndarray) and a.dtype == f64:
                a = a.astype(f32)
            args.append(a)
        out = kw.get("out")
        if out is not None:
            kw["out"] = tuple(o.view(np.ndarray) if isinstance(o, Vec) else o for o in out)
        res = getattr(ufunc, method)(*args, **kw)
        if out is not None:
            return out[0]
        if isinstance(res, np.ndarray):
            if res.dtype == f64:
                res = res.astype(f32)
            return res.view(Vec)
        if isinstance(res, f64):
            return f32(res)
        return res

    # component access
    @property
    def x(self):
        return self._scalar(self[0])

    @property
    def y(self):
        return self._scalar(self[1])

    @property
    def z(self):
        return self._scalar(self[2])

    @staticmethod
    def _scalar(v):
        if isinstance(v, np.ndarray) and v.shape == ():
            v = v[()]
        if isinstance(v, np.integer):
            return int(v)
        return v

    def __getitem__(self, idx):
        r = np.ndarray.__getitem__(self, idx)
        if isinstance(r, np.ndarray) and r.shape != ():
            return r
        return self._scalar(r)

    def dot(self, other):
        a = np.asarray(self)
        b = np.asarray(other)
        if a.dtype.kind == "f" or b.dtype.kind == "f":
            a = a.astype(f32)
            b = b.astype(f32)
            acc = a[0] * b[0]
            for n in range(1, a.shape[0]):
                acc = f32(acc + a[n] * b[n])
            return f32(acc)
        acc = int(a[0]) * int(b[0])
        for n in range(1, a.shape[0]):
            acc += int(a[n]) * int(b[n])
        return acc

    def norm_sqr(self):
        return self.dot(self)

    def norm(self):
        return f32(np.sqrt(f32(self.dot(self))))

    def sum(self, *a, **k):  # sequential left-to-right
        v = np.asarray(self)
        acc = v[0]
        for n in range(1, v.shape[0]):
            acc = acc + v[n]
        return self._scalar(acc)

    def __matmul__(self, other):
        A = np.asarray(self).astype(f32)
        b = np.asarray(other).astype(f32)
        prod = A * b[None, :]                      # exact per-product f32 rounding
        acc = np.add.accumulate(prod, axis=1, dtype=f32)  # sequential accumulate
        return acc[:, -1].copy().view(Vec)


def _make_vec(data, dtype=None):
    arr = np.array(data)
    if dtype is None:
        dtype = f32 if arr.dtype.kind == "f" else i32
    return arr.astype(dtype).view(Vec)


class _VectorNS:
    def __call__(self, data, dt=None):
        return _make_vec(data, dt)

    def field(self, n, dtype, shape=None, **kw):
        return Field(dtype, shape, (n,))


class _MatrixNS:
    def __call__(self, data, dt=None):
        return _make_vec(data, dt)

    def field(self, n, m, dtype, shape=None, **kw):
        return Field(dtype, shape, (n, m))


Vector = _VectorNS()
Matrix = _MatrixNS()


def _flatten_index(idx):
    if idx is None:
        return ()
    if not isinstance(idx, tuple):
        idx = (idx,)
    out = []
    for it in idx:
        if it is None:
            continue
        if isinstance(it, np.ndarray):
            out.extend(int(x) for x in np.asarray(it).ravel())
        else:
            out.append(int(it))
    return tuple(out)


class Field:
    def __init__(self, dtype, shape, elem=()):
        self.dtype = dtype
        self.elem = elem
        self.data = None
        if shape is not None:
            if isinstance(shape, int):
                shape = (shape,)
            self._alloc(tuple(shape))

    def _alloc(self, shape):
        self.shape = tuple(shape)
        self.data = np.zeros(self.shape + tuple(self.elem), dtype=self.dtype)

    def __getitem__(self, idx):
        ix = _flatten_index(idx)
        if self.elem:
            return self.data[ix].view(Vec)
        if len(ix) == 0:
            return self.data[...]          # 0-d view, so ti.atomic_max can write it
        v = self.data[ix]
        if isinstance(v, np.integer):
            return int(v)
        return v

    def __setitem__(self, idx, val):
        ix = _flatten_index(idx)
        if len(ix) == 0:
            self.data[...] = np.asarray(val).astype(self.dtype)
        else:
            self.data[ix] = np.asarray(val).astype(self.dtype)

    def __iter__(self):
        return itertools.product(*[range(n) for n in self.shape])

    def from_numpy(self, arr):
        self.data[...] = np.asarray(arr).astype(self.dtype)

    def to_numpy(self):
        return self.data.copy()


class _SNode:
    def __init__(self, shape=()):
        self.shape = tuple(shape)

    def pointer(self, axes, shape):
        return _SNode(self.shape + (tuple(shape),))

    dense = pointer
    bitmasked = pointer

    def place(self, *fields):
        levels = self.shape
        total = tuple(int(np.prod([lv[d] for lv in levels])) for d in range(len(levels[0])))
        for fld in fields:
            fld._alloc(total)
        return self


root = _SNode()


def grouped(fld):
    for idx in fld:
        yield _make_vec(idx, i32)


def ndrange(*ranges):
    rr = [range(*r) if isinstance(r, tuple) else range(r) for r in ranges]
    return itertools.product(*rr)


def static(x, *a):
    return x


def kernel(fn):
    return fn


func = kernel
data_oriented = kernel


def init(*a, **k):
    return None


def atomic_max(target, val):
    old = target[()]
    if val > old:
        target[...] = val
    return old


def sqrt(x):
    return f32(math.sqrt(x))


class _Profiler:
    def __getattr__(self, name):
        return lambda *a, **k: None


profiler = _Profiler()


def install():
    """Register this module as ``taichi`` and no-op ``pyevtk.hl`` / ``evtk.hl``
    (the grey-scale script imports the package under its old name) in sys.modules."""
    sys.modules["taichi"] = sys.modules[__name__]
    for name in ("pyevtk", "evtk"):
        pe = types.ModuleType(name)
        hl = types.ModuleType(name + ".hl")
        hl.gridToVTK = lambda *a, **k: None
        pe.hl = hl
        sys.modules[name] = pe
        sys.modules[name + ".hl"] = hl


def field(dtype, shape=None, **kw):
    return Field(dtype, shape)

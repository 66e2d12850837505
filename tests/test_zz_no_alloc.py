"""lbm_reduce_macros_noalloc: the reduction entry point that allocates nothing.

It serves callers that cannot call cudaMalloc: a host framework whose pool
allocator already owns the GPU's memory, or a time-critical loop that must not
risk the device-wide synchronisation of cudaMalloc/cudaFree.  This test calls it
through the C ABI on device arrays the test itself owns, twice in a row on two
different lattices (the larger first, so partials a previous call left in the
shared static scratch would show up), and checks each result against the
existing entry point, lbm_reductions, on the same data.  This file sorts last so
that a run stopping at the first failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-12   # FP64 sums of the same FP32 values in a different order


def _fn():
    from taichi_lbm3d_gb300 import _native
    fn = _native.load().lbm_reduce_macros_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                   ctypes.POINTER(_native.LbmStats)]
    fn.restype = ctypes.c_int
    return fn


def _lattice(shape, seed):
    from taichi_lbm3d_gb300 import _native
    from taichi_lbm3d_gb300.geometry import sphere_pack
    solid = sphere_pack(shape, 2.5, 5.0, 0.45, seed=seed)
    lat = _native.Lattice(_native.make_params(shape, niu=0.1, force=(1e-5, -2e-6, 0), visc_convention=1,
                                              guo_convention=2))
    lat.set_geometry(solid)
    lat.init()
    lat.step(40)
    return lat


def _node_arrays(lat):
    import torch
    rho, v = lat.macros()
    idx = lat.fluid_index()
    rho_n = np.ascontiguousarray(rho.ravel(order="F")[idx])
    v_n = np.ascontiguousarray(np.stack([v[..., c].ravel(order="F")[idx] for c in range(3)]))
    return torch.from_numpy(rho_n).cuda(), torch.from_numpy(v_n).cuda(), idx.size


def test_noalloc_reduction_matches_lbm_reductions_twice():
    import torch
    from taichi_lbm3d_gb300 import _native
    fn = _fn()
    for shape, seed in (((56, 48, 40), 31), ((24, 20, 16), 32)):
        lat = _lattice(shape, seed)
        ref = lat.stats()                      # existing entry point
        d_rho, d_v, n = _node_arrays(lat)
        torch.cuda.synchronize()
        st = _native.LbmStats()
        rc = fn(d_rho.data_ptr(), d_v.data_ptr(), n, n, None, ctypes.byref(st))
        assert rc == 0, _native.last_error()
        assert st.n_fluid == ref.n_fluid == n
        assert abs(st.mass - ref.mass) <= REL * abs(ref.mass)
        for c in range(3):
            assert abs(st.mom[c] - ref.mom[c]) <= REL * np.abs(lat.macros()[1][..., c]).sum() + 1e-300
        assert st.max_v == ref.max_v
        assert st.n_nonfinite == ref.n_nonfinite == 0
        lat.close()


def test_noalloc_padded_stride_on_a_caller_stream():
    """The layout real callers hand over: v components padded to a stride above
    n (the library's own node arrays pad to 64), the padding filled with NaN so
    that reading it would show, and a non-default stream owned by the caller."""
    import torch
    from taichi_lbm3d_gb300 import _native
    fn = _fn()
    lat = _lattice((40, 36, 28), 33)
    ref = lat.stats()
    d_rho, d_v, n = _node_arrays(lat)
    stride = (n + 63) // 64 * 64 + 64
    v_pad = torch.full((3, stride), float("nan"), dtype=torch.float32, device="cuda")
    v_pad[:, :n] = d_v
    rho_pad = torch.full((stride,), float("nan"), dtype=torch.float32, device="cuda")
    rho_pad[:n] = d_rho
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    for _ in range(2):
        st = _native.LbmStats()
        rc = fn(rho_pad.data_ptr(), v_pad.data_ptr(), n, stride, ctypes.c_void_p(s.cuda_stream), ctypes.byref(st))
        assert rc == 0, _native.last_error()
        assert st.n_fluid == ref.n_fluid == n
        assert st.n_nonfinite == 0
        assert abs(st.mass - ref.mass) <= REL * abs(ref.mass)
        for c in range(3):
            assert abs(st.mom[c] - ref.mom[c]) <= REL * np.abs(lat.macros()[1][..., c]).sum() + 1e-300
        assert st.max_v == ref.max_v
    lat.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from taichi_lbm3d_gb300 import _native
    fn = _fn()
    st = _native.LbmStats()
    limit = 67108864
    rc = fn(None, None, limit + 1, limit + 1, None, ctypes.byref(st))
    assert rc == _native.LBM_EINVAL
    assert "67108864" in _native.last_error()

"""The U-Net's memory kernels (pool, upsample, concat, split and their
backward passes) run as 16-byte vectors when channel counts are multiples of 8
and the tensors are 16-byte aligned, else element by element.  Both forms do
the same per-element arithmetic in the same order, so a call on aligned
tensors must equal, bit for bit, the same call on tensors shifted by one BF16
element (which takes the element form).  The one-pass head weight gradient
(16 -> 4) is checked against FP64 and against its general form."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, D, H, W = 1, 6, 8, 10


def _lib():
    from taichi_lbm3d_gb300 import unet
    return unet._lib()


def _pair(t, shape, dtype):
    """The same values twice: an aligned tensor and a view one element past a 16-byte boundary."""
    import torch
    n = int(np.prod(shape))
    a = t.reshape(shape).to(dtype).contiguous().cuda()
    buf = torch.zeros(n + 1, dtype=dtype, device="cuda")
    buf[1:] = a.reshape(-1)
    return a, buf[1:].view(shape)


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _s():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _same(x, y):
    import torch
    torch.cuda.synchronize()
    assert torch.equal(x.view(torch.int16) if x.dtype == torch.bfloat16 else x,
                       y.view(torch.int16) if y.dtype == torch.bfloat16 else y)


@pytest.mark.parametrize("c", [16, 48])
def test_pool_and_its_gradient_vector_equals_elementwise(c):
    import torch
    L = _lib()
    torch.manual_seed(c)
    x = torch.randn(N, D, H, W, c)
    xa, xu = _pair(x, (N, D, H, W, c), torch.bfloat16)
    oa = torch.empty(N, D // 2, H // 2, W // 2, c, dtype=torch.bfloat16, device="cuda")
    ou = torch.zeros((oa.numel() + 1,), dtype=torch.bfloat16, device="cuda")[1:].view(oa.shape)
    aa = torch.empty(oa.shape, dtype=torch.uint8, device="cuda")
    au = torch.zeros((oa.numel() + 1,), dtype=torch.uint8, device="cuda")[1:].view(oa.shape)
    assert L.lbm_nn_pool2(_p(xa), _p(oa), _p(aa), N, D, H, W, c, _s()) == 0
    assert L.lbm_nn_pool2(_p(xu), _p(ou), _p(au), N, D, H, W, c, _s()) == 0
    _same(oa, ou)
    _same(aa, au)
    g = torch.randn(oa.shape)
    ga, gu = _pair(g, oa.shape, torch.bfloat16)
    m = torch.randn(N, D, H, W, c)
    ma, mu = _pair(m, (N, D, H, W, c), torch.bfloat16)
    prev = torch.randn(N, D, H, W, c)
    for acc in (0, 1):
        ia, iu = _pair(prev, (N, D, H, W, c), torch.bfloat16)
        assert L.lbm_nn_pool2_bwd(_p(ga), _p(aa), _p(ia), _p(ma), N, D, H, W, c, acc, _s()) == 0
        assert L.lbm_nn_pool2_bwd(_p(gu), _p(au), _p(iu), _p(mu), N, D, H, W, c, acc, _s()) == 0
        _same(ia, iu)


@pytest.mark.parametrize("c", [16, 64])
def test_upsample_and_its_gradient_vector_equals_elementwise(c):
    import torch
    L = _lib()
    torch.manual_seed(c + 1)
    d, h, w = D // 2, H // 2, W // 2
    x = torch.randn(N, d, h, w, c)
    xa, xu = _pair(x, (N, d, h, w, c), torch.bfloat16)
    oa = torch.empty(N, D, H, W, c, dtype=torch.bfloat16, device="cuda")
    ou = torch.zeros((oa.numel() + 1,), dtype=torch.bfloat16, device="cuda")[1:].view(oa.shape)
    assert L.lbm_nn_upsample2(_p(xa), _p(oa), N, d, h, w, c, _s()) == 0
    assert L.lbm_nn_upsample2(_p(xu), _p(ou), N, d, h, w, c, _s()) == 0
    _same(oa, ou)
    g = torch.randn(N, D, H, W, c)
    ga, gu = _pair(g, (N, D, H, W, c), torch.bfloat16)
    m = torch.randn(N, d, h, w, c)
    ma, mu = _pair(m, (N, d, h, w, c), torch.bfloat16)
    ia = torch.empty(N, d, h, w, c, dtype=torch.bfloat16, device="cuda")
    iu = torch.zeros((ia.numel() + 1,), dtype=torch.bfloat16, device="cuda")[1:].view(ia.shape)
    assert L.lbm_nn_upsample2_bwd(_p(ga), _p(ia), _p(ma), N, d, h, w, c, _s()) == 0
    assert L.lbm_nn_upsample2_bwd(_p(gu), _p(iu), _p(mu), N, d, h, w, c, _s()) == 0
    _same(ia, iu)


@pytest.mark.parametrize("ca,cb", [(32, 16), (64, 32)])
def test_concat_and_split_vector_equals_elementwise(ca, cb):
    import torch
    L = _lib()
    torch.manual_seed(ca + cb)
    nv = N * D * H * W
    a = torch.randn(nv, ca)
    b = torch.randn(nv, cb)
    aa, au = _pair(a, (nv, ca), torch.bfloat16)
    ba, bu = _pair(b, (nv, cb), torch.bfloat16)
    oa = torch.empty(nv, ca + cb, dtype=torch.bfloat16, device="cuda")
    ou = torch.zeros((oa.numel() + 1,), dtype=torch.bfloat16, device="cuda")[1:].view(oa.shape)
    assert L.lbm_nn_concat(_p(aa), ca, _p(ba), cb, _p(oa), nv, _s()) == 0
    assert L.lbm_nn_concat(_p(au), ca, _p(bu), cb, _p(ou), nv, _s()) == 0
    _same(oa, ou)
    torch.cuda.synchronize()
    assert torch.equal(oa[:, :ca], aa) and torch.equal(oa[:, ca:], ba)
    g = torch.randn(nv, ca + cb)
    gA, gU = _pair(g, (nv, ca + cb), torch.bfloat16)
    m = torch.randn(nv, cb)
    ma, mu = _pair(m, (nv, cb), torch.bfloat16)
    prev = torch.randn(nv, cb)
    for acc in (0, 1):
        xa = torch.empty(nv, ca, dtype=torch.bfloat16, device="cuda")
        xu = torch.zeros((xa.numel() + 1,), dtype=torch.bfloat16, device="cuda")[1:].view(xa.shape)
        ya, yu = _pair(prev, (nv, cb), torch.bfloat16)
        assert L.lbm_nn_split(_p(gA), ca, cb, _p(xa), _p(ya), _p(ma), acc, nv, _s()) == 0
        assert L.lbm_nn_split(_p(gU), ca, cb, _p(xu), _p(yu), _p(mu), acc, nv, _s()) == 0
        _same(xa, xu)
        _same(ya, yu)


def test_head_weight_gradient_one_pass_matches_fp64_and_general_form():
    import torch
    L = _lib()
    torch.manual_seed(7)
    nv, cin, cout = 50_000, 16, 4
    gy = torch.randn(nv, cout, device="cuda")
    w = torch.randn(cout, cin, device="cuda")
    x = torch.randn(nv, cin)
    xa, xu = _pair(x, (nv, cin), torch.bfloat16)
    scr = torch.empty(256 * (cout * cin + cout), device="cuda")
    gx = torch.empty(nv, cin, dtype=torch.bfloat16, device="cuda")
    out = []
    for xx in (xa, xu):
        dwdb = torch.empty(cout * cin + cout, device="cuda")
        assert L.lbm_nn_head_bwd_act(_p(gy), _p(w), _p(xx), None, _p(gx), _p(dwdb), _p(scr), nv, cin, cout, 0,
                                     _s()) == 0
        torch.cuda.synchronize()
        out.append(dwdb.cpu().numpy().astype(np.float64))
    g64 = gy.cpu().numpy().astype(np.float64)
    x64 = xa.float().cpu().numpy().astype(np.float64)
    ref = np.concatenate([(g64.T @ x64).reshape(-1), g64.sum(axis=0)])
    for o in out:
        assert np.abs(o - ref).max() / np.abs(ref).max() < 1e-5
    assert np.abs(out[0] - out[1]).max() / np.abs(ref).max() < 1e-5

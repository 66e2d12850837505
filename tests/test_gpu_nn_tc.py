"""Tensor-core (tcgen05) 3x3x3 convolution against an FP64 numpy reference,
for the channel counts of the network, all four epilogue modes (ReLU and GELU
forward, their backward-data factors), and a voxel count that
leaves a partial 128-voxel tile; the pipeline's timeout flag stays clear."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (96, 32), (48, 16), (32, 96), (16, 48), (64, 32)]


def ref_conv(x, w, b, mask, mode):
    """x (D,H,W,cin), w (cout,27,cin); FP64.  Returns (out, pre-activation)."""
    from oracle.unet_oracle import conv_fwd, gelu, gelu_grad
    y = conv_fwd(x, w, np.zeros(w.shape[0]) if b is None else b)
    if mode == 0:
        return np.maximum(y, 0.0), y
    if mode == 2:
        return gelu(y), y
    if mask is None:
        return y, y
    return (y * (mask > 0) if mode == 1 else y * gelu_grad(mask)), y


@pytest.mark.parametrize("cin,cout", SHAPES)
@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_tc_conv_matches_reference(cin, cout, mode):
    """Modes: 0 relu(conv + b), 1 conv * (mask > 0), 2 gelu(conv + b) with the
    pre-activation written, 3 conv * gelu'(mask)."""
    import torch
    from taichi_lbm3d_gb300 import unet
    L = unet._lib()
    rng = np.random.default_rng(cin * 131 + cout + mode)
    D, H, W = 5, 7, 11                       # 385 voxels: three full tiles and a partial one
    x = torch.from_numpy(rng.standard_normal((1, D, H, W, cin)).astype(np.float32)).to(torch.bfloat16)
    w = torch.from_numpy((rng.standard_normal((cout, 27, cin)) / np.sqrt(27 * cin)).astype(np.float32)).to(torch.bfloat16)
    b = torch.from_numpy(rng.standard_normal(cout).astype(np.float32) * 0.1)
    m = torch.from_numpy(rng.standard_normal((1, D, H, W, cout)).astype(np.float32)).to(torch.bfloat16)
    xg, wg, bg, mg = x.cuda().contiguous(), w.cuda().contiguous(), b.cuda(), m.cuda().contiguous()
    out_tc = torch.zeros((1, D, H, W, cout), dtype=torch.bfloat16, device="cuda")
    pre_tc = torch.zeros((1, D, H, W, cout), dtype=torch.bfloat16, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    fwd = mode in (0, 2)
    if mode < 2:
        rc = L.lbm_nn_conv3d(p(xg), p(wg), p(bg) if fwd else None, None if fwd else p(mg), p(out_tc),
                             1, D, H, W, cin, cout, mode, ctypes.c_void_p(s))
    else:
        rc = L.lbm_nn_conv3d_act(p(xg), p(wg), p(bg) if fwd else None, None if fwd else p(mg), p(out_tc),
                                 p(pre_tc) if mode == 2 else None, 1, D, H, W, cin, cout, mode, ctypes.c_void_p(s))
    assert rc == 0
    torch.cuda.synchronize()
    flag = ctypes.c_int32(7)
    assert L.lbm_nn_tc_status(ctypes.byref(flag)) == 0 and flag.value == 0
    y = out_tc.float().cpu().numpy()[0].astype(np.float64)
    r, r_pre = ref_conv(x.float().numpy()[0].astype(np.float64), w.float().numpy().astype(np.float64),
                        b.numpy().astype(np.float64) if fwd else None, m.float().numpy()[0].astype(np.float64), mode)
    err = np.abs(y - r).max() / max(np.abs(r).max(), 1e-30)
    assert err < 1e-2, err
    if mode == 2:
        y_pre = pre_tc.float().cpu().numpy()[0].astype(np.float64)
        e_pre = np.abs(y_pre - r_pre).max() / max(np.abs(r_pre).max(), 1e-30)
        assert e_pre < 1e-2, e_pre


@pytest.mark.parametrize("cin,cout", [(16, 16), (16, 32), (32, 64), (64, 64), (96, 32), (48, 16), (32, 32)])
def test_tc_weight_gradient_matches_reference(cin, cout):
    """dw[co][tap][ci] = sum_v g[v][co] x[v + off(tap)][ci] and db = sum_v g,
    against FP64 on a volume whose voxel count is not a multiple of the
    4096-voxel chunk."""
    import torch
    from oracle.unet_oracle import conv_bwd
    from taichi_lbm3d_gb300 import unet
    L = unet._lib()
    rng = np.random.default_rng(cin * 7 + cout)
    D, H, W = 9, 23, 25                      # 5175 voxels: one full chunk and a partial one
    x = torch.from_numpy(rng.standard_normal((1, D, H, W, cin)).astype(np.float32)).to(torch.bfloat16)
    g = torch.from_numpy(rng.standard_normal((1, D, H, W, cout)).astype(np.float32)).to(torch.bfloat16)
    xg, gg = x.cuda().contiguous(), g.cuda().contiguous()
    dw = torch.zeros((cout, 27, cin), device="cuda")
    db = torch.zeros(cout, device="cuda")
    nscr = L.lbm_nn_wgrad_scratch_floats(1, D, H, W, cin, cout)
    scr = torch.empty(int(nscr), device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.lbm_nn_conv3d_wgrad(p(xg), p(gg), p(dw), p(db), p(scr), scr.numel(), 1, D, H, W, cin, cout, s) == 0
    torch.cuda.synchronize()
    flag = ctypes.c_int32(7)
    assert L.lbm_nn_tc_status(ctypes.byref(flag)) == 0 and flag.value == 0
    _, dw_ref, db_ref = conv_bwd(x.float().numpy()[0].astype(np.float64), np.zeros((cout, 27, cin)),
                                 g.float().numpy()[0].astype(np.float64))
    e_w = np.abs(dw.cpu().numpy() - dw_ref).max() / np.abs(dw_ref).max()
    e_b = np.abs(db.cpu().numpy() - db_ref).max() / np.abs(db_ref).max()
    assert e_w < 1e-4 and e_b < 1e-4, (e_w, e_b)


def test_tc_wait_timeout_sets_the_flag_and_keeps_the_context():
    """The bounded mbarrier wait gives up on a phase that nothing completes,
    records it, frees its tensor memory and returns; later work still runs."""
    import torch
    from taichi_lbm3d_gb300 import unet
    L = unet._lib()
    flag = ctypes.c_int32(0)
    assert L.lbm_nn_tc_status(ctypes.byref(flag)) == 0          # clear
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.lbm_nn_tc_timeout_selftest(s) == 0
    assert L.lbm_nn_tc_status(ctypes.byref(flag)) == 0 and flag.value == 1
    assert L.lbm_nn_tc_status(ctypes.byref(flag)) == 0 and flag.value == 0   # cleared by the read
    test_tc_conv_matches_reference(16, 16, 0)                               # the context still works

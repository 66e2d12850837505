"""3D U-Net warm start for the porous-flow solver.

The network maps (fluid indicator, distance to solid) on a cubic subvolume to
the steady (vx, vy, vz, rho - 1) field; the solver then starts from
f = feq(rho, v) instead of rest (``LB3D_Solver_Single_Phase.init_simulation(rho, v)``)
and runs to the same convergence criterion, so it judges the prediction and
falls back to plain iteration where the prediction is poor.

Architecture (3 levels, channels 16/32/64): two 3x3x3 conv + activation per
level (ReLU, or the exact GELU with ``activation="gelu"``), 2x max-pool down, 2x
nearest upsample + skip concat up, 1x1 head to 4 outputs.
Forward and backward run entirely in the project's CUDA kernels
(csrc/nn_unet.cu, C ABI include/lbm_nn.h); torch provides device memory and the
stream only.  Weights are kept in FP32 (Adam master copy) and used in BF16.
"""
import ctypes

import numpy as np

from . import _native

# name, input channels, output channels, level (0 = full resolution)
LAYERS = [("e1", 16, 16, 0), ("e1b", 16, 16, 0), ("e2", 16, 32, 1), ("e2b", 32, 32, 1), ("b1", 32, 64, 2),
          ("b1b", 64, 64, 2), ("d2", 96, 32, 1), ("d2b", 32, 32, 1), ("d1", 48, 16, 0), ("d1b", 16, 16, 0)]
IN_REAL = 2          # channels of the input that carry data (the rest of the 16 are zero)
OUT = 4

_P = ctypes.c_void_p
_I = ctypes.c_int32
_L = ctypes.c_int64
_F = ctypes.c_float
_SIGS = {
    "lbm_nn_conv3d": ([_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _P], ctypes.c_int),
    "lbm_nn_conv3d_act": ([_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _P], ctypes.c_int),
    "lbm_nn_head_bwd_act": ([_P, _P, _P, _P, _P, _P, _P, _L, _I, _I, _I, _P], ctypes.c_int),
    "lbm_nn_act_bwd": ([_P, _P, _L, _I, _P], ctypes.c_int),
    "lbm_nn_tc_status": ([_P], ctypes.c_int),
    "lbm_nn_tc_timeout_selftest": ([_P], ctypes.c_int),
    "lbm_nn_flip_transpose": ([_P, _P, _I, _I, _P], ctypes.c_int),
    "lbm_nn_wgrad_scratch_floats": ([_I, _I, _I, _I, _I, _I], ctypes.c_int64),
    "lbm_nn_conv3d_wgrad": ([_P, _P, _P, _P, _P, _L, _I, _I, _I, _I, _I, _I, _P], ctypes.c_int),
    "lbm_nn_pool2": ([_P, _P, _P, _I, _I, _I, _I, _I, _P], ctypes.c_int),
    "lbm_nn_pool2_bwd": ([_P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _P], ctypes.c_int),
    "lbm_nn_upsample2": ([_P, _P, _I, _I, _I, _I, _I, _P], ctypes.c_int),
    "lbm_nn_upsample2_bwd": ([_P, _P, _P, _I, _I, _I, _I, _I, _P], ctypes.c_int),
    "lbm_nn_concat": ([_P, _I, _P, _I, _P, _L, _P], ctypes.c_int),
    "lbm_nn_split": ([_P, _I, _I, _P, _P, _P, _I, _L, _P], ctypes.c_int),
    "lbm_nn_head": ([_P, _P, _P, _P, _L, _I, _I, _P], ctypes.c_int),
    "lbm_nn_head_bwd": ([_P, _P, _P, _P, _P, _P, _L, _I, _I, _P], ctypes.c_int),
    "lbm_nn_mse": ([_P, _P, _P, _P, _P, _P, _L, _I, _F, _P], ctypes.c_int),
    "lbm_nn_adam": ([_P, _P, _P, _P, _P, _L, _F, _F, _F, _F, _I, _F, _P], ctypes.c_int),
}


def _lib():
    L = _native.load()
    if not getattr(L, "_nn_bound", False):
        for n, (a, r) in _SIGS.items():
            f = getattr(L, n)
            f.argtypes = a
            f.restype = r
        L._nn_bound = True
    return L


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _ck(rc):
    if rc != 0:
        raise _native.LbmError(rc, _native.last_error())


ACTIVATIONS = {"relu": 0, "gelu": 1}


class UNet3D:
    def __init__(self, seed=0, activation="relu"):
        import torch
        if activation not in ACTIVATIONS:
            raise ValueError("activation must be 'relu' or 'gelu'")
        self.torch = torch
        self.activation = activation
        g = torch.Generator().manual_seed(seed)
        self.w, self.b, self.w16, self.wt16 = {}, {}, {}, {}
        self.params = []          # (name, master, grad, m, v, bf16 copy or None)
        for name, cin, cout, _ in LAYERS:
            real = IN_REAL if name == "e1" else cin
            std = (2.0 / (27 * real)) ** 0.5
            w = torch.zeros(cout, 27, cin)
            w[:, :, :real] = torch.randn(cout, 27, real, generator=g) * std
            self.w[name] = w.cuda().contiguous()
            self.b[name] = torch.zeros(cout, device="cuda")
            self.w16[name] = torch.empty(cout, 27, cin, dtype=torch.bfloat16, device="cuda")
            self.wt16[name] = torch.empty(cin, 27, cout, dtype=torch.bfloat16, device="cuda")
        self.hw = (torch.randn(OUT, 16, generator=g) * (1.0 / 4.0)).cuda()
        self.hb = torch.zeros(OUT, device="cuda")
        self.gw = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.gb = {k: torch.zeros_like(v) for k, v in self.b.items()}
        self.ghw_hb = torch.zeros(OUT * 16 + OUT, device="cuda")
        self.adam = {}
        self.step_count = 0
        self.scales = np.ones(OUT, np.float32)     # target normalisation (set by training data)
        self.refresh()

    # ----------------------------------------------------------- parameters
    def n_params(self):
        n = sum(int(LAYERS[i][2]) * 27 * (IN_REAL if LAYERS[i][0] == "e1" else LAYERS[i][1]) + LAYERS[i][2]
                for i in range(len(LAYERS)))
        return n + OUT * 16 + OUT

    def _stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def refresh(self):
        """BF16 copies and flip-transposed backward weights from the masters."""
        L = _lib()
        for name, cin, cout, _ in LAYERS:
            self.w16[name].copy_(self.w[name].to(self.torch.bfloat16))
            _ck(L.lbm_nn_flip_transpose(_p(self.w16[name]), _p(self.wt16[name]), cin, cout, self._stream()))

    def state_dict(self):
        d = {"w_" + k: v.cpu().numpy() for k, v in self.w.items()}
        d.update({"b_" + k: v.cpu().numpy() for k, v in self.b.items()})
        d["hw"] = self.hw.cpu().numpy()
        d["hb"] = self.hb.cpu().numpy()
        d["scales"] = self.scales
        d["activation"] = np.array(ACTIVATIONS[self.activation], np.int32)
        return d

    def load_state_dict(self, d):
        for k in self.w:
            self.w[k].copy_(self.torch.from_numpy(np.asarray(d["w_" + k])))
            self.b[k].copy_(self.torch.from_numpy(np.asarray(d["b_" + k])))
        self.hw.copy_(self.torch.from_numpy(np.asarray(d["hw"])))
        self.hb.copy_(self.torch.from_numpy(np.asarray(d["hb"])))
        self.scales = np.asarray(d["scales"], np.float32)
        if "activation" in d:
            code = int(np.asarray(d["activation"]))
            self.activation = next(k for k, v in ACTIVATIONS.items() if v == code)
        self.refresh()

    # ----------------------------------------------------------- forward
    def _buf(self, key, shape, dtype):
        t = self.torch
        b = self._bufs.get(key)
        if b is None or tuple(b.shape) != tuple(shape) or b.dtype != dtype:
            b = t.empty(*shape, dtype=dtype, device="cuda")
            self._bufs[key] = b
        return b

    def forward(self, x16):
        """x16: (N, D, H, W, 16) bf16 cuda tensor.  Returns y (N, D, H, W, 4) fp32."""
        t = self.torch
        L = _lib()
        s = self._stream()
        if not hasattr(self, "_bufs"):
            self._bufs = {}
        N, D, H, W, _ = x16.shape
        dims = {0: (N, D, H, W), 1: (N, D // 2, H // 2, W // 2), 2: (N, D // 4, H // 4, W // 4)}
        a = {"x": x16}

        gelu = self.activation == "gelu"

        def conv(name, src):
            _, cin, cout, lv = next(l for l in LAYERS if l[0] == name)
            out = self._buf("a_" + name, dims[lv] + (cout,), t.bfloat16)
            pre = self._buf("pre_" + name, dims[lv] + (cout,), t.bfloat16) if gelu else None
            _ck(L.lbm_nn_conv3d_act(_p(src), _p(self.w16[name]), _p(self.b[name]), None, _p(out), _p(pre),
                                    *dims[lv], cin, cout, 2 if gelu else 0, s))
            a[name] = out
            if gelu:
                a["pre_" + name] = pre
            return out

        def pool(name, src, lv, c):
            out = self._buf("a_" + name, dims[lv + 1] + (c,), t.bfloat16)
            arg = self._buf("arg_" + name, dims[lv + 1] + (c,), t.uint8)
            _ck(L.lbm_nn_pool2(_p(src), _p(out), _p(arg), *dims[lv], c, s))
            a[name] = out
            a["arg_" + name] = arg
            return out

        def up_cat(name, src, lv_low, c, skip, cs):
            up = self._buf("up_" + name, dims[lv_low - 1] + (c,), t.bfloat16)
            _ck(L.lbm_nn_upsample2(_p(src), _p(up), *dims[lv_low], c, s))
            cat = self._buf("a_" + name, dims[lv_low - 1] + (c + cs,), t.bfloat16)
            nv = int(np.prod(dims[lv_low - 1]))
            _ck(L.lbm_nn_concat(_p(up), c, _p(skip), cs, _p(cat), nv, s))
            a[name] = cat
            return cat

        conv("e1", x16)
        conv("e1b", a["e1"])
        pool("p1", a["e1b"], 0, 16)
        conv("e2", a["p1"])
        conv("e2b", a["e2"])
        pool("p2", a["e2b"], 1, 32)
        conv("b1", a["p2"])
        conv("b1b", a["b1"])
        up_cat("c2", a["b1b"], 2, 64, a["e2b"], 32)
        conv("d2", a["c2"])
        conv("d2b", a["d2"])
        up_cat("c1", a["d2b"], 1, 32, a["e1b"], 16)
        conv("d1", a["c1"])
        conv("d1b", a["d1"])
        y = self._buf("y", dims[0] + (OUT,), t.float32)
        _ck(L.lbm_nn_head(_p(a["d1b"]), _p(self.hw), _p(self.hb), _p(y), int(np.prod(dims[0])), 16, OUT, s))
        self._a, self._dims = a, dims
        return y

    # ----------------------------------------------------------- backward
    def backward(self, gy):
        """gy: dLoss/dy (N, D, H, W, 4) fp32.  Fills the parameter gradients."""
        t = self.torch
        L = _lib()
        s = self._stream()
        a, dims = self._a, self._dims
        nv0 = int(np.prod(dims[0]))
        gelu = self.activation == "gelu"
        act = ACTIVATIONS[self.activation]

        def dmask(name):
            """What the masked kernels multiply by: ReLU -> the activation (factor > 0),
            GELU -> the pre-activation (factor gelu')."""
            return a["pre_" + name] if gelu else a[name]

        def act_bwd(g, name):
            """GELU only: the pooling/upsampling backward kernels know the ReLU mask
            alone, so their GELU factor is applied by a separate pass."""
            if gelu:
                _ck(L.lbm_nn_act_bwd(_p(g), _p(a["pre_" + name]), g.numel(), act, s))

        def g_buf(name, lv, c):
            return self._buf("g_" + name, dims[lv] + (c,), t.bfloat16)

        def wgrad(name, src, g):
            _, cin, cout, lv = next(l for l in LAYERS if l[0] == name)
            need = int(L.lbm_nn_wgrad_scratch_floats(*dims[lv], cin, cout))
            scr = self._bufs.get("wg_scratch")
            if scr is None or scr.numel() < need:
                scr = t.empty(max(need, 1), dtype=t.float32, device="cuda")
                self._bufs["wg_scratch"] = scr
            _ck(L.lbm_nn_conv3d_wgrad(_p(src), _p(g), _p(self.gw[name]), _p(self.gb[name]), _p(scr), scr.numel(),
                                      *dims[lv], cin, cout, s))

        def bwd_data(name, g, mask, out_key):
            _, cin, cout, lv = next(l for l in LAYERS if l[0] == name)
            out = g_buf(out_key, lv, cin)
            _ck(L.lbm_nn_conv3d_act(_p(g), _p(self.wt16[name]), None, _p(mask), _p(out), None, *dims[lv], cout, cin,
                                    3 if gelu else 1, s))
            return out

        # head
        g_d1b = g_buf("d1b", 0, 16)
        hs = self._buf("head_scratch", (256 * (OUT * 16 + OUT),), t.float32)
        _ck(L.lbm_nn_head_bwd_act(_p(gy), _p(self.hw), _p(a["d1b"]), _p(a.get("pre_d1b")), _p(g_d1b),
                                  _p(self.ghw_hb), _p(hs), nv0, 16, OUT, act, s))
        # level 0 decoder
        wgrad("d1b", a["d1"], g_d1b)
        g_d1 = bwd_data("d1b", g_d1b, dmask("d1"), "d1")
        wgrad("d1", a["c1"], g_d1)
        g_c1 = bwd_data("d1", g_d1, None, "c1")
        g_u1 = g_buf("u1", 0, 32)
        g_e1b = g_buf("e1b", 0, 16)
        _ck(L.lbm_nn_split(_p(g_c1), 32, 16, _p(g_u1), _p(g_e1b), None, 0, nv0, s))
        g_d2b = g_buf("d2b", 1, 32)
        _ck(L.lbm_nn_upsample2_bwd(_p(g_u1), _p(g_d2b), None if gelu else _p(a["d2b"]), *dims[1], 32, s))
        act_bwd(g_d2b, "d2b")
        # level 1 decoder
        wgrad("d2b", a["d2"], g_d2b)
        g_d2 = bwd_data("d2b", g_d2b, dmask("d2"), "d2")
        wgrad("d2", a["c2"], g_d2)
        g_c2 = bwd_data("d2", g_d2, None, "c2")
        nv1 = int(np.prod(dims[1]))
        g_u2 = g_buf("u2", 1, 64)
        g_e2b = g_buf("e2b", 1, 32)
        _ck(L.lbm_nn_split(_p(g_c2), 64, 32, _p(g_u2), _p(g_e2b), None, 0, nv1, s))
        g_b1b = g_buf("b1b", 2, 64)
        _ck(L.lbm_nn_upsample2_bwd(_p(g_u2), _p(g_b1b), None if gelu else _p(a["b1b"]), *dims[2], 64, s))
        act_bwd(g_b1b, "b1b")
        # bottleneck
        wgrad("b1b", a["b1"], g_b1b)
        g_b1 = bwd_data("b1b", g_b1b, dmask("b1"), "b1")
        wgrad("b1", a["p2"], g_b1)
        g_p2 = bwd_data("b1", g_b1, None, "p2")
        _ck(L.lbm_nn_pool2_bwd(_p(g_p2), _p(a["arg_p2"]), _p(g_e2b), None if gelu else _p(a["e2b"]), *dims[1], 32,
                               1, s))
        act_bwd(g_e2b, "e2b")
        # level 1 encoder
        wgrad("e2b", a["e2"], g_e2b)
        g_e2 = bwd_data("e2b", g_e2b, dmask("e2"), "e2")
        wgrad("e2", a["p1"], g_e2)
        g_p1 = bwd_data("e2", g_e2, None, "p1")
        _ck(L.lbm_nn_pool2_bwd(_p(g_p1), _p(a["arg_p1"]), _p(g_e1b), None if gelu else _p(a["e1b"]), *dims[0], 16,
                               1, s))
        act_bwd(g_e1b, "e1b")
        # level 0 encoder
        wgrad("e1b", a["e1"], g_e1b)
        g_e1 = bwd_data("e1b", g_e1b, dmask("e1"), "e1")
        wgrad("e1", a["x"], g_e1)

    def grads(self):
        """Parameter gradients as numpy arrays (FP32), keyed like state_dict."""
        d = {"w_" + k: v.cpu().numpy() for k, v in self.gw.items()}
        d.update({"b_" + k: v.cpu().numpy() for k, v in self.gb.items()})
        hw_hb = self.ghw_hb.cpu().numpy()
        d["hw"] = hw_hb[:OUT * 16].reshape(OUT, 16)
        d["hb"] = hw_hb[OUT * 16:]
        return d

    # ----------------------------------------------------------- loss, optimiser
    def loss(self, y, target, mask, count):
        """Masked MSE over `count` (voxel, channel) entries; returns (loss tensor, gy)."""
        t = self.torch
        L = _lib()
        gy = self._buf("gy", tuple(y.shape), t.float32)
        loss = self._buf("loss", (1,), t.float32)
        scr = self._buf("mse_scratch", (256,), t.float32)
        nv = int(np.prod(y.shape[:-1]))
        _ck(L.lbm_nn_mse(_p(y), _p(target), _p(mask), _p(gy), _p(loss), _p(scr), nv, OUT, 1.0 / count,
                         self._stream()))
        return loss, gy

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, weight_decay=0.0):
        L = _lib()
        s = self._stream()
        self.step_count += 1
        hw_hb_g = self.ghw_hb
        items = [(self.w[k], self.gw[k], None) for k in self.w] + [(self.b[k], self.gb[k], None) for k in self.b]
        items += [(self.hw, hw_hb_g[:OUT * 16].view(OUT, 16), None), (self.hb, hw_hb_g[OUT * 16:], None)]
        for p, g, _ in items:
            key = p.data_ptr()
            if key not in self.adam:
                self.adam[key] = (self.torch.zeros_like(p), self.torch.zeros_like(p))
            m, v = self.adam[key]
            _ck(L.lbm_nn_adam(_p(p), _p(g.contiguous()), _p(m), _p(v), None, p.numel(), lr, b1, b2, eps,
                              self.step_count, weight_decay, s))
        self.refresh()


def features(solid):
    """Network input of a solid mask (nx, ny, nz): channel 0 = fluid indicator,
    channel 1 = distance to solid / 8, channels 2..15 = 0; shape (D=nz, H=ny, W=nx, 16)
    (the network's channels-last order is z, y, x)."""
    from .geometry import distance_to_solid
    fluid = (np.asarray(solid) == 0).astype(np.float32)
    dist = distance_to_solid(solid) / 8.0
    x = np.zeros(solid.shape[::-1] + (16,), np.float32)
    x[..., 0] = fluid.transpose(2, 1, 0)
    x[..., 1] = dist.transpose(2, 1, 0)
    return x


def targets(rho, v, scales):
    """Network target (D, H, W, 4) from the solver's dense rho, v: (vx, vy, vz, rho - 1) / scales."""
    t = np.zeros(rho.shape[::-1] + (OUT,), np.float32)
    for c in range(3):
        t[..., c] = v[..., c].transpose(2, 1, 0) / scales[c]
    t[..., 3] = (rho - 1.0).transpose(2, 1, 0) / scales[3]
    return t


def fields_from_output(y, scales):
    """Inverse of targets(): dense rho (nx,ny,nz) and v (nx,ny,nz,3) from y (D,H,W,4)."""
    y = np.asarray(y)
    v = np.stack([(y[..., c] * scales[c]).transpose(2, 1, 0) for c in range(3)], axis=-1)
    rho = 1.0 + (y[..., 3] * scales[3]).transpose(2, 1, 0)
    return rho.astype(np.float32), v.astype(np.float32)

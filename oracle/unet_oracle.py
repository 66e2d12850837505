"""FP64 CPU oracle of the warm-start U-Net (forward and hand-written backward).

TEST INFRASTRUCTURE ONLY: the GPU network's gradient check compares the
project's CUDA forward/backward kernels against this restatement (same
architecture and parameter layout as taichi_lbm3d_gb300/unet.py, numpy FP64,
no autograd).  tests/test_unet_oracle.py checks this backward against central
finite differences.

Tensors are channels last (D, H, W, C) for one sample; conv weights are
[cout][27][cin] with tap = (dz+1)*9 + (dy+1)*3 + (dx+1), zero padding.
"""
import numpy as np

LAYERS = [("e1", 16, 16, 0), ("e1b", 16, 16, 0), ("e2", 16, 32, 1), ("e2b", 32, 32, 1), ("b1", 32, 64, 2),
          ("b1b", 64, 64, 2), ("d2", 96, 32, 1), ("d2b", 32, 32, 1), ("d1", 48, 16, 0), ("d1b", 16, 16, 0)]
TAPS = [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]


def _shift(xp, dz, dy, dx, D, H, W):
    return xp[1 + dz:1 + dz + D, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W]


def conv_fwd(x, w, b):
    D, H, W, _ = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((D, H, W, w.shape[0]))
    for t, (dz, dy, dx) in enumerate(TAPS):
        out += _shift(xp, dz, dy, dx, D, H, W) @ w[:, t, :].T
    return out + b


def conv_bwd(x, w, g):
    """g: dL/d(pre-activation output).  Returns (dx, dw, db)."""
    D, H, W, _ = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    dxp = np.zeros_like(xp)
    dw = np.zeros_like(w)
    gf = g.reshape(-1, g.shape[-1])
    for t, (dz, dy, dx) in enumerate(TAPS):
        sh = _shift(xp, dz, dy, dx, D, H, W)
        dw[:, t, :] = gf.T @ sh.reshape(-1, sh.shape[-1])
        dxp[1 + dz:1 + dz + D, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W] += g @ w[:, t, :]
    return dxp[1:-1, 1:-1, 1:-1], dw, gf.sum(axis=0)


def pool_fwd(x):
    D, H, W, C = x.shape
    best = np.full((D // 2, H // 2, W // 2, C), -np.inf)
    arg = np.zeros((D // 2, H // 2, W // 2, C), np.int64)
    for k in range(8):
        v = x[(k >> 2)::2, ((k >> 1) & 1)::2, (k & 1)::2]
        upd = v > best
        best = np.where(upd, v, best)
        arg = np.where(upd, k, arg)
    return best, arg


def pool_bwd(g, arg, shape):
    out = np.zeros(shape)
    for k in range(8):
        out[(k >> 2)::2, ((k >> 1) & 1)::2, (k & 1)::2] = np.where(arg == k, g, 0.0)
    return out


def up_fwd(x):
    return x.repeat(2, 0).repeat(2, 1).repeat(2, 2)


def up_bwd(g):
    D, H, W, C = g.shape
    return g.reshape(D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(1, 3, 5))


def relu(x):
    return np.maximum(x, 0.0)


def _erf(x):
    from scipy.special import erf
    return erf(x)


def gelu(x):
    """Exact GELU, x * Phi(x) = x/2 (1 + erf(x / sqrt 2))."""
    return 0.5 * x * (1.0 + _erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    """d gelu / dx = Phi(x) + x phi(x)."""
    return 0.5 * (1.0 + _erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def act_fwd(x, act):
    return relu(x) if act == "relu" else gelu(x)


def act_grad(pre, act):
    return (pre > 0).astype(np.float64) if act == "relu" else gelu_grad(pre)


def forward(P, x, act="relu"):
    """P: parameter dict (w_<name>, b_<name>, hw, hb) as FP64 arrays; x (D,H,W,16);
    act: "relu" or "gelu" after every 3x3x3 convolution."""
    a = {"x": x}

    def conv(name, src):
        a["pre_" + name] = conv_fwd(src, P["w_" + name], P["b_" + name])
        a[name] = act_fwd(a["pre_" + name], act)
        return a[name]

    conv("e1", x)
    conv("e1b", a["e1"])
    a["p1"], a["arg1"] = pool_fwd(a["e1b"])
    conv("e2", a["p1"])
    conv("e2b", a["e2"])
    a["p2"], a["arg2"] = pool_fwd(a["e2b"])
    conv("b1", a["p2"])
    conv("b1b", a["b1"])
    a["c2"] = np.concatenate([up_fwd(a["b1b"]), a["e2b"]], axis=-1)
    conv("d2", a["c2"])
    conv("d2b", a["d2"])
    a["c1"] = np.concatenate([up_fwd(a["d2b"]), a["e1b"]], axis=-1)
    conv("d1", a["c1"])
    conv("d1b", a["d1"])
    y = a["d1b"] @ P["hw"].T + P["hb"]
    return y, a


def loss_and_grads(P, x, target, mask, act="relu"):
    """Masked MSE (mean over mask voxels x 4 channels) and its gradient w.r.t. every parameter."""
    y, a = forward(P, x, act)

    def dact(name):
        return act_grad(a["pre_" + name], act)

    m = mask[..., None].astype(np.float64)
    count = float(mask.sum()) * y.shape[-1]
    d = (y - target) * m
    loss = float((d * d).sum() / count)
    gy = 2.0 * d / count
    G = {}
    G["hw"] = gy.reshape(-1, gy.shape[-1]).T @ a["d1b"].reshape(-1, 16)
    G["hb"] = gy.reshape(-1, gy.shape[-1]).sum(axis=0)
    g = (gy @ P["hw"]) * dact("d1b")

    def back(name, src, g):
        dx, G["w_" + name], G["b_" + name] = conv_bwd(src, P["w_" + name], g)
        return dx

    g = back("d1b", a["d1"], g) * dact("d1")
    g_c1 = back("d1", a["c1"], g)
    g_d2b = up_bwd(g_c1[..., :32]) * dact("d2b")
    g_e1b_skip = g_c1[..., 32:]
    g = back("d2b", a["d2"], g_d2b) * dact("d2")
    g_c2 = back("d2", a["c2"], g)
    g_b1b = up_bwd(g_c2[..., :64]) * dact("b1b")
    g_e2b_skip = g_c2[..., 64:]
    g = back("b1b", a["b1"], g_b1b) * dact("b1")
    g_p2 = back("b1", a["p2"], g)
    g_e2b = (pool_bwd(g_p2, a["arg2"], a["e2b"].shape) + g_e2b_skip) * dact("e2b")
    g = back("e2b", a["e2"], g_e2b) * dact("e2")
    g_p1 = back("e2", a["p1"], g)
    g_e1b = (pool_bwd(g_p1, a["arg1"], a["e1b"].shape) + g_e1b_skip) * dact("e1b")
    g = back("e1b", a["e1"], g_e1b) * dact("e1")
    back("e1", x, g)
    return loss, G, y


def random_params(seed, in_real=2):
    rng = np.random.default_rng(seed)
    P = {}
    for name, cin, cout, _ in LAYERS:
        real = in_real if name == "e1" else cin
        w = np.zeros((cout, 27, cin))
        w[:, :, :real] = rng.standard_normal((cout, 27, real)) * np.sqrt(2.0 / (27 * real))
        P["w_" + name] = w
        P["b_" + name] = rng.standard_normal(cout) * 0.05
    P["hw"] = rng.standard_normal((4, 16)) * 0.25
    P["hb"] = rng.standard_normal(4) * 0.05
    return P

"""The warm-start network's CUDA forward and backward kernels against the FP64
CPU oracle (oracle/unet_oracle.py) on a 16^3 sample.  The GPU keeps weights and
activations in BF16 (FP32 accumulation), so the comparison uses the same
BF16-rounded weights and input and a tolerance for BF16 activations."""
import numpy as np
import pytest

from oracle import unet_oracle as U

pytestmark = pytest.mark.gpu

Y_TOL = 1e-2       # normwise, forward output
G_TOL = 5e-2       # normwise, per parameter tensor
G_COS = 0.999      # cosine similarity, per parameter tensor


def bf16_round(a):
    import torch
    return torch.from_numpy(np.asarray(a, np.float32)).to(torch.bfloat16).to(torch.float64).numpy()


def case(seed=3, n=16):
    rng = np.random.default_rng(seed)
    P = U.random_params(seed)
    for k in list(P):
        if k.startswith("w_"):
            P[k] = bf16_round(P[k])
    x = np.zeros((n, n, n, 16))
    x[..., 0] = rng.random((n, n, n)) > 0.3
    x[..., 1] = bf16_round(rng.random((n, n, n)))
    t = rng.standard_normal((n, n, n, 4)).astype(np.float32)
    mask = (x[..., 0] > 0)
    return P, x, t, mask


def gpu_model(P, act="relu"):
    from taichi_lbm3d_gb300.unet import UNet3D
    m = UNet3D(seed=0, activation=act)
    d = {k: np.asarray(v, np.float32) for k, v in P.items()}
    d["scales"] = np.ones(4, np.float32)
    m.load_state_dict(d)
    return m


def to_gpu(x, t, mask):
    import torch
    xg = torch.from_numpy(np.asarray(x, np.float32)[None]).to(torch.bfloat16).cuda().contiguous()
    tg = torch.from_numpy(np.asarray(t, np.float32)[None]).cuda().contiguous()
    mg = torch.from_numpy(np.asarray(mask, np.uint8)[None]).cuda().contiguous()
    return xg, tg, mg


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("act", ["relu", "gelu"])
def test_forward_and_gradients_match_cpu_oracle(act):
    pytest.importorskip("scipy")
    P, x, t, mask = case()
    loss_ref, G_ref, y_ref = U.loss_and_grads(P, x, t, mask, act)
    m = gpu_model(P, act)
    xg, tg, mg = to_gpu(x, t, mask)
    y = m.forward(xg)
    loss, gy = m.loss(y, tg, mg, float(mask.sum()) * 4)
    m.backward(gy)
    y_gpu = y.cpu().numpy()[0]
    e_y = rel(y_gpu, y_ref)
    e_l = abs(float(loss.cpu().numpy()[0]) - loss_ref) / loss_ref
    G = m.grads()
    worst = []
    for k, ref in G_ref.items():
        g = np.asarray(G[k], np.float64)
        if k == "w_e1":
            g, ref = g[:, :, :2], ref[:, :, :2]
        e = rel(g, ref)
        cos = float((g * ref).sum() / (np.linalg.norm(g) * np.linalg.norm(ref) + 1e-30))
        worst.append((e, cos, k))
    print("%s forward %.3e loss %.3e worst grads %s" % (act, e_y, e_l, sorted(worst)[-3:]))
    assert e_y < Y_TOL and e_l < Y_TOL
    for e, cos, k in worst:
        assert e < G_TOL and cos > G_COS, (k, e, cos)


@pytest.mark.parametrize("act", ["relu", "gelu"])
def test_training_reduces_loss(act):
    P, x, t, mask = case(seed=4)
    m = gpu_model(P, act)
    xg, tg, mg = to_gpu(x, 0.1 * t, mask)
    losses = []
    for _ in range(40):
        y = m.forward(xg)
        loss, gy = m.loss(y, tg, mg, float(mask.sum()) * 4)
        m.backward(gy)
        m.adam_step(lr=3e-3)
        losses.append(float(loss.cpu().numpy()[0]))
    assert losses[-1] < 0.5 * losses[0], losses[::8]

"""The FP64 CPU oracle of the warm-start network: its hand-written backward
matches central finite differences (so it can check the GPU kernels)."""
import numpy as np
import pytest

from oracle import unet_oracle as U


def small_case(seed=0, n=8):
    rng = np.random.default_rng(seed)
    P = U.random_params(seed)
    x = np.zeros((n, n, n, 16))
    x[..., 0] = rng.random((n, n, n)) > 0.3
    x[..., 1] = rng.random((n, n, n))
    t = rng.standard_normal((n, n, n, 4))
    mask = x[..., 0] > 0
    return P, x, t, mask


@pytest.mark.parametrize("act", ["relu", "gelu"])
def test_backward_matches_finite_differences(act):
    pytest.importorskip("scipy")
    P, x, t, mask = small_case()
    loss, G, _ = U.loss_and_grads(P, x, t, mask, act)
    rng = np.random.default_rng(1)
    eps = 1e-6
    for key in ["w_e1", "w_e2b", "w_b1b", "b_d2", "w_d1", "b_d1b", "hw", "hb"]:
        arr = P[key]
        for _ in range(4):
            idx = tuple(rng.integers(0, s) for s in arr.shape)
            if key == "w_e1" and idx[2] >= 2:
                idx = idx[:2] + (int(idx[2]) % 2,)
            old = arr[idx]
            arr[idx] = old + eps
            lp = U.loss_and_grads(P, x, t, mask, act)[0]
            arr[idx] = old - eps
            lm = U.loss_and_grads(P, x, t, mask, act)[0]
            arr[idx] = old
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - G[key][idx]) <= 1e-6 * max(1.0, abs(fd)), (act, key, idx, fd, G[key][idx])

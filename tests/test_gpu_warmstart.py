"""What the trained warm-start network gains over the start from rest.

Held-out 96^3 packs of the training distribution (seeds 20000..20003; the
network was trained on seeds 10000..11999), body force fx = 1e-6, periodic,
FP32 deviation-form storage, convergence |dk/k| <= 1e-6 checked every 100
steps.  The network's (rho, v) initialise the populations at equilibrium and
the solver runs to the same criterion; the test pins the measured gain (fewer
steps on every pack, about 1.17x on these four, 1.11x over 16 held-out packs)
and the prediction errors (rho - 1 about 60% of its norm, v about 50%).

The gain is bounded by the density field: a start from the exact steady
velocity with rho = 1 saves about 4% of the steps, the exact steady density
with v = 0 about 30% and both about 2.7x (every 100 steps), so the network
would have to predict the pore-scale pressure field to within ~20-50% to save
1.5x; at its ~60% density error it saves ~10%.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEEDS = (20000, 20001, 20002, 20003)


def _steps(solid, rho=None, v=None):
    from taichi_lbm3d_gb300 import warmstart as W
    lb = W._solver(solid, "f32dev")
    lb.init_simulation(rho, v)
    r = lb.run_to_convergence(tol=1e-6, check_every=100)
    lb.close()
    assert r["converged"]
    return r["steps"]


def test_warm_start_takes_fewer_steps_than_rest():
    from taichi_lbm3d_gb300 import warmstart as W
    model = W.load_model()
    rest, warm = [], []
    for seed in SEEDS:
        solid, feat = W._pack_and_features((seed, 96))
        rho, v = W.predict(model, feat)
        fl = solid == 0
        assert abs(float(rho[fl].astype(np.float64).mean()) - 1.0) < 1e-6     # same mass as a start from rest
        rest.append(_steps(solid))
        warm.append(_steps(solid, rho, v))
    ratio = np.array(rest, float) / np.array(warm, float)
    print("rest", rest, "warm", warm, "ratio", ratio)
    assert all(w < r for w, r in zip(warm, rest))
    assert ratio.mean() >= 1.05


def test_prediction_errors_on_a_held_out_pack():
    from taichi_lbm3d_gb300 import warmstart as W
    model = W.load_model()
    solid, feat = W._pack_and_features((SEEDS[0], 96))
    lb = W._solver(solid, "f32dev")
    lb.init_simulation()
    lb.run_to_convergence(tol=1e-9, check_every=500)
    rho, v = [a.copy() for a in lb._macros()]
    lb.close()
    (e_rho, e_v), = W.field_errors(model, [solid], [feat], [(W.smooth_density(solid, rho), v)])
    print("smoothed rho error %.3f, v error %.3f" % (e_rho, e_v))
    assert e_rho < 0.8 and e_v < 0.7

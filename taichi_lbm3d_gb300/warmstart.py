"""Learned warm start: dataset generation, training and the rest-vs-warm evaluation.

    python -m taichi_lbm3d_gb300.warmstart --train-n 2000 --edge 96 --epochs 30 \\
        --eval-n 100 --eval-edge 192 --fp64-subset 4 --out weights.npz --report report.json

The committed weights (weights/warmstart_unet_96.npz, WEIGHTS) are the training
half of that command (seeds 10000..11999, 30 epochs, lr 1e-3, density weight 4,
density target smoothed over 2 cells).

1. Training data: seeded sphere packs (edge ``--edge``, radii U[3,8], porosity
   U[0.25,0.5], percolating), body force fx = 1e-6, periodic faces, niu 0.1
   (tau = 3 niu + 1/2, standard Guo term), solved to steady state
   (|dk/k| <= 1e-6 over 500 steps) by the batched solver in FP32 deviation form.
2. Training: the U-Net (unet.py) on (fluid indicator, distance to solid) ->
   (v, rho - 1), masked MSE on fluid voxels, Adam; all forward/backward work in
   the project's CUDA kernels.
3. Evaluation on held-out packs (edge ``--eval-edge``): steps and wall time to
   the same convergence criterion (a) for the plain FP32 kernel from rest,
   (b) for FP16 storage started from the network's prediction (inference and
   initialisation included), (c) the same with the predicted velocity only
   (rho = 1) and (d) FP16 storage from rest, which separates what the network
   gains from what the storage gains; and the permeability of each against the
   FP64 run of the same solver on a subset.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

NIU, FX = 0.1, 1e-6
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "warmstart_unet_96.npz")


def load_model(path=WEIGHTS):
    """The trained warm-start network (UNet3D with its target scales)."""
    from .unet import UNet3D
    m = UNet3D(seed=0)
    m.load_state_dict(dict(np.load(path)))
    return m


def pack(seed, edge):
    from .geometry import sphere_pack
    rng = np.random.default_rng(seed)
    phi = float(rng.uniform(0.25, 0.50))
    return sphere_pack((edge, edge, edge), 3.0, 8.0, phi, seed)


def _pack_and_features(args):
    from .unet import features
    seed, edge = args
    s = pack(seed, edge)
    f = features(s)[..., :2].astype(np.float32)
    return s, f


def make_inputs(seeds, edge, workers=None):
    """Solids and 2-channel features, generated in spawned processes (call
    before the first CUDA call of the process)."""
    import multiprocessing as mp
    workers = workers or max(1, min(16, len(os.sched_getaffinity(0))))
    jobs = [(s, edge) for s in seeds]
    if workers == 1:
        return [_pack_and_features(j) for j in jobs]
    with mp.get_context("spawn").Pool(workers) as pool:
        return pool.map(_pack_and_features, jobs, chunksize=1)


def solve_targets(solids, chunk=200, log=print):
    """Steady (rho, v) of every solid with the batched solver (FP32 deviation form)."""
    from . import autotune
    from .batch import Batch
    out = []
    for a in range(0, len(solids), chunk):
        part = solids[a:a + chunk]
        b = Batch(part, niu=NIU, force=(FX, 0, 0), storage="f32dev")
        tuned = autotune.tune({part[0].shape[0]: part[:4]}, storage="f32dev")
        tiles, block = autotune.plan([s.shape[0] for s in part], tuned)
        b.configure(tiles, block)
        b.init()
        t = time.perf_counter()
        _, st, cv = b.run_to_convergence(tol=1e-6, check_every=500, max_steps=100_000)
        for q in range(len(part)):
            out.append(b.macros(q))
        log("solved %d-%d in %.1f s (%d/%d converged, mean %d steps)" % (a, a + len(part), time.perf_counter() - t,
                                                                         cv.sum(), len(part), st.mean()))
        b.close()
    return out


def _to_net(feat2):
    import torch
    x = torch.zeros(feat2.shape[:-1] + (16,), dtype=torch.bfloat16)
    x[..., :2] = torch.from_numpy(feat2)
    return x


def smooth_density(solid, rho, sigma=2.0):
    """rho - 1 averaged over the fluid with a periodic Gaussian of width sigma
    (cells), zero mean over the fluid, 1 in solid cells.  A start from the
    steady density smoothed this way saves as many steps as the exact field;
    what the smoothing removes (pore-corner fluctuations) saves none, and a
    network cannot predict it from the geometry, so it is left out of the target."""
    from scipy.ndimage import gaussian_filter
    fl = np.asarray(solid) == 0
    d = np.where(fl, np.asarray(rho, np.float64) - 1.0, 0.0)
    w = gaussian_filter(fl.astype(np.float64), sigma, mode="wrap")
    low = gaussian_filter(d, sigma, mode="wrap") / np.maximum(w, 1e-6)
    low = np.where(fl, low, 0.0)
    if fl.any():
        low[fl] -= low[fl].mean()
    return (1.0 + low).astype(np.float32)


def _gauss_periodic(x, sigma):
    """Separable periodic Gaussian (truncated at 4 sigma) of a 3D torch tensor."""
    import torch
    r = int(4 * sigma + 0.5)
    k = torch.exp(-0.5 * (torch.arange(-r, r + 1, dtype=torch.float64, device=x.device) / sigma) ** 2)
    k = k / k.sum()
    for ax in range(3):
        acc = torch.zeros_like(x)
        for o in range(-r, r + 1):
            acc += k[o + r] * torch.roll(x, o, dims=ax)
        x = acc
    return x


def _smooth_density_gpu(solid, rho, sigma, device="cuda"):
    """smooth_density with torch on `device` (same periodic masked Gaussian, FP64)."""
    import torch
    fl = torch.from_numpy(np.asarray(solid) == 0).to(device)
    d = torch.where(fl, torch.from_numpy(np.asarray(rho, np.float64)).to(device) - 1.0,
                    torch.zeros((), dtype=torch.float64, device=device))
    w = _gauss_periodic(fl.to(torch.float64), sigma)
    low = _gauss_periodic(d, sigma) / torch.clamp(w, min=1e-6)
    low = torch.where(fl, low, torch.zeros_like(low))
    if bool(fl.any()):
        low = torch.where(fl, low - low[fl].mean(), low)
    return (1.0 + low).to(torch.float32).cpu().numpy()


def train(model, feats, solids, fields, epochs=4, lr=1e-3, batch=2, log=print, seed=0, rho_weight=4.0,
          rho_sigma=2.0):
    """Masked MSE on (v, rho - 1), each channel normalised by its spread over the
    training set; the density target is the steady density smoothed over
    ``rho_sigma`` cells (smooth_density) and counts ``rho_weight`` times as much
    (its scale is divided by sqrt(rho_weight)): the steady pressure field is what
    a start from rest takes longest to build (the exact velocity with rho = 1
    saves about 4% of the steps, the exact density with v = 0 about 30%).
    Learning rate on a cosine schedule from ``lr`` to 0 over the epochs."""
    import torch
    from .unet import targets
    if rho_sigma:
        fields = [(_smooth_density_gpu(s, r, rho_sigma), v) for s, (r, v) in zip(solids, fields)]
    fl = np.concatenate([(s == 0).ravel() for s in solids[: min(64, len(solids))]])
    vv = np.concatenate([f[1].reshape(-1, 3) for f in fields[: min(64, len(fields))]])[fl]
    rr = np.concatenate([f[0].ravel() for f in fields[: min(64, len(fields))]])[fl]
    scales = np.array([vv[:, 0].std(), vv[:, 1].std(), vv[:, 2].std(),
                       max(np.abs(rr - 1).std(), 1e-12) / np.sqrt(rho_weight)], np.float32)
    scales = np.maximum(scales, 1e-12)
    model.scales = scales
    F2 = torch.from_numpy(np.stack(feats)).cuda()                                  # (N, D, H, W, 2) fp32
    X = torch.zeros(F2.shape[:-1] + (16,), dtype=torch.bfloat16, device="cuda")    # (N, D, H, W, 16) bf16
    X[..., :2] = F2.to(torch.bfloat16)
    del F2
    T = torch.empty(X.shape[:-1] + (4,), dtype=torch.float32, device="cuda")
    for q, (r, v) in enumerate(fields):
        T[q] = torch.from_numpy(targets(r, v, scales)).cuda()
    M = torch.stack([torch.from_numpy((s == 0).transpose(2, 1, 0).astype(np.uint8).copy()) for s in solids]).cuda()
    n = X.shape[0]
    rng = np.random.default_rng(seed)
    hist = []
    for ep in range(epochs):
        order = rng.permutation(n)
        tot, t0 = 0.0, time.perf_counter()
        for a in range(0, n - batch + 1, batch):
            idx = torch.from_numpy(order[a:a + batch]).cuda()
            x, t, m = X[idx].contiguous(), T[idx].contiguous(), M[idx].contiguous()
            y = model.forward(x)
            loss, gy = model.loss(y, t, m, float(m.sum().item()) * 4)
            model.backward(gy)
            model.adam_step(lr=lr * 0.5 * (1.0 + np.cos(np.pi * (ep + a / n) / epochs)))
            tot += float(loss.item())
        torch.cuda.synchronize()
        hist.append({"epoch": ep, "loss": tot / max(1, n // batch), "seconds": time.perf_counter() - t0})
        log("epoch %d loss %.4f (%.1f s)" % (ep, hist[-1]["loss"], hist[-1]["seconds"]))
    return hist


def predict(model, feat2):
    """Dense (rho, v) predicted for a feature volume; rho - 1 is shifted to
    zero mean over the fluid cells, so a start from it holds the mass of a
    start from rest (the steady state it converges to has the same mass)."""
    import torch
    from .unet import fields_from_output
    x = _to_net(feat2)[None].cuda().contiguous()
    y = model.forward(x)
    torch.cuda.synchronize()
    rho, v = fields_from_output(y[0].cpu().numpy(), model.scales)
    fluid = feat2[..., 0].transpose(2, 1, 0) > 0.5
    if fluid.any():
        rho = (rho - (rho[fluid].astype(np.float64).mean() - 1.0)).astype(np.float32)
    rho[~fluid] = 1.0
    v[~fluid] = 0.0
    return rho, v


def field_errors(model, solids, feats, fields):
    """Normwise relative errors of the predicted rho - 1 and v on the fluid
    cells of solved packs: ||pred - ref|| / ||ref||."""
    out = []
    for s, f, (r, v) in zip(solids, feats, fields):
        fl = s == 0
        pr, pv = predict(model, f)
        er = np.linalg.norm((pr - r)[fl]) / max(np.linalg.norm((r - 1.0)[fl]), 1e-30)
        ev = np.linalg.norm((pv - v)[fl]) / max(np.linalg.norm(v[fl]), 1e-30)
        out.append((float(er), float(ev)))
    return out


def _solver(solid, storage):
    from .solver import LB3D_Solver_Single_Phase
    lb = LB3D_Solver_Single_Phase(*solid.shape, storage=storage, viscosity_convention="standard",
                                  guo_convention="standard")
    lb.solid.from_numpy(solid)
    lb.set_viscosity(NIU)
    lb.set_force([FX, 0.0, 0.0])
    return lb


def evaluate(model, solids, feats, fp64_subset=4, log=print):
    rows = []
    for q, (s, f) in enumerate(zip(solids, feats)):
        row = {"edge": s.shape[0], "n_fluid": int((s == 0).sum())}
        lb = _solver(s, "f32")
        lb.init_simulation()
        t = time.perf_counter()
        r = lb.run_to_convergence()
        row.update(rest_f32_steps=r["steps"], rest_f32_seconds=time.perf_counter() - t, rest_f32_k=r["k"])
        lb.close()
        t = time.perf_counter()
        rho, v = predict(model, f)
        lb = _solver(s, "f16")
        lb.init_simulation(rho, v)
        t_inf = time.perf_counter() - t
        r = lb.run_to_convergence()
        row.update(warm_f16_steps=r["steps"], warm_f16_seconds=time.perf_counter() - t, warm_f16_k=r["k"],
                   inference_and_init_seconds=t_inf)
        lb.close()
        # the same prediction with rho = 1: velocity only
        t = time.perf_counter()
        lb = _solver(s, "f16")
        lb.init_simulation(np.ones_like(rho), v)
        r = lb.run_to_convergence()
        row.update(warm_v_f16_steps=r["steps"], warm_v_f16_seconds=time.perf_counter() - t + t_inf,
                   warm_v_f16_k=r["k"])
        lb.close()
        lb = _solver(s, "f16")
        lb.init_simulation()
        t = time.perf_counter()
        r = lb.run_to_convergence()
        row.update(rest_f16_steps=r["steps"], rest_f16_seconds=time.perf_counter() - t, rest_f16_k=r["k"])
        lb.close()
        if q < fp64_subset:
            lb = _solver(s, "f64")
            lb.init_simulation()
            t = time.perf_counter()
            r = lb.run_to_convergence()
            row.update(f64_k=r["k"], f64_steps=r["steps"], f64_seconds=time.perf_counter() - t)
            for key in ("rest_f32", "warm_f16", "warm_v_f16", "rest_f16"):
                row[key + "_k_err"] = abs(row[key + "_k"] - r["k"]) / abs(r["k"])
            lb.close()
        row["speedup_warm_f16_vs_rest_f32"] = row["rest_f32_seconds"] / row["warm_f16_seconds"]
        row["step_ratio_warm_vs_rest_f16"] = row["rest_f16_steps"] / max(1, row["warm_f16_steps"])
        row["step_ratio_warm_v_vs_rest_f16"] = row["rest_f16_steps"] / max(1, row["warm_v_f16_steps"])
        log("eval %d: rest f32 %d steps %.2f s | warm f16 %d steps %.2f s | warm v-only f16 %d | rest f16 %d steps" % (
            q, row["rest_f32_steps"], row["rest_f32_seconds"], row["warm_f16_steps"], row["warm_f16_seconds"],
            row["warm_v_f16_steps"], row["rest_f16_steps"]))
        rows.append(row)
    return rows


def summarize(rows):
    def med(k):
        v = [r[k] for r in rows if k in r]
        return float(np.median(v)) if v else None

    def mx(k):
        v = [r[k] for r in rows if k in r]
        return float(np.max(v)) if v else None

    tot_rest = sum(r["rest_f32_seconds"] for r in rows)
    tot_warm = sum(r["warm_f16_seconds"] for r in rows)
    return {"n": len(rows), "wall_rest_f32_total_s": tot_rest, "wall_warm_f16_total_s": tot_warm,
            "speedup_total": tot_rest / tot_warm, "speedup_median": med("speedup_warm_f16_vs_rest_f32"),
            "steps_rest_f32_median": med("rest_f32_steps"), "steps_warm_f16_median": med("warm_f16_steps"),
            "steps_rest_f16_median": med("rest_f16_steps"),
            "step_ratio_rest_over_warm_f16_median": med("step_ratio_warm_vs_rest_f16"),
            "step_ratio_rest_over_warm_f16_mean": float(np.mean([r["step_ratio_warm_vs_rest_f16"] for r in rows])),
            "steps_warm_v_f16_median": med("warm_v_f16_steps"),
            "step_ratio_rest_over_warm_v_f16_mean": float(np.mean([r["step_ratio_warm_v_vs_rest_f16"] for r in rows])),
            "warm_fewer_steps": int(sum(r["warm_f16_steps"] < r["rest_f16_steps"] for r in rows)),
            "warm_more_steps": int(sum(r["warm_f16_steps"] > r["rest_f16_steps"] for r in rows)),
            "warm_v_fewer_steps": int(sum(r["warm_v_f16_steps"] < r["rest_f16_steps"] for r in rows)),
            "warm_v_more_steps": int(sum(r["warm_v_f16_steps"] > r["rest_f16_steps"] for r in rows)),
            "k_err_warm_f16_vs_f64_max": mx("warm_f16_k_err"), "k_err_rest_f32_vs_f64_max": mx("rest_f32_k_err"),
            "k_err_rest_f16_vs_f64_max": mx("rest_f16_k_err"), "k_err_warm_v_f16_vs_f64_max": mx("warm_v_f16_k_err")}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-n", type=int, default=2000)
    ap.add_argument("--edge", type=int, default=96)
    ap.add_argument("--train-seed0", type=int, default=10000)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--rho-weight", type=float, default=4.0, help="weight of the density channel in the loss")
    ap.add_argument("--rho-sigma", type=float, default=2.0,
                    help="Gaussian width (cells) of the smoothed density target; 0 = the raw density")
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--eval-n", type=int, default=100)
    ap.add_argument("--eval-edge", type=int, default=192)
    ap.add_argument("--eval-seed0", type=int, default=20000)
    ap.add_argument("--fp64-subset", type=int, default=4)
    ap.add_argument("--activation", default="relu", choices=["relu", "gelu"],
                    help="activation after every 3x3x3 convolution of the network")
    ap.add_argument("--weights", default=None, help="load trained weights instead of training")
    ap.add_argument("--out", default="warmstart_weights.npz")
    ap.add_argument("--report", default="warmstart_report.json")
    a = ap.parse_args(argv)

    def log(m):
        print(m, file=sys.stderr, flush=True)

    t0 = time.perf_counter()
    train_in = make_inputs(range(a.train_seed0, a.train_seed0 + a.train_n), a.edge) if not a.weights else []
    eval_in = make_inputs(range(a.eval_seed0, a.eval_seed0 + a.eval_n), a.eval_edge)
    log("inputs ready in %.1f s" % (time.perf_counter() - t0))
    from .unet import UNet3D
    model = UNet3D(seed=0, activation=a.activation)
    report = {"n_params": model.n_params(), "activation": a.activation, "train_n": a.train_n, "edge": a.edge,
              "eval_n": a.eval_n,
              "eval_edge": a.eval_edge}
    if a.weights:
        model.load_state_dict(dict(np.load(a.weights)))
    else:
        solids = [s for s, _ in train_in]
        feats = [f for _, f in train_in]
        t = time.perf_counter()
        fields = solve_targets(solids, log=log)
        report["data_seconds"] = time.perf_counter() - t
        t = time.perf_counter()
        report["train_history"] = train(model, feats, solids, fields, epochs=a.epochs, lr=a.lr, log=log,
                                        rho_weight=a.rho_weight, rho_sigma=a.rho_sigma)
        report["train_seconds"] = time.perf_counter() - t
        np.savez(a.out, **model.state_dict())
    rows = evaluate(model, [s for s, _ in eval_in], [f for _, f in eval_in], fp64_subset=a.fp64_subset, log=log)
    report["summary"] = summarize(rows)
    report["rows"] = rows
    with open(a.report, "w") as fh:
        json.dump(report, fh, indent=1)
    print(json.dumps(report["summary"]))
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Trains the warm-start network on converged weights of the plain solver.

    python -m geogram_gb300.train_warmstart --out geogram_gb300/data/warmstart_mlp.npz

Synthetic training set: Gaussian mixtures with 4 to 16 components (means
uniform in [0.2, 0.8]^3, one standard deviation per component uniform in
[0.02, 0.1], seeds rejected outside the unit cube), n uniform in
[nmin, nmax]; the targets are (H0 w*)_i / vol_i(0), w* the weights of
gbv_ot_solve from zero to a relative mass error of 1e-6, H0 the Hessian
and vol(0) the cell volumes at zero weights (the cell-averaged Laplacian
of w* on the zero-weight cell graph).  Training runs on the GPU with the library's tensor-core
forward/backward kernels and Adam.  Held-out mixtures are then solved
from zero and from the network's prediction, and the Newton iterations
and times of both are written with the model.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def mixture(n: int, rng: np.random.Generator, kmin: int = 4, kmax: int = 16,
            smin: float = 0.02, smax: float = 0.1) -> np.ndarray:
    k = int(rng.integers(kmin, kmax + 1))
    mu = rng.uniform(0.2, 0.8, (k, 3))
    sig = rng.uniform(smin, smax, k)
    out, have = [], 0
    while have < n:
        c = rng.integers(0, k, n)
        p = mu[c] + sig[c, None] * rng.standard_normal((n, 3))
        p = p[((p > 0.0) & (p < 1.0)).all(1)]
        out.append(p)
        have += len(p)
    return np.concatenate(out)[:n]


def solve(g, x_dev, w0=None, tol=1e-6):
    import torch
    w = torch.zeros(x_dev.shape[0], dtype=torch.float64, device="cuda") if w0 is None else w0
    torch.cuda.synchronize()
    t = time.perf_counter()
    rep = g.ot_solve_device(x_dev, w, tol=tol)
    torch.cuda.synchronize()
    return w, rep, time.perf_counter() - t


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--out", required=True)
    ap.add_argument("--solves", type=int, default=24)
    ap.add_argument("--nmin", type=int, default=20000)
    ap.add_argument("--nmax", type=int, default=100000)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--heldout", type=int, default=4)
    ap.add_argument("--heldout-n", type=int, default=100000)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args(argv)

    import torch
    import geogram_gb300 as g
    from geogram_gb300.warmstart import WarmStartModel, features, laplacian_target

    rng = np.random.default_rng(args.seed)
    raws, targets, stats = [], [], []
    t0 = time.perf_counter()
    for s in range(args.solves):
        n = int(rng.integers(args.nmin, args.nmax + 1))
        x = torch.tensor(mixture(n, rng), device="cuda")
        w, rep, dt = solve(g, x)
        if not rep["converged"]:
            print(f"solve {s}: n={n} did not converge, skipped", flush=True)
            continue
        raws.append(features(x))
        b = laplacian_target(x.cpu().numpy(), w.cpu().numpy())
        targets.append(torch.tensor(b, dtype=torch.float32, device="cuda"))
        stats.append(dict(n=n, newton=rep["newton_iters"], seconds=dt,
                          w_std=float(w.std().item())))
        print(f"solve {s}: n={n} newton={rep['newton_iters']} {dt:.1f}s "
              f"w_std={stats[-1]['w_std']:.4g}", flush=True)
    raw = torch.cat(raws)
    target = torch.cat(targets)
    t_data = time.perf_counter() - t0

    model = WarmStartModel(seed=args.seed)
    model.fit_normalisation(raw, target)
    t1 = time.perf_counter()
    losses = model.train(raw, target, steps=args.steps, batch=args.batch, lr=args.lr,
                         seed=args.seed, log_every=max(1, args.steps // 10))
    t_train = time.perf_counter() - t1

    report = dict(config=vars(args), training_solves=stats, data_seconds=t_data,
                  train_seconds=t_train, loss_first=losses[0],
                  loss_last=float(np.mean(losses[-50:])))
    model.save(args.out, report=json.dumps(report))

    held = []
    for h in range(args.heldout):
        x = torch.tensor(mixture(args.heldout_n, rng), device="cuda")
        _, rp, tp = solve(g, x)
        entry = dict(n=args.heldout_n, plain_newton=rp["newton_iters"], plain_s=tp,
                     plain_calls=rp["cell_calls"], plain_converged=rp["converged"])
        w = torch.empty(args.heldout_n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        ta = time.perf_counter()
        rw = model.solve(x, w, tol=1e-6)
        torch.cuda.synchronize()
        entry.update(warm_newton=rw["newton_iters"], warm_s=time.perf_counter() - ta,
                     warm_calls=rw["cell_calls"], warm_converged=rw["converged"],
                     start_ms=rw["ms_start"], start_scale=rw["start_scale"])
        held.append(entry)
        print("held-out", h, json.dumps(entry), flush=True)
    report["heldout"] = held
    model.save(args.out, report=json.dumps(report))
    print(json.dumps(dict(loss_first=report["loss_first"], loss_last=report["loss_last"],
                          train_seconds=t_train), indent=1))


if __name__ == "__main__":
    main()

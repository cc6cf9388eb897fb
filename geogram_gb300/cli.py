"""Command-line program: cells or optimal transport of synthetic seeds.

    python -m geogram_gb300.cli cells --n 1000000 [--mixture 8 --sigma 0.05]
                                      [--weights 1e-4] [--precision fp32|fp64]
                                      [--certification security_radius|power_range]
    python -m geogram_gb300.cli ot --n 1000000 [--mixture 8 --sigma 0.05]
                                   [--learned | --levels | --start separable]
                                   [--max-newton N] [--tol 1e-6]

The counterpart of the reference's compute_RVD / compute_OTM programs for
meshless cells in the unit cube (src/examples/exploragram/compute_OTM/
main.cpp:109-321): seeds are generated here (uniform, or a Gaussian
mixture with means uniform in [0.2, 0.8]^3), everything else runs on the
GPU.  Prints one JSON line with the report.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def seeds(n: int, mixture: int, sigma: float, seed: int,
          sigma_range: tuple[float, float] | None = None) -> np.ndarray:
    """Uniform seeds, or a Gaussian mixture: one standard deviation sigma,
    or per component log-uniform in sigma_range."""
    rng = np.random.default_rng(seed)
    if mixture <= 0:
        return rng.random((n, 3))
    mu = rng.uniform(0.2, 0.8, (mixture, 3))
    sig = (np.exp(rng.uniform(np.log(sigma_range[0]), np.log(sigma_range[1]), mixture))
           if sigma_range else np.full(mixture, sigma))
    out, have = [], 0
    while have < n:
        c = rng.integers(0, mixture, n)
        p = mu[c] + sig[c, None] * rng.standard_normal((n, 3))
        p = p[((p > 0.0) & (p < 1.0)).all(1)]
        out.append(p)
        have += len(p)
    return np.concatenate(out)[:n]


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    for name in ("cells", "ot"):
        p = sub.add_parser(name)
        p.add_argument("--n", type=int, default=1_000_000)
        p.add_argument("--mixture", type=int, default=0, help="components (0: uniform seeds)")
        p.add_argument("--sigma", type=float, default=0.05)
        p.add_argument("--sigma-range", default=None,
                       help="lo,hi: per-component sigma log-uniform in [lo, hi]")
        p.add_argument("--seed", type=int, default=0)
        p.add_argument("--precision", default="fp32")
        p.add_argument("--repeat", type=int, default=1)
    c = sub.choices["cells"]
    c.add_argument("--weights", type=float, default=0.0, help="weights uniform in [0, w]")
    c.add_argument("--certification", default="security_radius")
    o = sub.choices["ot"]
    o.add_argument("--learned", action="store_true", help="start from the learned warm start")
    o.add_argument("--levels", action="store_true",
                   help="multilevel solve (optimize_levels): coarse-to-fine subsets")
    o.add_argument("--start", default="zero", choices=("zero", "separable"),
                   help="plain solve from zero weights or from the separable marginal-CDF start")
    o.add_argument("--ratio", type=int, default=8)
    o.add_argument("--min-level", type=int, default=20000)
    o.add_argument("--max-newton", type=int, default=100)
    o.add_argument("--tol", type=float, default=1e-6)
    args = ap.parse_args(argv)

    import torch
    import geogram_gb300 as g
    sr = tuple(float(v) for v in args.sigma_range.split(",")) if args.sigma_range else None
    x = torch.tensor(seeds(args.n, args.mixture, args.sigma, args.seed, sr), device="cuda")
    ctx = g.default_context()
    out = {}
    for _ in range(args.repeat):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if args.cmd == "cells":
            w = None
            if args.weights > 0:
                w = torch.tensor(np.random.default_rng(args.seed + 1).random(args.n) * args.weights,
                                 device="cuda")
            rep = g.compute_cells_device(x, w, precision=args.precision,
                                         certification=args.certification)
        else:
            w = torch.zeros(args.n, dtype=torch.float64, device="cuda")
            if args.levels:
                rep = g.ot_solve_levels_device(x, w, ratio=args.ratio, min_level=args.min_level,
                                               tol=args.tol, max_newton=args.max_newton,
                                               precision=args.precision)
            elif args.learned:
                from geogram_gb300.warmstart import WarmStartModel
                rep = WarmStartModel.load().solve(x, w, tol=args.tol, max_newton=args.max_newton,
                                                  precision=args.precision)
            else:
                ts = time.perf_counter()
                if args.start == "separable":
                    w = g.ot_separable_start_device(x)
                t_start = time.perf_counter() - ts
                rep = g.ot_solve_device(x, w, tol=args.tol, max_newton=args.max_newton,
                                        precision=args.precision)
                rep = dict(rep, start=args.start, start_s=t_start)
        torch.cuda.synchronize()
        out = dict(rep, wall_s=time.perf_counter() - t0)
    now, peak = ctx.device_bytes()
    out["device_bytes_peak"] = peak
    out["device_bytes_inputs"] = int(x.numel() * 8 * 2)
    print(json.dumps(out))


if __name__ == "__main__":
    main()

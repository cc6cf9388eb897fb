"""Generates the golden fixtures of tests/golden/ from the reference itself.

Runs geogram's own BalancedKdTree and VBW::ConvexCell (compiled from the
reference sources into oracle/_ref/libgbv_ref.so by oracle/ref/Makefile) on
small seeded inputs and saves inputs and outputs as compressed .npz files.
Needs the reference checkout; the fixtures are committed so that the tests
run without it.

    python tests/golden/make_golden.py [case names]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402


def gmm(rng, n, k, sigma_lo, sigma_hi, lo=0.2, hi=0.8):
    means = rng.uniform(lo, hi, (k, 3))
    sig = rng.uniform(sigma_lo, sigma_hi, k)
    out = []
    while len(out) < n:
        c = rng.integers(0, k, n)
        p = means[c] + rng.normal(size=(n, 3)) * sig[c, None]
        ok = np.all((p > 0) & (p < 1), axis=1)
        out.extend(p[ok])
    return np.array(out[:n])


def cases():
    rng = np.random.default_rng(0)
    yield "uniform_1500", rng.random((1500, 3)), None
    x = rng.random((1500, 3))
    # weights on the scale of the squared spacing, as in a 1M-seed diagram
    # with weights in [0, 1e-4] (w * (1e6 / n)^(2/3))
    w = rng.random(1500) * 1e-4 * (1e6 / 1500) ** (2 / 3)
    yield "power_1500", x, w
    yield "clustered_1500", gmm(np.random.default_rng(1), 1500, 8, 0.05, 0.05), None
    g = (np.arange(6) + 0.5) / 6
    yield "lattice_216", np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3), None
    x = np.random.default_rng(2).random((400, 3))
    yield "duplicates_405", np.concatenate([x, x[[3, 17, 17, 99, 250]]]), None
    # a seed at the centre of a thin spherical shell of m seeds (radii
    # jittered by 2% so that no five seeds are co-spherical): its cell has
    # hundreds of facets, beyond the fixed-capacity clipping shapes
    yield "shell_901", shell(300, 600, 300), None
    yield "shell_1601", shell(1000, 600, 1000), None


def shell(m, n_background, seed):
    rng = np.random.default_rng(seed)
    k = np.arange(m) + 0.5
    phi = np.arccos(1 - 2 * k / m)
    th = np.pi * (1 + 5 ** 0.5) * k
    d = np.stack([np.cos(th) * np.sin(phi), np.sin(th) * np.sin(phi), np.cos(phi)], 1)
    r = 0.1 * (1 + 0.02 * rng.random(m))
    bg = rng.random((3 * n_background, 3))
    bg = bg[np.linalg.norm(bg - 0.5, axis=1) > 0.2][:n_background]
    return np.concatenate([[[0.5, 0.5, 0.5]], 0.5 + d * r[:, None], bg])


def laguerre_cases():
    """Laguerre cells without the security radius: every other seed is a
    candidate (k0 = n - 1), so weights of any spread give the exact cells --
    the cells of the optimal-transport solver.  The weights are the optimal
    transport weights of the seeds (uniform measure on the cube), from the
    oracle's Newton solver: every cell has volume 1/n, the weights spread
    far beyond the squared spacing."""
    from oracle import ot
    x = gmm(np.random.default_rng(5), 1200, 6, 0.04, 0.08)
    w, _ = ot.newton(x, tol=1e-9, nthreads=8)
    yield "laguerre_ot_1200", x, w


def kuhn_grid(k: int, keep=lambda i, j, l: True):
    """The cubes (i, j, l) of a k^3 grid on [0,1]^3 that keep() accepts, each
    split into the 6 Kuhn tetrahedra (conforming across cubes), positively
    oriented."""
    import itertools
    vid = lambda i, j, l: (l * (k + 1) + j) * (k + 1) + i
    g = np.arange(k + 1) / k
    verts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).transpose(2, 1, 0, 3).reshape(-1, 3)
    tets = []
    for i, j, l in itertools.product(range(k), repeat=3):
        if not keep(i, j, l):
            continue
        for perm in itertools.permutations(range(3)):
            p = [i, j, l]
            tv = [vid(*p)]
            for a in perm:
                p[a] += 1
                tv.append(vid(*p))
            a, b, c, d = verts[tv]
            if np.dot(np.cross(b - a, c - a), d - a) < 0:
                tv[1], tv[2] = tv[2], tv[1]
            tets.append(tv)
    return verts, np.array(tets, np.uint32)


def rvd_cases():
    cases = {}
    v, t = kuhn_grid(1)
    cases["cube_300"] = (v, t, np.random.default_rng(6).random((300, 3)))
    # an L-shaped (non-convex) domain: the 4^3 grid without the cubes where
    # x > 1/2 and z > 1/2; seeds inside it
    v, t = kuhn_grid(4, lambda i, j, l: not (i >= 2 and l >= 2))
    x = np.random.default_rng(7).random((1200, 3))
    x = x[~((x[:, 0] > 0.5) & (x[:, 2] > 0.5))][:500]
    cases["lshape_500"] = (v, t, x)
    return cases


def main(only=None):
    """Writes every fixture, or only those whose names are listed."""
    oracle.build_ref()
    for name, x, w in laguerre_cases():
        if only and name not in only:
            continue
        x = np.ascontiguousarray(x)
        r = oracle.cells(x, w, k0=len(x) - 1, check_sr=False, nthreads=8, which="ref",
                         max_nbr=400)
        np.savez_compressed(os.path.join(HERE, f"cells_{name}.npz"), x=x, w=w, vol=r["vol"],
                            mg=r["mg"], rowptr=r["rowptr"], nbr=r["nbr"], area=r["area"],
                            status=r["status"], n_clip=r["n_clip"], k_list=r["k_list"])
        print(name, len(x), "cells (every seed a candidate), nnz", len(r["nbr"]))
    for name, x, w in cases():
        if only and name not in only:
            continue
        x = np.ascontiguousarray(x)
        r = oracle.cells(x, w, nthreads=8, which="ref", max_nbr=2100)
        np.savez_compressed(os.path.join(HERE, f"cells_{name}.npz"), x=x,
                            w=np.zeros(0) if w is None else w, vol=r["vol"], mg=r["mg"],
                            rowptr=r["rowptr"], nbr=r["nbr"], area=r["area"],
                            status=r["status"], n_clip=r["n_clip"], k_list=r["k_list"])
        print(name, len(x), "cells, nnz", len(r["nbr"]))
    if not only or "fast" in only:
        # the reference's other clipping variants: inexact predicates
        # (use_exact_predicates(false)) and clip_by_plane_fast.  Not on the
        # lattice: with inexact predicates the reference crashes there
        # (inconsistent signs on exactly degenerate configurations).
        variants = [("fast_clustered_1500", "clustered_1500", False, False),
                    ("walk_power_1500", "power_1500", True, True),
                    ("fastwalk_uniform_1500", "uniform_1500", False, True)]
        for name, src, exact, walk in variants:
            d = np.load(os.path.join(HERE, f"cells_{src}.npz"))
            x, w = d["x"], (d["w"] if d["w"].size else None)
            r = oracle.cells(x, w, exact=exact, walk=walk, nthreads=8, which="ref", max_nbr=2100)
            np.savez_compressed(os.path.join(HERE, f"cells_{name}.npz"), x=x,
                                w=np.zeros(0) if w is None else w, vol=r["vol"], mg=r["mg"],
                                rowptr=r["rowptr"], nbr=r["nbr"], area=r["area"],
                                status=r["status"], n_clip=r["n_clip"], k_list=r["k_list"],
                                exact=np.array(exact), walk=np.array(walk))
            print(name, "exact" if exact else "fast", "walk" if walk else "scan")
    if not only or "periodic" in only:
        # Laguerre cells in the periodic unit cube by the reference's
        # PeriodicDelaunay3d (weights at 0.2 x the squared spacing: the
        # reference crashes once cells become empty)
        x = np.random.default_rng(8).random((1000, 3))
        for name, w in (("periodic_1000", None),
                        ("periodic_power_1000",
                         np.random.default_rng(9).random(1000) * 0.2 * (1 / 1000) ** (2 / 3))):
            r = oracle.ref_periodic_cells(x, w)
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), x=x,
                                w=np.zeros(0) if w is None else w, vol=r["vol"], mg=r["mg"],
                                rowptr=r["rowptr"], nbr=r["nbr"], shift=r["shift"], area=r["area"])
            print(name, "facets", len(r["nbr"]), "volume", r["vol"].sum())
    if not only or "obj" in only:
        # ConvexCell::save text of some cells (interior, at the box, of
        # weighted seeds), plain and shrunk
        for src in ("uniform_1500", "power_1500"):
            d = np.load(os.path.join(HERE, f"cells_{src}.npz"))
            x, w = d["x"], (d["w"] if d["w"].size else None)
            which = np.array([0, 1, 2, 7, 42, 100, 333, 777, 1200, 1499], np.uint32)
            txt = oracle.ref_cells_obj(x, w, which)
            txt_s = oracle.ref_cells_obj(x, w, which[:4], shrink=0.2)
            np.savez_compressed(os.path.join(HERE, f"obj_{src}.npz"), which=which,
                                obj=np.array(txt), obj_shrink=np.array(txt_s))
            print(f"obj_{src}", len(txt), "bytes")
    if not only or "rvd" in only:
        # cells restricted to tetrahedral meshes, by the reference's own
        # Delaunay + RestrictedVoronoiDiagram (volumetric)
        for name, (v, t, x) in rvd_cases().items():
            r = oracle.ref_rvd_volume(v, t, x)
            np.savez_compressed(os.path.join(HERE, f"rvd_{name}.npz"), mesh_xyz=v, tets=t, x=x,
                                m=r["m"], mg=r["mg"], f=np.array(r["f"]), g=r["g"])
            print(f"rvd_{name}", len(t), "tets", len(x), "seeds, sum m", r["m"].sum())
    if not only or "cvt" in only:
        # the reference's CVT::Newton_iterations (HLBFGS, m = 7) on the
        # restricted cells: after 1 and after 10 iterations
        for name in ("cube_300", "lshape_500"):
            v, t, x = rvd_cases()[name]
            out = dict(mesh_xyz=v, tets=t, x=x)
            for it in (1, 10):
                xi, fi = oracle.ref_cvt_newton(v, t, x, it)
                out[f"x{it}"] = xi
                out[f"f{it}"] = np.array(fi)
            np.savez_compressed(os.path.join(HERE, f"cvt_newton_{name}.npz"), **out)
            print(f"cvt_newton_{name}", "f1", float(out["f1"]), "f10", float(out["f10"]))
    if only:
        return
    x = np.random.default_rng(3).random((2000, 3))
    idx, d2 = oracle.knn(x, 21, nthreads=8, which="ref")
    np.savez_compressed(os.path.join(HERE, "knn_2000.npz"), x=x, idx=idx, d2=d2)
    x4 = np.concatenate([x, np.random.default_rng(4).random((2000, 1)) * 0.01], axis=1)
    idx, d2 = oracle.knn(x4, 21, nthreads=8, which="ref")
    np.savez_compressed(os.path.join(HERE, "knn4_2000.npz"), x=x4, idx=idx, d2=d2)
    print("knn fixtures written")


if __name__ == "__main__":
    main(sys.argv[1:])

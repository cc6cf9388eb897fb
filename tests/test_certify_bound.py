"""The FP32 leaf test of the power-range certification walk (gbv_geom.cu,
certify_cell), emulated in numpy float32 operation by operation.

The kernel evaluates, for a corner c of cell i and a candidate seed j, in
the seed's frame: c' = c - p_i (FP64, rounded to FP32), q = p_j - p_i and
dw = w_j - w_i from FP32 value/remainder pairs, d = |c' - q|^2 - dw and
base = |c'|^2.  Its comment claims d within 1e-6 (base + |d| + |dw|) of the
exact value (and base within 1e-6 base), and the test it applies,
d <= (base (1 + 4e-6) + 1e-12) (1 + 5e-6) + 4.1e-6 |dw|, must keep every
seed whose exact power at c is not above the cell's own (a seed that cuts).
These tests check both on configurations like optimal-transport cells
(corners far from their seeds, weights large next to the power gaps) and
Voronoi cells, with near ties on both sides."""
import numpy as np

f32 = np.float32


def split(x):
    """FP32 value and remainder of FP64 x (the library's seed layout)."""
    hi = x.astype(f32)
    lo = (x - hi.astype(np.float64)).astype(f32)
    return hi, lo


def kernel_terms(c, pi, pj, wi, wj):
    """d, base and dw as the kernel forms them (each operation in FP32)."""
    ih, il = split(pi)
    jh, jl = split(pj)
    q = (jh - ih) + (jl - il)                    # float32 ops
    cl = (c - pi).astype(f32)                    # FP64 difference, rounded
    wih, wil = split(wi)
    wjh, wjl = split(wj)
    dw = (wjh - wih) + (wjl - wil)
    dx = cl - q
    d = dx[:, 0] * dx[:, 0] + dx[:, 1] * dx[:, 1] + dx[:, 2] * dx[:, 2] - dw
    base = cl[:, 0] * cl[:, 0] + cl[:, 1] * cl[:, 1] + cl[:, 2] * cl[:, 2]
    return d, base, dw


def keeps(d, base, dw):
    """The kernel's test: may seed j cut at this corner?"""
    thr = (base * f32(1.0 + 4e-6) + f32(1e-12)) * f32(1.0 + 5e-6)
    return d <= thr + f32(4.1e-6) * np.abs(dw)


def configurations(rng, n, far, weighted, gap_rel):
    """Corners c of cell i at distance ~far from p_i, a seed j a few
    spacings away with its weight set so that its power at c is the cell's
    own plus gap_rel * base (negative: j cuts there)."""
    pi = rng.uniform(0.2, 0.8, (n, 3))
    u = rng.standard_normal((n, 3))
    c = pi + far * rng.uniform(0.3, 1.0, (n, 1)) * u / np.linalg.norm(u, axis=1, keepdims=True)
    pj = pi + rng.uniform(-1.0, 1.0, (n, 3)) * 5e-3
    wi = rng.uniform(-0.05, 0.05, n) if weighted else np.zeros(n)
    base = np.sum((c - pi) ** 2, axis=1)
    gap = gap_rel * base
    # |c - p_j|^2 - (w_j - w_i) = base + gap
    wj = wi + np.sum((c - pj) ** 2, axis=1) - base - gap
    if not weighted:
        # Voronoi: no weights; move p_j instead along c - p_j so that
        # |c - p_j|^2 = base + gap
        v = pj - c
        pj = c + v * np.sqrt((base + gap) / np.sum(v * v, axis=1))[:, None]
        wj = np.zeros(n)
    return c, pi, pj, wi, wj


def exact_terms(c, pi, pj, wi, wj):
    d = np.sum((c - pj) ** 2, axis=1) - (wj - wi)
    base = np.sum((c - pi) ** 2, axis=1)
    return d, base, wj - wi


def test_rounding_within_the_stated_bound():
    rng = np.random.default_rng(0)
    worst_d = worst_b = 0.0
    for far, weighted in ((0.15, True), (0.02, True), (3e-3, False), (0.1, False)):
        for gap in (-1e-5, -1e-7, 0.0, 1e-7, 1e-5, 1e-3):
            c, pi, pj, wi, wj = configurations(rng, 20000, far, weighted, gap)
            d, base, dw = kernel_terms(c, pi, pj, wi, wj)
            de, be, dwe = exact_terms(c, pi, pj, wi, wj)
            scale = be + np.abs(de) + np.abs(dwe)
            worst_d = max(worst_d, np.max(np.abs(d.astype(np.float64) - de) / scale))
            worst_b = max(worst_b, np.max(np.abs(base.astype(np.float64) - be) / be))
    assert worst_d < 1e-6, worst_d
    assert worst_b < 1e-6, worst_b


def test_no_cutting_seed_is_dropped():
    rng = np.random.default_rng(1)
    for far, weighted in ((0.2, True), (0.05, True), (3e-3, False), (0.1, False)):
        for gap in (-1e-4, -1e-6, -1e-8, -1e-10, 0.0):
            c, pi, pj, wi, wj = configurations(rng, 20000, far, weighted, gap)
            de, be, _ = exact_terms(c, pi, pj, wi, wj)
            cuts = de <= be
            d, base, dw = kernel_terms(c, pi, pj, wi, wj)
            assert np.all(keeps(d, base, dw)[cuts])


def test_seeds_clear_of_the_band_are_dropped():
    """The test is tight: seeds whose power is above the cell's own by 1e-4
    of the corner's power are not kept (the walk's former FP32 margin,
    1e-5 |pi_i| + 1e-7 in the global frame, kept many of them)."""
    rng = np.random.default_rng(2)
    c, pi, pj, wi, wj = configurations(rng, 20000, 0.15, True, 1e-4)
    d, base, dw = kernel_terms(c, pi, pj, wi, wj)
    assert not np.any(keeps(d, base, dw))


def test_folded_threshold_covers_the_exact_condition():
    """d - 4e-6 (|d| + |dw|) <= base (1 + 4e-6) + 1e-12 for d >= 0 is what
    the kernel tests as d <= T + s with the two slacks folded in."""
    rng = np.random.default_rng(3)
    base = (10.0 ** rng.uniform(-8, -1, 100000)).astype(f32)
    dw = (rng.choice([-1, 1], 100000) * 10.0 ** rng.uniform(-9, 0, 100000)).astype(f32)
    bp = base.astype(np.float64) * (1 + 4e-6) + 1e-12
    # the largest d the exact condition allows, with a little room below
    dmax = (bp + 4e-6 * np.abs(dw.astype(np.float64))) / (1 - 4e-6)
    d = (dmax * (1 - 1e-7)).astype(f32)
    ok = d.astype(np.float64) <= dmax
    assert np.all(keeps(d, base, dw)[ok])

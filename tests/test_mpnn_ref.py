"""The CPU restatement of the learned-guess network (oracle/mpnn_ref.py): its gradient
against central finite differences, on a small O-grid graph.  This pins the oracle that
the GPU gradient tests compare with."""
import numpy as np

from conftest import small_case
from oracle import mpnn_ref as M
from oracle import oracle as O


def mpnn_graph(k):
    """Neighbour CSR = the Laplacian pattern without its diagonal (the library's order),
    boundary kinds from I_M (body) and IFM (outer)."""
    rp, idx = O.laplace_pattern(k.inpoel, k.npoin)
    ptr, nbr = [0], []
    for i in range(k.npoin):
        row = idx[rp[i]:rp[i + 1]] - 1
        nbr.extend(row[1:])
        ptr.append(len(nbr))
    kind = np.zeros(k.npoin, int)
    kind[np.asarray(k.i_m) - 1] = 1
    kind[np.asarray(k.ifm) - 1] = 2
    return np.array(ptr), np.array(nbr), kind


def rigid(k, kind, heave, pitch_deg):
    body = kind == 1
    cx, cy = k.x[body].mean(), k.y[body].mean()
    th = np.radians(pitch_deg)
    dx, dy = k.x - cx, k.y - cy
    g = np.zeros((k.npoin, 2))
    g[body, 0] = ((np.cos(th) - 1) * dx - np.sin(th) * dy)[body]
    g[body, 1] = (np.sin(th) * dx + (np.cos(th) - 1) * dy + heave)[body]
    return g


def test_reference_gradient_matches_finite_differences():
    k = small_case(1, scale=8, seed=5)
    ptr, nbr, kind = mpnn_graph(k)
    g = rigid(k, kind, 0.2, 7.0)
    G = M.globals_(k.x, k.y, kind, g)
    f = M.features(k.x, k.y, kind, G)
    i, j, e, deg = M.edges(k.x, k.y, ptr, nbr, G["L"])
    rng = np.random.default_rng(0)
    w = M.init_params(1).astype(np.float64) + 0.05 * rng.normal(size=M.n_params())
    target = 0.1 * rng.normal(size=(k.npoin, M.OUT))
    free = (kind == 0).astype(float)
    _, grad = M.loss_and_grad(w, f, i, j, e, deg, target, free)
    errs = []
    for q in rng.choice(w.size, 80, replace=False):
        h = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[q] += h
        wm[q] -= h
        lp, _ = M.loss_and_grad(wp, f, i, j, e, deg, target, free)
        lm, _ = M.loss_and_grad(wm, f, i, j, e, deg, target, free)
        fd = (lp - lm) / (2 * h)
        errs.append(abs(fd - grad[q]) / max(abs(fd) + abs(grad[q]), 1e-9))
    assert np.median(errs) < 1e-7
    assert max(errs) < 1e-3  # a ReLU kink within h of a sample is possible


def test_reference_packing_and_affine_fit():
    assert M.n_params() == 64 * 10 + 64 + 4 * 16704 + 3 * 64 + 3
    k = small_case(1, scale=8, seed=5)
    ptr, nbr, kind = mpnn_graph(k)
    # a rigid motion is affine: the fit recovers its translation and rotation exactly
    for heave, pitch in ((0.1, 0.0), (0.0, 3.0), (-0.2, -7.0)):
        g = rigid(k, kind, heave, pitch)
        G = M.globals_(k.x, k.y, kind, g)
        th = np.radians(pitch)
        assert abs(G["tx"]) < 1e-14 and abs(G["ty"] - heave) < 1e-14
        ref = np.array([[np.cos(th) - 1, -np.sin(th)], [np.sin(th), np.cos(th) - 1]])
        got = np.array([[G["m11"], G["m12"]], [G["m21"], G["m22"]]])
        assert np.abs(got - ref).max() < 1e-12
    # the guess from the exact fields reproduces the boundary data's linear response
    g = rigid(k, kind, 0.2, 5.0)
    G = M.globals_(k.x, k.y, kind, g)
    y = np.random.default_rng(0).normal(size=(k.npoin, 3))
    u = M.guess(y, G, kind, g)
    free = kind == 0
    px, py = G["L"] * y[:, 1], G["L"] * y[:, 2]
    assert np.allclose(u[free, 0], (G["tx"] * y[:, 0] + G["m11"] * px + G["m12"] * py)[free])
    assert np.array_equal(u[~free], g[~free])

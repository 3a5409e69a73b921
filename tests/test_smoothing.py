"""The mesh smoothing (smoothing.f90) on the GPU in its two visiting orders.  The colour-by-
colour variant moves one colour of mutually non-adjacent nodes at a time: it is the
sequential pass visiting the nodes colour by colour, so the oracle run in the GPU's colour
order must give the GPU's mesh bit for bit, and against the node-order oracle the checks are
the properties the algorithm guarantees (fixed nodes stay, no node makes its worst element
worse, the worst element improves about as far as the oracle's).  The node-order variant
visits the nodes as the reference does and must give the node-order oracle's mesh."""
import numpy as np
import pytest

from conftest import small_case


def quality(x, y, inpoel):
    """mu (smoothing.f90:351-362) of every element."""
    i = inpoel - 1
    X, Y = x[i], y[i]
    area = X[:, 1] * Y[:, 2] + X[:, 2] * Y[:, 0] + X[:, 0] * Y[:, 1] - (
        X[:, 1] * Y[:, 0] + X[:, 2] * Y[:, 1] + X[:, 0] * Y[:, 2])
    l = ((X[:, 2] - X[:, 1]) ** 2 + (Y[:, 2] - Y[:, 1]) ** 2 + (X[:, 0] - X[:, 2]) ** 2 +
         (Y[:, 0] - Y[:, 2]) ** 2 + (X[:, 1] - X[:, 0]) ** 2 + (Y[:, 1] - Y[:, 0]) ** 2)
    return 3.46410161513775 * area / l


def jittered(seed=1):
    """The jittered cylinder O-grid: about half its elements are below mu = 0.85."""
    k = small_case(1, scale=16, seed=seed)
    fixed = np.zeros(k.npoin, np.int32)
    fixed[k.ilaux() - 1] = 1
    return k, k.x.copy(), k.y.copy(), fixed


def test_oracle_smoothing_improves(oracle):
    k, x, y, fixed = jittered()
    q0 = quality(x, y, k.inpoel).min()
    xs, ys, it, q = oracle.smoothing(x, y, k.inpoel, fixed)
    assert it >= 1 and q > q0 and np.isclose(q, quality(xs, ys, k.inpoel).min())
    assert np.array_equal(xs[fixed == 1], x[fixed == 1])


@pytest.mark.gpu
def test_gpu_smoothing_properties(gpu_lib, oracle):
    from cfd_gb300 import solver
    k, x, y, fixed = jittered()
    q0 = quality(x, y, k.inpoel)
    xs, ys, it, q = solver.smoothing(x, y, k.inpoel, fixed)
    qs = quality(xs, ys, k.inpoel)
    assert it >= 1 and np.isclose(q, qs.min(), rtol=1e-12, atol=0)
    assert qs.min() >= q0.min() and (qs > 0).all()
    assert np.array_equal(xs[fixed == 1], x[fixed == 1])
    assert np.array_equal(ys[fixed == 1], y[fixed == 1])
    _, _, _, qo = oracle.smoothing(x, y, k.inpoel, fixed)
    assert qs.min() >= qo - 0.05


@pytest.mark.gpu
def test_gpu_smoothing_leaves_good_mesh(gpu_lib):
    """Every element at mu >= 0.85 (right isosceles triangles, mu = 0.866): no move at all."""
    from cfd_gb300 import solver
    n = 6
    xs, ys = np.meshgrid(np.arange(n, dtype=float), np.arange(n, dtype=float))
    x, y = xs.ravel(), ys.ravel()
    tri = []
    for j in range(n - 1):
        for i in range(n - 1):
            a = j * n + i + 1
            tri += [(a, a + 1, a + n + 1), (a, a + n + 1, a + n)]
    inpoel = np.array(tri, np.int32)
    fixed = np.zeros(n * n, np.int32)
    x2, y2, it, q = solver.smoothing(x, y, inpoel, fixed)
    assert it == 0 and np.array_equal(x2, x) and np.array_equal(y2, y)
    assert np.isclose(q, 3.46410161513775 * 1.0 / 4.0)


@pytest.mark.gpu
def test_resident_smoothing_then_step(gpu_lib):
    """cfd_ctx_smooth moves the context's mesh and recomputes its geometry: the FP64
    areas and dNx equal deriv of the smoothed coordinates, and the steps run on it."""
    from cfd_gb300 import solver
    from oracle import oracle as O
    k = small_case(2, scale=16, seed=3)
    s = solver.Solver(k)
    it, q = s.smooth()
    st = s.state()
    assert it >= 1 and q >= quality(k.x, k.y, k.inpoel).min()
    g = s.geometry()
    ref = O.deriv(st["X"], st["Y"], k.inpoel)
    assert np.array_equal(g["area"], ref["area"]) and np.array_equal(g["dNx"], ref["dNx"])
    rep = s.step(2)
    assert np.isfinite(s.state()["U"]).all() and rep.iter == 2
    s.close()


def _pair(prec, every, **over):
    """Two contexts of the jittered moving cylinder, the second smoothing its moved mesh
    every `every` steps."""
    from cfd_gb300 import abi, solver
    k = small_case(2, scale=16, seed=1, **over)
    P = abi.CFD_PREC_FP64 if prec == "fp64" else abi.CFD_PREC_MIXED
    a, b = solver.Solver(k, precision=P), solver.Solver(k, precision=P)
    b.set_smoothing(every)
    return k, a, b


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_smoothing_in_time_loop_step(gpu_lib, oracle, prec):
    """One step with the moved mesh smoothed (the setTol_move path with the step's
    displacement) against the same step without: no node moves further than the two
    Laplace passes and NITER sweeps allow (1.5 + 1.5 + 1 times |XPOS| + |YPOS|), a node
    that the motion did not move stays, the worst element does not get worse, W is the
    whole move over DTMIN, and the next step's geometry is the smoothed mesh's."""
    k, a, b = _pair(prec, 1)
    x0, y0 = k.x.copy(), k.y.copy()
    ra, rb = a.step(1), b.step(1)
    assert ra.dtmin == rb.dtmin
    sa, sb = a.state(), b.state()
    xp, yp = a.motion()
    tol = np.abs(xp) + np.abs(yp)
    assert tol.max() > 0
    move = np.abs(sb["X"] - sa["X"]) + np.abs(sb["Y"] - sa["Y"])
    scale = np.abs(x0).max()
    assert (move <= 4.0 * tol * (1 + 1e-9) + 1e-15 * scale).all()
    assert move.max() > 0
    assert (move[tol == 0] == 0).all()
    assert quality(sb["X"], sb["Y"], k.inpoel).min() >= quality(sa["X"], sa["Y"], k.inpoel).min()
    fb = b.fields()
    dt = rb.dtmin
    for w, xn, xs in (("W_X", "X", x0), ("W_Y", "Y", y0)):
        whole = sb[xn] - xs
        assert np.abs(fb[w] * dt - whole).max() <= 1e-9 * np.abs(whole).max()
    # the geometry of the smoothed mesh (the mixed form keeps it in FP32)
    area_b = oracle.deriv(sb["X"], sb["Y"], k.inpoel)["area"]
    area_a = oracle.deriv(sa["X"], sa["Y"], k.inpoel)["area"]
    rtol = 1e-12 if prec == "fp64" else 2e-6
    assert np.allclose(b.geometry()["area"], area_b, rtol=rtol, atol=0)
    assert (np.abs(area_a - area_b) > 10 * rtol * np.abs(area_b)).any()
    assert b.smoothing_stats()[0] == 1 and b.smoothing_stats()[1] >= 0
    a.close()
    b.close()


@pytest.mark.gpu
def test_gpu_smoothing_in_time_loop_mixed_matches_fp64(gpu_lib):
    """The mixed form with per-step smoothing against the FP64 form with it, over 12 steps
    smoothing every 2nd: the same state within the mixed form's tolerance; the graph replays
    the steps in between."""
    from cfd_gb300 import abi, solver
    k = small_case(2, scale=16, seed=1, estab_mode=2)
    k.params.fsafe = min(k.params.fsafe, 0.25)
    f = solver.Solver(k, precision=abi.CFD_PREC_FP64)
    m = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    for s in (f, m):
        s.set_smoothing(2)
    worst = 0.0
    for _ in range(12):
        rf, rm = f.step(1), m.step(1)
        assert abs(rm.dtmin - rf.dtmin) <= 1e-6 * rf.dtmin
        uf, um = f.state()["U"], m.state()["U"]
        worst = max(worst, max(np.linalg.norm(um[:, q] - uf[:, q]) / np.linalg.norm(uf[:, q])
                               for q in (0, 1, 3)))
    xf, xm = f.state()["X"], m.state()["X"]
    print("worst rel L2", worst, "mesh", np.abs(xf - xm).max())
    assert worst <= 1e-6
    assert np.abs(xf - xm).max() <= 1e-6 * np.abs(xf).max()
    assert f.smoothing_stats()[0] == 6 and m.smoothing_stats()[0] == 6
    assert m.graph_state()[1] > 0
    f.close()
    m.close()



def test_oracle_ordered_smoothing_node_order_is_the_reference(oracle):
    """The oracle's ordered smoothing with the identity order is its reference smoothing."""
    k, x, y, fixed = jittered()
    a = oracle.smoothing(x, y, k.inpoel, fixed)
    b = oracle.smoothing(x, y, k.inpoel, fixed, order=np.arange(k.npoin, dtype=np.int32))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]


@pytest.mark.gpu
def test_gpu_smoothing_is_the_reference_in_colour_order(gpu_lib, oracle):
    """Nodes of one colour share no element, so the GPU's colour-by-colour smoothing is the
    reference's sequential smoothing visiting the nodes colour by colour: with that order
    the oracle gives the same mesh, bit for bit, and the same iteration count."""
    from cfd_gb300 import solver
    k, x, y, fixed = jittered()
    order = oracle.colour_order(k.inpoel, k.npoin)
    xs, ys, it, q = solver.smoothing(x, y, k.inpoel, fixed)
    xo, yo, ito, qo = oracle.smoothing(x, y, k.inpoel, fixed, order=order)
    print("iterations", it, ito, "max |dx|", np.abs(xs - xo).max(), np.abs(ys - yo).max())
    assert it == ito
    assert np.array_equal(xs, xo) and np.array_equal(ys, yo)
    assert q == qo


def _displacement(k, seed=5):
    rng = np.random.default_rng(seed)
    scale = 0.02 * np.abs(k.x).max() / np.sqrt(k.npoin)
    return scale * rng.normal(size=k.npoin), scale * rng.normal(size=k.npoin)


def test_oracle_tol_move_bounds_the_moves(oracle):
    """The setTol_move path: a node moves at most 1.5 + 1.5 + 1 times |dX| + |dY| (two
    Laplacian passes of tol/2 * FACTOR_STEP, NITER sweeps of tol / NITER)."""
    k, x, y, fixed = jittered()
    dX, dY = _displacement(k)
    xs, ys, it, q = oracle.smoothing(x, y, k.inpoel, fixed, dX=dX, dY=dY)
    tol = np.abs(dX) + np.abs(dY)
    move = np.abs(xs - x) + np.abs(ys - y)
    assert it >= 1 and move.max() > 0
    assert (move <= 4.0 * tol * (1 + 1e-12)).all()


@pytest.mark.gpu
def test_gpu_tol_move_smoothing_is_the_reference_in_colour_order(gpu_lib, oracle):
    """cfd_smoothing's setTol_move path (dX, dY given) against the oracle's, both visiting
    the nodes in the GPU's colour order: the same mesh bit for bit."""
    from cfd_gb300 import solver
    k, x, y, fixed = jittered()
    dX, dY = _displacement(k)
    order = oracle.colour_order(k.inpoel, k.npoin)
    xs, ys, it, q = solver.smoothing(x, y, k.inpoel, fixed, dX, dY)
    xo, yo, ito, qo = oracle.smoothing(x, y, k.inpoel, fixed, order=order, dX=dX, dY=dY)
    print("iterations", it, ito, "max |dx|", np.abs(xs - xo).max(), np.abs(ys - yo).max())
    assert it == ito
    assert np.array_equal(xs, xo) and np.array_equal(ys, yo)


def test_oracle_case_smooths_in_the_loop(oracle):
    """The oracle's time loop with the per-step smoothing: the state stays finite and the
    mesh differs from the unsmoothed run's."""
    k = small_case(2, scale=16, seed=1)
    a, b = oracle.OracleCase(k), oracle.OracleCase(k)
    b.set_smoothing(1)
    a.step(2)
    b.step(2)
    sa, sb = a.state(), b.state()
    assert np.isfinite(sb["U"]).all()
    assert not np.array_equal(sa["X"], sb["X"])
    a.close()
    b.close()


@pytest.mark.gpu
def test_gpu_fp64_smoothing_in_the_loop_bit_exact(gpu_lib, oracle):
    """The FP64 form with the moved mesh smoothed every 2nd step against the oracle's loop
    with the same smoothing in the GPU's colour order: state, mesh, DTMIN and BiCG counts
    equal bit for bit over 6 steps."""
    from cfd_gb300 import abi, solver
    k = small_case(2, scale=16, seed=1)
    g = solver.Solver(k, precision=abi.CFD_PREC_FP64)
    o = oracle.OracleCase(k)
    g.set_smoothing(2)
    o.set_smoothing(2)
    for s in range(6):
        rg, ro = g.step(1), o.step(1)
        assert rg.dtmin == ro.dtmin and tuple(rg.bicg_iters) == tuple(ro.bicg_iters), s
        sg, so = g.state(), o.state()
        for key in ("U", "T", "X", "Y"):
            assert np.array_equal(sg[key], so[key]), (s, key, np.abs(sg[key] - so[key]).max())
    assert g.smoothing_stats()[0] == 3
    g.close()
    o.close()


@pytest.mark.gpu
def test_gpu_node_order_smoothing_is_the_reference(gpu_lib, oracle):
    """CFD_SMOOTH_NODE_ORDER visits the nodes one at a time in node order, as the reference
    does (smoothing.f90:55-67, :80-114): the mesh, the sweep count and the quality are the
    node-order oracle's, bit for bit, on the setup path and on the setTol_move path."""
    from cfd_gb300 import abi, solver
    k, x, y, fixed = jittered()
    xs, ys, it, q = solver.smoothing(x, y, k.inpoel, fixed, order=abi.CFD_SMOOTH_NODE_ORDER)
    xo, yo, ito, qo = oracle.smoothing(x, y, k.inpoel, fixed)
    assert (it, q) == (ito, qo) and it >= 1
    assert np.array_equal(xs, xo) and np.array_equal(ys, yo)
    rng = np.random.default_rng(4)
    h = 1e-3
    dX, dY = h * rng.uniform(-1, 1, k.npoin), h * rng.uniform(-1, 1, k.npoin)
    xs, ys, it, q = solver.smoothing(x, y, k.inpoel, fixed, dX=dX, dY=dY,
                                     order=abi.CFD_SMOOTH_NODE_ORDER)
    xo, yo, ito, qo = oracle.smoothing(x, y, k.inpoel, fixed, dX=dX, dY=dY)
    assert (it, q) == (ito, qo)
    assert np.array_equal(xs, xo) and np.array_equal(ys, yo)


@pytest.mark.gpu
def test_gpu_setup_smoothing_in_node_order_then_steps_are_the_references(gpu_lib):
    """A host that smooths at setup (ns2DComp.ALE.f90:76) through cfd_ctx_smooth_ex with the
    node order gets the reference's mesh, and the steps after it match the oracle's run of
    the same setup bit for bit."""
    from cfd_gb300 import abi, solver
    from oracle import oracle as O
    from test_gpu_parity import eq
    k = small_case(2, scale=16, seed=3)
    g = solver.Solver(k)
    g.smooth(order=abi.CFD_SMOOTH_NODE_ORDER)
    o = O.OracleCase(k, smoothing=True)
    sg, so = g.state(), o.state()
    eq(sg["X"], so["X"], "X after setup smoothing")
    eq(sg["Y"], so["Y"], "Y after setup smoothing")
    for s in range(2):
        rg, ro = g.step(1), o.step(1)
        assert rg.dtmin == ro.dtmin and tuple(rg.bicg_iters) == tuple(ro.bicg_iters)
        sg, so = g.state(), o.state()
        for key in ("U", "T", "X", "Y"):
            eq(sg[key], so[key], f"step {s + 1}: {key}")
    g.close()
    o.close()

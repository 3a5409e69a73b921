"""Known-answer tests of the oracle (the CPU restatement), derived from the mathematics of
the discretisation: they pin the restatement where the reference has no tests."""
import math

import numpy as np
import pytest

from conftest import perturbed_state, small_case


@pytest.fixture(scope="module")
def mesh():
    return small_case(1, scale=12, seed=5)


def test_deriv_exact_on_linear_fields(oracle, mesh):
    g = oracle.deriv(mesh.x, mesh.y, mesh.inpoel)
    assert np.all(g["area"] > 0), "generator must produce counter-clockwise triangles"
    n = mesh.inpoel - 1
    f = 2.5 * mesh.x - 1.25 * mesh.y + 3.0
    fx = np.sum(g["dNx"] * f[n], 1)
    fy = np.sum(g["dNy"] * f[n], 1)
    np.testing.assert_allclose(fx, 2.5, rtol=0, atol=1e-9)
    np.testing.assert_allclose(fy, -1.25, rtol=0, atol=1e-9)
    # partition of unity of the gradients
    np.testing.assert_allclose(g["dNx"].sum(1), 0.0, atol=1e-9)
    assert g["hmin"] == pytest.approx(np.sqrt(g["area"]).min())


def test_mass_total_area_and_translation(oracle, mesh):
    g = oracle.deriv(mesh.x, mesh.y, mesh.inpoel)
    M = oracle.masas(g["area"], mesh.inpoel, mesh.npoin)
    assert M.sum() == pytest.approx(g["area"].sum(), rel=1e-13)
    # annulus area with a polygonal body and outer ring
    assert M.sum() == pytest.approx(math.pi * (20.0 ** 2 - 0.5 ** 2), rel=0.02)
    g2 = oracle.deriv(mesh.x + 0.375, mesh.y - 0.125, mesh.inpoel)
    M2 = oracle.masas(g2["area"], mesh.inpoel, mesh.npoin)
    np.testing.assert_allclose(M2, M, rtol=1e-12)


def test_adjacency_and_pattern(oracle, mesh):
    e1, e2 = oracle.esup(mesh.inpoel, mesh.npoin)
    assert e2[0] == 0 and e2[-1] == 3 * mesh.nelem
    for p in [0, 5, mesh.npoin // 2, mesh.npoin - 1]:
        els = e1[e2[p]:e2[p + 1]] - 1
        assert np.all(np.diff(els) > 0), "esup lists elements in increasing order"
        assert np.all(np.any(mesh.inpoel[els] == p + 1, axis=1))
    p1, p2 = oracle.psup(mesh.inpoel, mesh.npoin)
    pairs = set()
    for p in range(mesh.npoin):
        for q in p1[p2[p]:p2[p + 1]]:
            pairs.add((p + 1, int(q)))
    assert all((q, p) in pairs for p, q in pairs), "psup is symmetric"
    rp, idx = oracle.laplace_pattern(mesh.inpoel, mesh.npoin)
    assert len(idx) == mesh.npoin + len(p1)
    assert np.all(idx[rp[:-1]] == np.arange(1, mesh.npoin + 1)), "diagonal first"


def test_laplacian_rows_sum_to_zero_and_symmetric(oracle, mesh):
    g = oracle.deriv(mesh.x, mesh.y, mesh.inpoel)
    rp, idx = oracle.laplace_pattern(mesh.inpoel, mesh.npoin)
    vals, diag = oracle.laplace(mesh.inpoel, g["dNx"], g["dNy"], mesh.x, mesh.y, rp, idx)
    rows = np.repeat(np.arange(mesh.npoin), np.diff(rp))
    rowsum = np.bincount(rows, weights=vals, minlength=mesh.npoin)
    np.testing.assert_allclose(rowsum, 0.0, atol=1e-8 * np.abs(diag).max())
    A = {(int(r), int(c) - 1): v for r, c, v in zip(rows, idx, vals)}
    asym = max(abs(v - A[(c, r)]) for (r, c), v in A.items())
    assert asym <= 1e-12 * np.abs(diag).max()
    assert np.all(diag > 0)


def test_uniform_freestream_has_zero_residual(oracle, mesh):
    """U uniform => Ux = Uy = 0 up to round-off => every term of calcRHS and FUENTE ~ 0."""
    p = mesh.params
    g = oracle.deriv(mesh.x, mesh.y, mesh.inpoel)
    n, ne = mesh.npoin, mesh.nelem
    U, T, u, v = perturbed_state(mesh, amp=0.0)
    shoc, t1, t2, t3 = oracle.estab(U, T, np.full(n, p.gama), u, v, np.zeros(n), np.zeros(n),
                                    g["dNx"], g["dNy"], mesh.inpoel, p.gama, p.fr, 1e-3,
                                    p.rho_inf, p.t_inf)
    rhs = oracle.calcrhs(np.zeros((n, 4)), U, np.zeros((n, 4)), g["dNx"], g["dNy"], g["area"],
                         shoc, np.full(ne, 1e-3), t1, t2, t3, mesh.inpoel, T, p.gas6())
    scale = np.abs(U).max() * g["area"].max() * 1e-3 * np.abs(g["dNx"]).max()
    assert np.all(np.abs(rhs).max(0) <= 1e-10 * scale * 1e3)
    w = np.full(n, 0.3)
    f = oracle.fuente(np.zeros((n, 4)), U, w, -w, g["dNx"], g["dNy"], g["area"],
                      np.full(ne, 1e-3), mesh.inpoel)
    assert np.all(np.abs(f).max(0) <= 1e-10 * scale * 1e3)


def test_bicg_solves_the_dirichlet_problem(oracle, mesh):
    """The operator sum_e (grad Ni . grad Nj)/mu_e^2 has no area weight, so only constants
    are in its kernel (affine fields are not); check the solve against the system itself:
    free rows satisfy A.x = 0, fixed rows hold their data."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    g = oracle.deriv(mesh.x, mesh.y, mesh.inpoel)
    rp, idx = oracle.laplace_pattern(mesh.inpoel, mesh.npoin)
    vals, diag = oracle.laplace(mesh.inpoel, g["dNx"], g["dNy"], mesh.x, mesh.y, rp, idx)
    fix = mesh.ilaux()
    data = 0.01 * np.sin(mesh.x[fix - 1]) - 0.02 * mesh.y[fix - 1]
    x, info = oracle.bicg(vals, idx, rp, diag, np.zeros(mesh.npoin), np.zeros(mesh.npoin),
                          data, fix, tol=1e-26, maxit=4000)
    assert info.converged == 1
    A = sp.csr_matrix((vals, idx - 1, rp), shape=(mesh.npoin, mesh.npoin))
    free = np.ones(mesh.npoin, bool)
    free[fix - 1] = False
    np.testing.assert_array_equal(x[fix - 1], data)
    assert np.abs((A @ x)[free]).max() <= 1e-10 * np.abs(A).max() * np.abs(data).max()
    # the same system solved directly
    Aff = A[free][:, free]
    rhs = -(A[free][:, ~free] @ x[~free])
    xd = spla.spsolve(Aff.tocsc(), rhs)
    np.testing.assert_allclose(x[free], xd, atol=1e-9 * np.abs(data).max())


def test_bicg_rigid_translation_and_cap(oracle, mesh):
    g = oracle.deriv(mesh.x, mesh.y, mesh.inpoel)
    rp, idx = oracle.laplace_pattern(mesh.inpoel, mesh.npoin)
    vals, diag = oracle.laplace(mesh.inpoel, g["dNx"], g["dNy"], mesh.x, mesh.y, rp, idx)
    fix = mesh.ilaux()
    xf = np.full(len(fix), 0.01)
    x, info = oracle.bicg(vals, idx, rp, diag, np.zeros(mesh.npoin), np.zeros(mesh.npoin), xf,
                          fix, tol=1e-26, maxit=2000)
    np.testing.assert_allclose(x, 0.01, atol=1e-10)
    # the iteration cap ends a solve that cannot reach the tolerance, with the status set
    x, info = oracle.bicg(vals, idx, rp, diag, np.zeros(mesh.npoin), np.zeros(mesh.npoin), xf,
                          fix, tol=1e-300, maxit=3)
    assert info.iters == 3 and info.converged == 0


def test_vecdot_fixed_tree(oracle):
    rng = np.random.default_rng(1)
    for n in [0, 1, 255, 1024, 1025, 5000, 300001]:
        a, b = rng.normal(size=n), rng.normal(size=n)
        d = oracle.vecdot(a, b)
        assert d == pytest.approx(math.fsum(a * b), abs=1e-10 * max(1, n))
    # emulate the tree for a 2-chunk case in numpy
    n = 1500
    a, b = rng.normal(size=n), rng.normal(size=n)
    prod = np.zeros(2048)
    prod[:n] = a * b

    def tree256(s):
        s = s.copy()
        w = []
        for wi in range(8):
            v = s[32 * wi:32 * wi + 32].copy()
            off = 16
            while off:
                v[:off] = v[:off] + v[off:2 * off]
                off //= 2
            w.append(v[0])
        w = np.array(w)
        off = 4
        while off:
            w[:off] = w[:off] + w[off:2 * off]
            off //= 2
        return w[0]

    parts = []
    for c in range(2):
        base = prod[1024 * c:1024 * (c + 1)]
        s = np.zeros(256)
        for t in range(256):
            acc = base[t]
            for k in range(1, 4):
                if 1024 * c + t + 256 * k < n:
                    acc = acc + base[t + 256 * k]
            s[t] = acc
        parts.append(tree256(s))
    s = np.zeros(256)
    s[:2] = parts
    assert oracle.vecdot(a, b) == tree256(s)


def test_gcl_literal_vs_corrected(oracle, mesh):
    g = oracle.deriv(mesh.x, mesh.y, mesh.inpoel)
    M = oracle.masas(g["area"], mesh.inpoel, mesh.npoin)
    n = mesh.npoin
    wx, wy = np.zeros(n), np.full(n, 0.7)  # rigid heave: div W = 0
    Mc = oracle.gcl(M, wx, wy, wx, wy, g["dNx"], g["dNy"], g["area"], g["area"], mesh.inpoel,
                    1e-2, 2)
    np.testing.assert_allclose(Mc, M, rtol=1e-12)
    wx2 = np.full(n, 0.4)
    Ml = oracle.gcl(M, wx2, wy, wx2, wy, g["dNx"], g["dNy"], g["area"], g["area"],
                    mesh.inpoel, 1e-2, 1)
    # literal divW = sum(dNx + dNy) * W_x: nonzero only through round-off
    np.testing.assert_allclose(Ml, M, rtol=1e-10)


def test_normales_unit_and_outward_cw(oracle, mesh):
    ni, nx, ny = oracle.normales(mesh.wall, mesh.x, mesh.y)
    assert len(ni) == len(mesh.i_m)
    np.testing.assert_allclose(np.hypot(nx, ny), 1.0, rtol=1e-12)
    # clockwise body edges: the edge normal (dy, -dx) points into the body
    px, py = mesh.x[ni - 1], mesh.y[ni - 1]
    assert np.all(nx * px + ny * py < 0)


def test_smoothing_improves_quality(oracle):
    k = small_case(1, scale=10, seed=2)
    x, y = k.x.copy(), k.y.copy()
    fixed = np.zeros(k.npoin, np.int32)
    fixed[k.ilaux() - 1] = 1
    # disturb interior nodes to create bad elements
    rng = np.random.default_rng(0)
    inner = np.where(fixed == 0)[0]
    x[inner] += rng.uniform(-0.2, 0.2, len(inner)) * 0.05
    q0 = np.min(mesh_quality(x, y, k.inpoel))
    xs, ys, it, q1 = oracle.smoothing(x, y, k.inpoel, fixed)
    assert it >= 1
    assert q1 >= q0 - 1e-15
    np.testing.assert_array_equal(xs[fixed == 1], x[fixed == 1])


def mesh_quality(x, y, inpoel):
    n = inpoel - 1
    X, Y = x[n], y[n]
    a = (X[:, 1] * Y[:, 2] + X[:, 2] * Y[:, 0] + X[:, 0] * Y[:, 1]
         - (X[:, 1] * Y[:, 0] + X[:, 2] * Y[:, 1] + X[:, 0] * Y[:, 2]))
    l = ((X[:, 2] - X[:, 1]) ** 2 + (Y[:, 2] - Y[:, 1]) ** 2 + (X[:, 0] - X[:, 2]) ** 2
         + (Y[:, 0] - Y[:, 2]) ** 2 + (X[:, 1] - X[:, 0]) ** 2 + (Y[:, 1] - Y[:, 0]) ** 2)
    return 3.46410161513775 * a / l


def test_driver_freestream_fixed_mesh_stays_uniform(oracle):
    """Fixed mesh, uniform freestream on every boundary and inviscid gas: nothing moves."""
    k = small_case(1, scale=8, seed=1)
    k.params.fmu = 0.0
    # no wall: treat the body ring like the far field
    k.ifixv_node = np.concatenate([k.ifm, k.i_m]).astype(np.int32)
    k.rfixv_valuex = np.full(len(k.ifixv_node), k.params.u_inf)
    k.rfixv_valuey = np.full(len(k.ifixv_node), k.params.v_inf)
    k.ifixt_node = k.ifixv_node.copy()
    k.rfixt_value = np.full(len(k.ifixt_node), k.params.t_inf)
    k.wall = np.zeros((0, 2), np.int32)
    oc = oracle.OracleCase(k)
    s0 = oc.state()
    rep = oc.step(3)
    s1 = oc.state()
    np.testing.assert_allclose(s1["U"], s0["U"], rtol=1e-9, atol=1e-12 * np.abs(s0["U"]).max())
    assert rep.bicg_iters[0] == 0 and np.all(s1["X"] == s0["X"])


def test_driver_heave_moves_body_rigidly(oracle):
    k = small_case(2, scale=10, seed=4)
    oc = oracle.OracleCase(k)
    x0 = oc.state()
    rep = oc.step(2)
    st = oc.state()
    dy = st["Y"][k.i_m - 1] - x0["Y"][k.i_m - 1]
    np.testing.assert_allclose(dy, dy[0], rtol=1e-9)
    assert dy[0] == pytest.approx(0.2 * math.sin(2 * math.pi * 0.2 * rep.time), rel=1e-9)
    np.testing.assert_array_equal(st["Y"][k.ifm - 1], x0["Y"][k.ifm - 1])
    assert np.all(np.isfinite(st["U"]))


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_reference_estab_is_discontinuous(oracle):
    """The reference ESTAB makes the step discontinuous at round-off level: unit vectors
    of round-off gradients (subrutinas.f90:374-393).  A 1e-13 perturbation comes back
    ~1e-4; under CFD_ESTAB_REGULARIZED the response is proportional."""
    k = small_case(3, scale=96, seed=0, estab_mode=0)
    k.params.fsafe = 0.25
    a, b = oracle.OracleCase(k), oracle.OracleCase(k)
    a.step(1)
    b.step(1)
    st, f = a.state(), a.fields()
    rng = np.random.default_rng(0)
    b.set_state(st["U"] * (1 + 1e-13 * rng.uniform(-1, 1, st["U"].shape)), st["T"], f["VEL_X"],
                f["VEL_Y"])
    a.step(1)
    b.step(1)
    d = _rel(b.state()["U"][:, 0], a.state()["U"][:, 0])
    assert d > 1e-9, "the reference ESTAB should amplify a 1e-13 perturbation"
    k.params.estab_mode = 2
    a, b = oracle.OracleCase(k), oracle.OracleCase(k)
    a.step(1)
    b.step(1)
    st, f = a.state(), a.fields()
    b.set_state(st["U"] * (1 + 1e-13 * rng.uniform(-1, 1, st["U"].shape)), st["T"], f["VEL_X"],
                f["VEL_Y"])
    a.step(1)
    b.step(1)
    assert _rel(b.state()["U"][:, 0], a.state()["U"][:, 0]) < 1e-10

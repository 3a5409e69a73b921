"""The 2-DOF Newmark structural model (meshMove.f90:196-367, enabled as CFD_MOTION_NEWMARK):
the oracle's statement-by-statement restatement against the matrix form of the
average-acceleration scheme, its static limit, and the FP64 (bit for bit) and mixed
(to tolerance) CUDA forms against the oracle on a coupled case."""
import numpy as np
import pytest

from conftest import small_case

M = np.array([[51.5, -51.5 * 0.0429], [-51.5 * 0.0429, 2.275]])
C = np.diag([32.358, 5.718])
K = np.diag([50828.463, 35923.241])


def newmark_matrix_form(H, F, d, v, a, gamma=0.5, beta=0.25):
    """(K + M/(beta H^2) + gamma C/(beta H)) d' = F + M(...) + C(...), then a', v'."""
    a1, a2, a3 = 1 / (beta * H * H), 1 / (beta * H), 1 / (2 * beta) - 1
    a1d, a2d, a3d = gamma / (beta * H), gamma / beta - 1, 0.5 * H * (gamma / beta - 2)
    keff = K + a1 * M + a1d * C
    r = F + M @ (a1 * d + a2 * v + a3 * a) + C @ (a1d * d + a2d * v + a3d * a)
    dn = np.linalg.solve(keff, r)
    an = a1 * (dn - d) - a2 * v - a3 * a
    vn = v + (1 - gamma) * H * a + gamma * H * an
    return dn, vn, an


def test_oracle_newmark_matches_matrix_form(oracle):
    rng = np.random.default_rng(4)
    for _ in range(20):
        H = 10 ** rng.uniform(-5, -2)
        F = rng.normal(0, 100, 2)
        d, v, a = rng.normal(0, 1e-2, 2), rng.normal(0, 1e-1, 2), rng.normal(0, 10, 2)
        got = oracle.newmark_step(H, F, d, v, a)
        ref = newmark_matrix_form(H, F, d, v, a)
        for g, r in zip(got, ref):
            assert np.allclose(g, r, rtol=1e-10, atol=1e-13 * np.abs(r).max())


def test_oracle_newmark_rest_and_static_limit(oracle):
    z = np.zeros(2)
    d, v, a = oracle.newmark_step(1e-3, z, z, z, z)
    assert not d.any() and not v.any() and not a.any()
    # a constant load: the damped oscillation settles at K^-1 F
    F = np.array([500.0, -20.0])
    d, v, a = z, z, z
    for _ in range(40000):
        d, v, a = oracle.newmark_step(2e-3, F, d, v, a)
    assert np.allclose(d, np.linalg.solve(K, F), rtol=1e-4)


def coupled_case(scale=16, seed=9, **over):
    from cfd_gb300 import abi
    return small_case(2, scale=scale, seed=seed, motion_law=abi.CFD_MOTION_NEWMARK, **over)


def test_oracle_coupled_case_moves(oracle):
    k = coupled_case()
    o = oracle.OracleCase(k)
    x0 = o.state()["X"].copy()
    o.step(3)
    assert np.abs(o.state()["X"] - x0).max() > 0.0
    o.close()


@pytest.mark.gpu
def test_fp64_newmark_bit_exact(gpu_lib):
    from test_gpu_parity import run_pair
    run_pair(coupled_case(), 3)


@pytest.mark.gpu
def test_mixed_newmark_close(gpu_lib):
    from cfd_gb300 import abi, solver
    from oracle import oracle as O
    from test_gpu_mixed import REL_TOL_STATE, state_errors
    k = coupled_case(scale=24, estab_mode=abi.CFD_ESTAB_REGULARIZED)
    g = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    o = O.OracleCase(k)
    for _ in range(4):
        rg, ro = g.step(1), o.step(1)
    sg, so = g.state(), o.state()
    assert max(state_errors(sg["U"], so["U"])) <= REL_TOL_STATE
    # the body follows the structural model, driven by the pressure force and moment
    body = k.i_m - 1
    for c in ("X", "Y"):
        dg, do = sg[c][body] - getattr(k, c.lower())[body], so[c][body] - getattr(k, c.lower())[body]
        assert np.abs(do).max() > 0.0
        assert np.abs(dg - do).max() <= 1e-5 * np.abs(do).max()
    g.close()
    o.close()

"""Learned mesh-motion guess on the GPU: forward pass and gradients of the library's
training kernels against the CPU oracle (oracle/mpnn_ref.py), Adam, determinism, the BF16
tensor-core inference pass against the FP32 pass, and what the trained network gains over
the zero initial guess of the plain BiCG solve."""
import os

import numpy as np
import pytest

from conftest import small_case
from oracle import mpnn_ref as M
from test_mpnn_ref import mpnn_graph, rigid

pytestmark = pytest.mark.gpu


def setup(k, heave=0.2, pitch=7.0, seed=0):
    from cfd_gb300 import learned
    ptr, nbr, kind = mpnn_graph(k)
    gfull = rigid(k, kind, heave, pitch)
    G = learned.Graph(k)
    bn = G.bnode - 1
    G.set_bc(gfull[bn, 0], gfull[bn, 1])
    Gr = M.globals_(k.x, k.y, kind, gfull)
    f = M.features(k.x, k.y, kind, Gr)
    i, j, e, deg = M.edges(k.x, k.y, ptr, nbr, Gr["L"])
    return G, kind, gfull, Gr, (f, i, j, e, deg)


def test_globals_match_oracle(gpu_lib):
    k = small_case(1, scale=12, seed=2)
    G, kind, gfull, Gr, _ = setup(k)
    gg = G.globals()
    for key in ("cx", "cy", "L", "R", "tx", "ty", "m11", "m12", "m21", "m22"):
        assert abs(gg[key] - Gr[key]) <= 1e-12 * max(1.0, abs(Gr[key])), key


def test_forward_and_gradient_match_oracle(gpu_lib):
    from cfd_gb300 import learned
    k = small_case(1, scale=12, seed=2)
    G, kind, gfull, Gr, (f, i, j, e, deg) = setup(k)
    rng = np.random.default_rng(4)
    w = (M.init_params(7) + 0.05 * rng.normal(size=M.n_params())).astype(np.float32)
    net = learned.Net(w)
    phi, psx, psy = (0.3 * rng.normal(size=k.npoin) for _ in range(3))
    G.set_target(phi, psx, psy)
    # forward (FP32 pass) and the guess it gives
    px, py = net.forward(G, bf16=False)
    y = M.forward(w.astype(np.float64), f, i, j, e, deg)
    free = kind == 0
    ref = M.guess(y, Gr, kind, gfull)
    got = np.stack([px, py], 1)
    assert np.abs(got[free] - ref[free]).max() <= 1e-5 * np.abs(ref[free]).max()
    assert np.array_equal(got[~free], gfull[~free])
    # loss and gradient
    loss, grad = net.loss_grad(G)
    target = np.stack([phi, psx / Gr["L"], psy / Gr["L"]], 1)
    lref, gref = M.loss_and_grad(w.astype(np.float64), f, i, j, e, deg, target,
                                 free.astype(float))
    assert abs(loss - lref) <= 1e-5 * lref
    P, Pr = M.unpack(grad.astype(np.float64)), M.unpack(gref)
    for name in Pr:
        nr = np.linalg.norm(Pr[name])
        assert np.linalg.norm(P[name] - Pr[name]) <= 2e-4 * max(nr, 1e-8), name


def test_adam_step_and_determinism(gpu_lib):
    from cfd_gb300 import learned
    k = small_case(1, scale=12, seed=3)
    G, kind, gfull, Gr, _ = setup(k, 0.1, -4.0)
    rng = np.random.default_rng(1)
    G.set_target(*(0.3 * rng.normal(size=k.npoin) for _ in range(3)))
    w0 = learned.init_weights(3)
    a, b = learned.Net(w0), learned.Net(w0)
    _, g0 = a.loss_grad(G)
    a.train_step(G, 1e-3)
    wa = a.weights()
    m, v, t = a.adam_state()
    wr, mr, vr = M.adam(w0, g0, np.zeros_like(w0), np.zeros_like(w0), 1, 1e-3)
    assert t == 1
    assert np.allclose(m, mr, rtol=1e-6, atol=1e-12) and np.allclose(v, vr, rtol=1e-6, atol=1e-18)
    assert np.abs(wa - wr).max() <= 1e-6
    for _ in range(3):
        a.train_step(G, 1e-3)
    b.train_step(G, 1e-3)
    for _ in range(3):
        b.train_step(G, 1e-3)
    assert np.array_equal(a.weights(), b.weights())


def test_bf16_inference_matches_fp32(gpu_lib):
    from cfd_gb300 import learned
    k = small_case(1, scale=24, seed=6)
    G, kind, gfull, Gr, _ = setup(k, -0.15, 5.0)
    rng = np.random.default_rng(9)
    net = learned.Net((learned.init_weights(2) + 0.02 * rng.normal(size=learned.n_params()))
                      .astype(np.float32))
    fx, fy = net.forward(G, bf16=False)
    bx, by = net.forward(G, bf16=True)
    free = kind == 0
    d = np.hypot(bx - fx, by - fy)[free]
    nrm = np.hypot(fx, fy)[free]
    assert np.linalg.norm(d) <= 3e-2 * np.linalg.norm(nrm)
    assert np.array_equal(bx[~free], fx[~free]) and np.array_equal(by[~free], fy[~free])


@pytest.mark.parametrize("scale", [22, 5])
def test_tcgen05_inference_matches_mma_sync(gpu_lib, monkeypatch, scale):
    """The tcgen05 passes (the default: accumulators in tensor memory) and the mma.sync
    passes (CFD_MPNN_TC=0) take the same BF16 operands and round the same FP32 sums to
    BF16; only the order of the FP32 sums differs.  968 nodes: a ragged last tile; 50
    nodes: less than one 128-node tile."""
    from cfd_gb300 import learned
    k = small_case(1, scale=scale, seed=6)
    assert k.npoin % 128 != 0
    G, kind, gfull, Gr, _ = setup(k, -0.15, 5.0)
    rng = np.random.default_rng(4)
    net = learned.Net((learned.init_weights(3) + 0.02 * rng.normal(size=learned.n_params()))
                      .astype(np.float32))
    monkeypatch.setenv("CFD_MPNN_TC", "0")
    mx, my = net.forward(G, bf16=True)
    monkeypatch.delenv("CFD_MPNN_TC")
    tx, ty = net.forward(G, bf16=True)
    tx2, ty2 = net.forward(G, bf16=True)
    fx, fy = net.forward(G, bf16=False)
    assert np.array_equal(tx, tx2) and np.array_equal(ty, ty2)
    free = kind == 0
    nrm = np.linalg.norm(np.hypot(fx, fy)[free])
    d_mma = np.linalg.norm(np.hypot(tx - mx, ty - my)[free]) / nrm
    d_f32 = np.linalg.norm(np.hypot(tx - fx, ty - fy)[free]) / nrm
    print("tcgen05 vs mma.sync", d_mma, "vs FP32", d_f32)
    assert d_mma <= 5e-3
    assert d_f32 <= 3e-2


def test_trained_guess_beats_zero_guess(gpu_lib):
    """The shipped weights: on a mesh and motions not in the training set, BiCG from the
    network's guess reaches the same solution (to the solve tolerance) in fewer
    iterations than from the zero guess of the plain method."""
    from cfd_gb300 import case as cs, learned
    if not os.path.exists(learned.DEFAULT_WEIGHTS):
        pytest.skip("no trained weights in the package")
    net = learned.Net.load()
    c = cs.ogrid_case("heldout", 96, 160, cs.flow_params(mach=0.3, re=100.0), body="ellipse",
                      r_body=0.5, semi_b=0.17, incidence_deg=3.0, r_out=22.0, seed=777)
    tot0 = tot1 = 0
    for heave, pitch in ((0.25, 0.0), (0.0, 8.0), (-0.12, -5.0)):
        r = learned.guess_gain(net, c, heave, pitch)
        assert all(r["converged"][0]) and all(r["converged"][1])
        # both solves meet the absolute r.z tolerance; their solutions agree to ~1e-5 of
        # the displacement
        assert r["max_diff"] < 1e-4 * max(abs(heave), 0.5 * np.radians(abs(pitch)))
        assert r["guess_rel_l2"] < 0.1
        tot0 += sum(r["iters_zero"])
        tot1 += sum(r["iters_net"])
    assert tot1 < 0.85 * tot0, (tot1, tot0)

"""The learned guess inside the resident mixed-form step (CFD_GUESS_LEARNED): the network
is evaluated when the gate opens, its guess is taken only when its residual is smaller,
and BiCG still finishes to the plain tolerance.  The solve's tolerance is absolute
(r.z < 1e-10, biconjGrad.f90:26) and loose against the per-step increments of these
cases, so two guesses give two admissible mesh motions: the flow is compared with the
previous-step-guess run to the bound that this allows."""
import os

import numpy as np
import pytest

from conftest import small_case

pytestmark = pytest.mark.gpu


def run(k, steps, net=None, gate=0.0):
    from cfd_gb300 import abi, solver
    S = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    if net is not None:
        S.set_guess_net(net, gate)
    reps = [S.step(1) for _ in range(steps)]
    st = S.state()
    stats = S.guess_stats() if net is not None else None
    S.close()
    return reps, st, stats


def test_learned_guess_in_the_step(gpu_lib):
    from cfd_gb300 import abi, learned
    if not os.path.exists(learned.DEFAULT_WEIGHTS):
        pytest.skip("no trained weights in the package")
    net = learned.Net.load()
    kw = dict(scale=48, seed=13, estab_mode=abi.CFD_ESTAB_REGULARIZED, fsafe=0.25)
    kp = small_case(3, **kw)
    kl = small_case(3, **kw)
    kl.params.guess_mode = abi.CFD_GUESS_LEARNED
    steps = 6
    rp, sp, _ = run(kp, steps)
    rl, sl, stats = run(kl, steps, net, gate=0.0)
    # gate 0: evaluated every step; the cold first step takes the network's guess
    assert stats[0] == steps and stats[3] == steps
    assert stats[2] >= 1
    it_prev = sum(rp[0].bicg_iters)
    it_net = sum(rl[0].bicg_iters)
    assert it_net < it_prev, (it_net, it_prev)
    for r in rl:
        assert all(r.bicg_converged)
    for q in range(4):
        d = np.linalg.norm(sl["U"][:, q] - sp["U"][:, q])
        assert d <= 2e-5 * np.linalg.norm(sp["U"][:, q]) + 1e-12


def test_gate_runs_the_network_on_the_cold_solve_only(gpu_lib):
    """gate = iteration threshold: the network runs on the first solve after attaching and
    again only after a solve that took more iterations than the gate."""
    from cfd_gb300 import abi, learned
    if not os.path.exists(learned.DEFAULT_WEIGHTS):
        pytest.skip("no trained weights in the package")
    net = learned.Net.load()
    kw = dict(scale=48, seed=13, estab_mode=abi.CFD_ESTAB_REGULARIZED, fsafe=0.25)
    kl = small_case(3, **kw)
    kl.params.guess_mode = abi.CFD_GUESS_LEARNED
    reps, _, stats = run(kl, 6, net, gate=1.0e9)
    assert stats[0] == 1 and stats[3] == 6
    reps2, _, stats2 = run(small_case(3, **dict(kw, guess_mode=abi.CFD_GUESS_LEARNED)), 6, net,
                           gate=0.5)
    # after the cold solve, steps whose solve took >= 1 iteration trigger the next one
    expect = 1 + sum(1 for r in reps2[:-1] if max(r.bicg_iters) > 0.5)
    assert stats2[0] == expect and stats2[3] == 6


def test_refined_guess_under_the_relative_test(gpu_lib):
    """Under the 1e-10 relative test the mixed form assembles the mesh-motion operator in
    FP64 as well (the first residual's precise product): the refined learned guess then
    meets the test in far fewer iterations than the previous step's increment, and every
    solve still reaches the test."""
    from cfd_gb300 import abi, learned, solver
    if not os.path.exists(learned.DEFAULT_WEIGHTS):
        pytest.skip("no trained weights in the package")
    net = learned.Net.load()
    its = {}
    for refined in (False, True):
        k = small_case(3, scale=96, seed=13, estab_mode=abi.CFD_ESTAB_REGULARIZED, fsafe=0.25,
                       bicg_tol_mode=abi.CFD_BICG_TOL_REL, bicg_maxit=20000)
        if refined:
            k.params.guess_mode = abi.CFD_GUESS_LEARNED
        S = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
        if refined:
            S.set_guess_net(net, 1.0e9)
            S.set_guess_refine(True)
        per_step = []
        for _ in range(8):
            r = S.step(1)
            assert all(r.bicg_converged) and max(r.bicg_relres) <= 1e-10
            per_step.append(sum(r.bicg_iters))
        its[refined] = per_step
        S.close()
    assert sum(its[True][3:]) * 4 < sum(its[False][3:]), its


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["learned", "learned_extrapolated"])
def test_refined_guess_graph_replay_matches_launches(gpu_lib, monkeypatch, mode):
    """The refined learned guess's kernels run on a side stream beside the mesh-motion
    branch (the fields' guess beside the first residual pass, their update beside the mesh
    update), joined by events.  Steps replayed from the captured graph give the iterations,
    the guess statistics and the state of the same steps enqueued launch by launch
    (CFD_GRAPHS=0), bit for bit."""
    from cfd_gb300 import abi, learned, solver
    if not os.path.exists(learned.DEFAULT_WEIGHTS):
        pytest.skip("no trained weights in the package")
    net = learned.Net.load()
    gm = abi.CFD_GUESS_LEARNED if mode == "learned" else abi.CFD_GUESS_LEARNED_EXTRAPOLATED
    k = small_case(3, scale=48, seed=13, estab_mode=abi.CFD_ESTAB_REGULARIZED, fsafe=0.25,
                   bicg_tol_mode=abi.CFD_BICG_TOL_REL, bicg_maxit=20000, guess_mode=gm)
    monkeypatch.setenv("CFD_GRAPHS", "0")
    a = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    monkeypatch.delenv("CFD_GRAPHS")
    b = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    for s in (a, b):
        s.set_guess_net(net, 1.0e9)
        s.set_guess_refine(True)
    for n in (1, 1, 3, 4):
        ra, rb = a.step(n), b.step(n)
        assert list(ra.bicg_iters) == list(rb.bicg_iters)
        assert list(ra.bicg_relres) == list(rb.bicg_relres)
        assert all(rb.bicg_converged) and max(rb.bicg_relres) <= 1e-10
        sa, sb = a.state(), b.state()
        for key in ("U", "X", "Y"):
            assert np.array_equal(sa[key], sb[key]), key
    assert list(a.guess_stats_ex()) == list(b.guess_stats_ex())
    assert a.graph_state()[0] == 0 and b.graph_state()[0] == 1 and b.graph_state()[1] > 0
    a.close()
    b.close()

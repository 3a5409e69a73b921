"""The mixed-precision form (FP32 calcRHS/FUENTE/ESTAB/deltat/Laplacian values with
compensated node sums; FP64 state update, areas, gcl and BiCG) against the FP64 oracle.

Accuracy is measured under CFD_ESTAB_REGULARIZED: with the reference's ESTAB the step is
discontinuous at round-off level (unit vectors of round-off gradients), so no two
implementations that differ in rounding agree to better than ~1e-4 after one step
(test_reference_estab_is_discontinuous shows it on the oracle alone)."""
import numpy as np
import pytest

from conftest import perturbed_state, small_case

pytestmark = pytest.mark.gpu

REL_TOL_STATE = 1.0e-6   # rel L2 per conserved variable vs the FP64 oracle
REL_TOL_FORCE = 1.0e-3   # lift/drag (pressure force) relative error


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def state_errors(ug, uo):
    """rel L2 per conserved variable; rho*v (zero in the freestream) is measured against
    the momentum scale max(|rho*v|, |rho*u|) so that round-off-sized fields do not count."""
    out = []
    for q in range(4):
        den = np.linalg.norm(uo[:, q])
        if q == 2:
            den = max(den, np.linalg.norm(uo[:, 1]))
        out.append(float(np.linalg.norm(ug[:, q] - uo[:, q]) / den))
    return out


def run_mixed_vs_oracle(k, steps):
    from cfd_gb300 import abi, solver
    from oracle import oracle as O
    g = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    o = O.OracleCase(k)
    worst = [0.0] * 4
    fg, fo = [], []
    for s in range(steps):
        rg, ro = g.step(1), o.step(1)
        assert abs(rg.dtmin - ro.dtmin) <= 1e-6 * ro.dtmin
        e = state_errors(g.state()["U"], o.state()["U"])
        worst = [max(a, b) for a, b in zip(worst, e)]
        fg.append((rg.fx[0], rg.fy[0]))
        fo.append((ro.fx[0], ro.fy[0]))
    g.close()
    o.close()
    fg, fo = np.array(fg), np.array(fo)
    # lift/drag error over the run, against the largest force of the run
    fworst = float(np.abs(fg - fo).max() / np.abs(fo).max())
    return worst, fworst


@pytest.mark.parametrize("which,scale,steps", [(1, 16, 20), (3, 32, 20), (2, 32, 20)])
def test_mixed_matches_fp64_regularized(gpu_lib, which, scale, steps):
    k = small_case(which, scale=scale, seed=21, estab_mode=2)
    # coarse meshes need FSAFE 0.25 (deltat has no acoustic limit; the reference's own
    # step diverges at 0.5 on these sizes)
    k.params.fsafe = min(k.params.fsafe, 0.25)
    worst, fworst = run_mixed_vs_oracle(k, steps)
    print("worst rel L2 per variable", worst, "force", fworst)
    assert max(worst) <= REL_TOL_STATE
    assert fworst <= REL_TOL_FORCE


@pytest.mark.parametrize("mode", [1, 2])
def test_fp64_estab_modes_bit_exact(gpu_lib, mode):
    from test_gpu_parity import run_pair
    k = small_case(3, scale=20, seed=5, estab_mode=mode)
    run_pair(k, 3)


def test_mixed_deterministic(gpu_lib):
    from cfd_gb300 import abi, solver
    k = small_case(3, scale=32, seed=2, estab_mode=2)
    a = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    b = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    a.step(5)
    b.step(5)
    assert np.array_equal(a.state()["U"], b.state()["U"])
    assert np.array_equal(a.state()["X"], b.state()["X"])


def test_mixed_from_perturbed_state(gpu_lib):
    from cfd_gb300 import abi, solver
    from oracle import oracle as O
    k = small_case(3, scale=32, seed=4, estab_mode=2)
    U, T, u, v = perturbed_state(k, seed=3, amp=0.05)
    g = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    o = O.OracleCase(k)
    for side in (g, o):
        side.set_state(U, T, u, v)
    g.step(3)
    o.step(3)
    assert max(state_errors(g.state()["U"], o.state()["U"])) <= REL_TOL_STATE


def test_graph_replay_matches_launches(gpu_lib, monkeypatch):
    """Steps replayed from the captured CUDA graph give the state, clock and forces of the
    same steps enqueued launch by launch (CFD_GRAPHS=0), bit for bit, across downloads
    and a restart of the clock between steps."""
    from cfd_gb300 import abi, solver
    k = small_case(3, scale=32, seed=6, estab_mode=2)
    monkeypatch.setenv("CFD_GRAPHS", "0")
    a = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    monkeypatch.delenv("CFD_GRAPHS")
    b = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    for n in (1, 3, 2):
        if n == 2:
            for s in (a, b):
                s.set_clock(iter=10, time=0.25, dtmin1=ra.dtmin, bandera=3, disn1=0.01,
                            disn2=0.02)
        ra, rb = a.step(n), b.step(n)
        assert (ra.time, ra.dtmin, ra.iter) == (rb.time, rb.dtmin, rb.iter)
        assert list(ra.fx) == list(rb.fx) and list(ra.fy) == list(rb.fy)
        assert list(ra.bicg_iters) == list(rb.bicg_iters)
        sa, sb = a.state(), b.state()
        for key in ("U", "X", "Y"):
            assert np.array_equal(sa[key], sb[key]), key
    assert a.graph_state()[0] == 0
    on, replays, kernels = b.graph_state()
    assert on == 1 and replays == 5 and kernels > 10
    a.close()
    b.close()


def test_mixed_local_time_step(gpu_lib):
    """ITLOCAL != 0 (ns2DComp.ALE.f90:159-162): the element time step DTL enters calcRHS and
    FUENTE through area*dtl/3; the mixed form forms it from its FP32 DT per element."""
    k = small_case(1, scale=16, seed=21, estab_mode=2, itlocal=5)
    k.params.fsafe = min(k.params.fsafe, 0.25)
    worst, fworst = run_mixed_vs_oracle(k, 8)
    print("worst rel L2 per variable", worst, "force", fworst)
    assert max(worst) <= REL_TOL_STATE
    assert fworst <= REL_TOL_FORCE


def test_bulk_copy_node_pass_matches_plain_loads(gpu_lib, monkeypatch):
    """The node passes that stage their slot records with bulk copies (the default) sum the
    same products in the same order as the plain-load passes (CFD_NODE_BULK=0)."""
    from cfd_gb300 import abi, solver
    k = small_case(3, scale=32, seed=8, estab_mode=2)
    monkeypatch.setenv("CFD_NODE_BULK", "0")
    a = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    monkeypatch.delenv("CFD_NODE_BULK")
    b = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    a.step(4)
    b.step(4)
    ua, ub = a.state()["U"], b.state()["U"]
    assert np.abs(ua - ub).max() <= 1e-14 * np.abs(ua).max()
    a.close()
    b.close()


def test_full_size_mixed_learned_matches_fp64(gpu_lib):
    """The 1M-node ellipse O-grid (1024 x 1024) with the regularized ESTAB: the mixed form
    with the learned guess attached (it runs on the cold first solve) against the FP64
    form over 4 steps (the later ones replayed from the captured graph): the state within
    the mixed form's tolerance, DTMIN to 1e-6, the mesh to 1e-8 of the domain's size."""
    from cfd_gb300 import abi, case as C, learned, solver
    k = C.config_case(3)
    k.params.estab_mode = abi.CFD_ESTAB_REGULARIZED
    f = solver.Solver(k, precision=abi.CFD_PREC_FP64)
    k.params.guess_mode = abi.CFD_GUESS_LEARNED
    m = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    net = learned.Net.load()
    m.set_guess_net(net)
    for _ in range(4):
        rf, rm = f.step(1), m.step(1)
        assert abs(rm.dtmin - rf.dtmin) <= 1e-6 * rf.dtmin
    sf, sm = f.state(), m.state()
    err = state_errors(sm["U"], sf["U"])
    print("1M mixed+learned vs FP64, rel L2 per variable", err)
    assert max(err) <= REL_TOL_STATE
    for key in ("X", "Y"):  # two BiCG solves per step, each stopped at |r.z| <= 1e-10
        assert np.abs(sm[key] - sf[key]).max() <= 1e-8 * np.abs(sf[key]).max()
    assert m.guess_stats()[0] >= 1 and m.graph_state()[1] >= 2
    f.close()
    m.close()
    net.close()

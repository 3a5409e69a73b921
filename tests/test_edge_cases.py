"""Edge cases of the resident step: a mesh with no boundary lists at all (no Dirichlet
nodes, no wall, no force set, no mesh-motion nodes) and a single-triangle mesh, on the
oracle (CPU) and on both CUDA forms (GPU: FP64 bit for bit, mixed to tolerance, the
captured graph included)."""
import numpy as np
import pytest

from conftest import small_case


def square(n, perturbed=True):
    from cfd_gb300 import case as C
    xs, ys = np.meshgrid(np.arange(n, dtype=float), np.arange(n, dtype=float))
    x, y = xs.ravel().copy(), ys.ravel().copy()
    tri = []
    for j in range(n - 1):
        for i in range(n - 1):
            a = j * n + i + 1
            tri += [(a, a + 1, a + n + 1), (a, a + n + 1, a + n)]
    p = C.flow_params(0.3, 100.0, maxiter=10, moving=0)
    I, D = np.zeros(0, np.int32), np.zeros(0)
    k = C.Case(name="square", params=p, x=x, y=y, inpoel=np.array(tri, np.int32),
               ifixrho_node=I, rfixrho_value=D, ifixv_node=I, rfixv_valuex=D,
               rfixv_valuey=D, ifixt_node=I, rfixt_value=D, wall=np.zeros((0, 2), np.int32),
               iset_entries=np.zeros((0, 4), np.int32), i_m=I, ifm=I)
    state = None
    if perturbed:  # a non-uniform start, so that the step does something
        rng = np.random.default_rng(1)
        nn = k.npoin
        rho = p.rho_inf * (1 + 0.05 * rng.uniform(-1, 1, nn))
        u = p.u_inf * (1 + 0.05 * rng.uniform(-1, 1, nn))
        v = 0.05 * p.u_inf * rng.uniform(-1, 1, nn)
        T = p.t_inf * (1 + 0.05 * rng.uniform(-1, 1, nn))
        E = rho * p.fr * T / ((p.gama - 1) * rho) + 0.5 * (u * u + v * v)
        state = (np.stack([rho, rho * u, rho * v, rho * E], 1), T, u, v)
    return k, state


def single_triangle():
    k, _ = square(2, perturbed=False)
    k.inpoel = k.inpoel[:1].copy()
    keep = np.unique(k.inpoel)
    k.x, k.y = k.x[keep - 1].copy(), k.y[keep - 1].copy()
    remap = np.zeros(keep.max() + 1, np.int32)
    remap[keep] = np.arange(1, keep.size + 1)
    k.inpoel = remap[k.inpoel]
    return k


def test_oracle_runs_without_boundary_lists(oracle):
    k, st = square(5)
    o = oracle.OracleCase(k)
    o.set_state(*st)
    r = o.step(3)
    assert np.isfinite(o.state()["U"]).all() and r.dtmin > 0 and r.nset_numb == 0
    o.close()


@pytest.mark.gpu
def test_fp64_without_boundary_lists_bit_exact(gpu_lib):
    from test_gpu_parity import run_pair
    k, st = square(6)
    run_pair(k, 3, setup=lambda g, o: [s.set_state(*st) for s in (g, o)])


@pytest.mark.gpu
def test_mixed_without_boundary_lists(gpu_lib):
    from cfd_gb300 import abi, solver
    from oracle import oracle as O
    from test_gpu_mixed import state_errors
    k, st = square(8)
    k.params.estab_mode = abi.CFD_ESTAB_REGULARIZED
    g = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    o = O.OracleCase(k)
    for s in (g, o):
        s.set_state(*st)
    for _ in range(4):  # the first step runs launch by launch, the others replay the graph
        g.step(1)
        o.step(1)
    assert g.graph_state()[1] == 3
    assert max(state_errors(g.state()["U"], o.state()["U"])) <= 1e-6
    g.close()
    o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_single_triangle(gpu_lib, precision):
    from cfd_gb300 import solver
    from oracle import oracle as O
    k = single_triangle()
    g = solver.Solver(k, precision=precision)
    o = O.OracleCase(k)
    rg, ro = g.step(2), o.step(2)
    assert np.isfinite(g.state()["U"]).all()
    if precision == 0:
        assert rg.dtmin == ro.dtmin and np.array_equal(g.state()["U"], o.state()["U"])
    else:
        assert abs(rg.dtmin - ro.dtmin) <= 1e-6 * ro.dtmin
    g.close()
    o.close()


@pytest.mark.gpu
def test_bounded_waits_give_up_and_the_device_stays_usable(gpu_lib):
    """Failure detection without a fault: the library's grid barrier (a second block that
    never arrives) and its mbarrier wait (nothing arrives) give up after their poll limit
    and report CFD_ERR_BARRIER; a full step runs afterwards in the same process."""
    import ctypes as C
    from cfd_gb300 import abi, solver
    b, m = C.c_int(-1), C.c_int(-1)
    abi.check(abi.lib().cfd_selftest_waits(100000, C.byref(b), C.byref(m)), "selftest")
    assert b.value == abi.CFD_ERR_BARRIER and m.value == abi.CFD_ERR_BARRIER
    assert abi.lib().cfd_selftest_waits(0, C.byref(b), C.byref(m)) == abi.CFD_ERR_ARG
    k = small_case(3, scale=16, seed=3, estab_mode=2)
    s = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    rep = s.step(2)
    assert rep.iter == 2 and np.isfinite(s.state()["U"]).all()
    s.close()


@pytest.mark.gpu
def test_div3_equals_the_division(gpu_lib):
    """The FP64 kernels' division by 3 (a multiply and two FMAs) gives the IEEE quotient
    x / 3.0 bit for bit over 2^32 inputs: raw bit patterns (every exponent, zeros,
    subnormals, infinities, NaNs), values in 2^-40 .. 2^40, and values next to 3 * 2^k."""
    import ctypes as C
    from cfd_gb300 import abi
    bad = C.c_ulonglong(12345)
    abi.check(abi.lib().cfd_selftest_div3(1 << 32, 0x5eed, C.byref(bad)), "div3 self-test")
    assert bad.value == 0
    assert abi.lib().cfd_selftest_div3(0, 1, C.byref(bad)) == abi.CFD_ERR_ARG


@pytest.mark.gpu
def test_div_rcp_equals_the_division(gpu_lib):
    """The FP64 BiCG's quotients r/diag from the reciprocal and two FMA corrections give the
    IEEE quotient bit for bit over 2^31 pairs (raw bit patterns, 2^-60 .. 2^60, quotients
    next to binade edges and halfway cases)."""
    import ctypes as C
    from cfd_gb300 import abi
    bad = C.c_ulonglong(12345)
    abi.check(abi.lib().cfd_selftest_div_rcp(1 << 31, 0xd1f, C.byref(bad)), "div_rcp self-test")
    assert bad.value == 0

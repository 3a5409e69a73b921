"""Parity of the sm_103a FP64 path with the oracle, through the C-ABI.

The FP64 kernels evaluate every expression in the reference's order without FMA
contraction, sum per-node contributions in element order and take the dot products in
the oracle's fixed tree, so the bar here is bit-for-bit equality (np.array_equal).
"""
import math

import numpy as np
import pytest

from conftest import perturbed_state, small_case

pytestmark = pytest.mark.gpu


def eq(a, b, what=""):
    a, b = np.asarray(a), np.asarray(b)
    if not np.array_equal(a, b):
        d = np.abs(a - b)
        i = np.unravel_index(np.argmax(d), d.shape)
        rel = d.max() / max(np.abs(b).max(), 1e-300)
        raise AssertionError(f"{what}: not bit-exact; max |diff| {d.max():.3e} at {i} "
                             f"(rel {rel:.3e}); {np.count_nonzero(d)} of {d.size} differ")


@pytest.fixture(scope="module")
def mesh():
    return small_case(1, scale=24, seed=11)


@pytest.fixture(scope="module")
def S(gpu_lib):
    from cfd_gb300 import solver
    return solver


def test_deriv_masas_gcl(S, oracle, mesh):
    g = S.deriv(mesh.x, mesh.y, mesh.inpoel)
    o = oracle.deriv(mesh.x, mesh.y, mesh.inpoel)
    for k in ("area", "dNx", "dNy", "HH", "HHX", "HHY"):
        eq(g[k], o[k], k)
    assert g["hmin"] == o["hmin"]
    eq(S.MASAS(g["area"], mesh.inpoel, mesh.npoin),
       oracle.masas(o["area"], mesh.inpoel, mesh.npoin), "MASAS")
    rng = np.random.default_rng(0)
    n = mesh.npoin
    M = oracle.masas(o["area"], mesh.inpoel, n)
    w = [rng.normal(size=n) for _ in range(4)]
    ao = o["area"] * (1 + 0.01 * rng.normal(size=mesh.nelem))
    for mode in (1, 2):
        eq(S.gcl_main(M, *w, o["dNx"], o["dNy"], o["area"], ao, mesh.inpoel, 1.3e-3, mode),
           oracle.gcl(M, *w, o["dNx"], o["dNy"], o["area"], ao, mesh.inpoel, 1.3e-3, mode),
           f"gcl mode {mode}")


def test_deltat_estab(S, oracle, mesh):
    p = mesh.params
    o = oracle.deriv(mesh.x, mesh.y, mesh.inpoel)
    U, T, u, v = perturbed_state(mesh, seed=1)
    rng = np.random.default_rng(2)
    wx, wy = 0.05 * rng.normal(size=mesh.npoin), 0.05 * rng.normal(size=mesh.npoin)
    DTg, dtg = S.deltat(T, u, v, wx, wy, o["area"], mesh.inpoel, p.fsafe, p.fr, p.gama, p.t_inf)
    DTo, dto = oracle.deltat(T, u, v, wx, wy, o["area"], mesh.inpoel, p.fsafe, p.fr, p.gama,
                             p.t_inf)
    assert dtg == dto
    eq(DTg, DTo, "DT")
    G = np.full(mesh.npoin, p.gama)
    args = (U, T, G, u, v, wx, wy, o["dNx"], o["dNy"], mesh.inpoel, p.gama, p.fr, dto,
            p.rho_inf, p.t_inf)
    for a, b, k in zip(S.ESTAB(*args), oracle.estab(*args), ("SHOC", "T_SUGN1", "T_SUGN2", "T_SUGN3")):
        eq(a, b, k)


@pytest.mark.parametrize("variant", ["viscous", "viscous_theta", "inviscid"])
def test_calcrhs_fuente(S, oracle, mesh, variant):
    p = mesh.params
    o = oracle.deriv(mesh.x, mesh.y, mesh.inpoel)
    U, T, u, v = perturbed_state(mesh, seed=3)
    n, ne = mesh.npoin, mesh.nelem
    rng = np.random.default_rng(4)
    shoc = 1e-3 * rng.uniform(0, 1, ne)
    ts = [1e-3 * rng.uniform(0.1, 1, ne) for _ in range(3)]
    dtl = 1e-3 * rng.uniform(0.5, 1, ne)
    gas = p.gas6()
    if variant == "inviscid":
        gas[2] = 0.0
    theta = 1e-2 * rng.normal(size=(n, 4)) if variant == "viscous_theta" else np.zeros((n, 4))
    rhs0 = 1e-3 * rng.normal(size=(n, 4))
    rg = S.calcRHS(rhs0.copy(), U, theta if variant == "viscous_theta" else None, o["dNx"],
                   o["dNy"], o["area"], shoc, dtl, *ts, mesh.inpoel, T, gas)
    ro = oracle.calcrhs(rhs0, U, theta, o["dNx"], o["dNy"], o["area"], shoc, dtl, *ts,
                        mesh.inpoel, T, gas)
    eq(rg, ro, f"calcRHS {variant}")
    wx, wy = 0.1 * rng.normal(size=n), 0.1 * rng.normal(size=n)
    eq(S.FUENTE(rg.copy(), U, wx, wy, o["dNx"], o["dNy"], o["area"], dtl, mesh.inpoel),
       oracle.fuente(ro, U, wx, wy, o["dNx"], o["dNy"], o["area"], dtl, mesh.inpoel), "FUENTE")


def test_adjacency_laplace_bicg(S, oracle, mesh):
    e1, e2 = S.getEsup(mesh.inpoel, mesh.npoin)
    o1, o2 = oracle.esup(mesh.inpoel, mesh.npoin)
    eq(e1, o1, "esup1")
    eq(e2, o2, "esup2")
    p1, p2 = S.getPsup(mesh.inpoel, mesh.npoin)
    q1, q2 = oracle.psup(mesh.inpoel, mesh.npoin)
    eq(p1, q1, "psup1")
    eq(p2, q2, "psup2")
    rp, idx = S.laplace_pattern(mesh.inpoel, mesh.npoin)
    orp, oidx = oracle.laplace_pattern(mesh.inpoel, mesh.npoin)
    eq(rp, orp, "lap_rowptr")
    eq(idx, oidx, "lap_idx")
    o = oracle.deriv(mesh.x, mesh.y, mesh.inpoel)
    vg, dg = S.laplace(mesh.inpoel, o["area"], o["dNx"], o["dNy"], mesh.x, mesh.y, idx, rp)
    vo, do = oracle.laplace(mesh.inpoel, o["dNx"], o["dNy"], mesh.x, mesh.y, rp, idx)
    eq(vg, vo, "lap_sparse")
    eq(dg, do, "lap_diag")
    fix = mesh.ilaux()
    rng = np.random.default_rng(5)
    data = 1e-3 * rng.normal(size=len(fix))
    x0 = 1e-4 * rng.normal(size=mesh.npoin)
    b = np.zeros(mesh.npoin)
    xg, ig = S.biCG(vo, oidx, orp, do, x0, b, data, fix)
    xo, io = oracle.bicg(vo, oidx, orp, do, x0, b, data, fix)
    assert (ig.iters, ig.converged) == (io.iters, io.converged)
    assert ig.rz == io.rz
    eq(xg, xo, "biCG x")
    # iteration cap: returns with converged = 0 after exactly maxit iterations
    xg, ig = S.biCG(vo, oidx, orp, do, x0, b, data, fix, tol=1e-300, maxit=5)
    xo, io = oracle.bicg(vo, oidx, orp, do, x0, b, data, fix, tol=1e-300, maxit=5)
    assert ig.iters == io.iters == 5 and ig.converged == io.converged == 0
    eq(xg, xo, "biCG x (capped)")


def run_pair(case, steps, check_each=True, setup=None, on_step=None):
    from cfd_gb300 import solver
    g = solver.Solver(case)
    o = None
    from oracle import oracle as O
    o = O.OracleCase(case)
    if setup:
        setup(g, o)
    for s in range(steps):
        rg, ro = g.step(1), o.step(1)
        assert rg.dtmin == ro.dtmin, f"step {s + 1}: DTMIN"
        assert rg.time == ro.time
        assert tuple(rg.bicg_iters) == tuple(ro.bicg_iters), f"step {s + 1}: BiCG iterations"
        assert tuple(rg.bicg_relres) == tuple(ro.bicg_relres), f"step {s + 1}: BiCG ||r||"
        if on_step:
            on_step(rg, ro)
        for i in range(rg.nset_numb):
            assert (rg.fx[i], rg.fy[i], rg.rm[i]) == (ro.fx[i], ro.fy[i], ro.rm[i]), "FORCES"
        if check_each or s == steps - 1:
            sg, so = g.state(), o.state()
            for k in ("U", "T", "X", "Y"):
                eq(sg[k], so[k], f"step {s + 1}: {k}")
    fg, fo = g.fields(), o.fields()
    for k in fg:
        eq(fg[k], fo[k], k)
    gg, go = g.geometry(), o.geometry()
    for k in gg:
        eq(gg[k], go[k], k)
    mg, mo = g.motion(), o.motion()
    eq(mg[0], mo[0], "xpos")
    eq(mg[1], mo[1], "ypos")
    g.close()
    o.close()


def test_step_fixed_mesh(gpu_lib):
    run_pair(small_case(1, scale=16, seed=7), 4)


def test_step_inviscid(gpu_lib):
    # FMU = 0: calcRHS has no viscous terms, so the stage-1 element pass is final for all
    # four stages
    run_pair(small_case(2, scale=16, seed=5, fmu=0.0, pitch_amp=math.radians(3.0),
                        motion_freq=2.0), 3)


@pytest.mark.parametrize("mass_mode", [0, 1, 2])
def test_step_heave_pitch(gpu_lib, mass_mode):
    k = small_case(2, scale=16, seed=8, pitch_amp=math.radians(4.0), motion_freq=2.0,
                   mass_mode=mass_mode)
    run_pair(k, 3)


def test_step_reference_motion_law_itlocal(gpu_lib):
    k = small_case(1, scale=12, seed=9, motion_law=0, moving=1, itlocal=50)
    run_pair(k, 3)


def test_step_from_shared_perturbed_state(gpu_lib):
    """Per-step parity from the same non-trivial state on both sides."""
    k = small_case(3, scale=24, seed=12)
    U, T, u, v = perturbed_state(k, seed=9, amp=0.1)

    def setup(g, o):
        for side in (g, o):
            side.set_state(U, T, u, v)
            side.set_clock(iter=10, time=0.5, dtmin1=0.0, bandera=1, disn1=0.0, disn2=0.0)

    run_pair(k, 2, setup=setup)


def test_step_after_upload_of_U_only(gpu_lib):
    """cfd_ctx_upload_state with U and T only: the velocities come from U (rho u / rho,
    rho v / rho) as the oracle forms them; the steps after it are bit-exact."""
    k = small_case(3, scale=16, seed=5)
    U, T, _, _ = perturbed_state(k, seed=4, amp=0.05)

    def setup(g, o):
        for side in (g, o):
            side.set_state(U, T)

    run_pair(k, 2, setup=setup)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_upload_from_pinned_memory(gpu_lib, prec):
    """cfd_ctx_upload_state with U in pinned host memory reads it with one kernel
    (k_upload_U: U, the velocities and the mixed form's shadows); the state, the fields and
    the steps after it equal those of the copy-engine path (pageable U) bit for bit."""
    import torch
    from cfd_gb300 import abi, solver
    k = small_case(3, scale=16, seed=5)
    U, T, _, _ = perturbed_state(k, seed=4, amp=0.05)
    p = abi.CFD_PREC_FP64 if prec == "fp64" else abi.CFD_PREC_MIXED
    hU = torch.empty(U.shape, dtype=torch.float64, pin_memory=True).numpy()
    hU[:] = U
    L = abi.lib()
    for withT in (True, False):
        a, b = solver.Solver(k, precision=p), solver.Solver(k, precision=p)
        a.set_state(U, T if withT else None)
        l0 = L.cfd_kernel_launches()
        b.set_state(hU, T if withT else None)
        if prec == "mixed" and not withT:  # one kernel instead of k_vel_from_U + k_narrow_state
            assert L.cfd_kernel_launches() - l0 == 1
        for key in ("U", "T"):
            eq(a.state()[key], b.state()[key], f"{prec} upload {key}")
        fa, fb = a.fields(), b.fields()
        for key in ("VEL_X", "VEL_Y"):
            eq(fa[key], fb[key], f"{prec} upload {key}")
        a.step(2)
        b.step(2)
        sa, sb = a.state(), b.state()
        for key in ("U", "T", "X", "Y"):
            eq(sa[key], sb[key], f"{prec} 2 steps after the upload {key}")
        a.close()
        b.close()


def test_bad_inputs_return_status(gpu_lib):
    from cfd_gb300 import abi, solver
    k = small_case(1, scale=8)
    bad = k.inpoel.copy()
    bad[3, 1] = k.npoin + 5
    with pytest.raises(abi.CfdError) as e:
        solver.MASAS(np.ones(k.nelem), bad, k.npoin)
    assert e.value.status == abi.CFD_ERR_MESH
    k.inpoel = bad
    with pytest.raises(abi.CfdError) as e:
        solver.Solver(k)
    assert e.value.status == abi.CFD_ERR_MESH


def test_full_size_one_step_parity_and_properties(gpu_lib):
    """The 1M-node ellipse O-grid (1024 x 1024): one full step against the oracle, then
    size-independent properties over more steps (finite state, mass = total area under
    MASAS, rigid body motion of the wall ring, run-to-run determinism)."""
    from cfd_gb300 import case as C, solver
    from oracle import oracle as O
    k = C.config_case(3)
    k.params.mass_mode = 0
    o = O.OracleCase(k)
    g = solver.Solver(k)
    rg, ro = g.step(1), o.step(1)
    assert rg.dtmin == ro.dtmin and tuple(rg.bicg_iters) == tuple(ro.bicg_iters)
    sg, so = g.state(), o.state()
    for key in ("U", "T", "X", "Y"):
        eq(sg[key], so[key], f"1M step 1 {key}")
    o.close()
    g.step(2)
    st = g.state()
    assert np.all(np.isfinite(st["U"]))
    geo = g.geometry()
    assert geo["M"].sum() == pytest.approx(geo["area"].sum(), rel=1e-12)
    dy = st["Y"][k.i_m - 1] - k.y[k.i_m - 1]
    np.testing.assert_allclose(dy, dy[0], rtol=1e-8)
    g2 = solver.Solver(k)
    g2.step(3)
    eq(g2.state()["U"], st["U"], "determinism")
    g.close()
    g2.close()

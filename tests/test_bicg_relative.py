"""The relative stopping tests of BiCG (CFD_BICG_TOL_REL, CFD_BICG_TOL_REL_R0).

The reference stops on an absolute |r.z| (biconjGrad.f90:26, :35, :47).  The relative modes
keep the reference's iterates and stop when ||r|| <= tol * ||ref||: ref = b - A.x_D (the
residual of the guess that is zero off the Dirichlet rows, so every guess solves to the
same accuracy) or ref = r_0.  CPU tests pin the oracle's modes on known answers; the GPU
tests check the FP64 kernels against the oracle bit for bit (drop-in and resident step)
and the mixed form's solve against its own test.
"""
import math

import numpy as np
import pytest

from conftest import small_case


def _system(oracle, scale=16, seed=3):
    k = small_case(1, scale=scale, seed=seed)
    g = oracle.deriv(k.x, k.y, k.inpoel)
    rp, idx = oracle.laplace_pattern(k.inpoel, k.npoin)
    vals, diag = oracle.laplace(k.inpoel, g["dNx"], g["dNy"], k.x, k.y, rp, idx)
    fix = k.ilaux()
    rng = np.random.default_rng(seed)
    data = 1e-3 * rng.normal(size=len(fix))
    return vals, idx, rp, diag, fix, data


def _true_relres(vals, idx, rp, diag, x, b, fix, data):
    """||b - A.x|| over the free rows against ||b - A.x_D|| (numpy, from the CSR)."""
    n = len(diag)
    rows = np.repeat(np.arange(n), np.diff(rp))
    cols = idx - 1
    Ax = np.bincount(rows, weights=vals * x[cols], minlength=n)
    xd = np.zeros(n)
    xd[fix - 1] = data
    Axd = np.bincount(rows, weights=vals * xd[cols], minlength=n)
    free = np.ones(n, bool)
    free[fix - 1] = False
    return (np.linalg.norm((b - Ax)[free]) / np.linalg.norm((b - Axd)[free]))


def test_oracle_relative_mode_reaches_its_tolerance(oracle):
    from cfd_gb300 import abi
    vals, idx, rp, diag, fix, data = _system(oracle)
    n = len(diag)
    b = np.zeros(n)
    x0 = np.zeros(n)
    iters = []
    for tol in (1e-4, 1e-7, 1e-10):
        x, info = oracle.bicg(vals, idx, rp, diag, x0, b, data, fix, tol=tol, maxit=5000,
                              tol_mode=abi.CFD_BICG_TOL_REL)
        assert info.converged == 1 and 0.0 < info.relres <= tol
        iters.append(info.iters)
        # the recursively updated residual the test measures tracks the true one
        true = _true_relres(vals, idx, rp, diag, x, b, fix, data)
        assert true <= 10 * tol, (tol, true)
    assert iters[0] < iters[1] < iters[2]


def test_oracle_relative_modes_agree_from_the_zero_guess(oracle):
    """From the guess that is 0 off the Dirichlet rows, r_0 = b - A.x_D: both relative
    modes take the same reference norm, hence the same iterations and the same x."""
    from cfd_gb300 import abi
    vals, idx, rp, diag, fix, data = _system(oracle, seed=5)
    n = len(diag)
    b = np.zeros(n)
    xa, ia = oracle.bicg(vals, idx, rp, diag, np.zeros(n), b, data, fix, tol=1e-9,
                         maxit=5000, tol_mode=abi.CFD_BICG_TOL_REL)
    xb, ib = oracle.bicg(vals, idx, rp, diag, np.zeros(n), b, data, fix, tol=1e-9,
                         maxit=5000, tol_mode=abi.CFD_BICG_TOL_REL_R0)
    assert (ia.iters, ia.converged, ia.relres) == (ib.iters, ib.converged, ib.relres)
    np.testing.assert_array_equal(xa, xb)


def test_oracle_modes_share_the_iterates(oracle):
    """Only the stopping test differs: with the same iteration count forced by maxit the
    absolute and relative modes return the same x bit for bit."""
    from cfd_gb300 import abi
    vals, idx, rp, diag, fix, data = _system(oracle, seed=7)
    n = len(diag)
    rng = np.random.default_rng(1)
    x0 = 1e-4 * rng.normal(size=n)
    b = np.zeros(n)
    out = []
    for mode in (abi.CFD_BICG_TOL_ABS, abi.CFD_BICG_TOL_REL, abi.CFD_BICG_TOL_REL_R0):
        x, info = oracle.bicg(vals, idx, rp, diag, x0, b, data, fix, tol=1e-300, maxit=17,
                              tol_mode=mode)
        assert info.iters == 17 and info.converged == 0
        out.append(x)
    np.testing.assert_array_equal(out[0], out[1])
    np.testing.assert_array_equal(out[0], out[2])


def test_oracle_better_guess_fewer_iterations_relative(oracle):
    """CFD_BICG_TOL_REL is guess-independent: a guess closer to the solution needs fewer
    iterations to reach the same accuracy (the point of a learned or previous-step guess),
    while r_0-relative stopping asks the same reduction from any guess."""
    from cfd_gb300 import abi
    vals, idx, rp, diag, fix, data = _system(oracle, scale=20, seed=2)
    n = len(diag)
    b = np.zeros(n)
    xs, _ = oracle.bicg(vals, idx, rp, diag, np.zeros(n), b, data, fix, tol=1e-13, maxit=5000,
                        tol_mode=abi.CFD_BICG_TOL_REL)
    rng = np.random.default_rng(3)
    near = xs * (1 + 1e-4 * rng.normal(size=n))
    _, i0 = oracle.bicg(vals, idx, rp, diag, np.zeros(n), b, data, fix, tol=1e-10, maxit=5000,
                        tol_mode=abi.CFD_BICG_TOL_REL)
    _, i1 = oracle.bicg(vals, idx, rp, diag, near, b, data, fix, tol=1e-10, maxit=5000,
                        tol_mode=abi.CFD_BICG_TOL_REL)
    assert i1.converged and i0.converged
    assert i1.iters < 0.8 * i0.iters, (i1.iters, i0.iters)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2])
def test_gpu_bicg_relative_bit_exact(gpu_lib, oracle, mode):
    from cfd_gb300 import solver
    vals, idx, rp, diag, fix, data = _system(oracle, scale=24, seed=4)
    n = len(diag)
    rng = np.random.default_rng(6)
    b = np.zeros(n)
    for x0 in (np.zeros(n), 1e-4 * rng.normal(size=n)):
        xg, ig = solver.biCG(vals, idx, rp, diag, x0, b, data, fix, tol=1e-10, maxit=3000,
                             tol_mode=mode)
        xo, io = oracle.bicg(vals, idx, rp, diag, x0, b, data, fix, tol=1e-10, maxit=3000,
                             tol_mode=mode)
        assert (ig.iters, ig.converged) == (io.iters, io.converged)
        assert ig.rz == io.rz and ig.relres == io.relres
        assert io.converged and io.relres <= 1e-10
        np.testing.assert_array_equal(xg, xo)
    # a non-zero right-hand side enters the reference norm
    bb = 1e-6 * rng.normal(size=n)
    xg, ig = solver.biCG(vals, idx, rp, diag, np.zeros(n), bb, data, fix, tol=1e-9, maxit=3000,
                         tol_mode=mode)
    xo, io = oracle.bicg(vals, idx, rp, diag, np.zeros(n), bb, data, fix, tol=1e-9, maxit=3000,
                         tol_mode=mode)
    assert (ig.iters, ig.relres) == (io.iters, io.relres)
    np.testing.assert_array_equal(xg, xo)


@pytest.mark.gpu
def test_gpu_step_relative_mode_bit_exact(gpu_lib):
    """The resident FP64 step with the mesh-motion solve under CFD_BICG_TOL_REL against the
    oracle's loop: every step's iterations, relative residuals, state and mesh."""
    from test_gpu_parity import run_pair
    from cfd_gb300 import abi
    k = small_case(2, scale=16, seed=8, pitch_amp=math.radians(4.0), motion_freq=2.0,
                   mass_mode=abi.CFD_MASS_GCL_CORRECTED, bicg_tol_mode=abi.CFD_BICG_TOL_REL,
                   bicg_maxit=3000)
    reps = []
    run_pair(k, 3, on_step=lambda rg, ro: reps.append((tuple(rg.bicg_relres),
                                                       tuple(ro.bicg_relres),
                                                       tuple(rg.bicg_iters))))
    for g, o, it in reps:
        assert g == o
        assert max(g) <= 1e-10 and min(it) > 0


@pytest.mark.gpu
def test_gpu_mixed_relative_mode(gpu_lib, oracle):
    """The mixed form's solve under CFD_BICG_TOL_REL: FP32 iterations against the precise
    residual of the FP64-assembled matrix, with a refinement pass when the first pass's
    recursive residual met the test before the precise one did; it takes at most about
    twice the FP64 form's iterations (the first pass and the refinement), and the mesh
    increments it solves for stay within the FP32 iterations' accuracy of the FP64 form's
    (the solve amplifies the FP32 matrix's ~1e-7 by the operator's conditioning, ~1e3 here,
    so the increments agree to ~1e-4)."""
    from cfd_gb300 import abi, solver
    k = small_case(2, scale=24, seed=8, pitch_amp=math.radians(4.0), motion_freq=2.0,
                   mass_mode=abi.CFD_MASS_GCL_CORRECTED, bicg_tol_mode=abi.CFD_BICG_TOL_REL,
                   bicg_maxit=3000, estab_mode=abi.CFD_ESTAB_REGULARIZED)
    gm = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    gd = solver.Solver(k)
    for s in range(4):
        rm, rd = gm.step(1), gd.step(1)
        assert all(rm.bicg_converged) and max(rm.bicg_relres) <= 1e-10
        for q in range(2):
            assert 0.8 * rd.bicg_iters[q] - 3 <= rm.bicg_iters[q] <= 2 * rd.bicg_iters[q] + 10, (
                s, tuple(rm.bicg_iters), tuple(rd.bicg_iters))
        for q, (a, b) in enumerate(zip(gm.motion(), gd.motion())):
            d = np.abs(a - b).max() / np.abs(b).max()
            assert d <= 1e-3, (s, q, d)
    gm.close()
    gd.close()


# a start at t = 0.4 with the heave's position there, so that the first step's increment
# is the motion's (not the jump from rest to A sin(w t0))
_T0 = dict(iter=0, time=0.4, disn1=0.2 * math.sin(2.0 * math.pi * 0.2 * 0.4))


def _heave_case(scale, **over):
    from cfd_gb300 import abi
    kw = dict(heave_amp=0.2, motion_freq=0.2, mass_mode=abi.CFD_MASS_GCL_CORRECTED,
              bicg_tol_mode=abi.CFD_BICG_TOL_REL, bicg_maxit=5000)
    kw.update(over)
    return small_case(2, scale=scale, seed=8, **kw)


def test_oracle_extrapolated_guess(oracle):
    """CFD_GUESS_EXTRAPOLATED on the oracle's loop: from the third step on the solves start
    from the last two increments extrapolated to the step's DTMIN and need far fewer
    iterations than from the previous increment, to the same relative tolerance; the flow
    and mesh stay within the solve's tolerance of the previous-guess run."""
    from cfd_gb300 import abi
    runs = {}
    for mode in (abi.CFD_GUESS_PREVIOUS, abi.CFD_GUESS_EXTRAPOLATED):
        o = oracle.OracleCase(_heave_case(48, guess_mode=mode))
        o.set_clock(**_T0)
        its = []
        for s in range(7):
            r = o.step(1)
            assert all(r.bicg_converged) and max(r.bicg_relres) <= 1e-10
            its.append(r.bicg_iters[1])
        runs[mode] = (its, o.state())
        o.close()
    ip, ie = runs[abi.CFD_GUESS_PREVIOUS][0], runs[abi.CFD_GUESS_EXTRAPOLATED][0]
    assert ip[:2] == ie[:2]                     # the previous increment until two are kept
    # this coarse mesh takes large steps (DTMIN ~5e-3): the extrapolation's error, O((w dt)^2),
    # is ~5e-5 of the increment against 4e-3 .. 4e-2 for the previous increment
    assert sum(ie[2:]) < 0.8 * sum(ip[2:]), (ie, ip)
    sp, se = runs[abi.CFD_GUESS_PREVIOUS][1], runs[abi.CFD_GUESS_EXTRAPOLATED][1]
    # ||r|| <= 1e-10 ||b - A x_D|| bounds the residual, not the error in the operator's slow
    # modes (its smallest eigenvalues are tiny against the boundary rows'): two runs whose
    # solves start from different guesses end 7 steps apart by ~1.4e-3 of the accumulated
    # displacement here
    d = np.abs(sp["Y"] - se["Y"]).max() / np.abs(sp["Y"] - _heave_case(48).y).max()
    assert d < 1e-2, d


@pytest.mark.gpu
@pytest.mark.parametrize("scale", [16, 40])
def test_gpu_extrapolated_guess_bit_exact(gpu_lib, scale):
    """The FP64 form with CFD_GUESS_EXTRAPOLATED against the oracle's loop: every step's
    iterations and relative residuals, the state and the mesh, bit for bit."""
    from test_gpu_parity import run_pair
    from cfd_gb300 import abi
    k = _heave_case(scale, guess_mode=abi.CFD_GUESS_EXTRAPOLATED)

    def setup(g, o):
        for side in (g, o):
            side.set_clock(**_T0)

    reps = []
    run_pair(k, 6, setup=setup,
             on_step=lambda rg, ro: reps.append((tuple(rg.bicg_iters), tuple(ro.bicg_iters))))
    assert all(g == o for g, o in reps)


@pytest.mark.gpu
def test_gpu_mixed_extrapolated_guess(gpu_lib):
    """The mixed form with CFD_GUESS_EXTRAPOLATED: the solves reach the relative tolerance,
    in fewer iterations than from the previous increment, and the mesh increments stay
    within the FP32 operator's accuracy of the previous-guess run's."""
    from cfd_gb300 import abi, solver
    runs = {}
    for mode in (abi.CFD_GUESS_PREVIOUS, abi.CFD_GUESS_EXTRAPOLATED):
        k = _heave_case(32, guess_mode=mode, estab_mode=abi.CFD_ESTAB_REGULARIZED)
        g = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
        g.set_clock(**_T0)
        its, mot = [], []
        for s in range(7):
            r = g.step(1)
            assert all(r.bicg_converged) and max(r.bicg_relres) <= 1e-10
            its.append(sum(r.bicg_iters))
            mot.append(g.motion()[1])
        runs[mode] = (its, mot)
        g.close()
    ip, ie = runs[abi.CFD_GUESS_PREVIOUS][0], runs[abi.CFD_GUESS_EXTRAPOLATED][0]
    assert sum(ie[2:]) < sum(ip[2:]), (ie, ip)
    for a, b in zip(runs[abi.CFD_GUESS_EXTRAPOLATED][1], runs[abi.CFD_GUESS_PREVIOUS][1]):
        assert np.abs(a - b).max() <= 1e-3 * np.abs(b).max()


@pytest.mark.gpu
def test_gpu_mesh_motion_matrix_assemblies(gpu_lib, oracle):
    """The mesh-motion matrix each form assembles (cfd_ctx_download_laplace) against the
    oracle's laplace (mLaplace.f90:7-58) of the context's own mesh: the FP64 form bit for
    bit at set-up; the mixed form's FP64 assembly (relative tests: element matrices formed
    once per element, rows summed per node, held as FP32 hi + lo) within FP64 rounding at
    set-up and after steps that moved the mesh (it assembles for the next step from the
    moved mesh); its FP32 assembly (absolute test) within FP32 rounding."""
    from cfd_gb300 import abi, solver
    kw = dict(pitch_amp=math.radians(4.0), motion_freq=2.0, heave_amp=0.1,
              mass_mode=abi.CFD_MASS_GCL_CORRECTED, bicg_maxit=3000,
              estab_mode=abi.CFD_ESTAB_REGULARIZED)
    krel = small_case(2, scale=24, seed=8, bicg_tol_mode=abi.CFD_BICG_TOL_REL, **kw)
    kabs = small_case(2, scale=24, seed=8, **kw)
    rp, idx = oracle.laplace_pattern(krel.inpoel, krel.npoin)
    rows = np.repeat(np.arange(krel.npoin), np.diff(rp))

    def ref(X, Y):
        g = oracle.deriv(X, Y, krel.inpoel)
        vals, _ = oracle.laplace(krel.inpoel, g["dNx"], g["dNy"], X, Y, rp, idx)
        return vals

    def rel_err(v, r):  # per entry, against the largest entry of its row
        scale = np.maximum.reduceat(np.abs(r), rp[:-1])[rows]
        return float((np.abs(v - r) / scale).max())

    gd = solver.Solver(krel)
    np.testing.assert_array_equal(gd.laplace_values(), ref(krel.x, krel.y))
    gd.close()
    for k, bound in ((krel, 1e-13), (kabs, 1e-6)):
        gm = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
        for s in range(3):
            st = gm.state()
            e = rel_err(gm.laplace_values(), ref(st["X"], st["Y"]))
            assert e <= bound, (k.params.bicg_tol_mode, s, e)
            gm.step(2)
        moved = np.abs(gm.state()["Y"] - k.y).max()
        assert moved > 1e-4, moved
        gm.close()

"""FORCE_VISC (ns2DComp.ALE.f90:819-893): known answers of the oracle's restatement (a
uniform state exerts no net viscous force on a closed body and no skin friction; a linear
shear flow gives the analytic skin friction), and the CUDA drop-in and resident forms
against the oracle (FP64 bit for bit, the mixed form to tolerance)."""
import numpy as np
import pytest

from conftest import small_case


def wall_inputs(k, vx, vy, P, T):
    from oracle import oracle as O
    g = O.deriv(k.x, k.y, k.inpoel)
    iset, ielem_sets, nset = k.iset_array()
    return dict(NELEM=k.nelem, npoin=k.npoin, nsets=iset.shape[0], IELEM_SETS=ielem_sets,
                ISET=iset, inpoel=k.inpoel, NSET_NUMB=nset, U_inf=k.params.u_inf,
                V_inf=k.params.v_inf, RHO_inf=k.params.rho_inf, T_inf=k.params.t_inf,
                X=k.x, Y=k.y, P=P, T=T, VEL_X=vx, VEL_Y=vy, DNX=g["dNx"], DNY=g["dNy"])


def oracle_force_visc(a):
    import ctypes as C
    from oracle import oracle as O
    fvx, fvy = np.zeros(10), np.zeros(10)
    ne = int(np.asarray(a["IELEM_SETS"])[:a["NSET_NUMB"]].sum())
    skin = np.zeros((ne, 3))
    f, i = O.f64, O.i32
    O.lib().or_force_visc(a["NELEM"], a["npoin"], a["nsets"], O.ip(i(a["IELEM_SETS"])),
                          O.ip(i(a["ISET"])), O.ip(i(a["inpoel"])), a["NSET_NUMB"],
                          a["U_inf"], a["V_inf"], a["RHO_inf"], a["T_inf"],
                          *[O.dp(f(a[k])) for k in ("X", "Y", "P", "T", "VEL_X", "VEL_Y",
                                                    "DNX", "DNY")],
                          O.dp(fvx), O.dp(fvy), O.dp(skin))
    return fvx, fvy, skin


def test_uniform_state_no_viscous_force(oracle):
    k = small_case(1, scale=12, seed=2)
    n = k.npoin
    a = wall_inputs(k, np.full(n, 0.3), np.full(n, -0.1), np.full(n, 90.0), np.full(n, 288.15))
    fvx, fvy, skin = oracle_force_visc(a)
    assert abs(fvx[0]) < 1e-10 * 90.0 and abs(fvy[0]) < 1e-10 * 90.0
    assert np.abs(skin[:, 0]).max() < 1e-12
    assert np.allclose(skin[:, 2], 90.0 / 82713.27, rtol=1e-14)


def test_linear_shear_skin_friction(oracle):
    """u = a y, v = 0, uniform T and p: tau_xy = mu a on every element, and the skin
    friction of an edge with unit normal (nx, ny) is mu a (nx^2 - ny^2) / (rho U^2 / 2)."""
    k = small_case(1, scale=12, seed=2)
    n, p = k.npoin, k.params
    a_sh, T0 = 0.7, 300.0
    a = wall_inputs(k, a_sh * k.y, np.zeros(n), np.full(n, 50.0), np.full(n, T0))
    fvx, fvy, skin = oracle_force_visc(a)
    mu = 0.017 * (T0 / p.t_inf) ** 1.5 * (p.t_inf + 110.0) / (T0 + 110.0)
    iset, ielem_sets, nset = k.iset_array()
    e = iset[:ielem_sets[0], 0, :]  # set 1's edges: (n1, n2, element)
    n1, n2 = e[:, 0] - 1, e[:, 1] - 1
    rlx, rly = k.y[n2] - k.y[n1], -(k.x[n2] - k.x[n1])
    m = np.hypot(rlx, rly)
    rlx, rly = rlx / m, rly / m
    want = mu * a_sh * (rlx ** 2 - rly ** 2) / (0.5 * p.rho_inf * (p.u_inf ** 2 + p.v_inf ** 2))
    assert np.allclose(skin[:, 0], want, rtol=1e-9, atol=1e-12 * np.abs(want).max())
    # a closed contour under a uniform stress: no net force
    assert abs(fvx[0]) < 1e-9 and abs(fvy[0]) < 1e-9


@pytest.mark.gpu
def test_drop_in_bit_exact(gpu_lib):
    from cfd_gb300 import solver
    from conftest import perturbed_state
    k = small_case(2, scale=20, seed=6)
    U, T, u, v = perturbed_state(k, seed=1, amp=0.1)
    P = U[:, 0] * k.params.fr * T
    a = wall_inputs(k, u, v, P, T)
    fvx, fvy, skin = solver.FORCE_VISC(**a, skin=True)
    ofx, ofy, oskin = oracle_force_visc(a)
    assert np.array_equal(fvx, ofx) and np.array_equal(fvy, ofy)
    assert np.array_equal(skin, oskin)


@pytest.mark.gpu
@pytest.mark.parametrize("each_step", [True, False])
def test_resident_fp64_bit_exact(gpu_lib, each_step):
    from cfd_gb300 import solver
    from oracle import oracle as O
    k = small_case(2, scale=16, seed=5)
    g, o = solver.Solver(k), O.OracleCase(k)
    for s in (g, o):
        s.set_force_visc(each_step)
        s.step(3)
    (gx, gy, gs), (ox, oy, os_) = g.force_visc(), o.force_visc()
    assert np.array_equal(gx, ox) and np.array_equal(gy, oy) and np.array_equal(gs, os_)
    assert np.abs(gx).max() > 0.0
    g.close()
    o.close()


@pytest.mark.gpu
def test_resident_mixed_close(gpu_lib):
    from cfd_gb300 import abi, solver
    from oracle import oracle as O
    k = small_case(2, scale=24, seed=5, estab_mode=abi.CFD_ESTAB_REGULARIZED)
    g, o = solver.Solver(k, precision=abi.CFD_PREC_MIXED), O.OracleCase(k)
    for s in (g, o):
        s.set_force_visc(True)
        s.step(3)
    (gx, gy, gs), (ox, oy, os_) = g.force_visc(), o.force_visc()
    scale = np.hypot(ox, oy).max()
    assert np.abs(gx - ox).max() <= 1e-4 * scale and np.abs(gy - oy).max() <= 1e-4 * scale
    assert np.abs(gs[:, 0] - os_[:, 0]).max() <= 1e-4 * np.abs(os_[:, 0]).max()
    g.close()
    o.close()

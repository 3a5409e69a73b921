"""How far a build of the reference that evaluates x**1.5d0, x**.5d0 and x**(-.5d0) with
the C library's pow sits from the oracle (test infrastructure, CPU only).

The oracle, and the bit-exact FP64 GPU path with it, evaluate those powers as the
correctly rounded compositions x*sqrt(x), sqrt(x) and 1/sqrt(x) (cfd_oracle.h).  A Fortran
compiler without unsafe-math options calls pow instead (the reference's sites:
subrutinas.f90:194, 196, 400, 429, 438-439; calcRHS.f90:50-51; ns2DComp.ALE.f90:845).
This script counts the values at which the two differ and the state difference after 1, 2,
3, 5 and 10 steps from the same start (the freestream, and a perturbed state) in the
oracle's two pow modes:

    python oracle/pow_exposure.py [--scale N]

--scale N runs the N x N version of the 1,048,576-node ellipse O-grid workload (default: the
full 1024 x 1024).  The oracle runs on one thread: its calcRHS and FUENTE scatter with OpenMP
atomics as the reference does, so more threads would add their own order-dependent
differences to the ones measured here.  Prints one JSON object.
"""
import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def perturbed(case, seed=0, amp=0.05):
    """Freestream with smooth and random perturbations of rho, velocity and T."""
    rng = np.random.default_rng(seed)
    p = case.params
    n = case.npoin
    x, y = case.x, case.y
    rho = p.rho_inf * (1 + amp * np.sin(0.7 * x) * np.cos(0.5 * y) + 0.2 * amp * rng.uniform(-1, 1, n))
    u = p.u_inf * (1 + amp * np.cos(0.3 * x + 0.2 * y)) + 0.1 * amp * p.u_inf * rng.uniform(-1, 1, n)
    v = p.u_inf * amp * np.sin(0.4 * y) + 0.1 * amp * p.u_inf * rng.uniform(-1, 1, n)
    T = p.t_inf * (1 + amp * np.sin(0.2 * x + 0.3 * y) + 0.1 * amp * rng.uniform(-1, 1, n))
    P = rho * p.fr * T
    E = P / ((p.gama - 1) * rho) + 0.5 * (u * u + v * v)
    return np.stack([rho, rho * u, rho * v, rho * E], 1), T, u, v


def element_ratios(case, T):
    """T_elem/T_inf as calcRHS.f90:49 and ESTAB/deltat form them (sum of three / 3)."""
    i = case.inpoel - 1
    Tel = ((T[i[:, 0]] + T[i[:, 1]]) + T[i[:, 2]]) / 3.0
    return Tel / case.params.t_inf


def trajectory(O, case, state, pow_mode, estab_mode, checkpoints):
    """U after each number of steps in checkpoints (ascending), from the same start."""
    case.params.estab_mode = estab_mode
    O.set_pow_mode(pow_mode)
    o = O.OracleCase(case)
    if state is not None:
        o.set_state(*state)
    out, done = [], 0
    for n in checkpoints:
        o.step(n - done)
        done = n
        out.append(o.state()["U"])
    o.close()
    O.set_pow_mode(0)
    return out


def rel_l2(a, b):
    return [float(np.linalg.norm(a[:, q] - b[:, q]) / np.linalg.norm(b[:, q])) for q in range(4)]


def measure(scale=None, checkpoints=(1, 2, 3, 5, 10)):
    from cfd_gb300 import abi, case as C
    from oracle import oracle as O
    O.set_threads(1)
    k = C.config_case(3, scale=scale, seed=0)
    out = {"workload": f"ellipse O-grid, {k.npoin} nodes, {k.nelem} triangles",
           "npoin": k.npoin, "nelem": k.nelem}
    fs = O.OracleCase(k)
    T0 = fs.state()["T"]
    fs.close()
    U, T, u, v = perturbed(k)
    for name, Tn in (("freestream", T0), ("perturbed", T)):
        r = element_ratios(k, Tn)
        c = O.pow_census(r)
        out[f"census_{name}"] = {"values": int(r.size), "pow1.5_differs": c[0],
                                 "pow-0.5_differs": c[1], "pow0.5_differs": c[2]}
    out["steps"] = list(checkpoints)
    for estab, ename in ((abi.CFD_ESTAB_REFERENCE, "reference"),
                         (abi.CFD_ESTAB_REGULARIZED, "regularized")):
        for name, st in (("freestream", None), ("perturbed", (U, T, u, v))):
            a = trajectory(O, k, st, 0, estab, checkpoints)
            b = trajectory(O, k, st, 1, estab, checkpoints)
            out[f"{name}_estab_{ename}"] = {
                "rel_l2_per_variable": [rel_l2(ub, ua) for ua, ub in zip(a, b)],
                "identical": [bool(np.array_equal(ua, ub)) for ua, ub in zip(a, b)]}
    k.params.estab_mode = abi.CFD_ESTAB_REFERENCE
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=int, default=None)
    a = ap.parse_args()
    print(json.dumps(measure(a.scale)))

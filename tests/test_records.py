"""Long lockstep runs of the FP64 form against the oracle on the configurations' workloads.

Minutes each, so they run only with CFD_RECORDS=1 (skipped otherwise); with
CFD_RECORD_DIR set, each writes its summary and histories there as JSON.

- config 1: the 8,192-node cylinder (64 x 128, fixed mesh, Mach 0.3, Re 100), 2000 steps
  against the oracle on one thread: DTMIN and drag/lift compared every step, the state
  (U, T, X, Y) every 100th step, bit for bit (ns2DComp.ALE.f90:138-282).
- config 5 with the reference's ESTAB (subrutinas.f90:374-393): the 4,194,304-node
  ellipse (2048 x 2048, Mach 0.8, Re 10000, heave 0.05 + pitch 3 deg at f = 0.1), FP64
  form against the oracle on all host threads with the element-order scatter (its
  one-thread result), up to 120 steps: DTMIN and the pressure forces every step, the state
  every 10th, and the step at which each side's state first stops being finite (both sides
  at the same step: the reference's method itself breaks down on this case; NaN counts as
  equal to NaN).
"""
import json
import math
import os
import time

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("CFD_RECORDS") != "1",
                                 reason="long record runs: set CFD_RECORDS=1")]


def _write(name, summary, history):
    d = os.environ.get("CFD_RECORD_DIR")
    if d:
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, f"{name}.json"), "w") as f:
            json.dump({"summary": summary, "history": history}, f)
    print(json.dumps(summary))


def _lift_drag(rep, side):
    """Drag and lift of body set 1 as the reference's FORCES file takes them: pressure
    (FX, FY of FORCES, meshMove.f90:153-194) plus viscous (F_VX, F_VY of FORCE_VISC,
    ns2DComp.ALE.f90:247-248)."""
    fvx, fvy, _ = side.force_visc()
    return float(rep.fx[0] + fvx[0]), float(rep.fy[0] + fvy[0])


def _same_bits(a, b):
    """Every entry the same double bit for bit, or NaN on both sides (the payloads of a NaN
    differ between the host's and the GPU's arithmetic)."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return bool(np.all((a.view(np.uint64) == b.view(np.uint64)) | (np.isnan(a) & np.isnan(b))))


def test_config1_fp64_2000_steps_bit_exact(gpu_lib, oracle):
    from cfd_gb300 import case as C, solver
    n = int(os.environ.get("CFD_RECORD_STEPS", "2000"))
    oracle.set_threads(1)
    k = C.config_case(1)
    S, Oc = solver.Solver(k), oracle.OracleCase(k)
    S.set_force_visc(True)
    Oc.set_force_visc(True)
    mism, checks, hist = [], 0, []
    t0 = time.perf_counter()
    for s in range(1, n + 1):
        rg, ro = S.step(1), Oc.step(1)
        fg, fo = _lift_drag(rg, S), _lift_drag(ro, Oc)
        same = rg.dtmin == ro.dtmin and fg == fo
        if s % 100 == 0 or s == n:
            sg, so = S.state(), Oc.state()
            checks += 1
            same = same and all(_same_bits(sg[q], so[q]) for q in ("U", "T", "X", "Y"))
            hist.append({"step": s, "time": rg.time, "dtmin": rg.dtmin, "drag": fg[0],
                         "lift": fg[1], "bit_exact": bool(same),
                         "rho_mean": float(sg["U"][:, 0].mean())})
        if not same:
            mism.append(s)
    summary = {"record": "config1",
               "workload": f"cylinder O-grid 64x128 ({k.npoin} nodes, {k.nelem} triangles), "
                           f"Mach 0.3, Re 100, fixed mesh, FP64",
               "steps": n, "state_checks": checks, "mismatched_steps": mism[:20],
               "bit_exact_every_step_and_checkpoint": not mism,
               "wall_s": time.perf_counter() - t0,
               "final_state_finite": bool(np.isfinite(S.state()["U"]).all())}
    S.close()
    Oc.close()
    _write("config1", summary, hist)
    assert not mism


def test_config5_fp64_reference_estab_lockstep(gpu_lib, oracle):
    from cfd_gb300 import abi, case as C, solver
    n = int(os.environ.get("CFD_RECORD_STEPS", "120"))
    oracle.set_threads(os.cpu_count() or 1)
    oracle.set_ordered_scatter(True)
    try:
        k = C.config_case(5)
        k.params.estab_mode = abi.CFD_ESTAB_REFERENCE
        S, Oc = solver.Solver(k), oracle.OracleCase(k)
        hist, mism = [], []
        first_bad = {"gpu": None, "oracle": None}
        t0 = time.perf_counter()
        for s in range(1, n + 1):
            rg, ro = S.step(1), Oc.step(1)
            fg = (float(rg.fx[0]), float(rg.fy[0]))
            fo = (float(ro.fx[0]), float(ro.fy[0]))
            same = _same_bits([rg.dtmin, *fg], [ro.dtmin, *fo])
            sg = so = None
            if s % 10 == 0 or not all(map(math.isfinite, fg + fo)):
                sg, so = S.state(), Oc.state()
                same = same and all(_same_bits(sg[q], so[q]) for q in ("U", "T", "X", "Y"))
                for side, st in (("gpu", sg), ("oracle", so)):
                    if first_bad[side] is None and not np.isfinite(st["U"]).all():
                        first_bad[side] = s
            hist.append({"step": s, "dtmin": [rg.dtmin, ro.dtmin], "fx": [fg[0], fo[0]],
                         "fy": [fg[1], fo[1]], "bit_exact": bool(same),
                         "state_checked": sg is not None,
                         "rho_min": None if sg is None else [float(np.nanmin(sg["U"][:, 0])),
                                                             float(np.nanmin(so["U"][:, 0]))]})
            if not same:
                mism.append(s)
            if first_bad["gpu"] is not None and first_bad["oracle"] is not None:
                break
        summary = {"record": "config5_fp64_reference_estab_lockstep",
                   "workload": f"ellipse O-grid 2048x2048 ({k.npoin} nodes, {k.nelem} "
                               f"triangles), Mach 0.8, Re 10000, heave 0.05 + pitch 3 deg @ "
                               f"f=0.1, ALE + gcl, FP64, reference ESTAB",
                   "oracle_threads": oracle.lib().or_get_threads(),
                   "steps_run": len(hist), "mismatched_steps": mism[:20],
                   "bit_exact_every_step": not mism,
                   "first_nonfinite_step": first_bad, "wall_s": time.perf_counter() - t0}
        S.close()
        Oc.close()
    finally:
        oracle.set_ordered_scatter(False)
        oracle.set_threads(1)
    _write("config5_reference_estab", summary, hist)
    assert not mism
    assert first_bad["gpu"] == first_bad["oracle"]

"""PROGRAM NSComp2D's run loop and its files (ns2DComp.ALE.f90:8-389) over a resident
context: the reference's case directory in (EULER.DAT, <name>-1.dat, <name>.dat, and
<name>.RST when IRESTART = 1), the reference's output files out.

    from cfd_gb300 import driver
    summary = driver.run_case("case_dir", out_dir="run")

Every print step (ITERPRINT = IPRINT, or the last iteration) writes, as the reference's
print block (ns2DComp.ALE.f90:186-254) does:

* ``<name>.cnv`` — ITER, TIME and the four relative residuals ||U_old - U||/||U|| (:195-203);
  the reference's format '(I7, 4E14.6)' has one E descriptor fewer than its six items,
  so the line here is '(I7, 5E14.6)';
* the fuse: a residual above 1e2 stops the run (:206-214);
* ``SKIN.DAT`` — FORCE_VISC's per-edge rows (:833-887) when FMU != 0; list-directed output
  is compiler-defined, the rows here are three ES25.16E3 fields;
* ``DESPLAZAMIENTO`` — TIME, F_VX(1), F_VY(1), RM(1), F_VX(2), F_VY(2), RM(2), '(7E13.5)';
* ``FORCES`` — per set the pressure, viscous and total forces (:237-250);
* ``<name>.RST`` — PRINTREST (:898-917), Fortran unformatted sequential records.

``FORCES_HISTORY`` is opened and left empty (:41).  The engine is a ``Solver`` by default;
anything with the same step/state/force_visc interface can drive the loop.

Setup differences: the reference smooths the mesh at setup (:72, smoothing.f90) — pass
``smoothing=callable`` to apply one; after a restart it restores U, T and GAMM only and
zeroes TIME and ITER (:107-109), leaving VEL_X, VEL_Y unset, which here are U(2)/U(1),
U(3)/U(1).
"""
import os
import struct

import numpy as np

from . import abi
from .case import read_case


# ------------------------------------------------------------------ Fortran edit descriptors
def fortran_e(v, w, d):
    """Ew.d: 0.ddddddE+ee, right-justified in w columns (three-digit exponents drop the E)."""
    v = float(v)
    if not np.isfinite(v):
        s = "NaN" if np.isnan(v) else ("-Infinity" if v < 0 else "Infinity")
        return s.rjust(w)[-w:]
    if v == 0.0:
        digits, e = "0" * d, 0
    else:
        m = f"{abs(v):.{d - 1}e}"
        digits = m[0] + m[2:2 + d - 1]
        e = int(m.split("e")[1]) + 1
    exp = f"E{'+' if e >= 0 else '-'}{abs(e):02d}" if abs(e) <= 99 else \
        f"{'+' if e >= 0 else '-'}{abs(e):03d}"
    s = ("-" if v < 0 else "") + "0." + digits + exp
    return s.rjust(w) if len(s) <= w else "*" * w


def fortran_i(v, w):
    s = str(int(v))
    return s.rjust(w) if len(s) <= w else "*" * w


def fortran_es(v, w=25, d=16):
    """ESw.dE3 (the SKIN.DAT rows): d.ddd...E+eee."""
    m = f"{float(v):.{d}e}"
    mant, e = m.split("e")
    return f"{mant}E{int(e):+04d}".rjust(w)


# ------------------------------------------------------------------ .RST
def _record(payload):
    n = struct.pack("<i", len(payload))
    return n + payload + n


def write_restart(path, iter_, time, U, T, GAMM):
    """PRINTREST (ns2DComp.ALE.f90:898-917): one record ITER (int32), TIME (real*8), then
    per node one record U(1:4), T, GAMM (six real*8); little-endian, 4-byte record markers
    (gfortran and ifort defaults)."""
    U = np.ascontiguousarray(U, dtype="<f8").reshape(-1, 4)
    rows = np.concatenate([U, np.asarray(T, "<f8")[:, None], np.asarray(GAMM, "<f8")[:, None]], 1)
    body = np.empty(rows.shape[0], dtype=[("a", "<i4"), ("v", "<f8", 6), ("b", "<i4")])
    body["a"] = 48
    body["v"] = rows
    body["b"] = 48
    with open(path, "wb") as f:
        f.write(_record(struct.pack("<id", int(iter_), float(time))))
        f.write(body.tobytes())


def read_restart(path, npoin):
    """RESTART (ns2DComp.ALE.f90:424-431) -> (ITER_OLD, TIME, U (npoin, 4), T, GAMM)."""
    with open(path, "rb") as f:
        data = f.read()
    n0 = struct.unpack_from("<i", data, 0)[0]
    if n0 != 12:
        raise ValueError(f"{path}: first record of {n0} bytes, expected 12 (ITER, TIME)")
    it, tm = struct.unpack_from("<id", data, 4)
    if struct.unpack_from("<i", data, 16)[0] != 12:
        raise ValueError(f"{path}: bad record marker")
    need = 20 + npoin * 56
    if len(data) < need:
        raise ValueError(f"{path}: {len(data)} bytes, {need} expected for {npoin} nodes")
    body = np.frombuffer(data, dtype=[("a", "<i4"), ("v", "<f8", 6), ("b", "<i4")],
                         count=npoin, offset=20)
    if not ((body["a"] == 48).all() and (body["b"] == 48).all()):
        raise ValueError(f"{path}: bad node record markers")
    v = body["v"]
    return int(it), float(tm), v[:, :4].copy(), v[:, 4].copy(), v[:, 5].copy()


# ------------------------------------------------------------------ the run
class Stop(RuntimeError):
    """The fuse of ns2DComp.ALE.f90:206-214 (a residual above 1e2)."""


def residuals(U_old, U_new):
    """ER/ERR of :195-203: per conserved variable sqrt(sum (U - U1)^2 / sum U1^2)."""
    er = ((U_old - U_new) ** 2).sum(0)
    err = (U_new ** 2).sum(0)
    return np.sqrt(er / err)


def run_case(directory, out_dir=None, precision=abi.CFD_PREC_FP64, maxiter=None, engine=None,
             smoothing=None, smooth_every=0, verbose=False):
    """Run the case in `directory` for MAXITER (or `maxiter`) iterations and write the
    reference's files into `out_dir` (default: the case directory).  `smooth_every` > 0
    smooths the moved mesh every that many steps (the smoothing module's setTol_move path,
    smoothing.f90:372-386, which the reference's loop never calls).  Returns a summary."""
    case = read_case(directory)
    out_dir = out_dir or directory
    os.makedirs(out_dir, exist_ok=True)
    p = case.params
    name = case.name
    if smoothing is not None:
        fixed = np.zeros(case.npoin, np.int32)
        fixed[case.ilaux() - 1] = 1
        case.x, case.y = smoothing(case.x, case.y, case.inpoel, fixed)
    if engine is None:
        from .solver import Solver
        engine = Solver(case, precision=precision)
    if p.irestart == 1:
        _, _, U, T, _ = read_restart(os.path.join(directory, name + ".RST"), case.npoin)
        engine.set_state(U, T, U[:, 1] / U[:, 0], U[:, 2] / U[:, 0])
    if smooth_every > 0:
        engine.set_smoothing(smooth_every)
    viscous = p.fmu != 0.0
    if viscous:
        engine.set_force_visc(True)
    open(os.path.join(out_dir, "FORCES_HISTORY"), "w").close()
    cnv = open(os.path.join(out_dir, name + ".cnv"), "w")
    desp = open(os.path.join(out_dir, "DESPLAZAMIENTO"), "w")
    last = {"iter": 0}
    maxiter = p.maxiter if maxiter is None else maxiter
    iprint = max(1, p.iprint)
    fvx, fvy = np.zeros(10), np.zeros(10)
    try:
        it, iterprint = 0, 0
        while it < maxiter:
            printing = iterprint + 1 == iprint or it + 1 == maxiter
            U_old = engine.state()["U"] if printing else None
            rep = engine.step(1)
            it += 1
            iterprint += 1
            if not printing:
                continue
            st = engine.state()
            res = residuals(U_old, st["U"])
            cnv.write(fortran_i(it, 7) + "".join(fortran_e(v, 14, 6) for v in (rep.time, *res))
                      + "\n")
            cnv.flush()
            if verbose:
                print(f"ITER {it} TIME {rep.time:.4e} DTMIN {rep.dtmin:.4e} residuals {res}")
            if np.max(res) > 1.0e2 or not np.isfinite(res).all():
                raise Stop(f"ERROR CONVERGENCIA / OVERFLOW at iteration {it}")
            iterprint = 0
            n = rep.nset_numb
            if viscous:
                gx, gy, skin = engine.force_visc()
                fvx[:n], fvy[:n] = gx, gy
                with open(os.path.join(out_dir, "SKIN.DAT"), "w") as f:
                    for row in skin:
                        f.write("".join(fortran_es(v) for v in row) + "\n")
            desp.write("".join(fortran_e(v, 13, 5) for v in (
                rep.time, fvx[0], fvy[0], rep.rm[0], fvx[1], fvy[1], rep.rm[1])) + "\n")
            desp.flush()
            with open(os.path.join(out_dir, "FORCES"), "w") as f:
                for s in range(n):
                    f.write("SET NUMERO" + fortran_i(s + 1, 2) + "\n")
                    f.write("FUERZA EN X:" + fortran_e(rep.fx[s], 14, 5) + "\n")
                    f.write("FUERZA EN Y:" + fortran_e(rep.fy[s], 14, 5) + "\n\n")
                    f.write("FUERZA VISCOSA EN X:" + fortran_e(fvx[s], 14, 5) + "\n")
                    f.write("FUERZA VISCOSA EN Y:" + fortran_e(fvy[s], 14, 5) + "\n\n")
                    f.write("FUERZA TOTAL EN X:" + fortran_e(rep.fx[s] + fvx[s], 14, 5) + "\n")
                    f.write("FUERZA TOTAL EN Y:" + fortran_e(rep.fy[s] + fvy[s], 14, 5) + "\n\n")
            gamm = np.full(case.npoin, p.gama)
            write_restart(os.path.join(out_dir, name + ".RST"), it, rep.time, st["U"], st["T"],
                          gamm)
            last = {"iter": it, "time": rep.time, "dtmin": rep.dtmin, "residuals": res.tolist(),
                    "fx": list(rep.fx[:n]), "fy": list(rep.fy[:n]), "rm": list(rep.rm[:n]),
                    "f_vx": fvx[:n].tolist(), "f_vy": fvy[:n].tolist()}
    finally:
        cnv.close()
        desp.close()
    return last


def main(argv=None):
    """Command line: run a case directory as the reference's executable does."""
    import argparse
    import json
    ap = argparse.ArgumentParser(description="Run a case directory (EULER.DAT, <name>-1.dat, "
                                 "<name>.dat) and write the reference's output files.")
    ap.add_argument("directory")
    ap.add_argument("--out", default=None, help="output directory (default: the case's)")
    ap.add_argument("--precision", choices=("fp64", "mixed"), default="fp64")
    ap.add_argument("--maxiter", type=int, default=None, help="steps (default: MAXITER)")
    ap.add_argument("--smooth-every", type=int, default=0,
                    help="smooth the moved mesh every this many steps (0: never)")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args(argv)
    prec = abi.CFD_PREC_FP64 if a.precision == "fp64" else abi.CFD_PREC_MIXED
    last = run_case(a.directory, a.out, precision=prec, maxiter=a.maxiter,
                    smooth_every=a.smooth_every, verbose=a.verbose)
    print(json.dumps(last))


if __name__ == "__main__":
    main()

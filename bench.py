#!/usr/bin/env python
"""bench.py — node-steps/s of the explicit SUPG compressible NS step with ALE mesh motion.

Workload: the 1,048,576-node ellipse O-grid (1024 x 1024, axes 1 and 0.12 at 2 degrees,
outer radius 30, +-10% seeded jitter), Mach 0.8, Re 5000, heave 0.05 at frequency 0.1,
ALE on with the gcl-corrected mass update.  A step is one iteration of the reference's
time loop: deltat, ESTAB, 4 RK stages of calcRHS+FUENTE and the lumped-mass update with
its boundary conditions, FORCES, TRANSF, two BiCG mesh-motion solves, the node update,
and the geometry of the moved mesh (normales, deriv, gcl, laplace).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0.  N > 1 runs N independent replicas (one per GPU; the path has
no exchange step on one mesh), value = all ranks' node-steps / max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "node-steps/s at 1M nodes: plain FP64 vs mixed+learned at ≤1e-6 rel L2"
UNIT = "node-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1500,
                    help="timed steps (the default times ~1 s, long enough for the clock "
                         "samples taken meanwhile)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--no-compare", action="store_true",
                    help="skip the plain-FP64 timing and the mixed-vs-FP64 error")
    ap.add_argument("--scale", type=int, default=None, help="nr = ntheta (reduced-size runs)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--large-nr", type=int, default=None,
                    help="nodes per direction of the large heave + pitch O-grid report "
                         "(default 2048, the 4,194,304-node workload; given, it also runs "
                         "under --no-compare)")
    ap.add_argument("--guess", choices=["learned", "learned_refined", "previous", "zero"],
                    default="learned",
                    help="initial guess of the mesh-motion solve in the mixed form "
                         "(learned_refined: the network once, then its refined fields judged "
                         "against the extrapolated increments)")
    ap.add_argument("--guess-gate", type=float, default=20.0,
                    help="learned guess: iterations of the previous solve above which the "
                         "network runs (it also runs on the first solve)")
    ap.add_argument("--accuracy-steps", type=int, default=0,
                    help="instead of the benchmark: run the mixed and the FP64 forms side by "
                         "side for this many steps and print their state and force errors")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="only run warmup + this many steps (for ncu captures)")
    ap.add_argument("--accuracy-compare-steps", type=int, default=2000,
                    help="steps of the default run's mixed-vs-FP64 and reference-vs-"
                         "regularized-ESTAB comparisons (the metric's condition is stated "
                         "after 2000 steps)")
    ap.add_argument("--record", choices=["config2", "config5"], default=None,
                    help="instead of the benchmark: the long run of a workload as its "
                         "configuration describes it (histories into --record-out)")
    ap.add_argument("--record-steps", type=int, default=None)
    ap.add_argument("--record-guess", choices=["previous", "extrapolated"], default="previous",
                    help="config2: the mesh-motion solves' initial guess (previous: the "
                         "reference's; extrapolated: CFD_GUESS_EXTRAPOLATED)")
    ap.add_argument("--record-out", default=None, help="JSON file of the record's histories")
    ap.add_argument("--bicg-tol-mode", type=int, default=0,
                    help="BiCG stopping test of the headline run and of --profile-steps "
                         "(0: the reference's absolute test; 1: relative 1e-10, cap 20000)")
    ap.add_argument("--guess-tol-mode", type=int, default=1,
                    help="BiCG stopping test of the guess report (0: the reference's "
                         "absolute r.z < 1e-10; 1: ||r|| <= 1e-10 ||b - A x_D||)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, use_gpu):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch
            import torch.distributed as td
            backend = "nccl" if use_gpu else "gloo"
            if use_gpu:
                torch.cuda.set_device(self.local)
            td.init_process_group(backend)
            self.td = td
            self.torch = torch
            self.use_gpu = use_gpu

    def barrier(self):
        if self.ws > 1:
            if self.use_gpu:
                self.td.barrier(device_ids=[self.local])
            else:
                self.td.barrier()

    def max(self, v):
        if self.ws == 1:
            return v
        t = self.torch.tensor([float(v)], dtype=self.torch.float64,
                              device=f"cuda:{self.local}" if self.use_gpu else "cpu")
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def replica_value(ws, npoin, sec_step):
    """Whole-job node-steps/s of ws replicas of an npoin-node mesh whose slowest rank took
    sec_step per step."""
    return ws * npoin / sec_step


def workload(args):
    from cfd_gb300 import case as C
    k = C.config_case(3, scale=args.scale)
    return k


def config_dict(k, args, ws):
    m = k.meta
    return {"workload": f"ellipse O-grid {m['nr']}x{m['ntheta']} ({k.npoin} nodes, {k.nelem} "
                        f"triangles), Mach 0.8, Re 5000, heave 0.05 @ f=0.1, ALE + gcl",
            "npoin": k.npoin, "nelem": k.nelem, "precision": args.precision,
            "guess": args.guess if args.precision == "mixed" else "previous",
            "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
            "l2": "inputs larger than L2 (state + element arrays ~0.9 GB at 1M nodes)",
            "data": "seeded synthetic O-grid (seed 0)"}


# Algorithmic bytes per launch of each timed group: every array a launch must touch, read
# or written once (gathers of node data count once per node).  N nodes, E elements, and
# 3E element-around-point slots (~6 per node).
# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per step of the timed groups
# of the mixed form on the 1,048,576-node workload, from the ncu capture summarised in
# profiles/step_mixed_1M_launches.md (the full-size workload fits the capture rules: ~2.5 GB
# on the device, kernels of 13-130 us).
NCU_TRAFFIC_PER_STEP = {
    "update_t": 1047.2e6,   # 4 node passes (934.0 MB) + 3 mu/lambda passes (113.2 MB)
    "calcrhs_t": 347.9e6,   # k_elem_stage1_mixed (ESTAB's DTMIN-free part included)
    "deltat_t": 62.9e6,     # k_deltat_mixed (the FP64 refinement reads a few chunks)
}


def algorithmic_bytes(k, iters, precision):
    """Algorithmic DRAM bytes per STEP of each timed group: every array element the group
    must read or write once (gathered node/element values counted once)."""
    N, E = k.npoin, k.nelem
    S = 3 * E          # (element, local node) slots
    nnz = 7 * N        # mesh-Laplacian entries (structured triangulation)
    it = float(iters)
    # BiCG: initial residual (both right-hand sides), then per iteration two passes over
    # the vectors and one FP32 SpMV per right-hand side
    bicg = nnz * 8 + N * 45 + it * (N * 234 + nnz * 16) + (N * 56 + nnz * 16 if it > 0 else 0)
    if precision == "mixed":
        # node pass of one RK stage: recVisc 16 + slot id 4 B/slot, element mu/lambda 8 B/E;
        # slot pointers 4, stage-invariant sums 16, 1/M 4, BC flags 1, U hi 16, T 4 B/N
        node_common = S * (16 + 4) + E * 8 + N * (4 + 16 + 4 + 1 + 16 + 4)
        return {
            # ESTAB + calcRHS + FUENTE: elem 16, slot_pos 12, geo 32 B/E; recInv + recVisc
            # 96 B/E; mu/lambda 8 B/E; U hi/lo 32 + W 8 + T 4 + VX, VY 8 B/N
            "calcrhs_t": E * (16 + 12 + 32 + 96 + 8) + N * 52,
            # stage 1 adds recInv (16 B/slot); stage 4 adds U 32, U1 32, six primitives 24,
            # U hi/lo 32 B/N; stages 2-4 recompute mu/lambda (elem 16 + 8 B/E, T 4 B/N)
            "update_t": 4 * node_common + S * 16 + N * 120 + 3 * (E * 24 + N * 4),
            # deltat: elem 16, area 4 B/E; T, VX, VY 12 + W 8 B/N
            "deltat_t": E * (16 + 4) + N * 20,
            "deriv_t": E * (16 + 32 + 4 + 8 + 8) + N * 32,
            "laplace_t": S * 8 + E * 40 + N * 52 + nnz * 4,
            "grad_t": bicg,
        }
    return {
        "calcrhs_t": 4 * (E * (16 + 48 + 8 + 8 + 24 + 96) + N * 40) + E * 96 + N * 16,
        "update_t": 4 * N * (24 + 2 * 6 * 32 + 32 + 8 + 32 + 56),
        "estab_t": E * (16 + 48 + 32) + N * (32 + 8 + 32),
        "deltat_t": E * (16 + 8 + 8) + N * 40,
        "grad_t": bicg,
    }


def main_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    k = workload(args)
    threads = os.cpu_count() or 1
    # bounded sample: each reported step is one real step of the full 1M-node workload
    n = max(1, min(args.steps, 3))
    w = 1 if args.warmup > 0 else 0
    from oracle import oracle as O
    O.set_threads(threads)
    oc = O.OracleCase(k)
    if w:
        oc.step(w)
    t = time.perf_counter()
    oc.step(n)
    sec = (time.perf_counter() - t) / n
    oc.close()
    v = k.npoin / sec
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": n, "warmup": w, "ms_per_step": sec * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(k, args, 1),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{n} full step(s) of the {k.npoin}-node workload after "
                                       f"{w} warm-up step(s) (oracle, OpenMP)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference is Fortran (ifort/OpenMP); no Fortran compiler here, so the "
                    "timed reference arm is the oracle's C++ restatement of it"}
    print(json.dumps(line), flush=True)


def timed_run(solver_mod, k, prec, W, K, L, net=None, gate=0.0, refine=False):
    """Create a context (with the learned-guess network attached when given, and its
    refined fields when refine), W warm-up steps, then K steps between CUDA events on the
    context's stream.  Returns (solver, ms per step, kernel launches, report)."""
    S = solver_mod.Solver(k, precision=prec)
    if net is not None:
        S.set_guess_net(net, gate)
        if refine:
            S.set_guess_refine(True)
    S.step(W)
    import torch
    torch.cuda.synchronize()
    l0 = L.cfd_kernel_launches()
    S.mark(0)
    rep = S.step(K)
    S.mark(1)
    ms = S.elapsed_ms(0, 1)
    return S, ms / K, L.cfd_kernel_launches() - l0, rep


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def main_accuracy(args):
    """Mixed form against the FP64 form (same ESTAB mode) on the workload, stepped in
    lockstep: state rel L2 per conserved variable every 100 steps and at the end, and the
    pressure-force (lift, drag) error over the run relative to the largest FP64 force."""
    from cfd_gb300 import abi, build, solver
    build.build()
    km, kd = workload(args), workload(args)
    for k in (km, kd):
        k.params.estab_mode = abi.CFD_ESTAB_REGULARIZED
    Sm = solver.Solver(km, precision=abi.CFD_PREC_MIXED)
    Sd = solver.Solver(kd, precision=abi.CFD_PREC_FP64)
    fmax, ferr, hist = 0.0, [0.0, 0.0], []
    for s in range(1, args.accuracy_steps + 1):
        rm, rd = Sm.step(1), Sd.step(1)
        fmax = max(fmax, abs(rd.fx[0]), abs(rd.fy[0]))
        ferr[0] = max(ferr[0], abs(rm.fx[0] - rd.fx[0]))
        ferr[1] = max(ferr[1], abs(rm.fy[0] - rd.fy[0]))
        if s % 100 == 0 or s == args.accuracy_steps:
            Um, Ud = Sm.state()["U"], Sd.state()["U"]
            mom = np.linalg.norm(Ud[:, 1:3])
            hist.append({"step": s, "rel_l2": [rel_l2(Um[:, q], Ud[:, q]) for q in range(4)],
                         "rel_l2_state": rel_l2(Um, Ud),
                         "rel_l2_momentum": float(np.linalg.norm(Um[:, 1:3] - Ud[:, 1:3]) / mom),
                         "finite": bool(np.isfinite(Um).all() and np.isfinite(Ud).all())})
    Sm.close()
    Sd.close()
    line = {"accuracy": "mixed vs fp64", "workload": config_dict(km, args, 1)["workload"],
            "npoin": km.npoin, "steps": args.accuracy_steps, "estab_mode": "regularized",
            "final_rel_l2": hist[-1]["rel_l2"] if hist else None,
            "max_rel_l2": [max(h["rel_l2"][q] for h in hist) for q in range(4)] if hist else None,
            "final_rel_l2_state": hist[-1]["rel_l2_state"] if hist else None,
            "final_rel_l2_momentum": hist[-1]["rel_l2_momentum"] if hist else None,
            "force_err_rel_max": [e / fmax if fmax > 0 else None for e in ferr],
            "history": hist}
    print(json.dumps(line), flush=True)


def large_mesh_report(W, net, gate, hbm_peak, nr=2048):
    """The nr x nr ellipse O-grid of config 5 (heave + pitch, Re 10000; nr = 2048: 4,194,304
    nodes) in the mixed form with the learned guess: node-steps/s over 200 event-timed
    steps, and the update_t group's algorithmic bandwidth and roofline fraction (timers on,
    own context)."""
    from cfd_gb300 import abi, case as C, solver
    k = C.config_case(5, scale=None if nr == 2048 else nr)
    k.params.estab_mode = abi.CFD_ESTAB_REGULARIZED
    if net is not None:
        k.params.guess_mode = abi.CFD_GUESS_LEARNED
    S = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    if net is not None:
        S.set_guess_net(net, gate)
    S.step(W)
    K = 200
    S.mark(0)
    S.step(K)
    S.mark(1)
    ms = S.elapsed_ms(0, 1) / K
    S.close()
    os.environ["CFD_TIMERS"] = "1"
    try:
        S2 = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    finally:
        os.environ.pop("CFD_TIMERS", None)
    S2.step(2)
    t0 = S2.timers()
    rep = S2.step(4)
    t1 = S2.timers()
    S2.close()
    upd = (t1["update_t"][0] - t0["update_t"][0]) / 4
    ab = algorithmic_bytes(k, float(np.mean(list(rep.bicg_iters))), "mixed")["update_t"]
    return {"workload": f"ellipse O-grid {k.meta['nr']}x{k.meta['ntheta']} ({k.npoin} nodes, "
                        f"{k.nelem} triangles), Mach 0.8, Re 10000, heave 0.05 + pitch 3 deg "
                        f"@ f=0.1, ALE + gcl",
            "npoin": k.npoin, "value": k.npoin / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
            "steps": K, "update_t": {"ms_per_step": upd * 1e3, "GBps_algorithmic": ab / upd / 1e9,
                                     "frac_of_hbm_peak": ab / upd / 1e9 / hbm_peak}}


def relative_test_report(args, W, net, K=300):
    """The metric's workload with the mesh-motion solves to the configurations' 1e-10
    relative test: the mixed form with the refined learned guess judged against the
    extrapolated increments (CFD_GUESS_LEARNED_EXTRAPOLATED), node-steps/s over K
    event-timed steps after the cold solve and W warm-up steps (graph replay, as the
    headline), with the iterations of the timed steps."""
    from cfd_gb300 import abi, solver
    k = workload(args)
    k.params.estab_mode = abi.CFD_ESTAB_REGULARIZED
    k.params.guess_mode = abi.CFD_GUESS_LEARNED_EXTRAPOLATED
    k.params.bicg_tol_mode = abi.CFD_BICG_TOL_REL
    k.params.bicg_tol = 1.0e-10
    k.params.bicg_maxit = 20000
    S = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
    S.set_guess_net(net, 1.0e9)
    S.set_guess_refine(True)
    r1 = S.step(1)
    S.step(max(W, 3))
    its, relres, conv = [], [], []
    S.mark(0)
    for _ in range(K):
        r = S.step(1)
        its.append(sum(r.bicg_iters))
        relres.append(max(r.bicg_relres))
        conv.append(min(r.bicg_converged))
    S.mark(1)
    ms = S.elapsed_ms(0, 1) / K
    S.close()
    return {"bicg_test": "||r|| <= 1e-10 ||b - A x_D|| (relative)",
            "guess": "learned_refined_extrapolated", "value": k.npoin / (ms / 1e3), "unit": UNIT,
            "ms_per_step": ms, "steps": K, "first_step_iters": list(r1.bicg_iters),
            "iters_per_step": float(np.mean(its)), "iters_per_step_max": int(max(its)),
            "all_converged": bool(min(conv) == 1), "max_relres": float(max(relres))}


def guess_report(args, W, K, tol_mode=0, tol=1.0e-10, maxit=1000, modes=None,
                 precision=None):
    """Mesh-motion solve with the previous-step, zero and learned guesses on the workload
    (mixed form): BiCG iterations (x + y solves) on the first (cold) step and per step after
    warm-up, the mesh-motion time per step (timer of the BiCG group, which holds the network
    and the fields), the step time, and for the learned guesses how often a guess was
    formed and how often it was taken.  tol_mode / tol / maxit: the solve's stopping test
    (0: the reference's absolute |r.z|; 1: ||r|| <= tol ||b - A x_D||).

    Learned variants: "learned" runs the network on the first solve and after solves above
    the gate; "learned_every_step" runs it on every solve; "learned_refined" runs it on the
    first solve and then tries, every step, the guess of the basis fields it seeded and
    the solves refine (cfd_ctx_set_guess_refine).  "extrapolated": CFD_GUESS_EXTRAPOLATED,
    the last two increments extrapolated to the step's DTMIN; "learned_refined_extrapolated":
    the refined learned guess judged against that extrapolation.  precision: the form that
    solves (the learned variants run in the mixed form only)."""
    from cfd_gb300 import abi, learned, solver
    net = learned.Net.load()
    out = {}
    all_modes = {"previous": (abi.CFD_GUESS_PREVIOUS, None, False),
                 "zero": (abi.CFD_GUESS_ZERO, None, False),
                 "learned_every_step": (abi.CFD_GUESS_LEARNED, 0.0, False),
                 "learned": (abi.CFD_GUESS_LEARNED, args.guess_gate, False),
                 "learned_refined": (abi.CFD_GUESS_LEARNED, 1.0e9, True)}
    all_modes["extrapolated"] = (abi.CFD_GUESS_EXTRAPOLATED, None, False)
    all_modes["learned_refined_extrapolated"] = (abi.CFD_GUESS_LEARNED_EXTRAPOLATED, 1.0e9, True)
    modes = modes or ["previous", "zero", "learned_every_step", "learned"]
    os.environ["CFD_TIMERS"] = "1"
    try:
        for name in modes:
            mode, gate, refine = all_modes[name]
            k = workload(args)
            k.params.estab_mode = abi.CFD_ESTAB_REGULARIZED
            k.params.guess_mode = mode
            k.params.bicg_tol_mode = tol_mode
            k.params.bicg_tol = tol
            k.params.bicg_maxit = maxit
            S = solver.Solver(k, precision=abi.CFD_PREC_MIXED if precision is None else precision)
            if gate is not None:
                S.set_guess_net(net, gate)
                if refine:
                    S.set_guess_refine(True)
            r1 = S.step(1)
            S.step(max(W - 1, 0))
            t0 = S.timers()
            its, conv, relres = [], [], []
            S.mark(0)
            for _ in range(K):
                r = S.step(1)
                its.append(sum(r.bicg_iters))
                conv.append(min(r.bicg_converged))
                relres.append(max(r.bicg_relres))
            S.mark(1)
            ms = S.elapsed_ms(0, 1) / K
            t1 = S.timers()
            d = {"first_step_iters": list(r1.bicg_iters), "iters_per_step": float(np.mean(its)),
                 "iters_per_step_min_max": [int(min(its)), int(max(its))],
                 "converged_steps": int(sum(conv)), "steps_timed": K,
                 "max_relres": float(max(relres)) if tol_mode else None,
                 "mesh_motion_ms_per_step": (t1["grad_t"][0] - t0["grad_t"][0]) * 1e3 / K,
                 "ms_per_step": ms}
            if gate is not None:
                st = S.guess_stats_ex()
                ev, tx, ty, n = st[:4]
                d.update({"gate": gate, "network_steps": ev, "network_taken": tx + ty,
                          "network_fallback_rate": (1.0 - (tx + ty) / (2.0 * ev)) if ev else None,
                          "steps": n})
                if refine:
                    dv, dx, dy = st[4:7]
                    d.update({"fields_steps": dv, "fields_taken": [dx, dy]})
            S.close()
            out[name] = d
    finally:
        os.environ.pop("CFD_TIMERS", None)
    return out


def e2e_loop(S, L, N, KE, dist, ws):
    """The metric through the C-ABI with host buffers: per step, upload U (the context
    derives the velocities and keeps T), one step, download U; pinned host memory, copies
    inside the timed region.  Returns the e2e dict."""
    import torch
    from cfd_gb300 import abi
    hU = torch.empty((N, 4), dtype=torch.float64, pin_memory=True).numpy()
    hU[:] = S.state()["U"]
    torch.cuda.synchronize()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(KE):
        abi.check(L.cfd_ctx_upload_state(S.h, abi.dptr(hU), None, None, None), "upload")
        S.step(1)
        abi.check(L.cfd_ctx_download_state(S.h, abi.dptr(hU), None, None, None), "download")
    torch.cuda.synchronize()
    sec = dist.max(time.perf_counter() - t0) / KE
    return {"value": ws * N / sec, "unit": UNIT, "h2d_bytes_per_step": int(N * 32),
            "d2h_bytes_per_step": int(N * 32), "ms_per_step": sec * 1e3, "steps": KE}


def forces(rep):
    return float(rep.fx[0]), float(rep.fy[0])


def accuracy_compare(args, NS):
    """Three runs of the workload in lockstep for NS steps: the mixed form (regularized
    ESTAB, previous-step guess), the FP64 form with the same ESTAB, and the FP64 form with
    the reference's ESTAB (subrutinas.f90:374-393).  Returns (a) the mixed form's error
    against the FP64 form of the same method: the whole state and each conserved variable
    (rel L2, rho*v also against the momentum scale) after NS steps, and the pressure force
    (drag, lift of body set 1) error over the run against the largest FP64 force; (b) how
    far the regularized method sits from the reference's: the same measures between the two
    FP64 runs."""
    from cfd_gb300 import abi, solver
    runs = {}
    for name, prec, estab in (("mixed", abi.CFD_PREC_MIXED, abi.CFD_ESTAB_REGULARIZED),
                              ("fp64_reg", abi.CFD_PREC_FP64, abi.CFD_ESTAB_REGULARIZED),
                              ("fp64_ref", abi.CFD_PREC_FP64, abi.CFD_ESTAB_REFERENCE)):
        k = workload(args)
        k.params.estab_mode = estab
        runs[name] = solver.Solver(k, precision=prec)
    hist = {n: [] for n in runs}
    t0 = time.perf_counter()
    for _ in range(NS):
        for n, S in runs.items():
            hist[n].append(forces(S.step(1)))
    wall = time.perf_counter() - t0
    U = {n: S.state()["U"] for n, S in runs.items()}
    for S in runs.values():
        S.close()
    F = {n: np.array(h) for n, h in hist.items()}

    def compare(a, b):
        Ua, Ub = U[a], U[b]
        fmax = float(np.abs(F[b]).max())
        return {"state_rel_l2": rel_l2(Ua, Ub),
                "rel_l2": [rel_l2(Ua[:, q], Ub[:, q]) for q in range(4)],
                "rho_v_rel_l2_momentum_scale": float(np.linalg.norm(Ua[:, 2] - Ub[:, 2]) / max(
                    np.linalg.norm(Ub[:, 1]), np.linalg.norm(Ub[:, 2]))),
                "force_err_rel_max": [float(np.abs(F[a][:, c] - F[b][:, c]).max() / fmax)
                                      for c in range(2)],
                "force_err_rel_final": [float(abs(F[a][-1, c] - F[b][-1, c]) / fmax)
                                        for c in range(2)],
                "finite": bool(np.isfinite(Ua).all() and np.isfinite(Ub).all())}
    return {"steps": NS, "wall_s": wall,
            "mixed_vs_fp64": dict(compare("mixed", "fp64_reg"), estab_mode="regularized",
                                  guess="previous"),
            "estab_regularized_vs_reference_fp64": compare("fp64_reg", "fp64_ref")}


def run_cpu_baselines(k_fn, threads_all):
    """The oracle on the host cores: all threads (3 steps after 1 warm-up step) and one
    thread (1 step), each on the full workload."""
    from oracle import oracle as O
    out = {}
    for label, threads, steps, warm in (("all_cores", threads_all, 3, 1), ("one_core", 1, 1, 0)):
        O.set_threads(threads)
        k = k_fn()
        oc = O.OracleCase(k)
        if warm:
            oc.step(warm)
        t = time.perf_counter()
        oc.step(steps)
        sec = (time.perf_counter() - t) / steps
        oc.close()
        out[label] = {"value": k.npoin / sec, "unit": UNIT, "cores": threads, "kind": "port",
                      "sample": f"{steps} full step(s) of the {k.npoin}-node workload after "
                                f"{warm} warm-up step(s) (oracle, OpenMP, {threads} "
                                f"thread(s), reference ESTAB), setup excluded",
                      "ms_per_step": sec * 1e3}
    return out


def config1_report(threads_all, steps=2000):
    """The reference's CPU-runnable case run fully (the 8,192-node cylinder, fixed mesh,
    2000 steps): the FP64 form on the GPU (device time over one cfd_step call) and the
    oracle on all host cores and on one core, node-steps/s each."""
    from cfd_gb300 import abi, case as C, solver
    from oracle import oracle as O
    out = {"workload": "cylinder O-grid 64x128 (8192 nodes, 16128 triangles), Mach 0.3, "
                       "Re 100, fixed mesh, FP64, reference ESTAB", "steps": steps}
    k = C.config_case(1)
    S = solver.Solver(k)
    S.step(3)
    S.mark(0)
    S.step(steps)
    S.mark(1)
    ms = S.elapsed_ms(0, 1) / steps
    S.close()
    out["gpu_fp64"] = {"value": k.npoin / (ms / 1e3), "unit": UNIT, "ms_per_step": ms}
    for label, threads in (("oracle_all_cores", threads_all), ("oracle_one_core", 1)):
        O.set_threads(threads)
        oc = O.OracleCase(C.config_case(1))
        oc.step(3)
        t = time.perf_counter()
        oc.step(steps)
        sec = (time.perf_counter() - t) / steps
        oc.close()
        out[label] = {"value": k.npoin / sec, "unit": UNIT, "cores": threads, "kind": "port",
                      "ms_per_step": sec * 1e3}
    O.set_threads(1)
    return out


def lift_drag(rep, S):
    """Drag and lift of body set 1 as the reference's FORCES file takes them: pressure
    (FX, FY of FORCES, meshMove.f90:153-194) plus viscous (F_VX, F_VY of FORCE_VISC,
    ns2DComp.ALE.f90:247-248)."""
    fvx, fvy, _ = S.force_visc()
    return float(rep.fx[0] + fvx[0]), float(rep.fy[0] + fvy[0])


def main_record(args):
    """Long runs of the workloads as their configurations describe them; the histories go
    to --record-out (JSON), one summary line to stdout.  (The runs that compare against the
    oracle step by step, the 8,192-node cylinder over 2000 steps among them, are
    tests/test_records.py.)

    config2: the 262,144-node cylinder (512 x 512, heave 0.2 sin(2 pi 0.2 t), Re 200), FP64
      form, the mesh-motion solve to ||r|| <= 1e-10 ||b - A x_D||, 5000 steps: BiCG
      iterations and relative residual per step and solve, drag and lift per step.
    config5: the 4,194,304-node ellipse (2048 x 2048, Mach 0.8, Re 10000, heave 0.05 + pitch
      3 deg at f = 0.1): the mixed form with the learned guess (refined fields) for 10000
      steps, node-steps/s, and its pressure forces over the first 500 steps against 500-step
      FP64 runs of the same case (regularized and reference ESTAB)."""
    from cfd_gb300 import abi, build, case as C, learned, solver
    build.build()
    abi.lib()
    out = {"record": args.record}
    hist = []
    if args.record == "config2":
        n = args.record_steps or 5000
        k = C.config_case(2)
        k.params.bicg_tol_mode = abi.CFD_BICG_TOL_REL
        k.params.bicg_tol = 1.0e-10
        k.params.bicg_maxit = 20000
        if args.record_guess == "extrapolated":
            k.params.guess_mode = abi.CFD_GUESS_EXTRAPOLATED
        S = solver.Solver(k)
        S.set_force_visc(True)
        t0 = time.perf_counter()
        S.mark(0)
        for s in range(1, n + 1):
            r = S.step(1)
            d, li = lift_drag(r, S)
            hist.append({"step": s, "time": r.time, "dtmin": r.dtmin, "drag": d, "lift": li,
                         "bicg_iters": list(r.bicg_iters), "bicg_relres": list(r.bicg_relres),
                         "converged": list(r.bicg_converged)})
        S.mark(1)
        ms = S.elapsed_ms(0, 1) / n
        its = np.array([h["bicg_iters"] for h in hist])
        out.update({"workload": f"cylinder O-grid 512x512 ({k.npoin} nodes, {k.nelem} "
                                f"triangles), Mach 0.3, Re 200, heave 0.2 sin(2 pi 0.2 t), ALE "
                                f"+ gcl, FP64, BiCG to ||r|| <= 1e-10 ||b - A x_D|| from "
                                f"the {args.record_guess} guess",
                    "steps": n, "ms_per_step": ms, "node_steps_per_s": k.npoin / (ms / 1e3),
                    "wall_s": time.perf_counter() - t0,
                    "bicg_iters_per_solve_mean": its.mean(0).tolist(),
                    "bicg_iters_per_solve_min": its.min(0).tolist(),
                    "bicg_iters_per_solve_max": its.max(0).tolist(),
                    "all_converged": all(min(h["converged"]) == 1 for h in hist),
                    "max_relres": max(max(h["bicg_relres"]) for h in hist),
                    "final_time": hist[-1]["time"],
                    "lift_range": [min(h["lift"] for h in hist), max(h["lift"] for h in hist)],
                    "drag_range": [min(h["drag"] for h in hist), max(h["drag"] for h in hist)],
                    "state_finite": bool(np.isfinite(S.state()["U"]).all())})
        S.close()
    elif args.record == "config5":
        n = args.record_steps or 10000
        nf = min(500, n)
        net = learned.Net.load()
        k = C.config_case(5)
        k.params.estab_mode = abi.CFD_ESTAB_REGULARIZED
        k.params.guess_mode = abi.CFD_GUESS_LEARNED
        if args.bicg_tol_mode:  # the configs' relative test instead of the reference's; the
            # learned guesses judged against the extrapolated increments (the pitching body's
            # x solve takes the extrapolation, the y solve the fields)
            k.params.bicg_tol_mode = args.bicg_tol_mode
            k.params.bicg_maxit = 20000
            k.params.guess_mode = abi.CFD_GUESS_LEARNED_EXTRAPOLATED
        S = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
        S.set_guess_net(net, 1.0e9)
        S.set_guess_refine(True)
        fm, its = [], []
        S.mark(0)
        for s in range(1, nf + 1):
            rs = S.step(1)
            fm.append(forces(rs))
            its.append(list(rs.bicg_iters))
        S.mark(2)
        r = S.step(n - nf) if n > nf else S.step(0)
        S.mark(1)
        ms = S.elapsed_ms(0, 1) / n
        ms_tail = S.elapsed_ms(2, 1) / (n - nf) if n > nf else None
        Um = S.state()["U"]
        gs = S.guess_stats_ex()
        S.close()
        out.update({"workload": f"ellipse O-grid 2048x2048 ({k.npoin} nodes, {k.nelem} "
                                f"triangles), Mach 0.8, Re 10000, heave 0.05 + pitch 3 deg @ "
                                f"f=0.1, ALE + gcl, mixed + learned guess (refined fields)",
                    "steps": n, "ms_per_step": ms, "value": k.npoin / (ms / 1e3),
                    "ms_per_step_after_force_window": ms_tail,
                    "bicg_iters_last": list(r.bicg_iters), "guess_stats_ex": list(gs),
                    "bicg_test": "relative" if args.bicg_tol_mode else "absolute (reference)",
                    "bicg_iters_per_step_force_window": {
                        "first": its[0], "mean_after_first": (np.array(its[1:]).sum(1).mean()
                                                              if len(its) > 1 else None)},
                    "state_finite": bool(np.isfinite(Um).all())})
        for estab, name in ((abi.CFD_ESTAB_REGULARIZED, "fp64_regularized"),
                            (abi.CFD_ESTAB_REFERENCE, "fp64_reference")):
            kd = C.config_case(5)
            kd.params.estab_mode = estab
            if args.bicg_tol_mode:  # the same test; from the previous increment the FP64
                # solves would take thousands of iterations a step, from the extrapolated
                # one none (the guess moves the solution only within the test)
                kd.params.bicg_tol_mode = args.bicg_tol_mode
                kd.params.bicg_maxit = 20000
                kd.params.guess_mode = abi.CFD_GUESS_EXTRAPOLATED
            Sd = solver.Solver(kd)
            fd = [forces(Sd.step(1)) for _ in range(nf)]
            Sd.close()
            Fm, Fd = np.array(fm), np.array(fd)
            # the reference's ESTAB breaks down on this case (its state stops being finite,
            # bit for bit with the oracle): compare over the steps before that
            bad = np.flatnonzero(~np.isfinite(Fd).all(axis=1))
            m = int(bad[0]) if bad.size else nf
            fmax = float(np.abs(Fd[:m]).max())
            out[f"forces_vs_{name}"] = {
                "steps": nf, "steps_compared": m,
                "first_nonfinite_step": int(bad[0]) + 1 if bad.size else None,
                "rel_err_max": [float(np.abs(Fm[:m, c] - Fd[:m, c]).max() / fmax)
                                for c in range(2)],
                "rel_err_final": [float(abs(Fm[m - 1, c] - Fd[m - 1, c]) / fmax)
                                  for c in range(2)]}
            hist.append({name: Fd.tolist()})
        hist.append({"mixed": fm, "bicg_iters": its})
    if args.record_out:
        with open(args.record_out, "w") as f:
            json.dump({"summary": out, "history": hist}, f)
    print(json.dumps(out), flush=True)


def main_ours(args):
    ws, rank, local = dist_env()
    import torch
    from cfd_gb300 import abi, build, solver
    build.build()
    L = abi.lib()
    abi.check(L.cfd_set_device(local), "cfd_set_device")
    dist = Dist(use_gpu=True)
    k = workload(args)
    mixed = args.precision == "mixed"
    prec = abi.CFD_PREC_MIXED if mixed else abi.CFD_PREC_FP64
    # the mixed form runs the regularized ESTAB (continuous in the state; the reference's
    # is discontinuous at round-off level); the plain form runs the reference's
    k.params.estab_mode = abi.CFD_ESTAB_REGULARIZED if mixed else abi.CFD_ESTAB_REFERENCE
    W, K = max(3, args.warmup), args.steps
    net, gate = None, 0.0
    refine = mixed and args.guess == "learned_refined"
    if mixed and args.guess in ("learned", "learned_refined"):
        from cfd_gb300 import learned
        k.params.guess_mode = (abi.CFD_GUESS_LEARNED_EXTRAPOLATED if refine
                               else abi.CFD_GUESS_LEARNED)
        net, gate = learned.Net.load(), (1.0e9 if refine else args.guess_gate)
    elif args.guess == "zero":
        k.params.guess_mode = abi.CFD_GUESS_ZERO
    if args.bicg_tol_mode:
        k.params.bicg_tol_mode = args.bicg_tol_mode
        k.params.bicg_maxit = 20000
    if args.profile_steps:
        S = solver.Solver(k, precision=prec)
        if net is not None:
            S.set_guess_net(net, gate)
            if refine:
                S.set_guess_refine(True)
        S.step(W)
        S.step(args.profile_steps)
        return
    # ---- headline form: timed region (device time, CUDA events on the launching stream)
    torch.cuda.synchronize()
    dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    S, ms_step, launches, rep = timed_run(solver, k, prec, W, K, L, net, gate, refine)
    guess_stats = S.guess_stats() if net is not None else None
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    sec_step = dist.max(ms_step) / 1e3
    value = replica_value(ws, k.npoin, sec_step)
    final_U = S.state()["U"]
    # ---- e2e through the C-ABI with pinned host buffers, copies inside the timed region
    N = k.npoin
    KE = max(2, min(K, 10))
    e2e = e2e_loop(S, L, N, KE, dist, ws)
    S.close()
    # ---- the other forms: plain FP64 (reference ESTAB) speed and e2e; the errors of the
    # mixed form and of the regularized ESTAB over the comparison run; the mesh-motion solve
    # with each initial guess under the relative stopping test
    forms = {}
    if mixed and not args.no_compare:
        kp = workload(args)
        Sp, msp, lp, repp = timed_run(solver, kp, abi.CFD_PREC_FP64, W, min(K, 10), L)
        forms["fp64_plain"] = {"value": ws * N / (dist.max(msp) / 1e3), "unit": UNIT,
                               "ms_per_step": msp, "estab_mode": "reference",
                               "gpu_launches_per_step": lp / min(K, 10),
                               "e2e": e2e_loop(Sp, L, N, 3, dist, ws)}
        Sp.close()
        forms["speedup_vs_fp64_plain"] = value / forms["fp64_plain"]["value"]
        forms["e2e_speedup_vs_fp64_plain"] = e2e["value"] / forms["fp64_plain"]["e2e"]["value"]
        if args.accuracy_compare_steps > 0:
            forms["accuracy"] = accuracy_compare(args, args.accuracy_compare_steps)
        if net is not None:
            # under the reference's absolute test the learned guess changes the mesh motion
            # within the solve's tolerance
            NC = W + min(K, 52)
            runs = {}
            for name, mode in (("previous", abi.CFD_GUESS_PREVIOUS),
                               ("learned", abi.CFD_GUESS_LEARNED)):
                kl = workload(args)
                kl.params.estab_mode = abi.CFD_ESTAB_REGULARIZED
                kl.params.guess_mode = mode
                Sl = solver.Solver(kl, precision=abi.CFD_PREC_MIXED)
                if mode == abi.CFD_GUESS_LEARNED:
                    Sl.set_guess_net(net, gate)
                Sl.step(NC)
                runs[name] = (Sl.state()["U"], Sl.guess_stats() if mode else None)
                Sl.close()
            Ul, Um = runs["learned"][0], runs["previous"][0]
            forms["learned_vs_previous_guess"] = {
                "steps": NC, "bicg_tol_mode": "absolute (reference)",
                "rel_l2": [rel_l2(Ul[:, q], Um[:, q]) for q in range(4)],
                "guess_stats": list(runs["learned"][1]),
                # (network evaluated, x and y guesses taken, steps) in the timed run
                "timed_run_guess_stats": list(guess_stats)}
        tm = args.guess_tol_mode
        forms["guess"] = guess_report(
            args, W, min(K, 10), tol_mode=tm, tol=1.0e-10, maxit=20000 if tm else 1000,
            modes=["previous", "zero", "learned", "learned_every_step", "learned_refined",
                   "extrapolated", "learned_refined_extrapolated"])
        forms["guess"]["bicg_test"] = ("||r|| <= 1e-10 ||b - A x_D|| (relative)" if tm else
                                       "|r.z| < 1e-10 (the reference's absolute test)")
        # the same solves in the plain FP64 form (its operator is assembled in FP64, so the
        # previous solutions carry no FP32 rounding of the operator into the next solve)
        forms["guess_fp64"] = guess_report(
            args, W, min(K, 10), tol_mode=tm, tol=1.0e-10, maxit=20000 if tm else 1000,
            modes=["previous", "extrapolated"], precision=abi.CFD_PREC_FP64)
        forms["guess_fp64"]["bicg_test"] = forms["guess"]["bicg_test"]
        if net is not None:
            forms["relative_test"] = relative_test_report(args, W, net)
    # ---- per-kernel breakdown and roofline of the dominant kernel (timers on, own ctx)
    os.environ["CFD_TIMERS"] = "1"
    S2 = solver.Solver(k, precision=prec)
    os.environ.pop("CFD_TIMERS")
    S2.step(2)
    t_before = S2.timers()
    KT = 4
    rep2 = S2.step(KT)
    t_after = S2.timers()
    S2.close()
    per_step, per_launch, calls_per_step = {}, {}, {}
    for n_, (sec, calls) in t_after.items():
        ds, dc = sec - t_before[n_][0], calls - t_before[n_][1]
        if dc > 0:
            per_step[n_] = ds / KT
            per_launch[n_] = ds / dc
            calls_per_step[n_] = dc / KT
    iters = float(np.mean(list(rep2.bicg_iters)))
    ab = algorithmic_bytes(k, iters, args.precision)
    total = sum(per_step.values())
    dom = max(per_step, key=lambda n_: per_step[n_])
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    ach = ab[dom] / per_step[dom] / 1e9 if dom in ab else None
    traffic = None
    if mixed and args.scale is None and dom in NCU_TRAFFIC_PER_STEP:
        traffic = NCU_TRAFFIC_PER_STEP[dom] / calls_per_step[dom]
    roofline = {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                "frac": (ach / hbm_peak) if ach else None, "traffic": traffic,
                "traffic_source": "ncu capture, profiles/step_mixed_1M_launches.md"
                if traffic else None,
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback",
                "share_of_step": per_step[dom] / total if total else None,
                "launch_ms": per_launch[dom] * 1e3,
                "launches_per_step": calls_per_step[dom],
                "algorithmic_bytes_per_launch": (ab[dom] / calls_per_step[dom]) if dom in ab else None}
    if mixed and args.scale is None and ws == 1:
        if args.large_nr is not None and args.large_nr != 2048:
            forms[f"config5_nr{args.large_nr}"] = large_mesh_report(W, net, gate, hbm_peak,
                                                                    args.large_nr)
        elif not args.no_compare or args.large_nr is not None:
            forms["config5_4M"] = large_mesh_report(W, net, gate, hbm_peak)
    kernels = {n_: {"ms_per_launch": per_launch[n_] * 1e3, "launches_per_step": calls_per_step[n_],
                    "GBps_algorithmic": (ab[n_] / per_step[n_] / 1e9) if n_ in ab else None,
                    "frac_of_hbm_peak": (ab[n_] / per_step[n_] / 1e9 / hbm_peak)
                    if n_ in ab else None}
               for n_ in per_launch}
    cpu, cpu1 = None, None
    if rank == 0 and not args.no_cpu_baseline:
        cb = run_cpu_baselines(lambda: workload(args), os.cpu_count() or 1)
        cpu, cpu1 = cb["all_cores"], cb["one_core"]
        if mixed and args.scale is None and not args.no_compare:
            forms["config1_gpu_vs_cpu"] = config1_report(os.cpu_count() or 1)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K,
                "warmup": W, "ms_per_step": sec_step * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64 (mixed)" if mixed else "f64", "data": "synthetic",
                "config": config_dict(k, args, ws), "e2e": e2e, "gpu_launches": int(launches),
                "clocks": clk, "roofline": roofline, "cpu_baseline": cpu,
                "cpu_baseline_one_core": cpu1, "forms": forms,
                "kernels": kernels,
                "breakdown_ms_per_step": {n_: v * 1e3 for n_, v in per_step.items()},
                "bicg_iters": list(rep.bicg_iters), "bicg_converged": list(rep.bicg_converged),
                "state_finite": bool(np.isfinite(final_U).all())}
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        main_reference(a)
    elif a.record:
        main_record(a)
    elif a.accuracy_steps > 0:
        main_accuracy(a)
    else:
        main_ours(a)

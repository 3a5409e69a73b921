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
    ap.add_argument("--guess", choices=["learned", "previous", "zero"], default="learned",
                    help="initial guess of the mesh-motion solve in the mixed form")
    ap.add_argument("--guess-gate", type=float, default=20.0,
                    help="learned guess: iterations of the previous solve above which the "
                         "network runs (it also runs on the first solve)")
    ap.add_argument("--accuracy-steps", type=int, default=0,
                    help="instead of the benchmark: run the mixed and the FP64 forms side by "
                         "side for this many steps and print their state and force errors")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="only run warmup + this many steps (for ncu captures)")
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
    "update_t": 1059.5e6,   # 4 node passes (946.4 MB) + 3 mu/lambda passes (113.1 MB)
    "calcrhs_t": 350.1e6,   # k_elem_stage1_mixed (ESTAB's DTMIN-free part included)
    "deltat_t": 63.3e6,     # k_deltat_mixed (the FP64 refinement reads a few chunks)
    "laplace_t": 181.8e6,
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


def run_cpu_reference(k, threads, steps):
    """The oracle (CPU restatement of the reference) with `threads` OpenMP threads:
    seconds per step over `steps` steps after setup."""
    from oracle import oracle as O
    O.set_threads(threads)
    oc = O.OracleCase(k)
    t = time.perf_counter()
    rep = oc.step(steps)
    dt = (time.perf_counter() - t) / steps
    oc.close()
    return dt, rep


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


def timed_run(solver_mod, k, prec, W, K, L, net=None, gate=0.0):
    """Create a context (with the learned-guess network attached when given), W warm-up
    steps, then K steps between CUDA events on the context's stream.  Returns (solver, ms
    per step, kernel launches, report)."""
    S = solver_mod.Solver(k, precision=prec)
    if net is not None:
        S.set_guess_net(net, gate)
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


def guess_report(args, W, K):
    """Mesh-motion solve with the previous-step, zero and learned guesses on the workload
    (mixed form): BiCG iterations on the first (cold) step and per step after warm-up, the
    mesh-motion time per step (timer of the BiCG group, which holds the network), the step
    time, and for the learned guess how often it ran and how often its guess was taken."""
    from cfd_gb300 import abi, learned, solver
    net = learned.Net.load()
    out = {}
    modes = (("previous", abi.CFD_GUESS_PREVIOUS, None), ("zero", abi.CFD_GUESS_ZERO, None),
             ("learned_every_step", abi.CFD_GUESS_LEARNED, 0.0),
             ("learned", abi.CFD_GUESS_LEARNED, args.guess_gate))
    os.environ["CFD_TIMERS"] = "1"
    try:
        for name, mode, gate in modes:
            k = workload(args)
            k.params.estab_mode = abi.CFD_ESTAB_REGULARIZED
            k.params.guess_mode = mode
            S = solver.Solver(k, precision=abi.CFD_PREC_MIXED)
            if gate is not None:
                S.set_guess_net(net, gate)
            r1 = S.step(1)
            S.step(max(W - 1, 0))
            t0 = S.timers()
            its = []
            S.mark(0)
            for _ in range(K):
                its.append(sum(S.step(1).bicg_iters))
            S.mark(1)
            ms = S.elapsed_ms(0, 1) / K
            t1 = S.timers()
            d = {"first_step_iters": list(r1.bicg_iters), "iters_per_step": float(np.mean(its)),
                 "mesh_motion_ms_per_step": (t1["grad_t"][0] - t0["grad_t"][0]) * 1e3 / K,
                 "ms_per_step": ms}
            if gate is not None:
                ev, tx, ty, n = S.guess_stats()
                d.update({"gate": gate, "network_steps": ev, "network_taken": tx + ty,
                          "fallback_rate": (1.0 - (tx + ty) / (2.0 * ev)) if ev else None,
                          "steps": n})
            S.close()
            out[name] = d
    finally:
        os.environ.pop("CFD_TIMERS", None)
    return out


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
    if mixed and args.guess == "learned":
        from cfd_gb300 import learned
        k.params.guess_mode = abi.CFD_GUESS_LEARNED
        net, gate = learned.Net.load(), args.guess_gate
    elif args.guess == "zero":
        k.params.guess_mode = abi.CFD_GUESS_ZERO
    if args.profile_steps:
        S = solver.Solver(k, precision=prec)
        if net is not None:
            S.set_guess_net(net, gate)
        S.step(W)
        S.step(args.profile_steps)
        return
    # ---- headline form: timed region (device time, CUDA events on the launching stream)
    torch.cuda.synchronize()
    dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    S, ms_step, launches, rep = timed_run(solver, k, prec, W, K, L, net, gate)
    guess_stats = S.guess_stats() if net is not None else None
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    sec_step = dist.max(ms_step) / 1e3
    value = replica_value(ws, k.npoin, sec_step)
    final_U = S.state()["U"]
    # ---- e2e through the C-ABI with pinned host buffers, copies inside the timed region
    N = k.npoin
    st, f = S.state(), S.fields()
    hU = torch.empty((N, 4), dtype=torch.float64, pin_memory=True).numpy()
    hT = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    hvx = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    hvy = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
    hU[:], hT[:], hvx[:], hvy[:] = st["U"], st["T"], f["VEL_X"], f["VEL_Y"]
    KE = max(2, min(K, 10))
    torch.cuda.synchronize()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(KE):
        S.set_state(hU, hT, hvx, hvy)
        S.step(1)
        abi.check(L.cfd_ctx_download_state(S.h, abi.dptr(hU), abi.dptr(hT), None, None),
                  "download")
    torch.cuda.synchronize()
    e2e_sec = dist.max(time.perf_counter() - t0) / KE
    e2e = {"value": ws * N / e2e_sec, "unit": UNIT, "h2d_bytes_per_step": int(N * (32 + 8 * 3)),
           "d2h_bytes_per_step": int(N * (32 + 8))}
    S.close()
    # ---- the other forms: plain FP64 (reference ESTAB) speed; FP64 with the same ESTAB
    # as the mixed run for its error
    forms = {}
    if mixed and not args.no_compare:
        kp = workload(args)
        Sp, msp, lp, repp = timed_run(solver, kp, abi.CFD_PREC_FP64, W, min(K, 10), L)
        forms["fp64_plain"] = {"value": ws * N / (dist.max(msp) / 1e3), "unit": UNIT,
                               "ms_per_step": msp, "estab_mode": "reference"}
        Sp.close()
        # the error runs: W + min(K, 52) steps (the FP64 form takes ~29 ms a step)
        NC = W + min(K, 52)
        kr = workload(args)
        kr.params.estab_mode = abi.CFD_ESTAB_REGULARIZED
        Sr = solver.Solver(kr, precision=abi.CFD_PREC_FP64)
        repr_ = Sr.step(NC)
        Ur = Sr.state()["U"]
        Sr.close()
        # precision error: the mixed form against the FP64 form, both with the previous-
        # step guess (the same mesh-motion solves)
        km = workload(args)
        km.params.estab_mode = abi.CFD_ESTAB_REGULARIZED
        Sm = solver.Solver(km, precision=abi.CFD_PREC_MIXED)
        repm = Sm.step(NC)
        Um = Sm.state()["U"]
        Sm.close()
        forms["mixed_vs_fp64"] = {
            "steps": NC, "estab_mode": "regularized", "guess": "previous",
            # the whole conserved state; per variable against its own norm; rho*v (small at
            # 2 degrees) also against the momentum scale max(|rho*u|, |rho*v|)
            "state_rel_l2": rel_l2(Um, Ur),
            "rel_l2": [rel_l2(Um[:, q], Ur[:, q]) for q in range(4)],
            "rho_v_rel_l2_momentum_scale": float(np.linalg.norm(Um[:, 2] - Ur[:, 2]) / max(
                np.linalg.norm(Ur[:, 1]), np.linalg.norm(Ur[:, 2]))),
            "force_rel_err": float(np.hypot(repm.fx[0] - repr_.fx[0], repm.fy[0] - repr_.fy[0])
                                   / np.hypot(repr_.fx[0], repr_.fy[0]))}
        if net is not None:
            # the learned guess changes the mesh motion within the solve's absolute tolerance
            kl = workload(args)
            kl.params.estab_mode = abi.CFD_ESTAB_REGULARIZED
            kl.params.guess_mode = abi.CFD_GUESS_LEARNED
            Sl = solver.Solver(kl, precision=abi.CFD_PREC_MIXED)
            Sl.set_guess_net(net, gate)
            Sl.step(NC)
            Ul = Sl.state()["U"]
            gs_l = Sl.guess_stats()
            Sl.close()
            forms["learned_vs_previous_guess"] = {
                "steps": NC, "rel_l2": [rel_l2(Ul[:, q], Um[:, q]) for q in range(4)],
                "guess_stats": list(gs_l),
                # (network evaluated, x and y guesses taken, steps) in the timed run
                "timed_run_guess_stats": list(guess_stats)}
        forms["speedup_vs_fp64_plain"] = value / forms["fp64_plain"]["value"]
        if mixed:
            forms["guess"] = guess_report(args, W, min(K, 10))
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
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        kc = workload(args)
        sec, _ = run_cpu_reference(kc, threads, 1)
        cpu = {"value": k.npoin / sec, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"1 full step of the {k.npoin}-node workload (oracle, OpenMP, "
                         f"{threads} threads, reference ESTAB), setup excluded"}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K,
                "warmup": W, "ms_per_step": sec_step * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64 (mixed)" if mixed else "f64", "data": "synthetic",
                "config": config_dict(k, args, ws), "e2e": e2e, "gpu_launches": int(launches),
                "clocks": clk, "roofline": roofline, "cpu_baseline": cpu, "forms": forms,
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
    elif a.accuracy_steps > 0:
        main_accuracy(a)
    else:
        main_ours(a)

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
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--scale", type=int, default=None, help="nr = ntheta (reduced-size runs)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
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


def workload(args):
    from cfd_gb300 import case as C
    k = C.config_case(3, scale=args.scale)
    return k


def config_dict(k, args, ws):
    m = k.meta
    return {"workload": f"ellipse O-grid {m['nr']}x{m['ntheta']} ({k.npoin} nodes, {k.nelem} "
                        f"triangles), Mach 0.8, Re 5000, heave 0.05 @ f=0.1, ALE + gcl",
            "npoin": k.npoin, "nelem": k.nelem, "precision": args.precision,
            "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
            "l2": "inputs larger than L2 (state + element arrays ~0.9 GB at 1M nodes)",
            "data": "seeded synthetic O-grid (seed 0)"}


# algorithmic bytes per launch of each timed group (FP64 path; the design doc lists them)
def algorithmic_bytes(k, iters):
    N, E = k.npoin, k.nelem
    nnz = 7 * N
    return {
        "calcrhs_t": E * (16 + 48 + 8 + 8 + 24 + 96) + N * 40 + (E * 96 + N * 16) / 4.0,
        "update_t": N * (24 + 2 * 6 * 32 + 32 + 8 + 32 + 56),
        "estab_t": E * (16 + 48 + 32) + N * (32 + 8 + 32),
        "deltat_t": E * (16 + 8 + 8) + N * 40,
        "grad_t": (nnz * 12 + N * 4) * (2 + iters) + N * 8 * 10 * (2 + iters),
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


def main_ours(args):
    ws, rank, local = dist_env()
    from cfd_gb300 import abi, build, solver
    build.build()
    L = abi.lib()
    abi.check(L.cfd_set_device(local), "cfd_set_device")
    dist = Dist(use_gpu=True)
    k = workload(args)
    prec = abi.CFD_PREC_FP64 if args.precision == "fp64" else abi.CFD_PREC_MIXED
    S = solver.Solver(k, precision=prec)
    W, K = max(3, args.warmup), args.steps
    if args.profile_steps:
        S.step(W)
        S.step(args.profile_steps)
        return
    S.step(W)
    # ---- timed region (device time, CUDA events on the launching stream)
    import torch
    torch.cuda.synchronize()
    dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    l0 = L.cfd_kernel_launches()
    S.mark(0)
    rep = S.step(K)
    S.mark(1)
    ms = S.elapsed_ms(0, 1)
    launches = L.cfd_kernel_launches() - l0
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    ms_max = dist.max(ms)
    sec_step = ms_max / 1e3 / K
    value = ws * k.npoin / sec_step
    # ---- e2e through the C-ABI with host buffers (pinned), copies inside the timed region
    N = k.npoin
    st = S.state()
    f = S.fields()
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
    # ---- per-kernel breakdown and roofline of the dominant kernel (timers on, separate ctx)
    os.environ["CFD_TIMERS"] = "1"
    S2 = solver.Solver(k, precision=prec)
    os.environ.pop("CFD_TIMERS")
    S2.step(2)
    t_before = S2.timers()
    KT = 4
    rep2 = S2.step(KT)
    t_after = S2.timers()
    per = {n: (t_after[n] - t_before.get(n, 0.0)) / KT for n in t_after}
    launches_per_step = {"calcrhs_t": 4, "update_t": 4, "estab_t": 1, "deltat_t": 1, "grad_t": 1}
    iters = float(np.mean(list(rep2.bicg_iters)))
    ab = algorithmic_bytes(k, iters)
    total = sum(per.values())
    dom = max(per, key=lambda n: per[n])
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    dom_launch_s = per[dom] / launches_per_step.get(dom, 1)
    ach = ab.get(dom, 0.0) / dom_launch_s / 1e9 if dom in ab else None
    roofline = {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                "frac": (ach / hbm_peak) if ach else None, "traffic": None,
                "peak_source": "measured" if peaks else "fallback",
                "share": per[dom] / total if total else None,
                "launch_ms": dom_launch_s * 1e3}
    S2.close()
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sec, _ = run_cpu_reference(k, threads, 1)
        cpu = {"value": k.npoin / sec, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"1 full step of the {k.npoin}-node workload (oracle, OpenMP, "
                         f"{threads} threads), setup excluded"}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K,
                "warmup": W, "ms_per_step": sec_step * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config_dict(k, args, ws), "e2e": e2e, "gpu_launches": int(launches),
                "clocks": clk, "roofline": roofline, "cpu_baseline": cpu,
                "breakdown_ms_per_step": {n: v * 1e3 for n, v in per.items() if v > 0},
                "bicg_iters": list(rep.bicg_iters), "bicg_converged": list(rep.bicg_converged)}
        print(json.dumps(line), flush=True)
    S.close()
    dist.close()


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        main_reference(a)
    else:
        main_ours(a)

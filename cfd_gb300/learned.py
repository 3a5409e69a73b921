"""Learned initial guess of the mesh-motion solve.

The reference starts each mesh-motion solve (meshMove.f90:97 and :119, biconjGrad.f90:8-62)
from the previous step's increment.  Here an edge message-passing network (4 layers,
width 64; cfd_gb300/csrc/mpnn.cuh) predicts, from the mesh geometry, the three fields
Phi, Psi_x, Psi_y of the solve (its response to the body data 1, x - c_x, y - c_y); the
guess for a prescribed body displacement g is t Phi + M (Psi_x, Psi_y) with (t, M) the
least-squares affine fit of g, exact for rigid motions once the fields are.  BiCG then
finishes the solve to the same tolerance.  Everything runs through libcfd_gb300: the
FP32 training forward/backward passes and Adam are the library's own CUDA kernels, the
inference pass uses BF16 tensor cores.

    Net            network parameters and Adam state on the GPU
    Graph          one mesh graph with its boundary nodes
    rigid_bc       boundary displacement of a rigid body motion (heave, pitch)
    Laplace        the mesh Laplacian of a mesh (mLaplace.f90), its plain solve, and the
                   fields (training targets) from three plain solves
    make_meshes / make_dataset / train   the training pipeline
    DEFAULT_WEIGHTS                      the trained parameters shipped with the package

Run `python -m cfd_gb300.learned --train OUT.npz` to regenerate the weights.
"""
import argparse
import ctypes as C
import os
import time

import numpy as np

from . import abi, case as cs, solver
from .abi import check, dptr, iptr

PKG = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(PKG, "data", "mpnn_guess.npz")
_fp = C.POINTER(C.c_float)


def _f32p(a):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_fp)


def n_params():
    return int(abi.lib().cfd_mpnn_nparams())


def init_weights(seed=0):
    """Uniform(+-1/sqrt(fan_in)) weights, zero biases, in the library's packing (the same
    draw as the test oracle's init_params)."""
    rng = np.random.default_rng(seed)
    F_IN, HID, E_F, LAYERS, OUT = 10, 64, 3, 4, 3
    shapes = [(HID, F_IN), (HID,)]
    for _ in range(LAYERS):
        shapes += [(HID, HID), (HID, HID), (HID, E_F), (HID,), (HID, 2 * HID), (HID,)]
    shapes += [(OUT, HID), (OUT,)]
    parts = []
    for sh in shapes:
        if len(sh) == 1:
            parts.append(np.zeros(sh, np.float32))
        else:
            b = 1.0 / np.sqrt(sh[1])
            parts.append(rng.uniform(-b, b, size=sh).astype(np.float32))
    return np.concatenate([p.reshape(-1) for p in parts])


class Net:
    def __init__(self, weights=None, seed=0):
        w = init_weights(seed) if weights is None else np.ascontiguousarray(weights, np.float32)
        assert w.size == n_params(), (w.size, n_params())
        h = C.c_void_p()
        check(abi.lib().cfd_mpnn_create(C.byref(h), _f32p(w)), "cfd_mpnn_create")
        self.h = h

    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS):
        return cls(np.load(path)["weights"])

    def save(self, path, **meta):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez(path, weights=self.weights(), **meta)

    def weights(self):
        w = np.zeros(n_params(), np.float32)
        check(abi.lib().cfd_mpnn_get_weights(self.h, _f32p(w)), "cfd_mpnn_get_weights")
        return w

    def set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        check(abi.lib().cfd_mpnn_set_weights(self.h, _f32p(w)), "cfd_mpnn_set_weights")

    def adam_state(self):
        m = np.zeros(n_params(), np.float32)
        v = np.zeros(n_params(), np.float32)
        t = C.c_int(0)
        check(abi.lib().cfd_mpnn_adam_state(self.h, _f32p(m), _f32p(v), C.byref(t)), "adam")
        return m, v, t.value

    def loss_grad(self, graph):
        loss = C.c_float(0)
        g = np.zeros(n_params(), np.float32)
        check(abi.lib().cfd_mpnn_loss_grad(self.h, graph.h, C.byref(loss), _f32p(g)),
              "cfd_mpnn_loss_grad")
        return loss.value, g

    def train_step(self, graph, lr):
        loss = C.c_float(0)
        check(abi.lib().cfd_mpnn_train_step(self.h, graph.h, C.c_float(lr), C.byref(loss)),
              "cfd_mpnn_train_step")
        return loss.value

    def forward(self, graph, bf16=True):
        ux, uy = np.zeros(graph.n), np.zeros(graph.n)
        check(abi.lib().cfd_mpnn_forward(self.h, graph.h, int(bool(bf16)), dptr(ux), dptr(uy)),
              "cfd_mpnn_forward")
        return ux, uy

    def close(self):
        if getattr(self, "h", None):
            abi.lib().cfd_mpnn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def boundary_of(case):
    """Boundary nodes (1-based) and kinds of a case: the moving nodes I_M (kind 1) and the
    fixed-movement nodes IFM (kind 2), in the reference's ilaux order."""
    bnode = np.concatenate([case.i_m, case.ifm]).astype(np.int32)
    bkind = np.concatenate([np.ones(len(case.i_m)), 2 * np.ones(len(case.ifm))]).astype(np.int32)
    return bnode, bkind


class Graph:
    def __init__(self, case):
        self.case = case
        self.n = case.npoin
        self.bnode, self.bkind = boundary_of(case)
        inp = np.ascontiguousarray(case.inpoel, np.int32)
        h = C.c_void_p()
        check(abi.lib().cfd_mpnn_graph_create(
            C.byref(h), int(case.npoin), int(inp.shape[0]), iptr(inp),
            dptr(np.ascontiguousarray(case.x)), dptr(np.ascontiguousarray(case.y)),
            int(len(self.bnode)), iptr(self.bnode), iptr(self.bkind)), "cfd_mpnn_graph_create")
        self.h = h

    def set_bc(self, gx, gy):
        check(abi.lib().cfd_mpnn_graph_set_bc(self.h, dptr(np.ascontiguousarray(gx, np.float64)),
                                              dptr(np.ascontiguousarray(gy, np.float64))),
              "cfd_mpnn_graph_set_bc")

    def set_target(self, phi, psi_x, psi_y):
        a = [dptr(np.ascontiguousarray(v, np.float64)) for v in (phi, psi_x, psi_y)]
        check(abi.lib().cfd_mpnn_graph_set_target(self.h, *a), "cfd_mpnn_graph_set_target")

    def globals(self):
        g = np.zeros(10)
        check(abi.lib().cfd_mpnn_graph_globals(self.h, dptr(g)), "cfd_mpnn_graph_globals")
        return dict(zip(["cx", "cy", "L", "R", "tx", "ty", "m11", "m12", "m21", "m22"], g))

    def close(self):
        if getattr(self, "h", None):
            abi.lib().cfd_mpnn_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rigid_bc(case, heave, pitch_deg, pivot=None):
    """Displacement of the boundary nodes (boundary_of order) for a rigid motion of the
    body: rotation by pitch about the pivot (default: the body centroid), then heave;
    the outer boundary stays fixed."""
    bnode, bkind = boundary_of(case)
    p = bnode - 1
    body = bkind == 1
    if pivot is None:
        pivot = (case.x[p[body]].mean(), case.y[p[body]].mean())
    th = np.radians(pitch_deg)
    dx, dy = case.x[p] - pivot[0], case.y[p] - pivot[1]
    gx = (np.cos(th) - 1.0) * dx - np.sin(th) * dy
    gy = np.sin(th) * dx + (np.cos(th) - 1.0) * dy + heave
    gx[~body] = 0.0
    gy[~body] = 0.0
    return gx, gy


class Laplace:
    """The mesh Laplacian of a case (mLaplace.f90:7-58, on the GPU) and the plain BiCG
    solve of the mesh motion (biconjGrad.f90:8-62, FP64 on the GPU)."""

    def __init__(self, case):
        self.case = case
        g = solver.deriv(case.x, case.y, case.inpoel)
        self.rp, self.idx = solver.laplace_pattern(case.inpoel, case.npoin)
        self.vals, self.diag = solver.laplace(case.inpoel, g["area"], g["dNx"], g["dNy"],
                                              case.x, case.y, self.idx, self.rp)
        self.bnode, _ = boundary_of(case)

    def solve(self, gx, gy, x0=None, y0=None, tol=1.0e-10, maxit=20000):
        """-> (ux, uy, (iters_x, iters_y)) from the guesses x0, y0 (default zero)."""
        n = self.case.npoin
        b = np.zeros(n)
        ux, ix = solver.biCG(self.vals, self.idx, self.rp, self.diag,
                             np.zeros(n) if x0 is None else x0, b, gx, self.bnode, tol, maxit)
        uy, iy = solver.biCG(self.vals, self.idx, self.rp, self.diag,
                             np.zeros(n) if y0 is None else y0, b, gy, self.bnode, tol, maxit)
        return ux, uy, (ix.iters, iy.iters), (ix.converged, iy.converged)

    def fields(self, tol=1.0e-10, maxit=20000):
        """(Phi, Psi_x, Psi_y): the plain solves for the body data 1, x - c_x, y - c_y
        (outer boundary 0), c = mean body position."""
        bnode, bkind = boundary_of(self.case)
        p = bnode - 1
        body = bkind == 1
        cx, cy = self.case.x[p[body]].mean(), self.case.y[p[body]].mean()
        one = np.where(body, 1.0, 0.0)
        dx = np.where(body, self.case.x[p] - cx, 0.0)
        dy = np.where(body, self.case.y[p] - cy, 0.0)
        phi, psx, _, c1 = self.solve(one, dx, tol=tol, maxit=maxit)
        psy, _, _, c2 = self.solve(dy, np.zeros_like(dy), tol=tol, maxit=maxit)
        return phi, psx, psy, bool(c1[0] and c1[1] and c2[0])


def make_meshes(seed=0, n=24, sizes=((64, 128), (96, 128), (128, 128), (96, 256),
                                      (128, 256), (192, 192), (256, 256)), big=(512, 512)):
    """Seeded O-grids around cylinders and ellipses (aspect ratio 0.1-1, incidence +-5 deg,
    outer radius 15-30 body lengths, +-10% jitter), 8k-65k nodes, plus one 262k-node mesh."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n + (1 if big else 0)):
        nr, nt = big if k == n else sizes[int(rng.integers(len(sizes)))]
        ar = float(rng.uniform(0.1, 1.0))
        body = "cylinder" if ar > 0.95 else "ellipse"
        p = cs.flow_params(mach=0.3, re=100.0)
        c = cs.ogrid_case(f"train{k}", nr, nt, p, body=body, r_body=0.5, semi_b=0.5 * ar,
                          incidence_deg=float(rng.uniform(-5, 5)),
                          r_out=float(rng.uniform(15.0, 30.0)), seed=int(rng.integers(1 << 30)))
        out.append(c)
    return out


def make_dataset(meshes, log=None):
    """Per mesh the fields (Phi, Psi_x, Psi_y) of three plain solves: the boundary-
    displacement / interior-displacement pairs of the unit translation and the two affine
    modes, from which the solve of any affine (rigid) motion is a combination."""
    data = []
    for mi, c in enumerate(meshes):
        phi, psx, psy, ok = Laplace(c).fields()
        if not ok:
            raise RuntimeError(f"plain solve did not converge on mesh {mi}")
        data.append((phi, psx, psy))
        if log:
            log(f"mesh {mi}: {c.npoin} nodes")
    return data


def train(meshes, data, steps, lr=1e-3, lr_end=1e-5, seed=0, log=None, net=None):
    """Adam on the library's kernels, one mesh per step, cosine learning-rate decay."""
    rng = np.random.default_rng(seed)
    net = net or Net(seed=seed)
    graphs = []
    for c, (phi, psx, psy) in zip(meshes, data):
        g = Graph(c)
        g.set_target(phi, psx, psy)
        graphs.append(g)
    hist = []
    t0 = time.time()
    for s in range(steps):
        g = graphs[int(rng.integers(len(graphs)))]
        r = lr_end + 0.5 * (lr - lr_end) * (1 + np.cos(np.pi * s / max(steps - 1, 1)))
        hist.append(net.train_step(g, r))
        if log and (s % max(steps // 20, 1) == 0 or s == steps - 1):
            log(f"step {s}: loss {np.mean(hist[-100:]):.4e} lr {r:.2e} ({time.time() - t0:.1f} s)")
    for g in graphs:
        g.close()
    return net, hist


def guess_gain(net, case, heave, pitch_deg, bf16=True):
    """Iterations of the plain solve from the zero guess and from the network's guess, and
    the max difference between the two solutions."""
    lap = Laplace(case)
    gx, gy = rigid_bc(case, heave, pitch_deg)
    ux0, uy0, it0, c0 = lap.solve(gx, gy)
    g = Graph(case)
    g.set_bc(gx, gy)
    px, py = net.forward(g, bf16=bf16)
    g.close()
    ux1, uy1, it1, c1 = lap.solve(gx, gy, px, py)
    err = float(max(np.abs(ux1 - ux0).max(), np.abs(uy1 - uy0).max()))
    rel_guess = float(np.sqrt(((px - ux0) ** 2 + (py - uy0) ** 2).sum() /
                              max((ux0 ** 2 + uy0 ** 2).sum(), 1e-300)))
    return {"iters_zero": it0, "iters_net": it1, "converged": (c0, c1), "max_diff": err,
            "guess_rel_l2": rel_guess}


def time_inference(reps=20, nr=1024):
    """BF16 inference on the nr x nr ellipse O-grid workload with the shipped weights: ms per
    forward (the guess and its download included) of the tcgen05 passes and of the mma.sync
    passes (CFD_MPNN_TC=0), and whether the two guesses are identical."""
    k = cs.config_case(3, scale=nr)
    G = Graph(k)
    net = Net.load()
    G.set_bc(*rigid_bc(k, 0.05, 2.0))
    out, guess = {}, {}
    prev = os.environ.get("CFD_MPNN_TC")
    try:
        for mode in ("1", "0"):
            os.environ["CFD_MPNN_TC"] = mode
            for _ in range(3):
                guess[mode] = net.forward(G, bf16=True)
            t = time.perf_counter()
            for _ in range(reps):
                net.forward(G, bf16=True)
            out["tcgen05" if mode == "1" else "mma.sync"] = (time.perf_counter() - t) / reps * 1e3
    finally:
        if prev is None:
            os.environ.pop("CFD_MPNN_TC", None)
        else:
            os.environ["CFD_MPNN_TC"] = prev
    out["identical"] = bool(all(np.array_equal(a, b) for a, b in zip(guess["1"], guess["0"])))
    out["nodes"] = k.npoin
    G.close()
    net.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", metavar="OUT", help="train and write the weights (.npz)")
    ap.add_argument("--time-inference", type=int, metavar="REPS",
                    help="time the BF16 inference passes on the ellipse O-grid workload")
    ap.add_argument("--nr", type=int, default=1024,
                    help="--time-inference: nodes per direction of the O-grid (default 1024)")
    ap.add_argument("--meshes", type=int, default=24)
    ap.add_argument("--steps", type=int, default=8000)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args()
    if a.time_inference:
        print(time_inference(a.time_inference, a.nr), flush=True)
        return
    if not a.train:
        ap.error("--train OUT or --time-inference REPS is required")

    def log(m):
        print(m, flush=True)

    meshes = make_meshes(a.seed, n=a.meshes)
    t = time.time()
    data = make_dataset(meshes, log=log)
    log(f"dataset: {len(data)} meshes in {time.time() - t:.1f} s")
    net, hist = train(meshes, data, a.steps, lr=a.lr, seed=a.seed, log=log)
    net.save(a.train, steps=a.steps, meshes=a.meshes, seed=a.seed,
             final_loss=float(np.mean(hist[-200:])))
    test = cs.ogrid_case("heldout", 160, 160, cs.flow_params(mach=0.3, re=100.0),
                         body="ellipse", r_body=0.5, semi_b=0.2, incidence_deg=2.0, r_out=25.0,
                         seed=12345)
    for heave, pitch in ((0.2, 0.0), (0.0, 6.0), (-0.1, -4.0)):
        log(str(guess_gain(net, test, heave, pitch)))


if __name__ == "__main__":
    main()

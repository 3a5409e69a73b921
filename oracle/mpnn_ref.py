"""CPU restatement of the learned mesh-motion guess network (TEST INFRASTRUCTURE ONLY).

The learned initial guess has no counterpart in the reference (its mesh-motion solve,
meshMove.f90:97/119 -> biconjGrad.f90:8-62, starts from the previous step's increment).
This module restates, in numpy (float64 by default), exactly the network the CUDA kernels
of cfd_gb300/csrc/kernels_mpnn.cu evaluate and differentiate, so that tests can check the
GPU forward pass, the GPU gradients (and these against finite differences) and the Adam
update.  Only tests/ use it.

Graph: mesh nodes; edges = the point-neighbour lists (both directions).  Node kinds:
0 free, 1 moving boundary (body), 2 fixed boundary (outer).  g = prescribed displacement
of the boundary nodes.

The solve is linear with one scalar operator for both components, so for an affine body
motion g = t + M (p - c) (outer boundary fixed) the displacement is
u = t Phi + M (Psi_x, Psi_y), Phi = L^-1[1], Psi_x = L^-1[x - c_x], Psi_y = L^-1[y - c_y]
(data on the body).  The network predicts (Phi, Psi_x / L, Psi_y / L) from geometry.

Globals: c = mean body position, L = 2 max |p - c| over the body, R = mean |p - c| over
the outer nodes; (t, M) = least-squares affine fit of g over the body nodes (t = mean g,
rows of M from the 2x2 normal equations of d = p - c).

Node features (10): d/L (2), log(|d|/L + 1e-6), log(R/L), body flag, outer flag, the
fields of the continuum model div(k grad u), k ~ 1/r^2, for a circular body of radius
a = L/2 in a circle of radius R: clamp((R^2 - r^2)/(R^2 - a^2), 0, 1) and
psi(rho) d / rho / L (2), psi(r) = a ((r/R)^p - (r/R)^q) / ((a/R)^p - (a/R)^q),
p, q = 1 +- sqrt(2), rho = r a / r_b(theta) with r_b the radius of the body's
second-moment ellipse along the node's direction (0 outside r < R); and the ellipse's
aspect ratio.
Edge features of i->j (3): unit vector of p_j - p_i, log(|p_j - p_i|/L).

Network: h0 = relu(W_in f + b_in); four layers of
    z_ij = A h_i + B h_j + C e_ij + c,  agg_i = mean_j relu(z_ij),
    h_i <- h_i + relu(U [h_i; agg_i] + u);
then y = W_out h + b_out (3 outputs).  The guess is t y_0 + L M (y_1, y_2) at free nodes
and g at boundary nodes.  Loss: mean over free nodes of |y - target|^2.
"""
import numpy as np

F_IN, HID, E_F, LAYERS, OUT = 10, 64, 3, 4, 3


def param_shapes():
    """(name, shape) in the flat packing order the CUDA library uses."""
    s = [("W_in", (HID, F_IN)), ("b_in", (HID,))]
    for l in range(LAYERS):
        s += [(f"A{l}", (HID, HID)), (f"B{l}", (HID, HID)), (f"C{l}", (HID, E_F)),
              (f"c{l}", (HID,)), (f"U{l}", (HID, 2 * HID)), (f"u{l}", (HID,))]
    s += [("W_out", (OUT, HID)), ("b_out", (OUT,))]
    return s


def n_params():
    return int(sum(np.prod(sh) for _, sh in param_shapes()))


def unpack(w):
    out, k = {}, 0
    for name, sh in param_shapes():
        n = int(np.prod(sh))
        out[name] = w[k:k + n].reshape(sh)
        k += n
    assert k == w.size
    return out


def pack(p):
    return np.concatenate([p[name].reshape(-1) for name, _ in param_shapes()])


def init_params(seed=0):
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases (float32)."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, sh in param_shapes():
        if len(sh) == 1:
            p[name] = np.zeros(sh, np.float32)
        else:
            b = 1.0 / np.sqrt(sh[1])
            p[name] = rng.uniform(-b, b, size=sh).astype(np.float32)
    return pack(p)


def globals_(x, y, kind, g):
    body, outer = kind == 1, kind == 2
    cx, cy = x[body].mean(), y[body].mean()
    dx, dy = x - cx, y - cy
    r = np.hypot(dx, dy)
    L = 2.0 * r[body].max()
    R = r[outer].mean() if outer.any() else L
    gb = g[body]
    t = gb.mean(axis=0)
    D = np.stack([dx[body], dy[body]], 1)
    S = D.T @ D
    M = np.linalg.solve(S, D.T @ gb).T  # rows: g_c ~ t_c + M[c] . d
    nb = body.sum()
    hx, mxy, tr = 0.5 * (S[0, 0] - S[1, 1]) / nb, S[0, 1] / nb, 0.5 * (S[0, 0] + S[1, 1]) / nb
    rt = np.hypot(hx, mxy)
    al = 0.5 * np.arctan2(2 * mxy, 2 * hx)
    return dict(cx=cx, cy=cy, L=L, R=R, tx=t[0], ty=t[1], m11=M[0, 0], m12=M[0, 1],
                m21=M[1, 0], m22=M[1, 1], ea=np.sqrt(2 * (tr + rt)),
                eb=np.sqrt(max(2 * (tr - rt), 0.0)), ec=np.cos(al), es=np.sin(al))


def features(x, y, kind, G):
    dx, dy = x - G["cx"], y - G["cy"]
    L = G["L"]
    f = np.zeros((x.size, F_IN))
    f[:, 0] = dx / L
    f[:, 1] = dy / L
    f[:, 2] = np.log(np.hypot(dx, dy) / L + 1e-6)
    f[:, 3] = np.log(G["R"] / L)
    f[:, 4] = kind == 1
    f[:, 5] = kind == 2
    r2 = dx * dx + dy * dy
    r = np.sqrt(r2)
    a, R = 0.5 * L, G["R"]
    p, q = 1.0 + np.sqrt(2.0), 1.0 - np.sqrt(2.0)
    phi, c = np.zeros_like(r), np.zeros_like(r)
    m = (r < R) if R > a else np.zeros_like(r, bool)
    if m.any():
        rs = np.maximum(r[m], 1e-6 * L)
        phi[m] = (R * R - r2[m]) / (R * R - a * a)
        ea, eb, ec, es = G["ea"], G["eb"], G["ec"], G["es"]
        u = (dx[m] * ec + dy[m] * es) / rs
        v = (-dx[m] * es + dy[m] * ec) / rs
        rb = ea * eb / np.maximum(np.sqrt(eb * eb * u * u + ea * ea * v * v), 1e-300)
        rho = np.minimum(rs * a / np.maximum(rb, 1e-6 * L), 0.999999 * R)
        psi = a * ((rho / R) ** p - (rho / R) ** q) / ((a / R) ** p - (a / R) ** q)
        c[m] = psi / rho
    f[:, 6] = np.clip(phi, 0.0, 1.0)
    f[:, 7] = c * dx / L
    f[:, 8] = c * dy / L
    f[:, 9] = G["eb"] / G["ea"] if G["ea"] > 0 else 1.0
    return f


def guess(y, G, kind, g):
    """Displacement guess from the network outputs y (n x 3)."""
    u = np.empty((y.shape[0], 2))
    px, py = G["L"] * y[:, 1], G["L"] * y[:, 2]
    u[:, 0] = G["tx"] * y[:, 0] + G["m11"] * px + G["m12"] * py
    u[:, 1] = G["ty"] * y[:, 0] + G["m21"] * px + G["m22"] * py
    fixed = kind > 0
    u[fixed] = g[fixed]
    return u


def edges(x, y, ptr, nbr, L):
    """Edge list (i, j) in CSR order and their features."""
    deg = np.diff(ptr)
    i = np.repeat(np.arange(ptr.size - 1), deg)
    j = nbr
    ddx, ddy = x[j] - x[i], y[j] - y[i]
    ln = np.hypot(ddx, ddy)
    e = np.stack([ddx / ln, ddy / ln, np.log(ln / L)], 1)
    return i, j, e, deg


def relu(a):
    return np.maximum(a, 0.0)


def forward(w, f, i, j, e, deg, keep=False):
    P = unpack(w.astype(np.float64))
    n = f.shape[0]
    a0 = f @ P["W_in"].T + P["b_in"]
    h = relu(a0)
    cache = {"a0": a0, "f": f, "layers": []}
    invdeg = 1.0 / np.maximum(deg, 1)
    for l in range(LAYERS):
        A, B, C, c, U, u = (P[f"{k}{l}"] for k in "ABCcUu")
        PA, QB = h @ A.T, h @ B.T
        z = PA[i] + QB[j] + e @ C.T + c
        agg = np.zeros((n, HID))
        np.add.at(agg, i, relu(z))
        agg *= invdeg[:, None]
        hc = np.concatenate([h, agg], 1)
        v = hc @ U.T + u
        cache["layers"].append({"h": h, "z": z, "agg": agg, "hc": hc, "v": v})
        h = h + relu(v)
    y = h @ P["W_out"].T + P["b_out"]
    cache["hL"] = h
    return (y, cache) if keep else y


def loss_and_grad(w, f, i, j, e, deg, target, free):
    """Loss (mean over free nodes of |y - target|^2) and its gradient w.r.t. the packed
    parameters (float64)."""
    P = unpack(w.astype(np.float64))
    y, cache = forward(w, f, i, j, e, deg, keep=True)
    nf = max(int(free.sum()), 1)
    diff = (y - target) * free[:, None]
    loss = float((diff ** 2).sum() / nf)
    dy = 2.0 * diff / nf
    G = {k: np.zeros_like(v) for k, v in P.items()}
    G["W_out"] = dy.T @ cache["hL"]
    G["b_out"] = dy.sum(0)
    dh = dy @ P["W_out"]
    n = f.shape[0]
    invdeg = 1.0 / np.maximum(deg, 1)
    for l in reversed(range(LAYERS)):
        A, B, C, c, U, u = (P[f"{k}{l}"] for k in "ABCcUu")
        L_ = cache["layers"][l]
        dv = dh * (L_["v"] > 0)
        G[f"U{l}"] = dv.T @ L_["hc"]
        G[f"u{l}"] = dv.sum(0)
        dhc = dv @ U
        dh = dh + dhc[:, :HID]
        dagg = dhc[:, HID:] * invdeg[:, None]
        dz = dagg[i] * (L_["z"] > 0)
        G[f"C{l}"] = dz.T @ e
        G[f"c{l}"] = dz.sum(0)
        dPA = np.zeros((n, HID))
        np.add.at(dPA, i, dz)
        dQB = np.zeros((n, HID))
        np.add.at(dQB, j, dz)
        G[f"A{l}"] = dPA.T @ L_["h"]
        G[f"B{l}"] = dQB.T @ L_["h"]
        dh = dh + dPA @ A + dQB @ B
    da0 = dh * (cache["a0"] > 0)
    G["W_in"] = da0.T @ f
    G["b_in"] = da0.sum(0)
    return loss, pack(G)


def adam(w, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (t counts from 1), float32 like the CUDA kernel."""
    w, g, m, v = (a.astype(np.float32) for a in (w, g, m, v))
    one, b1, b2 = np.float32(1), np.float32(b1), np.float32(b2)
    m = b1 * m + (one - b1) * g
    v = b2 * v + (one - b2) * g * g
    mh = m / (one - b1 ** np.float32(t))
    vh = v / (one - b2 ** np.float32(t))
    w = w - np.float32(lr) * mh / (np.sqrt(vh) + np.float32(eps))
    return w, m, v

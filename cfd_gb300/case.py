"""Cases in the reference's own data model and file formats.

* `Case` holds what readInputData + loadMeshData leave in the InputData/MeshData modules
  (dataLoader.f90:5-91): derived parameters, the mesh, and the boundary-condition lists.
* `read_case` / `write_case` speak the reference's files: EULER.DAT (the case name),
  `<name>-1.dat` (parameters, dataLoader.f90:26-56) and `<name>.dat` (mesh and BC sets,
  dataLoader.f90:98-268), so reference runs and cfd_gb300 runs can swap inputs.  Options
  the reference hard-codes (motion law, mass update, guess) go to `<name>-gb300.json`.
* `ogrid_case` generates the seeded synthetic O-grids used for every workload: a body
  ring (cylinder or ellipse), geometric radial spacing, quads split into two triangles
  along alternating diagonals, interior jitter of +-10% of the local spacing.
"""
import dataclasses
import json
import math
import os
from typing import Dict, Optional

import numpy as np

from . import abi

I32 = np.int32
F64 = np.float64


@dataclasses.dataclass
class Params:
    """InputData (dataLoader.f90:5-15) after readInputData (:58-64) + build options."""
    irestart: int = 0
    maxiter: int = 1
    iprint: int = 100
    movie: int = 0
    itlocal: int = 0
    fsafe: float = 0.5
    u_inf: float = 0.0
    v_inf: float = 0.0
    mach_inf: float = 0.3
    t_inf: float = 288.15
    rho_inf: float = 1.0
    p_inf: float = 0.0
    c_inf: float = 0.0
    fmu: float = 0.017
    fgx: float = 0.0
    fgy: float = 0.0
    qh: float = 0.0
    fk: float = 0.0
    fr: float = 0.0
    fcv: float = 0.0
    gama: float = 1.4
    ngas: int = 0
    cte: float = 1.0          # as stored: 1/CTE of the file (dataLoader.f90:59)
    moving: int = 0
    xref: tuple = (0.0,) * 10
    yref: tuple = (0.0,) * 10
    # build-side options (hard-coded in the reference)
    motion_law: int = abi.CFD_MOTION_HARMONIC
    heave_amp: float = 0.0
    pitch_amp: float = 0.0
    motion_freq: float = 0.0
    mass_mode: int = abi.CFD_MASS_MASAS
    guess_mode: int = abi.CFD_GUESS_PREVIOUS
    bicg_tol: float = 1.0e-10
    bicg_maxit: int = 1000
    estab_mode: int = abi.CFD_ESTAB_REFERENCE
    bicg_tol_mode: int = abi.CFD_BICG_TOL_ABS

    def to_c(self) -> abi.CfdParams:
        p = abi.CfdParams()
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if f.name in ("xref", "yref"):
                setattr(p, f.name, (abi.C.c_double * 10)(*[float(x) for x in v]))
            else:
                setattr(p, f.name, v)
        return p

    def gas6(self) -> np.ndarray:
        """{FCV, FK, FMU, GAMA, T_inf, CTE} as calcRHS.f90:5 imports them."""
        return np.array([self.fcv, self.fk, self.fmu, self.gama, self.t_inf, self.cte], F64)


@dataclasses.dataclass
class Case:
    name: str
    params: Params
    x: np.ndarray                  # (npoin,)
    y: np.ndarray
    inpoel: np.ndarray             # (nelem, 3) int32, 1-based  == Fortran inpoel(3,nelem)
    ifixrho_node: np.ndarray
    rfixrho_value: np.ndarray      # final values (after dataLoader.f90:136-140)
    ifixv_node: np.ndarray         # inflow entries then no-slip entries (:149-176)
    rfixv_valuex: np.ndarray
    rfixv_valuey: np.ndarray
    ifixt_node: np.ndarray         # no-slip T_wall entries then file entries (:161-198)
    rfixt_value: np.ndarray
    wall: np.ndarray               # (nwall, 2)
    iset_entries: np.ndarray       # (nsets, 4): NELE_SET, ISET1, ISET2, ISETNUMB (:208-215)
    i_m: np.ndarray                # moving nodes
    ifm: np.ndarray                # fixed-movement nodes
    nfixvi: int = 0                # inflow entries at the head of ifixv_node
    nfixt_file: int = 0            # file fixed-T entries at the tail of ifixt_node
    meta: Dict = dataclasses.field(default_factory=dict)

    @property
    def npoin(self):
        return int(self.x.shape[0])

    @property
    def nelem(self):
        return int(self.inpoel.shape[0])

    def ilaux(self):
        return np.concatenate([self.i_m, self.ifm]).astype(I32)

    def iset_array(self):
        """ISET(3,10,nsets), IELEM_SETS(10), NSET_NUMB as loadMeshData builds them."""
        nsets = max(1, int(self.iset_entries.shape[0]))
        iset = np.zeros((nsets, 10, 3), I32)  # C order of Fortran ISET(3,10,nsets)
        ielem_sets = np.zeros(10, I32)
        nset_numb = 0
        for nele, n1, n2, sn in self.iset_entries:
            nset_numb = max(nset_numb, int(sn))
            ielem_sets[sn - 1] += 1
            k = ielem_sets[sn - 1] - 1
            iset[k, sn - 1, :] = (n1, n2, nele)
        return iset, ielem_sets, nset_numb

    def to_c(self):
        """(CfdMesh, keepalive) — the struct points into arrays held by keepalive."""
        keep = {}

        def arr(name, a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            keep[name] = a
            return a

        m = abi.CfdMesh()
        m.npoin, m.nelem = self.npoin, self.nelem
        m.inpoel = abi.iptr(arr("inpoel", self.inpoel, I32))
        m.x = abi.dptr(arr("x", self.x, F64))
        m.y = abi.dptr(arr("y", self.y, F64))
        m.nfixrho = len(self.ifixrho_node)
        m.ifixrho_node = abi.iptr(arr("ifr", self.ifixrho_node, I32))
        m.rfixrho_value = abi.dptr(arr("rfr", self.rfixrho_value, F64))
        m.nfixv = len(self.ifixv_node)
        m.ifixv_node = abi.iptr(arr("ifv", self.ifixv_node, I32))
        m.rfixv_valuex = abi.dptr(arr("rfvx", self.rfixv_valuex, F64))
        m.rfixv_valuey = abi.dptr(arr("rfvy", self.rfixv_valuey, F64))
        m.nfixt = len(self.ifixt_node)
        m.ifixt_node = abi.iptr(arr("ift", self.ifixt_node, I32))
        m.rfixt_value = abi.dptr(arr("rft", self.rfixt_value, F64))
        m.nwall = len(self.wall)
        m.wall = abi.iptr(arr("wall", self.wall, I32))
        iset, ielem_sets, nset_numb = self.iset_array()
        m.nsets = iset.shape[0]
        m.nset_numb = nset_numb
        for i in range(10):
            m.ielem_sets[i] = int(ielem_sets[i])
        m.iset = abi.iptr(arr("iset", iset, I32))
        m.nmove, m.nfix_move = len(self.i_m), len(self.ifm)
        m.ilaux = abi.iptr(arr("ilaux", self.ilaux(), I32))
        return m, keep


# ----------------------------------------------------------------------------- flow setup
def flow_params(mach: float, re: float, aoa_deg: float = 0.0, fmu: float = 0.017,
                rho_inf: float = 1.0, t_inf: float = 288.15, gama: float = 1.4,
                pr: float = 0.72, length: float = 1.0, **kw) -> Params:
    """Perfect-gas non-dimensionalisation with FMU=0.017, rho_inf=1, D=1, so that the
    hard-coded mu=0.017*Sutherland of deltat/ESTAB (subrutinas.f90:195-197, :399-400)
    matches calcRHS's FMU.  U_inf = Re*FMU/(rho*D); FR = U^2/(M^2*gama*T_inf)."""
    u = re * fmu / (rho_inf * length)
    fr = u * u / (mach * mach * gama * t_inf)
    fcv = fr / (gama - 1.0)
    fk = fmu * gama * fcv / pr
    a = math.radians(aoa_deg)
    p = Params(u_inf=u * math.cos(a), v_inf=u * math.sin(a), mach_inf=mach, t_inf=t_inf,
               rho_inf=rho_inf, fmu=fmu, fk=fk, fr=fr, fcv=fcv, gama=gama, **kw)
    derive(p)
    return p


def derive(p: Params) -> Params:
    """readInputData's derivations (dataLoader.f90:58-64), with CTE already inverted."""
    if p.t_inf == 0.0:
        p.t_inf = p.p_inf / (p.fr * p.rho_inf)
    if p.p_inf == 0.0:
        p.p_inf = p.rho_inf * p.fr * p.t_inf
    if p.rho_inf == 0.0:
        p.rho_inf = p.p_inf / (p.fr * p.t_inf)
    p.c_inf = math.sqrt(p.gama * p.fr * p.t_inf)
    if math.sqrt(p.u_inf ** 2 + p.v_inf ** 2) == 0.0:
        p.u_inf = p.c_inf * p.mach_inf
    return p


# ----------------------------------------------------------------------------- O-grid
def _geometric_ratio(n_int: int, span: float, first: float) -> float:
    """q with first*(q^n - 1)/(q - 1) = span (bisection)."""
    if abs(first * n_int - span) < 1e-12 * span:
        return 1.0
    lo, hi = 1.0 + 1e-12, 2.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        try:
            s = first * (mid ** n_int - 1.0) / (mid - 1.0)
        except OverflowError:  # mid^n beyond the double range: far above the span
            s = float("inf")
        if s > span:
            hi = mid
        else:
            lo = mid
    return 0.5 * (lo + hi)


def ogrid_case(name: str, nr: int, ntheta: int, params: Params, body: str = "cylinder",
               r_body: float = 0.5, semi_b: float = 0.06, incidence_deg: float = 0.0,
               r_out: float = 20.0, ratio: Optional[float] = None, jitter: float = 0.1,
               seed: int = 0) -> Case:
    """Seeded O-grid around a cylinder (radius r_body) or an ellipse (semi-axes r_body,
    semi_b), out to a circle of radius r_out.  Node (i, j) -> 1 + i*ntheta + j with i the
    ring (0 = body).  With ratio None the geometric ratio makes the first radial spacing
    equal the mean body arc spacing, and is recorded in meta."""
    assert ntheta % 2 == 0 and nr >= 3
    th = 2.0 * np.pi * np.arange(ntheta) / ntheta
    if body == "cylinder":
        bx, by = r_body * np.cos(th), r_body * np.sin(th)
    elif body == "ellipse":
        ex, ey = r_body * np.cos(th), semi_b * np.sin(th)
        inc = math.radians(incidence_deg)  # nose-up incidence: rotate the body by -inc
        bx = ex * math.cos(-inc) - ey * math.sin(-inc)
        by = ex * math.sin(-inc) + ey * math.cos(-inc)
    else:
        raise ValueError(body)
    ox, oy = r_out * np.cos(th), r_out * np.sin(th)
    arc = np.hypot(np.roll(bx, -1) - bx, np.roll(by, -1) - by)
    span = r_out - float(np.mean(np.hypot(bx, by)))
    if ratio is None:
        first = float(np.mean(arc))
        ratio = _geometric_ratio(nr - 1, span, first)
    # s_i in [0, 1]: geometric increments
    inc_ = ratio ** np.arange(nr - 1)
    s = np.concatenate([[0.0], np.cumsum(inc_)])
    s /= s[-1]
    X = bx[None, :] + s[:, None] * (ox - bx)[None, :]
    Y = by[None, :] + s[:, None] * (oy - by)[None, :]
    rng = np.random.default_rng(seed)
    if jitter > 0 and nr > 2:
        # local spacings of interior nodes: along the radial line and along the ring
        dr = np.minimum(np.hypot(X[2:] - X[1:-1], Y[2:] - Y[1:-1]),
                        np.hypot(X[1:-1] - X[:-2], Y[1:-1] - Y[:-2]))
        xi, yi = X[1:-1], Y[1:-1]
        dt = np.minimum(np.hypot(np.roll(xi, -1, 1) - xi, np.roll(yi, -1, 1) - yi),
                        np.hypot(xi - np.roll(xi, 1, 1), yi - np.roll(yi, 1, 1)))
        erx, ery = X[2:] - X[:-2], Y[2:] - Y[:-2]
        n = np.hypot(erx, ery)
        erx, ery = erx / n, ery / n
        etx, ety = -ery, erx
        a = rng.uniform(-jitter, jitter, size=xi.shape) * dr
        b = rng.uniform(-jitter, jitter, size=xi.shape) * dt
        X[1:-1] = xi + a * erx + b * etx
        Y[1:-1] = yi + a * ery + b * ety
    x = X.reshape(-1).astype(F64)
    y = Y.reshape(-1).astype(F64)
    # triangles: quad a=(i,j) b=(i,j+1) c=(i+1,j+1) d=(i+1,j), counter-clockwise
    i = np.arange(nr - 1)[:, None]
    j = np.arange(ntheta)[None, :]
    jp = (j + 1) % ntheta
    a = 1 + i * ntheta + j
    b = 1 + i * ntheta + jp
    c = 1 + (i + 1) * ntheta + jp
    d = 1 + (i + 1) * ntheta + j
    even = ((i + j) % 2 == 0)
    t1 = np.where(even[..., None], np.stack([a, d, c], -1), np.stack([a, d, b], -1))
    t2 = np.where(even[..., None], np.stack([a, c, b], -1), np.stack([d, c, b], -1))
    inpoel = np.stack([t1, t2], axis=2).reshape(-1, 3).astype(I32)
    # boundary sets
    body_nodes = (1 + np.arange(ntheta)).astype(I32)
    outer_nodes = (1 + (nr - 1) * ntheta + np.arange(ntheta)).astype(I32)
    # body edges clockwise (fluid on the left): node j+1 -> node j
    e1 = (1 + (np.arange(ntheta) + 1) % ntheta).astype(I32)
    e2 = (1 + np.arange(ntheta)).astype(I32)
    wall = np.stack([e1, e2], 1).astype(I32)
    # element of each body edge: ring-0 quad j holds the edge (a=(0,j), b=(0,j+1))
    jj = np.arange(ntheta)
    even0 = (jj % 2 == 0)
    elem_t2 = 1 + 2 * jj + 1  # second triangle (a,c,b) holds a-b when even
    elem_t1 = 1 + 2 * jj      # first triangle (a,d,b) holds a-b when odd
    owner = np.where(even0, elem_t2, elem_t1).astype(I32)
    iset_entries = np.stack([owner, e1, e2, np.ones(ntheta, I32)], 1).astype(I32)
    p = params
    twall = p.t_inf * (1.0 + (p.gama - 1) / 2.0 * p.mach_inf * p.mach_inf)
    case = Case(
        name=name, params=p, x=x, y=y, inpoel=inpoel,
        ifixrho_node=outer_nodes.copy(), rfixrho_value=np.full(ntheta, 1.0 * p.rho_inf),
        ifixv_node=np.concatenate([outer_nodes, body_nodes]).astype(I32),
        rfixv_valuex=np.concatenate([np.full(ntheta, 1.0 * p.u_inf), np.zeros(ntheta)]),
        rfixv_valuey=np.concatenate([np.full(ntheta, 1.0 * p.v_inf), np.zeros(ntheta)]),
        ifixt_node=np.concatenate([body_nodes, outer_nodes]).astype(I32),
        rfixt_value=np.concatenate([np.full(ntheta, twall), np.full(ntheta, 1.0 * p.t_inf)]),
        wall=wall, iset_entries=iset_entries, i_m=body_nodes.copy(), ifm=outer_nodes.copy(),
        nfixvi=ntheta, nfixt_file=ntheta,
        meta=dict(generator="ogrid", nr=nr, ntheta=ntheta, body=body, r_body=r_body,
                  semi_b=semi_b, incidence_deg=incidence_deg, r_out=r_out,
                  ratio=float(ratio), jitter=jitter, seed=seed))
    return case


# ----------------------------------------------------------------------------- workloads
def config_case(which: int, scale: Optional[int] = None, seed: int = 0) -> Case:
    """The synthetic workloads (1: cylinder 64x128 fixed; 2: cylinder 512x512 heave;
    3: ellipse 1024x1024 Mach 0.8 heave; 5: ellipse 2048x2048 heave+pitch).  `scale`
    replaces the node counts (nr = ntheta = scale) for reduced-size tests."""
    if which == 1:
        p = flow_params(0.3, 100.0, maxiter=2000, moving=0,
                        motion_law=abi.CFD_MOTION_HARMONIC)
        nr, nt = (64, 128) if scale is None else (scale, 2 * scale)
        return ogrid_case("cylinder_8k", nr, nt, p, "cylinder", r_out=20.0,
                          ratio=1.05 if scale is None else None, seed=seed)
    if which == 2:
        p = flow_params(0.3, 200.0, maxiter=5000, moving=1, motion_law=abi.CFD_MOTION_HARMONIC,
                        heave_amp=0.2, motion_freq=0.2, mass_mode=abi.CFD_MASS_GCL_CORRECTED)
        n = 512 if scale is None else scale
        return ogrid_case("cylinder_262k_ale", n, n, p, "cylinder", r_out=20.0, seed=seed)
    if which == 3:
        # FSAFE 0.25: deltat has no acoustic limit (subrutinas.f90:179, 199-206) and the
        # impulsive Mach 0.8 start diverges within ~20 steps at FSAFE 0.5
        p = flow_params(0.8, 5000.0, aoa_deg=0.0, maxiter=2000, moving=1, fsafe=0.25,
                        motion_law=abi.CFD_MOTION_HARMONIC, heave_amp=0.05, motion_freq=0.1,
                        mass_mode=abi.CFD_MASS_GCL_CORRECTED)
        n = 1024 if scale is None else scale
        return ogrid_case("ellipse_1M", n, n, p, "ellipse", incidence_deg=2.0, r_out=30.0,
                          seed=seed)
    if which == 5:
        p = flow_params(0.8, 10000.0, maxiter=10000, moving=1, fsafe=0.25,
                        motion_law=abi.CFD_MOTION_HARMONIC, heave_amp=0.05,
                        pitch_amp=math.radians(3.0), motion_freq=0.1,
                        mass_mode=abi.CFD_MASS_GCL_CORRECTED)
        n = 2048 if scale is None else scale
        return ogrid_case("ellipse_4M", n, n, p, "ellipse", incidence_deg=2.0, r_out=30.0,
                          seed=seed)
    raise ValueError(which)


# ----------------------------------------------------------------------------- file I/O
_BUILD_KEYS = ("motion_law", "heave_amp", "pitch_amp", "motion_freq", "mass_mode",
               "guess_mode", "bicg_tol", "bicg_maxit", "estab_mode", "bicg_tol_mode")


def _fmt(v):
    return repr(float(v)).replace("e", "D") if isinstance(v, float) else str(v)


def write_case(case: Case, directory: str) -> None:
    """EULER.DAT, <name>-1.dat and <name>.dat in the reference's formats."""
    os.makedirs(directory, exist_ok=True)
    p = case.params
    with open(os.path.join(directory, "EULER.DAT"), "w") as f:
        f.write(case.name + "\n")
    L = [
        "IRESTART MAXITER IPRINT MOVIE ITLOCAL",
        f"{p.irestart} {p.maxiter} {p.iprint} {p.movie} {p.itlocal}",
        "FSAFE U_inf V_inf MACH_inf T_inf RHO_inf P_inf",
        " ".join(_fmt(float(v)) for v in (p.fsafe, p.u_inf, p.v_inf, p.mach_inf, p.t_inf,
                                         p.rho_inf, p.p_inf)),
        "FMU FGX FGY QH",
        " ".join(_fmt(float(v)) for v in (p.fmu, p.fgx, p.fgy, p.qh)),
        "FK FR FCv GAMA NGAS",
        " ".join(_fmt(float(v)) for v in (p.fk, p.fr, p.fcv, p.gama)) + f" {p.ngas}",
        "CTE (shock capturing)",
        _fmt(1.0 / p.cte),
        "ALE",
        "MOVING XREF YREF",
        f"{p.moving} {_fmt(float(p.xref[0]))} {_fmt(float(p.yref[0]))}",
        "OUTPUT",
        "RHO VEL2 MACH PRES TEMP ENER POS",
        ".si. .si. .si. .si. .si. .si. .si.",
        "REFINEMENT", "-", "-",
        "ETA_REFIN HHMAX_REFIN HHMIN_REFIN",
        "0.0 1.0 0.01",
    ]
    with open(os.path.join(directory, case.name + "-1.dat"), "w") as f:
        f.write("\n".join(L) + "\n")
    with open(os.path.join(directory, case.name + "-gb300.json"), "w") as f:
        json.dump({k: getattr(p, k) for k in _BUILD_KEYS} | {"meta": case.meta}, f, indent=1)
    nfv = case.nfixvi
    nnoslip = len(case.ifixv_node) - nfv
    nft_file = case.nfixt_file
    with open(os.path.join(directory, case.name + ".dat"), "w") as f:
        w = f.write
        w("NPOIN NELEM\n")
        w(f"{case.npoin} {case.nelem}\n")
        w("NFIXRHO NFIXVI NFIXV NWALL NFIXT NSETS NMASTER NSLAVE NFIX_MOVE NMOVE\n")
        w(f"{len(case.ifixrho_node)} {nfv} {nnoslip} {len(case.wall)} {nft_file} "
          f"{len(case.iset_entries)} 0 0 {len(case.ifm)} {len(case.i_m)}\n")
        w("-\n-\n-\nCOORDINATES\n")
        idx = np.arange(1, case.npoin + 1)
        w("".join(f"{i} {a!r} {b!r}\n" for i, a, b in zip(idx, case.x.tolist(), case.y.tolist())))
        w("ELEMENTS\n")
        w("".join(f"{k} {a} {b} {c}\n" for k, (a, b, c) in
                  zip(range(1, case.nelem + 1), case.inpoel.tolist())))
        w("FIX RHO\n")
        rr = [v / p.rho_inf for v in case.rfixrho_value.tolist()]
        w("".join(f"{n} {v!r}\n" for n, v in zip(case.ifixrho_node.tolist(), rr)))
        w("FIX VEL INFLOW\n")
        fx = [v / p.u_inf if p.u_inf != 0 else 1.0 for v in case.rfixv_valuex[:nfv].tolist()]
        fy = [v / p.v_inf if p.v_inf != 0 else 1.0 for v in case.rfixv_valuey[:nfv].tolist()]
        w("".join(f"{n} {a!r} {b!r}\n" for n, a, b in
                  zip(case.ifixv_node[:nfv].tolist(), fx, fy)))
        w("FIX VEL NO SLIP\n")
        w("".join(f"{n} 0.0 0.0\n" for n in case.ifixv_node[nfv:].tolist()))
        w("WALL\n")
        w("".join(f"{a} {b}\n" for a, b in case.wall.tolist()))
        w("FIX T\n")
        tail = len(case.ifixt_node) - nft_file
        w("".join(f"{n} {v / p.t_inf!r}\n" for n, v in
                  zip(case.ifixt_node[tail:].tolist(), case.rfixt_value[tail:].tolist())))
        w("SETS\n")
        w("".join(f"{a} {b} {c} {d}\n" for a, b, c, d in case.iset_entries.tolist()))
        w("PERIODIC MASTER\nPERIODIC SLAVE\n")
        w("FIX MOVE\n")
        w("".join(f"{n} 0\n" for n in case.ifm.tolist()))
        w("MOVE\n")
        w("".join(f"{n} 0\n" for n in case.i_m.tolist()))


class _Lines:
    def __init__(self, path):
        with open(path) as f:
            self.lines = f.read().splitlines()
        self.k = 0

    def skip(self, n=1):
        self.k += n

    def vals(self):
        s = self.lines[self.k]
        self.k += 1
        return s.replace(",", " ").split()

    def block(self, n):
        rows = self.lines[self.k:self.k + n]
        self.k += n
        return rows


def _num(s):
    return float(s.replace("D", "E").replace("d", "e"))


def read_case(directory: str) -> Case:
    """readInputData + loadMeshData (dataLoader.f90:17-275) over the reference files."""
    with open(os.path.join(directory, "EULER.DAT")) as f:
        name = f.readline().strip()
    L = _Lines(os.path.join(directory, name + "-1.dat"))
    p = Params()
    L.skip()
    p.irestart, p.maxiter, p.iprint, p.movie, p.itlocal = [int(v) for v in L.vals()[:5]]
    L.skip()
    p.fsafe, p.u_inf, p.v_inf, p.mach_inf, p.t_inf, p.rho_inf, p.p_inf = \
        [_num(v) for v in L.vals()[:7]]
    L.skip()
    p.fmu, p.fgx, p.fgy, p.qh = [_num(v) for v in L.vals()[:4]]
    L.skip()
    v = L.vals()
    p.fk, p.fr, p.fcv, p.gama = [_num(x) for x in v[:4]]
    p.ngas = int(v[4])
    L.skip()
    p.cte = 1.0 / _num(L.vals()[0])
    L.skip(2)
    v = L.vals()
    p.moving = int(v[0])
    p.xref = (_num(v[1]),) + (0.0,) * 9
    p.yref = (_num(v[2]),) + (0.0,) * 9
    derive(p)
    side = os.path.join(directory, name + "-gb300.json")
    meta = {}
    if os.path.exists(side):
        with open(side) as f:
            d = json.load(f)
        meta = d.pop("meta", {})
        for k in _BUILD_KEYS:
            if k in d:
                setattr(p, k, d[k])
    M = _Lines(os.path.join(directory, name + ".dat"))
    M.skip()
    npoin, nelem = [int(v) for v in M.vals()[:2]]
    M.skip()
    (nfixrho, nfixvi, nfixv, nwall, nfixt, nsets, nmaster, nslave, nfix_move,
     nmove) = [int(v) for v in M.vals()[:10]]
    M.skip(4)

    def table(n, ncol, conv=float):
        if n == 0:
            return np.zeros((0, ncol))
        txt = " ".join(M.block(n)).replace("D", "E").replace("d", "e")
        a = np.array(txt.split(), dtype=np.float64)
        return a.reshape(n, -1)[:, :ncol]

    co = table(npoin, 3)
    x = np.zeros(npoin)
    y = np.zeros(npoin)
    ii = co[:, 0].astype(np.int64) - 1
    x[ii], y[ii] = co[:, 1], co[:, 2]
    M.skip()
    el = table(nelem, 4).astype(np.int64)
    inpoel = np.zeros((nelem, 3), I32)
    inpoel[el[:, 0] - 1] = el[:, 1:4]
    M.skip()
    fr = table(nfixrho, 2)
    ifixrho = fr[:, 0].astype(I32)
    rfixrho = np.where(fr[:, 1] < 0, 1.225, fr[:, 1] * p.rho_inf)
    M.skip()
    fvi = table(nfixvi, 3)
    M.skip()
    fvn = table(nfixv, 3)
    twall = p.t_inf * (1.0 + (p.gama - 1) / 2.0 * p.mach_inf * p.mach_inf)
    ifixv = np.concatenate([fvi[:, 0], fvn[:, 0]]).astype(I32)
    rvx = np.concatenate([fvi[:, 1] * p.u_inf, np.zeros(nfixv)])
    rvy = np.concatenate([fvi[:, 2] * p.v_inf, np.zeros(nfixv)])
    M.skip()
    wall = table(nwall, 2).astype(I32)
    M.skip()
    ft = table(nfixt, 2)
    ifixt = np.concatenate([fvn[:, 0], ft[:, 0]]).astype(I32)
    rfixt = np.concatenate([np.full(nfixv, twall), ft[:, 1] * p.t_inf])
    M.skip()
    sets = table(nsets, 4).astype(I32)
    M.skip()
    M.block(nmaster)
    M.skip()
    M.block(nmaster)
    M.skip()
    ifm = table(nfix_move, 1)[:, 0].astype(I32)
    M.skip()
    i_m = table(nmove, 1)[:, 0].astype(I32)
    return Case(name=name, params=p, x=x, y=y, inpoel=inpoel, ifixrho_node=ifixrho,
                rfixrho_value=rfixrho, ifixv_node=ifixv, rfixv_valuex=rvx,
                rfixv_valuey=rvy, ifixt_node=ifixt, rfixt_value=rfixt, wall=wall,
                iset_entries=sets, i_m=i_m, ifm=ifm, nfixvi=nfixvi, nfixt_file=nfixt,
                meta=meta)


def main(argv=None):
    """Command line: write one of the synthetic workloads as a case directory in the
    reference's input formats."""
    import argparse
    ap = argparse.ArgumentParser(description="Write a synthetic workload as a case directory "
                                 "(EULER.DAT, <name>-1.dat, <name>.dat).")
    ap.add_argument("directory")
    ap.add_argument("--config", type=int, default=3, choices=(1, 2, 3, 5),
                    help="1: cylinder 64x128 fixed; 2: cylinder 512x512 heave; 3: ellipse "
                         "1024x1024 Mach 0.8 heave; 5: ellipse 2048x2048 heave + pitch")
    ap.add_argument("--scale", type=int, default=None,
                    help="nodes per direction instead of the workload's")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--maxiter", type=int, default=None)
    a = ap.parse_args(argv)
    c = config_case(a.config, scale=a.scale, seed=a.seed)
    if a.maxiter is not None:
        c.params.maxiter = a.maxiter
    write_case(c, a.directory)
    print(f"{a.directory}: {c.name}, {c.npoin} nodes, {c.nelem} triangles")


if __name__ == "__main__":
    main()

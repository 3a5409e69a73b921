"""ctypes wrapper of the oracle library (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg; never by the
cfd_gb300 product path.  See cfd_oracle.h for what the oracle restates and how.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from cfd_gb300 import abi  # noqa: E402  (ctypes struct types only)

from . import build_oracle  # noqa: E402

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p
_d, _i = C.c_double, C.c_int

_SIG = {
    "or_set_threads": (None, [_i]),
    "or_set_ordered_scatter": (None, [_i]),
    "or_set_estab_mode": (None, [_i]),
    "or_set_estab_eps": (None, [_d]),
    "or_get_threads": (_i, []),
    "or_deriv": (None, [_i, _i, _dp, _dp, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "or_masas": (None, [_i, _i, _dp, _ip, _dp]),
    "or_deltat": (None, [_i, _i, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _d, _d, _d, _d, _dp, _dp]),
    "or_estab": (None, [_i, _i, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _d, _d, _d,
                        _d, _d, _dp, _dp, _dp, _dp]),
    "or_calcrhs": (None, [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _i, _i,
                          _dp, _dp]),
    "or_fuente": (None, [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _i, _i]),
    "or_gcl": (None, [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _i, _i, _d, _i]),
    "or_get_esup": (_i, [_ip, _i, _i, _ip, _ip]),
    "or_get_psup": (_i, [_ip, _i, _i, _ip, _ip, _ip]),
    "or_laplace_pattern": (_i, [_ip, _i, _i, _ip, _ip, _ip]),
    "or_laplace": (None, [_ip, _dp, _dp, _i, _i, _dp, _dp, _ip, _ip, _dp, _ip, _ip, _dp]),
    "or_vecdot": (_d, [_i, _dp, _dp]),
    "or_bicg": (None, [_dp, _ip, _ip, _dp, _dp, _dp, _dp, _ip, _i, _i, _d, _i,
                       C.POINTER(abi.CfdSolveInfo)]),
    "or_set_pow_mode": (None, [_i]),
    "or_get_pow_mode": (_i, []),
    "or_pow_census": (None, [_i, _dp, C.POINTER(C.c_longlong)]),
    "or_bicg_mode": (None, [_dp, _ip, _ip, _dp, _dp, _dp, _dp, _ip, _i, _i, _d, _i, _i,
                            C.POINTER(abi.CfdSolveInfo)]),
    "or_normales": (_i, [_i, _i, _ip, _dp, _dp, _ip, _dp, _dp]),
    "or_smoothing": (None, [_dp, _dp, _ip, _ip, _i, _i, _ip, _dp]),
    "or_smoothing_ordered": (None, [_dp, _dp, _ip, _ip, _i, _i, _ip, _dp, _ip, _dp]),
    "or_newmark_step": (None, [C.c_double, _dp, _dp, _dp, _dp]),
    "or_force_visc": (None, [_i, _i, _i, _ip, _ip, _ip, _i, C.c_double, C.c_double, C.c_double,
                             C.c_double, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                             _dp]),
    "or_case_force_visc": (None, [_vp, _dp, _dp, _dp]),
    "or_case_set_force_visc": (None, [_vp, _i]),
    "or_case_set_smoothing": (None, [_vp, _i, _ip]),
    "or_case_create": (_vp, [C.POINTER(abi.CfdMesh), C.POINTER(abi.CfdParams), _i]),
    "or_case_destroy": (None, [_vp]),
    "or_case_step": (_i, [_vp, _i, C.POINTER(abi.CfdStepReport)]),
    "or_case_get": (None, [_vp, _dp, _dp, _dp, _dp]),
    "or_case_get_fields": (None, [_vp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "or_case_get_motion": (None, [_vp, _dp, _dp]),
    "or_case_get_geometry": (None, [_vp, _dp, _dp, _dp, _dp]),
    "or_case_set_state": (None, [_vp, _dp, _dp, _dp, _dp]),
    "or_case_set_mesh": (None, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "or_case_set_clock": (None, [_vp, _i, _d, _d, _i, _d, _d]),
    "or_case_timers": (None, [_vp, _dp, _i, _ip]),
}

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        for k, (r, a) in _SIG.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        # one thread by default: the element order of the serial loops (the parity
        # order); the CPU baseline raises it with set_threads()
        L.or_set_threads(1)
        _LIB = L
    return _LIB


dp, ip = abi.dptr, abi.iptr


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def set_threads(n):
    lib().or_set_threads(int(n))


def set_ordered_scatter(on):
    """True: calcRHS/FUENTE add their element rows in element order at any thread count
    (the one-thread result); False (default): OpenMP atomics, as the reference."""
    lib().or_set_ordered_scatter(1 if on else 0)


def set_pow_mode(mode):
    """0: the compositions x*sqrt(x), 1/sqrt(x), sqrt(x) (the GPU's); 1: the C library's
    pow for x**1.5d0, x**(-.5d0), x**.5d0 (a Fortran build without unsafe math)."""
    lib().or_set_pow_mode(int(mode))


def get_pow_mode():
    return lib().or_get_pow_mode()


def pow_census(x):
    """(#pow(x,1.5) != x*sqrt(x), #pow(x,-0.5) != 1/sqrt(x), #pow(x,0.5) != sqrt(x))."""
    x = f64(x)
    out = (C.c_longlong * 3)()
    lib().or_pow_census(len(x), dp(x), out)
    return tuple(out)


# ------------------------------------------------------------------ per-routine calls
def deriv(x, y, inpoel):
    x, y, inp = f64(x), f64(y), i32(inpoel)
    ne, n = inp.shape[0], x.shape[0]
    area = np.zeros(ne)
    dnx = np.zeros((ne, 3))
    dny = np.zeros((ne, 3))
    hh, hhx, hhy = np.zeros(ne), np.zeros(ne), np.zeros(ne)
    hmin = C.c_double(0)
    lib().or_deriv(n, ne, dp(x), dp(y), ip(inp), dp(area), dp(dnx), dp(dny), dp(hh), dp(hhx),
                   dp(hhy), C.byref(hmin))
    return dict(area=area, dNx=dnx, dNy=dny, HH=hh, HHX=hhx, HHY=hhy, hmin=hmin.value)


def masas(area, inpoel, npoin):
    M = np.zeros(npoin)
    inp = i32(inpoel)
    lib().or_masas(npoin, inp.shape[0], dp(f64(area)), ip(inp), dp(M))
    return M


def deltat(T, vx, vy, wx, wy, area, inpoel, fsafe, fr, gama, t_inf):
    inp = i32(inpoel)
    dt = np.zeros(inp.shape[0])
    dtmin = C.c_double(0)
    lib().or_deltat(len(T), inp.shape[0], dp(f64(T)), dp(f64(vx)), dp(f64(vy)), dp(f64(wx)),
                    dp(f64(wy)), dp(f64(area)), ip(inp), fsafe, fr, gama, t_inf, dp(dt),
                    C.byref(dtmin))
    return dt, dtmin.value


def estab(U, T, GAMM, vx, vy, wx, wy, dNx, dNy, inpoel, gama, fr, dtmin, rhoinf, tinf):
    inp = i32(inpoel)
    ne = inp.shape[0]
    out = [np.zeros(ne) for _ in range(4)]
    lib().or_estab(len(T), ne, dp(f64(U)), dp(f64(T)), dp(f64(GAMM)), dp(f64(vx)),
                   dp(f64(vy)), dp(f64(wx)), dp(f64(wy)), dp(f64(dNx)), dp(f64(dNy)),
                   ip(inp), gama, fr, dtmin, rhoinf, tinf, *[dp(o) for o in out])
    return out  # SHOC, T_SUGN1, T_SUGN2, T_SUGN3


def calcrhs(rhs, U, theta, dNx, dNy, area, shoc, dtl, ts1, ts2, ts3, inpoel, T, gas6):
    inp = i32(inpoel)
    rhs = f64(rhs).copy()
    lib().or_calcrhs(dp(rhs), dp(f64(U)), dp(f64(theta)), dp(f64(dNx)), dp(f64(dNy)),
                     dp(f64(area)), dp(f64(shoc)), dp(f64(dtl)), dp(f64(ts1)), dp(f64(ts2)),
                     dp(f64(ts3)), ip(inp), inp.shape[0], len(T), dp(f64(T)), dp(f64(gas6)))
    return rhs


def fuente(rhs, U, wx, wy, dNx, dNy, area, dtl, inpoel):
    inp = i32(inpoel)
    rhs = f64(rhs).copy()
    lib().or_fuente(dp(rhs), dp(f64(U)), dp(f64(wx)), dp(f64(wy)), dp(f64(dNx)),
                    dp(f64(dNy)), dp(f64(area)), dp(f64(dtl)), ip(inp), inp.shape[0],
                    len(wx))
    return rhs


def gcl(M, wx, wy, wxo, wyo, dNx, dNy, area, area_old, inpoel, dt, mode):
    inp = i32(inpoel)
    M = f64(M).copy()
    lib().or_gcl(dp(M), dp(f64(wx)), dp(f64(wy)), dp(f64(wxo)), dp(f64(wyo)), dp(f64(dNx)),
                 dp(f64(dNy)), dp(f64(area)), dp(f64(area_old)), ip(inp), inp.shape[0],
                 len(M), float(dt), int(mode))
    return M


def esup(inpoel, npoin):
    inp = i32(inpoel)
    e1 = np.zeros(3 * inp.shape[0], np.int32)
    e2 = np.zeros(npoin + 1, np.int32)
    assert lib().or_get_esup(ip(inp), inp.shape[0], npoin, ip(e1), ip(e2)) == 0
    return e1, e2


def psup(inpoel, npoin):
    inp = i32(inpoel)
    n = C.c_int(0)
    lib().or_get_psup(ip(inp), inp.shape[0], npoin, None, None, C.byref(n))
    p1 = np.zeros(max(n.value, 1), np.int32)
    p2 = np.zeros(npoin + 1, np.int32)
    lib().or_get_psup(ip(inp), inp.shape[0], npoin, ip(p1), ip(p2), None)
    return p1[:n.value], p2


def laplace_pattern(inpoel, npoin):
    inp = i32(inpoel)
    nnz = C.c_int(0)
    lib().or_laplace_pattern(ip(inp), inp.shape[0], npoin, None, None, C.byref(nnz))
    rp = np.zeros(npoin + 1, np.int32)
    idx = np.zeros(nnz.value, np.int32)
    lib().or_laplace_pattern(ip(inp), inp.shape[0], npoin, ip(rp), ip(idx), C.byref(nnz))
    return rp, idx


def laplace(inpoel, dNx, dNy, x, y, rowptr, idx):
    inp = i32(inpoel)
    npoin = len(x)
    e1, e2 = esup(inp, npoin)
    vals = np.zeros(len(idx))
    diag = np.zeros(npoin)
    lib().or_laplace(ip(inp), dp(f64(dNx)), dp(f64(dNy)), inp.shape[0], npoin, dp(f64(x)),
                     dp(f64(y)), ip(e1), ip(e2), dp(vals), ip(i32(idx)), ip(i32(rowptr)),
                     dp(diag))
    return vals, diag


def vecdot(x, y):
    return lib().or_vecdot(len(x), dp(f64(x)), dp(f64(y)))


def bicg(vals, idx, rowptr, diag, x, b, x_fix, fix_idx, tol=1e-10, maxit=1000,
         tol_mode=abi.CFD_BICG_TOL_ABS):
    x = f64(x).copy()
    info = abi.CfdSolveInfo()
    lib().or_bicg_mode(dp(f64(vals)), ip(i32(idx)), ip(i32(rowptr)), dp(f64(diag)), dp(x),
                       dp(f64(b)), dp(f64(x_fix)), ip(i32(fix_idx)), len(x), len(fix_idx), tol,
                       maxit, int(tol_mode), C.byref(info))
    return x, info


def normales(wall, x, y):
    n = len(x)
    w = i32(wall)
    ni = np.zeros(n, np.int32)
    nx, ny = np.zeros(n), np.zeros(n)
    m = lib().or_normales(n, w.shape[0], ip(w), dp(f64(x)), dp(f64(y)), ip(ni), dp(nx), dp(ny))
    return ni[:m], nx[:m], ny[:m]


def smoothing(x, y, inpoel, fixed, order=None, dX=None, dY=None):
    """smoothing.f90:21-72 -> (X, Y, iterations, min quality); `order` (0-based node
    permutation) replaces node order in the Laplacian passes and the sweeps; dX, dY turn on
    the setTol_move path (:372-386) with tol = |dX| + |dY|."""
    x, y = f64(x).copy(), f64(y).copy()
    inp = i32(inpoel)
    it = C.c_int(0)
    q = C.c_double(0)
    if order is None and dX is None:
        lib().or_smoothing(dp(x), dp(y), ip(inp), ip(i32(fixed)), len(x), inp.shape[0],
                           C.byref(it), C.byref(q))
    else:
        tol = None if dX is None else f64(np.abs(f64(dX)) + np.abs(f64(dY)))
        lib().or_smoothing_ordered(dp(x), dp(y), ip(inp), ip(i32(fixed)), len(x), inp.shape[0],
                                   None if order is None else ip(i32(order)),
                                   None if tol is None else dp(tol), C.byref(it), C.byref(q))
    return x, y, it.value, q.value


def colour_order(inpoel, npoin):
    """Nodes by colour of a greedy colouring of the point-neighbour graph in node order (each
    node takes the least colour none of its lower-numbered neighbours has), in node order
    within a colour: the order in which a colour-by-colour smoothing moves them."""
    nbr, ptr = psup(inpoel, npoin)  # 1-based neighbours, 0-based row pointers
    col = np.full(npoin, -1, np.int64)
    for p in range(npoin):
        used = {int(col[q - 1]) for q in nbr[ptr[p]:ptr[p + 1]] if col[q - 1] >= 0}
        c = 0
        while c in used:
            c += 1
        col[p] = c
    return np.argsort(col, kind="stable").astype(np.int32)


def newmark_step(H, F, dis, vel, acc):
    """meshMove.f90 NEWMARK_METHOD(H) with load F; returns the new (dis, vel, acc)."""
    d, v, a = f64(dis).copy(), f64(vel).copy(), f64(acc).copy()
    lib().or_newmark_step(float(H), dp(f64(F)), dp(d), dp(v), dp(a))
    return d, v, a


# ------------------------------------------------------------------ whole driver
class OracleCase:
    """PROGRAM NSComp2D (ns2DComp.ALE.f90:8-282) over a cfd_gb300.case.Case."""

    def __init__(self, case, smoothing=False):
        self.case = case
        self.n, self.ne = case.npoin, case.nelem
        self._mesh, self._keep = case.to_c()
        self._params = case.params.to_c()
        self.h = lib().or_case_create(C.byref(self._mesh), C.byref(self._params),
                                      1 if smoothing else 0)

    def close(self):
        if self.h:
            lib().or_case_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n=1):
        rep = abi.CfdStepReport()
        st = lib().or_case_step(self.h, int(n), C.byref(rep))
        assert st == 0
        return rep

    def state(self):
        U = np.zeros((self.n, 4))
        T, X, Y = np.zeros(self.n), np.zeros(self.n), np.zeros(self.n)
        lib().or_case_get(self.h, dp(U), dp(T), dp(X), dp(Y))
        return dict(U=U, T=T, X=X, Y=Y)

    def fields(self):
        names = ["RHO", "VEL_X", "VEL_Y", "E", "P", "RMACH", "W_X", "W_Y"]
        arrs = [np.zeros(self.n) for _ in names]
        lib().or_case_get_fields(self.h, *[dp(a) for a in arrs])
        return dict(zip(names, arrs))

    def motion(self):
        xp, yp = np.zeros(self.n), np.zeros(self.n)
        lib().or_case_get_motion(self.h, dp(xp), dp(yp))
        return xp, yp

    def set_force_visc(self, each_step):
        lib().or_case_set_force_visc(self.h, 1 if each_step else 0)

    def set_smoothing(self, every, order="colour"):
        """Smooth the moved mesh every `every` steps (setTol_move path); order "colour": the
        GPU's colour order, None: node order, or a 0-based permutation."""
        if isinstance(order, str):
            order = colour_order(self.case.inpoel, self.case.npoin)
        self._sm_order = None if order is None else i32(order)
        lib().or_case_set_smoothing(self.h, int(every),
                                    None if self._sm_order is None else ip(self._sm_order))

    def force_visc(self):
        """FORCE_VISC now: (F_VX[nset_numb], F_VY[nset_numb], skin rows (nedges, 3))."""
        fvx, fvy = np.zeros(10), np.zeros(10)
        ne = int(sum(self.case.iset_array()[1]))
        skin = np.zeros((max(ne, 1), 3))
        lib().or_case_force_visc(self.h, dp(fvx), dp(fvy), dp(skin))
        n = self.case.iset_array()[2]
        return fvx[:n], fvy[:n], skin[:ne]

    def geometry(self):
        a = np.zeros(self.ne)
        dnx, dny = np.zeros((self.ne, 3)), np.zeros((self.ne, 3))
        M = np.zeros(self.n)
        lib().or_case_get_geometry(self.h, dp(a), dp(dnx), dp(dny), dp(M))
        return dict(area=a, dNx=dnx, dNy=dny, M=M)

    def set_state(self, U=None, T=None, VEL_X=None, VEL_Y=None):
        lib().or_case_set_state(self.h, dp(None if U is None else f64(U)),
                                dp(None if T is None else f64(T)),
                                dp(None if VEL_X is None else f64(VEL_X)),
                                dp(None if VEL_Y is None else f64(VEL_Y)))

    def set_mesh(self, X=None, Y=None, W_X=None, W_Y=None, xpos=None, ypos=None):
        conv = [None if a is None else f64(a) for a in (X, Y, W_X, W_Y, xpos, ypos)]
        lib().or_case_set_mesh(self.h, *[dp(a) for a in conv])

    def set_clock(self, iter=0, time=0.0, dtmin1=0.0, bandera=1, disn1=0.0, disn2=0.0):
        lib().or_case_set_clock(self.h, iter, time, dtmin1, bandera, disn1, disn2)

    def timers(self):
        s = np.zeros(16)
        n = C.c_int(0)
        lib().or_case_timers(self.h, dp(s), 16, C.byref(n))
        return s[:n.value]

"""Host-side mirror of the reference's routines and driver over the CUDA library.

Drop-in routines keep the reference's names, argument order, array layout (U(4,npoin) as a
(npoin, 4) C array, dNx(3,nelem) as (nelem, 3), 1-based inpoel) and in/out meaning:

    calcRHS(rhs, U, theta, dNx, dNy, area, shoc, dtl, t_sugn1, t_sugn2, t_sugn3, inpoel,
            nelem, npoin, T, gas)                              calcRHS.f90:4
    FUENTE(rhs, U, W_X, W_Y, dNx, dNy, area, dtl, inpoel)     subrutinas.f90:1036
    ESTAB(...), deltat(...), deriv(...), MASAS(...)            subrutinas.f90:332/155/88/128
    gcl_main(...)                                              gcl.f90:8
    getEsup / getPsup / laplace_pattern / laplace              pointNeighbor.f90, mLaplace.f90
    biCG(spMtx, spIdx, spRowptr, diagMtx, x, b, x_fix, x_fixIdx)  biconjGrad.f90:8

`Solver` is PROGRAM NSComp2D (ns2DComp.ALE.f90:8-282) over a resident GPU context.
Every call runs the sm_103a kernels; a failing status raises abi.CfdError.
"""
import ctypes as C

import numpy as np

from . import abi
from .abi import check, dptr, iptr

_f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
_i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)  # noqa: E731


def _ci(v):
    return C.byref(C.c_int(int(v)))


# ------------------------------------------------------------------ drop-in routines
def calcRHS(rhs, U, theta, dNx, dNy, area, shoc, dtl, t_sugn1, t_sugn2, t_sugn3, inpoel, T,
            gas):
    """rhs += calcRHS contributions (calcRHS.f90:4-154).  gas = {FCV,FK,FMU,GAMA,T_inf,CTE}.
    rhs is updated in place and returned."""
    L = abi.lib()
    inp = _i32(inpoel)
    npoin, nelem = len(T), inp.shape[0]
    assert rhs.dtype == np.float64 and rhs.flags["C_CONTIGUOUS"]
    th = None if theta is None else _f64(theta)
    check(L.cfd_calcrhs(dptr(rhs), dptr(_f64(U)), dptr(th), dptr(_f64(dNx)), dptr(_f64(dNy)),
                        dptr(_f64(area)), dptr(_f64(shoc)), dptr(_f64(dtl)),
                        dptr(_f64(t_sugn1)), dptr(_f64(t_sugn2)), dptr(_f64(t_sugn3)),
                        iptr(inp), _ci(nelem), _ci(npoin), dptr(_f64(T)), dptr(_f64(gas))),
          "cfd_calcrhs")
    return rhs


def FUENTE(rhs, U, W_X, W_Y, dNx, dNy, area, dtl, inpoel):
    L = abi.lib()
    inp = _i32(inpoel)
    check(L.cfd_fuente(dptr(rhs), dptr(_f64(U)), dptr(_f64(W_X)), dptr(_f64(W_Y)),
                       dptr(_f64(dNx)), dptr(_f64(dNy)), dptr(_f64(area)), dptr(_f64(dtl)),
                       iptr(inp), _ci(inp.shape[0]), _ci(len(W_X))), "cfd_fuente")
    return rhs


def ESTAB(U, T, GAMM, VEL_X, VEL_Y, W_X, W_Y, dNx, dNy, inpoel, GAMA, FR, DTMIN, RHOINF, TINF):
    """-> SHOC, T_SUGN1, T_SUGN2, T_SUGN3 (subrutinas.f90:332-446)."""
    L = abi.lib()
    inp = _i32(inpoel)
    ne = inp.shape[0]
    out = [np.zeros(ne) for _ in range(4)]
    scal = np.array([GAMA, FR, DTMIN, RHOINF, TINF], np.float64)
    check(L.cfd_estab(dptr(_f64(U)), dptr(_f64(T)), dptr(_f64(GAMM)), dptr(_f64(VEL_X)),
                      dptr(_f64(VEL_Y)), dptr(_f64(W_X)), dptr(_f64(W_Y)), dptr(_f64(dNx)),
                      dptr(_f64(dNy)), iptr(inp), _ci(ne), _ci(len(T)), dptr(scal),
                      *[dptr(o) for o in out]), "cfd_estab")
    return out


def deltat(T, VEL_X, VEL_Y, W_X, W_Y, area, inpoel, FSAFE, FR, GAMA, T_inf):
    """-> DT (clamped at 10*DTMIN), DTMIN (subrutinas.f90:155-218)."""
    L = abi.lib()
    inp = _i32(inpoel)
    ne = inp.shape[0]
    DT = np.zeros(ne)
    dtmin = C.c_double(0.0)
    scal = np.array([FSAFE, FR, GAMA, T_inf], np.float64)
    check(L.cfd_deltat(dptr(_f64(T)), dptr(_f64(VEL_X)), dptr(_f64(VEL_Y)), dptr(_f64(W_X)),
                       dptr(_f64(W_Y)), dptr(_f64(area)), iptr(inp), _ci(ne), _ci(len(T)),
                       dptr(scal), dptr(DT), C.byref(dtmin)), "cfd_deltat")
    return DT, dtmin.value


def deriv(X, Y, inpoel):
    """-> dict(area, dNx, dNy, HH, HHX, HHY, hmin) (subrutinas.f90:88-126)."""
    L = abi.lib()
    inp = _i32(inpoel)
    ne = inp.shape[0]
    r = dict(area=np.zeros(ne), dNx=np.zeros((ne, 3)), dNy=np.zeros((ne, 3)), HH=np.zeros(ne),
             HHX=np.zeros(ne), HHY=np.zeros(ne))
    hmin = C.c_double(0.0)
    check(L.cfd_deriv(dptr(_f64(X)), dptr(_f64(Y)), iptr(inp), _ci(ne), _ci(len(X)),
                      dptr(r["area"]), dptr(r["dNx"]), dptr(r["dNy"]), dptr(r["HH"]),
                      dptr(r["HHX"]), dptr(r["HHY"]), C.byref(hmin)), "cfd_deriv")
    r["hmin"] = hmin.value
    return r


def FORCE_VISC(NELEM, npoin, nsets, IELEM_SETS, ISET, inpoel, NSET_NUMB, U_inf, V_inf, RHO_inf,
               T_inf, X, Y, P, T, VEL_X, VEL_Y, DNX, DNY, RMU=0.0, RHO=None, skin=False):
    """ns2DComp.ALE.f90:819-893 -> (F_VX(10), F_VY(10)[, skin rows (nedges, 3)]).  ISET is
    Fortran ISET(3,10,nsets) as a C array of shape (nsets, 10, 3); DNX, DNY (nelem, 3)."""
    L = abi.lib()
    fvx, fvy = np.zeros(10), np.zeros(10)
    ne = int(np.sum(np.asarray(IELEM_SETS)[:NSET_NUMB]))
    sk = np.zeros((max(ne, 1), 3)) if skin else None
    rho = _f64(np.zeros(npoin) if RHO is None else RHO)
    check(L.cfd_force_visc(_ci(NELEM), _ci(npoin), _ci(nsets), iptr(_i32(IELEM_SETS)),
                           iptr(_i32(ISET)), iptr(_i32(inpoel)), _ci(NSET_NUMB),
                           C.byref(C.c_double(U_inf)), C.byref(C.c_double(V_inf)),
                           C.byref(C.c_double(RHO_inf)), C.byref(C.c_double(T_inf)),
                           dptr(_f64(X)), dptr(_f64(Y)), dptr(_f64(P)), dptr(_f64(T)),
                           dptr(_f64(VEL_X)), dptr(_f64(VEL_Y)), dptr(_f64(DNX)),
                           dptr(_f64(DNY)), C.byref(C.c_double(RMU)), dptr(rho), dptr(fvx),
                           dptr(fvy), dptr(sk)), "cfd_force_visc")
    return (fvx, fvy, sk[:ne]) if skin else (fvx, fvy)


def smoothing(X, Y, inpoel, fixed, dX=None, dY=None, order=abi.CFD_SMOOTH_COLOUR):
    """smoothing.f90:21-72 -> (X, Y, iterations, min quality).  fixed: per node, True = does
    not move; dX, dY: the setTol_move path's displacements; order: CFD_SMOOTH_COLOUR (the
    GPU's colour-by-colour variant) or CFD_SMOOTH_NODE_ORDER (the reference's order)."""
    L = abi.lib()
    X, Y = _f64(X).copy(), _f64(Y).copy()
    inp = _i32(inpoel)
    it, q = C.c_int(0), C.c_double(0.0)
    check(L.cfd_smoothing_ex(dptr(X), dptr(Y), iptr(inp), iptr(_i32(fixed)), _ci(len(X)),
                             _ci(inp.shape[0]), dptr(None if dX is None else _f64(dX)),
                             dptr(None if dY is None else _f64(dY)), C.byref(it), C.byref(q),
                             int(order)), "cfd_smoothing")
    return X, Y, it.value, q.value


def MASAS(area, inpoel, npoin):
    L = abi.lib()
    inp = _i32(inpoel)
    M = np.zeros(npoin)
    check(L.cfd_masas(dptr(_f64(area)), iptr(inp), _ci(inp.shape[0]), _ci(npoin), dptr(M)),
          "cfd_masas")
    return M


def gcl_main(M, W_x, W_y, W_x_old, W_y_old, dNx, dNy, area, area_old, inpoel, dt,
             mode=abi.CFD_MASS_GCL_LITERAL):
    L = abi.lib()
    inp = _i32(inpoel)
    M = _f64(M).copy()
    dtv = C.c_double(float(dt))
    check(L.cfd_gcl(dptr(M), dptr(_f64(W_x)), dptr(_f64(W_y)), dptr(_f64(W_x_old)),
                    dptr(_f64(W_y_old)), dptr(_f64(dNx)), dptr(_f64(dNy)), dptr(_f64(area)),
                    dptr(_f64(area_old)), iptr(inp), _ci(inp.shape[0]), _ci(len(M)),
                    C.byref(dtv), int(mode)), "cfd_gcl")
    return M


def getEsup(inpoel, npoin):
    L = abi.load()
    inp = _i32(inpoel)
    e1 = np.zeros(3 * inp.shape[0], np.int32)
    e2 = np.zeros(npoin + 1, np.int32)
    check(L.cfd_get_esup(iptr(inp), _ci(inp.shape[0]), _ci(npoin), iptr(e1), iptr(e2)),
          "cfd_get_esup")
    return e1, e2


def getPsup(inpoel, npoin):
    L = abi.load()
    inp = _i32(inpoel)
    n = C.c_int(0)
    check(L.cfd_get_psup(iptr(inp), _ci(inp.shape[0]), _ci(npoin), None, None, C.byref(n)),
          "cfd_get_psup")
    p1 = np.zeros(max(1, n.value), np.int32)
    p2 = np.zeros(npoin + 1, np.int32)
    check(L.cfd_get_psup(iptr(inp), _ci(inp.shape[0]), _ci(npoin), iptr(p1), iptr(p2), None),
          "cfd_get_psup")
    return p1[:n.value], p2


def laplace_pattern(inpoel, npoin):
    L = abi.load()
    inp = _i32(inpoel)
    nnz = C.c_int(0)
    check(L.cfd_laplace_pattern(iptr(inp), _ci(inp.shape[0]), _ci(npoin), None, None,
                                C.byref(nnz)), "cfd_laplace_pattern")
    rp = np.zeros(npoin + 1, np.int32)
    idx = np.zeros(nnz.value, np.int32)
    check(L.cfd_laplace_pattern(iptr(inp), _ci(inp.shape[0]), _ci(npoin), iptr(rp), iptr(idx),
                                C.byref(nnz)), "cfd_laplace_pattern")
    return rp, idx


def laplace(inpoel, area, dNx, dNy, X, Y, lap_idx, lap_rowptr):
    """-> lap_sparse, lap_diag (mLaplace.f90:7-58) on the given pattern."""
    L = abi.lib()
    inp = _i32(inpoel)
    npoin = len(X)
    vals = np.zeros(len(lap_idx))
    diag = np.zeros(npoin)
    check(L.cfd_laplace(iptr(inp), dptr(_f64(area)), dptr(_f64(dNx)), dptr(_f64(dNy)),
                        _ci(inp.shape[0]), _ci(npoin), dptr(_f64(X)), dptr(_f64(Y)), dptr(vals),
                        iptr(_i32(lap_idx)), iptr(_i32(lap_rowptr)), dptr(diag)), "cfd_laplace")
    return vals, diag


def biCG(spMtx, spIdx, spRowptr, diagMtx, x, b, x_fix, x_fixIdx, tol=1.0e-10, maxit=1000,
         tol_mode=abi.CFD_BICG_TOL_ABS):
    """x (initial guess, copied) -> (solution, CfdSolveInfo) (biconjGrad.f90:8-62).
    tol_mode CFD_BICG_TOL_ABS is the reference's absolute test on |r.z|; the relative modes
    stop when ||r|| <= tol * ||ref|| (include/cfd_gpu.h)."""
    L = abi.lib()
    x = _f64(x).copy()
    info = abi.CfdSolveInfo()
    fi = _i32(x_fixIdx)
    check(L.cfd_bicg_mode(dptr(_f64(spMtx)), iptr(_i32(spIdx)), iptr(_i32(spRowptr)),
                          dptr(_f64(diagMtx)), dptr(x), dptr(_f64(b)), dptr(_f64(x_fix)),
                          iptr(fi), _ci(len(x)), _ci(len(fi)), float(tol), int(maxit),
                          int(tol_mode), C.byref(info)), "cfd_bicg")
    return x, info


# ------------------------------------------------------------------ resident driver
class Solver:
    """PROGRAM NSComp2D over a resident context: freestream start (RESTART, IRESTART=0),
    setup geometry, then `step(n)` runs n iterations of ns2DComp.ALE.f90:140-280."""

    def __init__(self, case, precision=abi.CFD_PREC_FP64):
        self.case = case
        self.n, self.ne = case.npoin, case.nelem
        self._mesh, self._keep = case.to_c()
        self._params = case.params.to_c()
        L = abi.lib()
        h = C.c_void_p()
        check(L.cfd_ctx_create(C.byref(h), C.byref(self._mesh), C.byref(self._params),
                               int(precision)), "cfd_ctx_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            abi.lib().cfd_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_guess_net(self, net, gate=20.0):
        """Attach a learned-guess network (cfd_gb300.learned.Net; None detaches) to this
        mixed-form context; used when the case's guess_mode is CFD_GUESS_LEARNED.  The
        network runs on the first solve and after any solve that took more than `gate`
        iterations (every solve when gate is 0)."""
        self._net = net
        check(abi.lib().cfd_ctx_set_guess_net(self.h, net.h if net is not None else None,
                                              float(gate)), "cfd_ctx_set_guess_net")

    def guess_stats(self):
        """(steps with the network evaluated, x solves and y solves that took its guess,
        steps) since the network was attached."""
        out = (C.c_longlong * 4)()
        check(abi.lib().cfd_ctx_guess_stats(self.h, out), "cfd_ctx_guess_stats")
        return tuple(int(v) for v in out)

    def set_guess_refine(self, on=True):
        """Refined learned guess: basis fields seeded by the network and corrected by every
        solve (see cfd_ctx_set_guess_refine)."""
        check(abi.lib().cfd_ctx_set_guess_refine(self.h, int(bool(on))),
              "cfd_ctx_set_guess_refine")

    def guess_stats_ex(self):
        """(network guesses formed, x and y taken, steps, fields guesses formed, x and y
        taken, 0) since the network was attached."""
        out = (C.c_longlong * 8)()
        check(abi.lib().cfd_ctx_guess_stats_ex(self.h, out), "cfd_ctx_guess_stats_ex")
        return tuple(int(v) for v in out)

    def smooth(self, order=abi.CFD_SMOOTH_COLOUR):
        """The reference's setup smoothing of the resident mesh, then its geometry again.
        order: CFD_SMOOTH_COLOUR or CFD_SMOOTH_NODE_ORDER.  -> (iterations, min quality)."""
        it, q = C.c_int(0), C.c_double(0.0)
        check(abi.lib().cfd_ctx_smooth_ex(self.h, int(order), C.byref(it), C.byref(q)),
              "cfd_ctx_smooth")
        return it.value, q.value

    def set_force_visc(self, each_step):
        """each_step: every step computes FORCE_VISC where the reference's print block does."""
        check(abi.lib().cfd_ctx_set_force_visc(self.h, 1 if each_step else 0),
              "cfd_ctx_set_force_visc")

    def set_smoothing(self, every):
        """Smooth the moved mesh every `every` steps inside the time loop (0: never)."""
        check(abi.lib().cfd_ctx_set_smoothing(self.h, int(every)), "cfd_ctx_set_smoothing")

    def smoothing_stats(self):
        """(steps smoothed, smoothing sweeps) so far."""
        out = (C.c_longlong * 2)()
        check(abi.lib().cfd_ctx_smoothing_stats(self.h, out), "cfd_ctx_smoothing_stats")
        return int(out[0]), int(out[1])

    def force_visc(self):
        """(F_VX[nset_numb], F_VY[nset_numb], SKIN.DAT rows (nedges, 3))."""
        fvx, fvy = np.zeros(10), np.zeros(10)
        iset, ielem_sets, n = self.case.iset_array()
        ne = int(ielem_sets[:n].sum())
        skin = np.zeros((max(ne, 1), 3))
        check(abi.lib().cfd_ctx_force_visc(self.h, dptr(fvx), dptr(fvy), dptr(skin)),
              "cfd_ctx_force_visc")
        return fvx[:n], fvy[:n], skin[:ne]

    def graph_state(self):
        """(1 if steps replay a captured CUDA graph, replays so far, kernels per replay)."""
        out = (C.c_longlong * 3)()
        check(abi.lib().cfd_ctx_graph_state(self.h, out), "cfd_ctx_graph_state")
        return tuple(int(v) for v in out)

    def step(self, n=1):
        rep = abi.CfdStepReport()
        check(abi.lib().cfd_step(self.h, int(n), C.byref(rep)), "cfd_step")
        return rep

    def state(self):
        U = np.zeros((self.n, 4))
        T, X, Y = np.zeros(self.n), np.zeros(self.n), np.zeros(self.n)
        check(abi.lib().cfd_ctx_download_state(self.h, dptr(U), dptr(T), dptr(X), dptr(Y)),
              "cfd_ctx_download_state")
        return dict(U=U, T=T, X=X, Y=Y)

    def fields(self):
        names = ["RHO", "VEL_X", "VEL_Y", "E", "P", "RMACH", "W_X", "W_Y"]
        arrs = [np.zeros(self.n) for _ in names]
        check(abi.lib().cfd_ctx_download_fields(self.h, *[dptr(a) for a in arrs]),
              "cfd_ctx_download_fields")
        return dict(zip(names, arrs))

    def motion(self):
        xp, yp = np.zeros(self.n), np.zeros(self.n)
        check(abi.lib().cfd_ctx_download_motion(self.h, dptr(xp), dptr(yp)),
              "cfd_ctx_download_motion")
        return xp, yp

    def geometry(self):
        a = np.zeros(self.ne)
        dnx, dny = np.zeros((self.ne, 3)), np.zeros((self.ne, 3))
        M = np.zeros(self.n)
        check(abi.lib().cfd_ctx_download_geometry(self.h, dptr(a), dptr(dnx), dptr(dny), dptr(M)),
              "cfd_ctx_download_geometry")
        return dict(area=a, dNx=dnx, dNy=dny, M=M)

    def laplace_values(self):
        """The mesh-motion matrix of the last assembly, in the order of laplace_pattern."""
        rp, _ = laplace_pattern(self.case.inpoel, self.n)
        v = np.zeros(int(rp[-1]))
        check(abi.lib().cfd_ctx_download_laplace(self.h, dptr(v)), "cfd_ctx_download_laplace")
        return v

    def set_state(self, U=None, T=None, VEL_X=None, VEL_Y=None):
        conv = [None if a is None else _f64(a) for a in (U, T, VEL_X, VEL_Y)]
        check(abi.lib().cfd_ctx_upload_state(self.h, *[dptr(a) for a in conv]),
              "cfd_ctx_upload_state")

    def set_mesh(self, X=None, Y=None, W_X=None, W_Y=None, xpos=None, ypos=None):
        conv = [None if a is None else _f64(a) for a in (X, Y, W_X, W_Y, xpos, ypos)]
        check(abi.lib().cfd_ctx_upload_mesh(self.h, *[dptr(a) for a in conv]),
              "cfd_ctx_upload_mesh")

    def set_clock(self, iter=0, time=0.0, dtmin1=0.0, bandera=1, disn1=0.0, disn2=0.0):
        check(abi.lib().cfd_ctx_set_clock(self.h, iter, time, dtmin1, bandera, disn1, disn2),
              "cfd_ctx_set_clock")

    def stream(self):
        """cudaStream_t (int) every kernel of this context runs on."""
        return abi.lib().cfd_ctx_stream(self.h)

    def mark(self, slot):
        """Record CUDA event `slot` on the context's stream."""
        check(abi.lib().cfd_ctx_mark(self.h, int(slot)), "cfd_ctx_mark")

    def elapsed_ms(self, a, b):
        ms = C.c_double(0.0)
        check(abi.lib().cfd_ctx_elapsed(self.h, int(a), int(b), C.byref(ms)), "cfd_ctx_elapsed")
        return ms.value

    def timers(self):
        """{timer name: (seconds, timed launches)} accumulated since create (CFD_TIMERS=1)."""
        s = np.zeros(16)
        c = (C.c_longlong * 16)()
        n = C.c_int(0)
        check(abi.lib().cfd_ctx_timers(self.h, dptr(s), 16, C.byref(n)), "cfd_ctx_timers")
        check(abi.lib().cfd_ctx_timer_calls(self.h, c, 16, C.byref(n)), "cfd_ctx_timer_calls")
        names = [abi.lib().cfd_timer_name(i).decode() for i in range(n.value)]
        return {nm: (float(s[i]), int(c[i])) for i, nm in enumerate(names)}

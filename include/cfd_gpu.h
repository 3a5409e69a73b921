/*
 * cfd_gpu.h — C-ABI of the GB300 (sm_103a) implementation of the explicit SUPG
 * compressible Navier–Stokes step on linear triangles with ALE mesh motion.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and returns an
 * int status (0 = CFD_OK; see cfd_strerror()).  Two layers:
 *
 *  1. Drop-in routines.  Same argument lists, argument meaning and array layout as the
 *     Fortran routines they replace: column-major arrays (U(4,npoin) is node-major
 *     interleaved), 1-based node/element indices, scalars passed by pointer (Fortran
 *     by-reference).  All pointers are HOST memory; each call stages its inputs to the
 *     GPU, runs the kernels and copies the outputs back.
 *
 *  2. Resident context.  Mesh, state and every per-step array live in GPU memory; the
 *     host uploads once, steps N times and downloads on demand.  This is the timed path.
 *
 * Nothing here holds global mutable state except the documented per-device buffers of
 * the drop-in layer; a context belongs to one host thread at a time.
 */
#ifndef CFD_GPU_H
#define CFD_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
enum {
    CFD_OK = 0,
    CFD_ERR_ARG = 1,          /* null pointer, non-positive size, bad enum value      */
    CFD_ERR_MESH = 2,         /* index out of 1..npoin, degenerate/inverted element   */
    CFD_ERR_CUDA = 3,         /* a CUDA runtime call failed                           */
    CFD_ERR_NOMEM = 4,        /* device allocation failed                             */
    CFD_ERR_NOT_CONVERGED = 5,/* BiCG hit its iteration cap (reference: silent)       */
    CFD_ERR_NONFINITE = 6,    /* NaN/Inf found in the state (reference: fuse > 1e2)   */
    CFD_ERR_BARRIER = 7,      /* a device-side bounded wait gave up                   */
    CFD_ERR_LIMIT = 8,        /* a size above a documented maximum                    */
    CFD_ERR_STATE = 9         /* call out of order (e.g. step before upload)          */
};

/* precision_mode for cfd_ctx_create */
enum {
    CFD_PREC_FP64 = 0,        /* plain: every operation FP64, reference evaluation order */
    CFD_PREC_MIXED = 1        /* calcRHS and SpMV in FP32 (compensated node sums);
                                 state update, gcl, BiCG dots and scalars in FP64        */
};

/* mass_mode: how the lumped mass follows a moving mesh */
enum {
    CFD_MASS_MASAS = 0,       /* recompute M = sum(area/3) (reference, MOVING=1)        */
    CFD_MASS_GCL_LITERAL = 1, /* gcl.f90 main as written (divW uses dNy*W_x)            */
    CFD_MASS_GCL_CORRECTED = 2/* gcl.f90 main with divW = dNx.W_x + dNy.W_y             */
};

/* motion_law: the prescribed body motion (reference hard-codes law 0) */
enum {
    CFD_MOTION_REFERENCE = 0, /* pitch pi/8*sin(10 t), no heave (meshMove.f90:55-71)    */
    CFD_MOTION_HARMONIC = 1,  /* heave A_h*sin(2 pi f t), pitch A_p*sin(2 pi f t)       */
    CFD_MOTION_NEWMARK = 2    /* heave and pitch from the 2-DOF Newmark structural model
                                 under set 1's pressure force and moment
                                 (meshMove.f90:61-62, :196-367, enabled)              */
};

/* guess_mode: initial guess of the two mesh-motion solves */
enum {
    CFD_GUESS_PREVIOUS = 0,   /* previous step's increment (reference, meshMove.f90:97) */
    CFD_GUESS_ZERO = 1,
    CFD_GUESS_LEARNED = 2,    /* edge message-passing network (falls back to PREVIOUS)  */
    /* the last two increments extrapolated to this step (no counterpart in the reference):
     * a solve's unknown is the step's mesh increment, the mean mesh velocity over the step
     * times DTMIN; with that velocity linear in time through the last two steps' midpoints
     * the guess on the free rows is x = c1 x_{n-1} + c2 x_{n-2}, h = (dt_n + dt_1)/(dt_1 +
     * dt_2), c1 = dt_n/dt_1 (1 + h), c2 = -(dt_n/dt_2) h (2 x_{n-1} - x_{n-2} at a constant
     * DTMIN); PREVIOUS until two solutions are kept.  The solves reach the same tolerance;
     * FP64 form and oracle stay bit-identical. */
    CFD_GUESS_EXTRAPOLATED = 3,
    /* LEARNED with EXTRAPOLATED as the guess the network's and the fields' guesses are
     * judged against (per solve: the x and y solves of a pitching body can prefer
     * different guesses) */
    CFD_GUESS_LEARNED_EXTRAPOLATED = 4
};

/* estab_mode: the "velocity gradient" of ESTAB (subrutinas.f90:380-383) is
 * DUX = VEL2*sum(dNx), zero in exact arithmetic; as written its round-off decides
 * whether H_RGN and T_SUGN2 vanish (a discontinuity at round-off level). */
enum {
    CFD_ESTAB_REFERENCE = 0,  /* evaluate DUX, DUY as written (bit-exact reference)     */
    CFD_ESTAB_EXACT = 1,      /* take DUX = DUY = 0, their exact-arithmetic value       */
    CFD_ESTAB_REGULARIZED = 2 /* unit vectors continuous in the state: grad(rho), grad(T)
                                 plus 1e-3*scale*sum|grad N_i| along the freestream
                                 direction d, normalised; the velocity-gradient direction
                                 (round-off in the reference) is d                      */
};

/* bicg_tol_mode: what the BiCG stopping test measures.  The reference's test is absolute
 * (biconjGrad.f90:26, :35, :47); the relative modes compare the 2-norm of the (Dirichlet-
 * rows-zeroed) residual r with a reference norm:  ||r|| <= tol * ||ref||. */
enum {
    CFD_BICG_TOL_ABS = 0,     /* |r.z| <= tol, early exit on r.r < tol (reference)      */
    CFD_BICG_TOL_REL = 1,     /* ref = b - A.x_D, the residual of the guess that is 0 off
                                 the Dirichlet rows: independent of the initial guess, so
                                 every guess solves to the same accuracy                 */
    CFD_BICG_TOL_REL_R0 = 2   /* ref = r_0, the residual of the initial guess           */
};

/* ---------------------------------------------------------------- plain structs */

/* InputData (dataLoader.f90:5-15) after readInputData's derivations (:58-64),
 * plus the options the reference hard-codes. */
typedef struct cfd_params {
    int irestart, maxiter, iprint, movie, itlocal, ngas, moving;
    double fsafe, u_inf, v_inf, mach_inf, t_inf, rho_inf, p_inf, c_inf;
    double fmu, fgx, fgy, qh, fk, fr, fcv, gama;
    double cte;               /* as stored by readInputData: 1/CTE of the file (:59)   */
    double xref[10], yref[10];
    /* build-side options (reference: hard-coded) */
    int motion_law;           /* CFD_MOTION_*                                          */
    double heave_amp, pitch_amp, motion_freq;
    int mass_mode;            /* CFD_MASS_*                                            */
    int guess_mode;           /* CFD_GUESS_*                                           */
    double bicg_tol;          /* 1e-10 in biconjGrad.f90:26 (absolute, on r.z)         */
    int bicg_maxit;           /* 1000 in biconjGrad.f90:47                             */
    int estab_mode;           /* CFD_ESTAB_*                                           */
    int bicg_tol_mode;        /* CFD_BICG_TOL_* (default 0: the reference's absolute test) */
    int reserved[5];
} cfd_params;

/* MeshData (dataLoader.f90:68-91) as loadMeshData leaves it.  Host pointers, Fortran
 * layout, 1-based indices.  iset is ISET(3,10,nsets) column-major. */
typedef struct cfd_mesh {
    int npoin, nelem;
    const int* inpoel;        /* 3*nelem                                               */
    const double* x;          /* npoin                                                 */
    const double* y;
    int nfixrho;  const int* ifixrho_node; const double* rfixrho_value;
    int nfixv;    const int* ifixv_node;   const double* rfixv_valuex; const double* rfixv_valuey;
    int nfixt;    const int* ifixt_node;   const double* rfixt_value;
    int nwall;    const int* wall;         /* 2*nwall                                  */
    int nsets;    int nset_numb;  int ielem_sets[10]; const int* iset; /* 3*10*nsets   */
    int nmove;    int nfix_move;  const int* ilaux;    /* nmove+nfix_move              */
} cfd_mesh;

/* Per-call report of cfd_step (the last step of the call). */
typedef struct cfd_step_report {
    int iter;                 /* ITER after the call                                   */
    int status;
    double time;              /* TIME                                                  */
    double dtmin;             /* DTMIN used by the step (after hysteresis)             */
    int bicg_iters[2];        /* x and y solves                                        */
    double bicg_rz[2];        /* final |r.z|                                           */
    int bicg_converged[2];
    double fx[10], fy[10], rm[10]; /* FORCES (pressure) per set, before the mesh moves */
    int nset_numb;
    int reserved0;
    double bicg_relres[2];    /* ||r||/||ref|| of the last iteration (relative modes; 0 in
                                 the absolute mode)                                    */
    int reserved[4];
} cfd_step_report;

typedef struct cfd_solve_info {
    int iters;                /* k of biconjGrad.f90:47-48                             */
    int converged;            /* 1 if the stopping test holds (or the early exit at :35) */
    double rz;                /* final |r.z| (at an early exit: r.r, as the reference)  */
    double relres;            /* relative modes: final ||r||/||ref||; absolute mode: 0  */
} cfd_solve_info;

typedef struct cfd_ctx cfd_ctx;

/* ---------------------------------------------------------------- drop-in routines */

/* calcRHS (calcRHS.f90:4-154).  rhs(4,npoin) is ACCUMULATED into (the caller zeroes it,
 * subrutinas.f90:680-682).  T(npoin) is the module temperature read at calcRHS.f90:6.
 * gas = {FCV, FK, FMU, GAMA, T_inf, CTE} as calcRHS.f90:5 imports them. */
int cfd_calcrhs(double* rhs, const double* U, const double* theta,
                const double* dNx, const double* dNy, const double* area,
                const double* shoc, const double* dtl, const double* t_sugn1,
                const double* t_sugn2, const double* t_sugn3, const int* inpoel,
                const int* nelem, const int* npoin, const double* T, const double* gas6);

/* FUENTE (subrutinas.f90:1036-1094): rhs += ALE source term. */
int cfd_fuente(double* rhs, const double* U, const double* W_X, const double* W_Y,
               const double* dNx, const double* dNy, const double* area, const double* dtl,
               const int* inpoel, const int* nelem, const int* npoin);

/* ESTAB (subrutinas.f90:332-446) -> SHOC, T_SUGN1..3 per element.
 * scal = {GAMA, FR, DTMIN, RHOINF, TINF} (RMU, UINF, VINF are read but unused). */
int cfd_estab(const double* U, const double* T, const double* GAMM, const double* VEL_X,
              const double* VEL_Y, const double* W_X, const double* W_Y,
              const double* dNx, const double* dNy, const int* inpoel,
              const int* nelem, const int* npoin, const double* scal5,
              double* SHOC, double* T_SUGN1, double* T_SUGN2, double* T_SUGN3);

/* deltat (subrutinas.f90:155-218) -> DT(nelem) (clamped at 10*DTMIN) and DTMIN.
 * scal = {FSAFE, FR, GAMA, T_inf}. */
int cfd_deltat(const double* T, const double* VEL_X, const double* VEL_Y,
               const double* W_X, const double* W_Y, const double* area,
               const int* inpoel, const int* nelem, const int* npoin,
               const double* scal4, double* DT, double* DTMIN);

/* smoothing (smoothing.f90:21-72), drop-in: X, Y in/out; fixed: per node, nonzero = does
 * not move (the reference's logical array); dX, dY: both NULL, or the step's displacement
 * for the setTol_move path (:372-386).  GPU colour-by-colour order (cfd_ctx_smooth). */
int cfd_smoothing(double* X, double* Y, const int* inpoel, const int* fixed, const int* npoin,
                  const int* nelem, const double* dX, const double* dY, int* iters,
                  double* min_quality);
/* The node visiting order of the smoothing: */
enum {
    CFD_SMOOTH_COLOUR = 0,    /* nodes coloured so that no two of a colour share an element,
                                 one colour at a time (parallel; a nearby smoothed mesh)    */
    CFD_SMOOTH_NODE_ORDER = 1 /* one node at a time in node order, as smoothing.f90:55-67
                                 and :80-114 visit them (the reference's mesh, bit for bit
                                 with its FP64 arithmetic; sequential by construction: one
                                 GPU thread, a setup-time step)                            */
};
/* smoothing (smoothing.f90:21-72) with the visiting order chosen (cfd_smoothing: colour). */
int cfd_smoothing_ex(double* X, double* Y, const int* inpoel, const int* fixed, const int* npoin,
                     const int* nelem, const double* dX, const double* dY, int* iters,
                     double* min_quality, int order);

/* FORCE_VISC (ns2DComp.ALE.f90:819-893), drop-in: the reference's argument list (RMU and
 * RHO are unused by its body), F_VX/F_VY 10 each; skin: NULL, or 3 doubles per set edge
 * (the SKIN.DAT rows the reference writes instead). */
int cfd_force_visc(const int* NELEM, const int* npoin, const int* nsets, const int* IELEM_SETS,
                   const int* ISET, const int* inpoel, const int* NSET_NUMB, const double* U_inf,
                   const double* V_inf, const double* RHO_inf, const double* T_inf,
                   const double* X, const double* Y, const double* P, const double* T,
                   const double* VEL_X, const double* VEL_Y, const double* DNX,
                   const double* DNY, const double* RMU, const double* RHO, double* F_VX,
                   double* F_VY, double* skin);

/* deriv (subrutinas.f90:88-126) -> area, dNx(3,nelem), dNy, HH, HHX, HHY, hmin. */
int cfd_deriv(const double* X, const double* Y, const int* inpoel, const int* nelem,
              const int* npoin, double* area, double* dNx, double* dNy,
              double* HH, double* HHX, double* HHY, double* hmin);

/* MASAS (subrutinas.f90:128-153) -> lumped mass M(npoin). */
int cfd_masas(const double* area, const int* inpoel, const int* nelem, const int* npoin,
              double* M);

/* gcl_mod::main (gcl.f90:8-46) with putW/putArea's saved state passed explicitly:
 * M += dt*(tot1+tot2)/2.  mode = CFD_MASS_GCL_LITERAL or CFD_MASS_GCL_CORRECTED. */
int cfd_gcl(double* M, const double* W_x, const double* W_y, const double* W_x_old,
            const double* W_y_old, const double* dNx, const double* dNy,
            const double* area, const double* area_old, const int* inpoel,
            const int* nelem, const int* npoin, const double* dt, int mode);

/* getEsup / getPsup (pointNeighbor.f90:5-91), host-side.  Output arrays are 1-based
 * like the reference: esup2(npoin+1) offsets, esup1(3*nelem); psup2(npoin+1) offsets,
 * psup1(*npsup).  Call once with psup1 == NULL to get *npsup. */
int cfd_get_esup(const int* inpoel, const int* nelem, const int* npoin,
                 int* esup1, int* esup2);
int cfd_get_psup(const int* inpoel, const int* nelem, const int* npoin,
                 int* psup1, int* psup2, int* npsup);

/* Mlaplace::initialize (mLaplace.f90:60-94): lap_rowptr(npoin+1) (0-based offsets),
 * lap_idx(nnz) (1-based, diagonal first).  Call with lap_idx == NULL to get *nnz. */
int cfd_laplace_pattern(const int* inpoel, const int* nelem, const int* npoin,
                        int* lap_rowptr, int* lap_idx, int* nnz);

/* Mlaplace::laplace (mLaplace.f90:7-58): values of the mesh-motion operator on a given
 * pattern (from cfd_laplace_pattern).  area is accepted and unused, as in the reference. */
int cfd_laplace(const int* inpoel, const double* area, const double* dNx, const double* dNy,
                const int* nelem, const int* npoin, const double* X, const double* Y,
                double* lap_sparse, const int* lap_idx, const int* lap_rowptr,
                double* lap_diag);

/* biCG (biconjGrad.f90:8-62): Jacobi-preconditioned CG with Dirichlet rows by
 * overwrite + 1e30 penalty.  x is the initial guess on entry, the solution on exit.
 * tol/maxit as the reference (1e-10 absolute on |r.z|, 1000) unless overridden by
 * cfd_bicg_ex.  info may be NULL.  Returns CFD_OK also when the cap is hit (like the
 * reference); info->converged says which. */
int cfd_bicg(const double* spMtx, const int* spIdx, const int* spRowptr,
             const double* diagMtx, double* x, const double* b, const double* x_fix,
             const int* x_fixIdx, const int* npoin, const int* nfix,
             cfd_solve_info* info);
int cfd_bicg_ex(const double* spMtx, const int* spIdx, const int* spRowptr,
                const double* diagMtx, double* x, const double* b, const double* x_fix,
                const int* x_fixIdx, const int* npoin, const int* nfix,
                double tol, int maxit, cfd_solve_info* info);
/* biCG with the stopping test chosen by tol_mode (CFD_BICG_TOL_*; tol is then the relative
 * tolerance, e.g. 1e-10).  The iterates are those of cfd_bicg_ex, only the iteration at
 * which the solve stops differs. */
int cfd_bicg_mode(const double* spMtx, const int* spIdx, const int* spRowptr,
                  const double* diagMtx, double* x, const double* b, const double* x_fix,
                  const int* x_fixIdx, const int* npoin, const int* nfix,
                  double tol, int maxit, int tol_mode, cfd_solve_info* info);

/* BiCG on arrays already in device memory, with no device allocation.  This entry has no
 * counterpart in the reference: it is for callers that cannot call cudaMalloc where they
 * solve (a host that owns all device memory itself, e.g. CUDA Fortran/OpenACC arrays or
 * a framework pool with a fixed budget, or a time loop that must not allocate).  Work
 * vectors live in one static device array of the library, reserved on every GPU that
 * loads it until the process exits, which caps npoin at CFD_NOALLOC_MAX_NPOIN
 * (about 2.5 MiB of device memory).
 * All pointers are DEVICE pointers: CSR with 0-based col/rowptr (diagonal entries as in
 * lap_*), isfix[npoin] nonzero on Dirichlet rows, x = initial guess that already holds the
 * Dirichlet values on those rows (the reference's copy1), b may be NULL (zero).  Same
 * arithmetic and result as cfd_bicg_ex.  Runs on `stream` (cudaStream_t, NULL = default)
 * and waits for it before returning.  The first call on a device looks up the array's
 * device address; under CUDA's lazy module loading (the default, CUDA_MODULE_LOADING=LAZY)
 * that lookup is also when the runtime creates the array on the device, so make the first
 * call during set-up, before a memory pool takes the free device memory and before any
 * stream capture.  Every call shares the one array: calls that overlap on the GPU (other
 * streams or threads) race.  npoin above the cap returns CFD_ERR_LIMIT. */
#define CFD_NOALLOC_MAX_NPOIN 65536
int cfd_bicg_device_noalloc(const double* spMtx, const int* col, const int* rowptr,
                            const double* diag, const unsigned char* isfix, double* x,
                            const double* b, int npoin, double tol, int maxit, void* stream,
                            cfd_solve_info* info);

/* ---------------------------------------------------------------- resident context */

/* Builds adjacency, BC tables, the Laplacian pattern and every device buffer.
 * Runs normales/deriv/MASAS/laplace on the device (ns2DComp.ALE.f90:88-100).
 * The freestream initial state of RESTART (ns2DComp.ALE.f90:404-420) is loaded. */
int cfd_ctx_create(cfd_ctx** ctx, const cfd_mesh* mesh, const cfd_params* p,
                   int precision_mode);
void cfd_ctx_destroy(cfd_ctx* ctx);

/* Overwrite the flow state.  U(4,npoin), T, VEL_X, VEL_Y may be NULL to keep the
 * current ones; when VEL_* are NULL they are derived from U.  With VEL_* NULL and U in
 * pinned host memory (cudaHostAlloc / cudaHostRegister, 16-byte aligned) one kernel reads
 * U over the host link and forms the device copies as it arrives; otherwise the arrays are
 * copied.  Returns when U, T, VEL_* may be reused by the caller. */
int cfd_ctx_upload_state(cfd_ctx* ctx, const double* U, const double* T,
                         const double* VEL_X, const double* VEL_Y);
/* Overwrite the mesh-motion state: X, Y, W_X, W_Y, xpos, ypos (any may be NULL), and
 * recompute the geometry of the new mesh (normales, deriv, mass, laplace). */
int cfd_ctx_upload_mesh(cfd_ctx* ctx, const double* X, const double* Y,
                        const double* W_X, const double* W_Y,
                        const double* xpos, const double* ypos);
/* Time-loop scalars: ITER, TIME, DTMIN1 (hysteresis memory), BANDERA, DISN(1:2). */
int cfd_ctx_set_clock(cfd_ctx* ctx, int iter, double time, double dtmin1, int bandera,
                      double disn1, double disn2);

/* nsteps iterations of the loop body ns2DComp.ALE.f90:140-280. */
int cfd_step(cfd_ctx* ctx, int nsteps, cfd_step_report* rep);

/* Any pointer may be NULL.  U(4,npoin) reference layout. */
int cfd_ctx_download_state(cfd_ctx* ctx, double* U, double* T, double* X, double* Y);
/* Primitive fields of the last stage: RHO, VEL_X, VEL_Y, E, P, RMACH, W_X, W_Y. */
int cfd_ctx_download_fields(cfd_ctx* ctx, double* RHO, double* VEL_X, double* VEL_Y,
                            double* E, double* P, double* RMACH, double* W_X, double* W_Y);
/* Mesh-motion increments of the last step (guess of the next). */
int cfd_ctx_download_motion(cfd_ctx* ctx, double* xpos, double* ypos);
/* Geometry of the current mesh: area(nelem), dNx(3,nelem), dNy(3,nelem), M(npoin). */
int cfd_ctx_download_geometry(cfd_ctx* ctx, double* area, double* dNx, double* dNy,
                              double* M);
/* The mesh-motion matrix of the last assembly (laplace, mLaplace.f90:7-58): its nnz values in
 * the CSR order of cfd_laplace_pattern (the diagonal first in each row).  The FP64 form
 * assembles it for each step's solve from the mesh before the step moves it, the mixed form
 * for the next step from the moved mesh.  FP64 form: the FP64 values; mixed form: the FP32
 * values, or under the relative BiCG tests the FP64-class ones (held as FP32 hi + lo,
 * to 2^-47). */
int cfd_ctx_download_laplace(cfd_ctx* ctx, double* val);

/* Per-kernel timers (CUDA events) accumulated since create, in seconds; names follow
 * the reference TIMERS module (commonModules.f90:31-35).  n = slots written. */
int cfd_ctx_timers(cfd_ctx* ctx, double* seconds, int max, int* n);
/* Number of timed launches accumulated in each timer slot. */
int cfd_ctx_timer_calls(cfd_ctx* ctx, long long* calls, int max, int* n);
const char* cfd_timer_name(int slot);

/* The cudaStream_t (as void*) every kernel of this context is launched on, so a caller
 * can record CUDA events around cfd_step on the launching stream. */
void* cfd_ctx_stream(cfd_ctx* ctx);
/* CUDA events on the context's stream: mark(slot) records event slot (0..7);
 * elapsed waits for event b and returns the time from a to b in milliseconds. */
int cfd_ctx_mark(cfd_ctx* ctx, int slot);
int cfd_ctx_elapsed(cfd_ctx* ctx, int a, int b, double* ms);

/* Select the device (ordinal) this library's contexts and drop-in calls use on the
 * calling host thread (one process per GPU sets its local rank). */
int cfd_set_device(int ordinal);

/* ---------------------------------------------------------------- learned guess */
/* An edge message-passing network (4 layers, width 64) that gives the initial guess of
 * the mesh-motion solve; BiCG then finishes the solve from it (no reference counterpart:
 * the reference starts from the previous step's increment, meshMove.f90:44,97).  From the
 * node coordinates and boundary kinds it predicts the three fields Phi, Psi_x, Psi_y whose
 * combination t Phi + M (Psi_x, Psi_y) is the solve's displacement for an affine body
 * motion g = t + M (p - c); (t, M) is the least-squares fit of the prescribed body
 * displacement.  Training runs on the GPU (FP32 forward/backward, Adam); inference uses
 * BF16 tensor cores with FP32 accumulation.  Parameters: cfd_mpnn_nparams() floats in the
 * packing of cfd_gb300/csrc/mpnn.cuh. */
typedef struct cfd_mpnn cfd_mpnn;
typedef struct cfd_mpnn_graph cfd_mpnn_graph;

int cfd_mpnn_nparams(void);
int cfd_mpnn_create(cfd_mpnn** net, const float* weights);
void cfd_mpnn_destroy(cfd_mpnn* net);
int cfd_mpnn_get_weights(cfd_mpnn* net, float* weights);
int cfd_mpnn_set_weights(cfd_mpnn* net, const float* weights);
/* Adam moments (may be NULL) and step count */
int cfd_mpnn_adam_state(cfd_mpnn* net, float* m, float* v, int* t);
/* Graph of a mesh; bnode (1-based) lists the boundary nodes with their kind: 1 moving body,
 * 2 fixed outer boundary. */
int cfd_mpnn_graph_create(cfd_mpnn_graph** g, int npoin, int nelem, const int* inpoel,
                          const double* x, const double* y, int nb, const int* bnode,
                          const int* bkind);
void cfd_mpnn_graph_destroy(cfd_mpnn_graph* g);
/* prescribed displacement of the boundary nodes (bnode order) and its affine fit */
int cfd_mpnn_graph_set_bc(cfd_mpnn_graph* g, const double* gx, const double* gy);
/* cx, cy, L, R (body geometry) and the fit tx, ty, m11, m12, m21, m22 */
int cfd_mpnn_graph_globals(cfd_mpnn_graph* g, double* out10);
/* training target: the fields the plain solve gives for the boundary data 1, x - c_x and
 * y - c_y on the body (0 on the outer boundary), npoin each */
int cfd_mpnn_graph_set_target(cfd_mpnn_graph* g, const double* phi, const double* psi_x,
                              const double* psi_y);
/* FP32 forward + backward: loss and (grad may be NULL) the gradient of every parameter */
int cfd_mpnn_loss_grad(cfd_mpnn* net, cfd_mpnn_graph* g, float* loss, float* grad);
/* loss_grad, then one Adam step (beta1 0.9, beta2 0.999, eps 1e-8) with rate lr */
int cfd_mpnn_train_step(cfd_mpnn* net, cfd_mpnn_graph* g, float lr, float* loss);
/* The guess (npoin each; the boundary nodes carry their prescribed values): bf16 = 1 for
 * the tensor-core pass, 0 for the FP32 pass. */
int cfd_mpnn_forward(cfd_mpnn* net, cfd_mpnn_graph* g, int bf16, double* ux, double* uy);

/* Learned guess in a resident context (mixed form, params.guess_mode = CFD_GUESS_LEARNED):
 * the network's guess is formed on the first mesh-motion solve after attaching, and then
 * whenever the previous step's solve took more than `gate` iterations (every step when
 * gate = 0); per solve it replaces the previous-step guess if its r.z (the solve's measure
 * of convergence) is the smaller, so the plain guess stays the fallback and the yardstick.
 * net = NULL detaches it (previous-step guess).  The network must outlive its use by the
 * context. */
int cfd_ctx_set_guess_net(cfd_ctx* ctx, cfd_mpnn* net, double gate);
/* counters since attach: steps with the network evaluated, solves 1 (x) and 2 (y) that
 * took the network's guess, steps */
int cfd_ctx_guess_stats(cfd_ctx* ctx, long long* out4);
/* Refined learned guess (on = 1; default off).  The context keeps the three fields
 * (Phi, Psi_x, Psi_y) per node in FP64: a network run seeds them with its prediction, and
 * after every pair of solves each node's fields take the smallest change that makes them
 * reproduce both solutions (x = t Phi + M Psi with each solve's affine fit).  Between network
 * runs each solve also tries the fields' guess t Phi + M Psi for its own data, and keeps it
 * when its r.z is smaller than the previous step's.  The fields then track the moving
 * mesh's operator, so the guess error is the change of the operator over a step rather
 * than the change of the motion, which pays under a relative stopping test
 * (CFD_BICG_TOL_REL).  Switching it makes the network run again on the next solve. */
int cfd_ctx_set_guess_refine(cfd_ctx* ctx, int on);
/* out8 = (steps with a network guess formed, x and y taken from it, steps, steps with a
 * fields guess formed, x and y taken from it, 0) */
int cfd_ctx_guess_stats_ex(cfd_ctx* ctx, long long* out8);

/* FORCE_VISC (ns2DComp.ALE.f90:819-893): viscous force per force set on its wall edges
 * (F_VX, F_VY: 10 each) and, when skin is not NULL, the SKIN.DAT row of every set edge in
 * set and edge order (3 doubles: skin friction, the edge's mean x, element-mean pressure /
 * 82713.27).  With each_step set (cfd_ctx_set_force_visc) every cfd_step computes it where
 * the reference's print block does (after the mesh moved, before its dNx are recomputed)
 * and cfd_ctx_force_visc returns the last step's values; otherwise cfd_ctx_force_visc
 * computes it on the context's current state, mesh and dNx. */
int cfd_ctx_set_force_visc(cfd_ctx* ctx, int each_step);
int cfd_ctx_force_visc(cfd_ctx* ctx, double* F_VX, double* F_VY, double* skin);

/* Mixed form: out3 = (1 if steps replay a captured CUDA graph, steps replayed so far,
 * kernels in one replay).  The first step of a context, and steps that run the learned
 * guess, are enqueued launch by launch; CFD_GRAPHS=0 or CFD_TIMERS=1 at create turn the
 * graph off.  No counterpart in the reference (its time loop calls the routines of
 * ns2DComp.ALE.f90:114-283 one by one). */
int cfd_ctx_graph_state(cfd_ctx* ctx, long long* out3);

/* Smooth the context's mesh as the reference does at setup (ns2DComp.ALE.f90:62-72,
 * smoothing.f90; the mesh-motion boundary nodes stay), then recompute its geometry (normals,
 * dNx/dNy/area, lumped mass, Laplacian).  The GPU colours the nodes so that no two nodes
 * of a colour share an element and moves one colour at a time (the reference moves one
 * node at a time, in node order), so the result is a nearby smoothed mesh, not the
 * reference's.  iters: the sweeps run (NITER + 1 when they did not settle, 0 when no
 * element is below the quality threshold 0.85); min_quality: the worst element's mu
 * afterwards.  Either may be NULL. */
int cfd_ctx_smooth(cfd_ctx* ctx, int* iters, double* min_quality);
/* cfd_ctx_smooth with the visiting order chosen: CFD_SMOOTH_NODE_ORDER gives the mesh the
 * reference's setup call (ns2DComp.ALE.f90:76) gives. */
int cfd_ctx_smooth_ex(cfd_ctx* ctx, int order, int* iters, double* min_quality);

/* Smooth the moved mesh inside the time loop every `every` steps (0: never, the default):
 * after the step's mesh update, the smoothing moves each node at most |XPOS| + |YPOS| (the
 * setTol_move path, smoothing.f90:372-386, with the step's displacement), W becomes the
 * whole move over DTMIN, and the new mesh's geometry is computed from the smoothed nodes.
 * The reference's time loop smooths nothing: its per-step calls of the older SMOOTH_MESH
 * are commented out (meshMove.f90:133, subrutinas.f90:795) and the smoothing module's
 * setTol_move, made for a moved mesh, has no caller.  A step that smooths runs launch by
 * launch and waits on the host for the sweeps' convergence.  cfd_ctx_smoothing_stats:
 * out2 = (steps smoothed, sweeps). */
int cfd_ctx_set_smoothing(cfd_ctx* ctx, int every);
int cfd_ctx_smoothing_stats(cfd_ctx* ctx, long long* out2);

/* Number of kernels this library launched since process start (all contexts). */
long long cfd_kernel_launches(void);

/* Failure-detection self-test (no counterpart in the reference): runs, in one block, the
 * library's two bounded device waits on conditions that never come true (a grid barrier
 * that a second block never reaches; an mbarrier nothing arrives on), each giving up after
 * `polls` polls (1 .. 2^24; the library's kernels use 2^24) or 1 s on the GPU's global
 * timer, whichever comes first (every wait of the library has both bounds).  Both statuses
 * come back as CFD_ERR_BARRIER and the device stays usable. */
int cfd_selftest_waits(long long polls, int* barrier_status, int* mbarrier_status);

/* Arithmetic self-test (no counterpart in the reference): the FP64 kernels divide by 3 with
 * a multiply and two FMAs (Markstein's correction of the quotient by the rounded reciprocal);
 * this compares it with the IEEE division x / 3.0 over n inputs (1 .. 2^36: raw 64-bit
 * patterns from `seed`, values in 2^-40 .. 2^40, and values next to 3 * 2^k) and returns
 * the number whose bits differ. */
int cfd_selftest_div3(long long n, unsigned long long seed, unsigned long long* mismatches);
/* The same for the FP64 BiCG's quotients r/diag: a multiply by RN(1/diag) and four FMAs
 * (two Markstein corrections) against the division, over n pairs from `seed` (raw bit
 * patterns, magnitudes 2^-60 .. 2^60, quotients next to binade edges and halfway cases). */
int cfd_selftest_div_rcp(long long n, unsigned long long seed, unsigned long long* mismatches);

const char* cfd_strerror(int status);
/* 1 if a CUDA device is usable by this library. */
int cfd_device_available(void);

#ifdef __cplusplus
}
#endif
#endif /* CFD_GPU_H */

/*
 * cfd_oracle.h — CPU restatement of the reference's FP64 step (chanshing/cfd).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline (cpu_baseline / --impl reference) may load this library; nothing in the
 * cfd_gb300 product path links, imports or calls it.
 *
 * Parity is UNPINNED by the reference itself: the reference ships no tests, fixtures or
 * sample inputs, and it is Fortran (ifort) with no Fortran compiler available to build
 * it.  The restatement is pinned instead by known-answer tests derived from the
 * mathematics (tests/test_oracle_*.py) and by golden vectors it produced on seeded
 * meshes (tests/golden/).
 *
 * Conventions (each routine cites the reference file:line it follows):
 *  - arrays in the reference's Fortran layout, indices 1-based;
 *  - every expression evaluated in Fortran's order (left to right, ** before * and /,
 *    unary minus over the whole product), compiled with -ffp-contract=off;
 *  - x**2 and x**2.d0 are x*x; x**.5d0 is sqrt(x); x**1.5d0 is x*sqrt(x) and
 *    x**(-.5d0) is 1/sqrt(x) (correctly rounded compositions, within about one ulp
 *    of the exact power, evaluated identically by any IEEE-754 double unit);
 *  - sums the reference leaves to OpenMP atomics or REDUCTION(+) are taken in element
 *    order (1 thread), except vecdot, whose order is pinned to or_vecdot's fixed tree.
 */
#ifndef CFD_ORACLE_H
#define CFD_ORACLE_H
#include "../include/cfd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

void or_set_threads(int n);
/* 0 (default): calcRHS and FUENTE scatter with OpenMP atomics, as the reference does (with
 * more than one thread the adds into a node come in thread order); 1: the element rows are
 * formed in parallel and added in element order, the one-thread result at any thread count */
void or_set_ordered_scatter(int on);
void or_set_estab_mode(int mode);  /* CFD_ESTAB_* for the per-routine or_estab */
/* 0 (default): the compositions above; 1: x**1.5d0, x**.5d0 and x**(-.5d0) through the C
 * library's pow, as a Fortran compiler without unsafe-math options evaluates them */
void or_set_pow_mode(int mode);
int or_get_pow_mode(void);
/* counts over x[0..n): pow(x,1.5) != x*sqrt(x), pow(x,-0.5) != 1/sqrt(x),
 * pow(x,0.5) != sqrt(x) */
void or_pow_census(int n, const double* x, long long* out3);
int or_get_threads(void);

void or_deriv(int npoin, int nelem, const double* X, const double* Y, const int* inpoel,
              double* area, double* dNx, double* dNy, double* HH, double* HHX,
              double* HHY, double* hmin);
void or_masas(int npoin, int nelem, const double* area, const int* inpoel, double* M);
void or_deltat(int npoin, int nelem, const double* T, const double* VEL_X,
               const double* VEL_Y, const double* W_X, const double* W_Y,
               const double* area, const int* inpoel, double FSAFE, double FR,
               double GAMA, double T_inf, double* DT, double* DTMIN);
void or_estab(int npoin, int nelem, const double* U, const double* T, const double* GAMM,
              const double* VEL_X, const double* VEL_Y, const double* W_X,
              const double* W_Y, const double* dNx, const double* dNy, const int* inpoel,
              double GAMA, double FR, double DTMIN, double RHOINF, double TINF,
              double* SHOC, double* TS1, double* TS2, double* TS3);
void or_calcrhs(double* rhs, const double* U, const double* theta, const double* dNx,
                const double* dNy, const double* area, const double* shoc,
                const double* dtl, const double* ts1, const double* ts2,
                const double* ts3, const int* inpoel, int nelem, int npoin,
                const double* T, const double* gas6);
void or_fuente(double* rhs, const double* U, const double* W_X, const double* W_Y,
               const double* dNx, const double* dNy, const double* area,
               const double* dtl, const int* inpoel, int nelem, int npoin);
void or_gcl(double* M, const double* W_x, const double* W_y, const double* W_x_old,
            const double* W_y_old, const double* dNx, const double* dNy,
            const double* area, const double* area_old, const int* inpoel, int nelem,
            int npoin, double dt, int mode);

int or_get_esup(const int* inpoel, int nelem, int npoin, int* esup1, int* esup2);
int or_get_psup(const int* inpoel, int nelem, int npoin, int* psup1, int* psup2,
                int* npsup);
int or_laplace_pattern(const int* inpoel, int nelem, int npoin, int* lap_rowptr,
                       int* lap_idx, int* nnz);
void or_laplace(const int* inpoel, const double* dNx, const double* dNy, int nelem,
                int npoin, const double* X, const double* Y, const int* esup1,
                const int* esup2, double* lap_sparse, const int* lap_idx,
                const int* lap_rowptr, double* lap_diag);

double or_vecdot(int n, const double* x, const double* y);
void or_bicg(const double* spMtx, const int* spIdx, const int* spRowptr,
             const double* diagMtx, double* x, const double* b, const double* x_fix,
             const int* x_fixIdx, int npoin, int nfix, double tol, int maxit,
             cfd_solve_info* info);
/* the same iterates with the stopping test of tol_mode (CFD_BICG_TOL_*) */
void or_bicg_mode(const double* spMtx, const int* spIdx, const int* spRowptr,
                  const double* diagMtx, double* x, const double* b, const double* x_fix,
                  const int* x_fixIdx, int npoin, int nfix, double tol, int maxit, int tol_mode,
                  cfd_solve_info* info);

int or_normales(int npoin, int nwall, const int* wall, const double* X, const double* Y,
                int* n_ipoin, double* n_x, double* n_y);

void or_smoothing(double* X, double* Y, const int* inpoel, const int* fixed, int npoin,
                  int nelem, int* iters_out, double* min_quality_out);
/* the same visiting the nodes in `order` (0-based permutation; NULL: node order), with
 * setTol_move's |dX| + |dY| per node when tol_move is not NULL */
void or_smoothing_ordered(double* X, double* Y, const int* inpoel, const int* fixed, int npoin,
                          int nelem, const int* order, const double* tol_move, int* iters_out,
                          double* min_quality_out);

void or_force_visc(int nelem, int npoin, int nsets, const int* ielem_sets, const int* iset,
                   const int* inpoel, int nset_numb, double u_inf, double v_inf, double rho_inf,
                   double t_inf, const double* X, const double* Y, const double* P,
                   const double* T, const double* VEL_X, const double* VEL_Y, const double* dNx,
                   const double* dNy, double* F_VX, double* F_VY, double* skin);

/* One NEWMARK_METHOD step (meshMove.f90:196-310) on dis, vel, acc (2 each) under load F. */
void or_newmark_step(double H, const double* F, double* dis, double* vel, double* acc);

/* Whole-driver restatement (ns2DComp.ALE.f90:8-282) over a cfd_mesh/cfd_params. */
typedef struct or_case or_case;
or_case* or_case_create(const cfd_mesh* mesh, const cfd_params* p, int do_smoothing);
void or_case_destroy(or_case* c);
int or_case_step(or_case* c, int nsteps, cfd_step_report* rep);
void or_case_get(or_case* c, double* U, double* T, double* X, double* Y);
void or_case_get_fields(or_case* c, double* RHO, double* VEL_X, double* VEL_Y, double* E,
                        double* P, double* RMACH, double* W_X, double* W_Y);
void or_case_get_motion(or_case* c, double* xpos, double* ypos);
/* FORCE_VISC: each_step = 1 computes it in every step at the print block's point (after
 * the move, before deriv) and or_case_force_visc returns the last step's values; 0 makes
 * or_case_force_visc compute it on the current state and mesh.  skin: 3 per set edge. */
void or_case_set_force_visc(or_case* c, int each_step);
/* smooth the moved mesh every `every` steps on the setTol_move path, visiting the nodes in
 * `order` (0-based; NULL: node order); W the whole move over DTMIN */
void or_case_set_smoothing(or_case* c, int every, const int* order);
void or_case_force_visc(or_case* c, double* F_VX, double* F_VY, double* skin);
void or_case_get_geometry(or_case* c, double* area, double* dNx, double* dNy, double* M);
void or_case_set_state(or_case* c, const double* U, const double* T, const double* VEL_X,
                       const double* VEL_Y);
void or_case_set_mesh(or_case* c, const double* X, const double* Y, const double* W_X,
                      const double* W_Y, const double* xpos, const double* ypos);
void or_case_set_clock(or_case* c, int iter, double time, double dtmin1, int bandera,
                       double disn1, double disn2);
/* seconds spent per reference TIMERS slot (same order as cfd_timer_name) */
void or_case_timers(or_case* c, double* seconds, int max, int* n);

#ifdef __cplusplus
}
#endif
#endif

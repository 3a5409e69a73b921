// cfd_kernels.cuh — kernel declarations and the small device-side structs.
#pragma once
#include "cfd_common.cuh"

namespace cfd {

// per-node boundary-condition bits (the reference's FIXVEL / NORMALVEL / FIX lists)
enum : unsigned char { BC_FIXV = 1, BC_NORMAL = 2, BC_FIXRHO = 4, BC_FIXT = 8 };

// Device-resident step scalars.
struct StepScal {
    unsigned long long dtmin_bits;  // atomicMin target of k_deltat
    unsigned long long dtmin32_bits;  // mixed form: FP32 candidate minimum
    double dtmin_raw;               // DTMIN from deltat
    double dtmin;                   // DTMIN after hysteresis (used by the step)
    double dtmin1;                  // hysteresis memory (ns2DComp.ALE.f90:146-156)
    double cota;                    // 10*DTMIN of deltat
    int bandera;
    int pad;
    double fx[10], fy[10], rm[10];  // FORCES per set
};

// calcRHS.f90:5 imports: Cv => FCV, lambda_ref => FK, mu_ref => FMU, gamma0 => GAMA, T_inf, CTE
struct GasConst {
    double cv, lambda_ref, mu_ref, gamma, t_inf, cte;
    double fr;  // FR (perfect-gas constant), used by the mixed node kernel
};

// ------------------------------------------------------------------ mixed precision
__global__ void k_deltat_mixed(int nelem, const int4* elem, const double* T, const double* VX,
                               const double* VY, const double* WX, const double* WY,
                               const double* area, float fsafe, float t_inf,
                               unsigned long long* dtmin_bits);
__global__ void k_deltat_refine(int nelem, const int4* elem, const double* T, const double* VX,
                                const double* VY, const double* WX, const double* WY,
                                const double* area, float fsafe, float t_inf, StepScal* sc);
__global__ void k_estab_mixed(int nelem, const int4* elem, const double* U, const double* T,
                              float gm, const double* VX, const double* VY, const double* WX,
                              const double* WY, const double* geo, float FR, const StepScal* sc,
                              float RHOINF, float TINF, int estab_mode, float eps_dir,
                              float dirx, float diry, float* SHOC, float* TS1, float* TS2,
                              float* TS3);
cudaError_t launch_elem_stage1_mixed(bool viscous, cudaStream_t st, int nelem, const int4* elem,
                                     const double* U, const double* geo, const double* area,
                                     const float* shoc, const double* dtl_arr,
                                     const double* dtl_scalar, const float* ts1, const float* ts2,
                                     const float* ts3, GasConst gc, const double* WX,
                                     const double* WY, const int* slot_pos, void* rec);
cudaError_t launch_node_mixed(cudaStream_t st, int npoin, const int* esup_ptr, const int* esup_slot,
                              const int4* elem, const void* rec, const double* T, GasConst gc,
                              int viscous, const double* U, const double* invM, double rk_fact,
                              const unsigned char* bcflag, const double* bcval, const double2* nrm,
                              const double* WX, const double* WY, double* U1, double* RHO,
                              double* VX, double* VY, double* E, double* P, double* To,
                              double* RMACH);
size_t slot_record_bytes();
__global__ void k_deriv_mixed(int nelem, const int4* elem, const double* X, const double* Y,
                              double* area, double* geo);
__global__ void k_gcl_elem(int nelem, const int4* elem, const double* geo, const double* area,
                           const double* area_old, const double* Wx, const double* Wy,
                           const double* Wxo, const double* Wyo, int literal, double2* terms);
__global__ void k_mass_mixed(int npoin, const int* esup_ptr, const int* esup_slot,
                             const double* area, const double2* terms, const double* dtp, int gcl,
                             double* M, double* invM);
cudaError_t launch_laplace_mixed(bool fp64, cudaStream_t st, int npoin, int nelem, const int4* elem,
                                 const int* esup_ptr, const int* esup_slot, const uchar4* lap_pos,
                                 const double* geo, const double* X, const double* Y,
                                 const int* rowptr, float* valf, double* vals, double* diag,
                                 double* invdiag);
__global__ void k_forces_tree(int nset_numb, const int* set_ptr, const int2* set_edges,
                              const double* P, const double* X, const double* Y,
                              const double* xref, const double* yref, StepScal* sc);

#define ELEM_RHS_ARGS                                                                    \
    int, const int4* __restrict__, const double* __restrict__, const double* __restrict__, \
        const double* __restrict__, const double* __restrict__, const double* __restrict__, \
        const double* __restrict__, const double* __restrict__, const double* __restrict__, \
        const double* __restrict__, const double* __restrict__, const double* __restrict__, \
        GasConst, double* __restrict__, const double* __restrict__,                        \
        const double* __restrict__, double* __restrict__

__global__ void k_deriv(int nelem, const int4* elem, const double* X, const double* Y,
                        double* area, double* geo, double* hh, double* hhx, double* hhy);
__global__ void k_mass(int npoin, const int* esup_ptr, const int* esup_slot, const double* area,
                       double* M);
__global__ void k_gcl(int npoin, int nelem, const int4* elem, const int* esup_ptr,
                      const int* esup_slot, const double* geo, const double* area,
                      const double* area_old, const double* Wx, const double* Wy,
                      const double* Wxo, const double* Wyo, const double* dtp, int literal,
                      double* M);
__global__ void k_deltat(int nelem, const int4* elem, const double* T, const double* VX,
                         const double* VY, const double* WX, const double* WY,
                         const double* area, double fsafe, double t_inf, double* DT,
                         unsigned long long* dtmin_bits);
__global__ void k_dt_finalize(StepScal* sc);
__global__ void k_dtl(int nelem, double* DT, double* DTL, const StepScal* sc, double dtfact);
__global__ void k_estab(int nelem, const int4* elem, const double* U, const double* T,
                        double gamm, const double* GAMM, const double* VX, const double* VY, const double* WX,
                        const double* WY, const double* geo, double FR, const StepScal* sc,
                        double RHOINF, double TINF, int estab_mode, double eps_dir,
                        double dirx, double diry, double* SHOC, double* TS1, double* TS2,
                        double* TS3);
// calcRHS (+ FUENTE when contribF != NULL) element kernel; contrib may be NULL (FUENTE only)
cudaError_t launch_elem_rhs(bool viscous, bool with_theta, cudaStream_t stream, int nelem,
                            const int4* elem, const double* U, const double* theta,
                            const double* T, const double* geo, const double* area,
                            const double* shoc, const double* dtl_arr, const double* dtl_scalar,
                            const double* ts1, const double* ts2, const double* ts3, GasConst gc,
                            double* contrib, const double* WX, const double* WY,
                            double* contribF);
__global__ void k_node_update(int npoin, const int* esup_ptr, const int* esup_slot,
                              const double* contrib, const double* contribF, const double* U,
                              const double* M, double rk_fact, double gamm, double FR,
                              const unsigned char* bcflag, const double* bcval,
                              const double2* nrm, const double* WX, const double* WY,
                              double* U1, double* RHO, double* VX, double* VY, double* Eo,
                              double* Po, double* To, double* RMACH, const double* rhs_init,
                              double* rhs_out);
__global__ void k_dt_clamp(int nelem, double* DT, const StepScal* sc);
__global__ void k_min_positive(long n, const double* x, unsigned long long* bits);
__global__ void k_normales(int nwn, const int* wnode, const int* wptr, const int2* wedge_of,
                           const int2* walls, const double* X, const double* Y,
                           unsigned char* bcflag, double2* nrm);
__global__ void k_laplace(int npoin, int nelem, const int4* elem, const int* esup_ptr,
                          const int* esup_slot, const uchar4* lap_pos, const double* geo,
                          const double* X, const double* Y, const int* rowptr, double* vals,
                          double* diag);
__global__ void k_forces(int nset_numb, const int* set_ptr, const int2* set_edges,
                         const double* P, const double* X, const double* Y, const double* xref,
                         const double* yref, StepScal* sc);
__global__ void k_transf(int nnmove, const int* fix_node, const int* fix_set, const double* X,
                         const double* Y, const double* xref, const double* yref, double ca,
                         double sa, double yposr, double* xfix_x, double* xfix_y);
__global__ void k_motion_update(int npoin, const double* xpos, const double* ypos,
                                const StepScal* sc, double* X, double* Y, double* WX,
                                double* WY);

// ------------------------------------------------------------------ PCG
struct PcgArgs {
    int n;
    int nsolve;                  // 1 or 2 right-hand sides on the same matrix
    const int* rowptr;           // CSR, 0-based, diagonal first in each row
    const int* col;
    const double* val;
    const double* diag;
    const unsigned char* isfix;  // per node: Dirichlet row
    int nfix;                    // unique fixed nodes (last entry of the reference list)
    const int* fix_node;
    const int* fix_src;          // index into fixval of the entry that wins
    const double* fixval[2];
    double* x[2];
    const double* b[2];          // NULL = zero right-hand side
    double* r[2];
    double* z[2];
    double* y[2];
    double* p[2][2];             // ping-pong search directions
    double* part;                // [2 phases][2 solves][nchunks] chunk partial sums
    // mixed form only: FP32 matrix values, 1/diag, FP32 shadows of p (ping-pong) and z
    const float* valf;
    const double* invdiag;
    float* pf[2][2];
    float* zf[2];
    GridBar* bar;
    double tol;
    int maxit;
    int* iters_out;              // [2]
    double* rz_out;              // [2]
    int* conv_out;               // [2]
};

__global__ void k_pcg_fp64(PcgArgs a);
__global__ void k_pcg_mixed(PcgArgs a);

}  // namespace cfd

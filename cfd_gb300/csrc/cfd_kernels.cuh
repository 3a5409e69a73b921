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
    int iter;                       // mixed form: ITER, advanced on the device
    double fx[10], fy[10], rm[10];  // FORCES per set
    double inv_dtmin;               // 1/DTMIN (mixed form: W = XPOS*(1/DTMIN))
    float dtmin_f;                  // (float)DTMIN for the FP32 kernels
    float pad_f;
    float dtfact_f, cota_f;         // mixed form, ITLOCAL != 0: DTFACT and COTA of DTL
    float pad2_f[2];
};

// DTMIN from the minimum DTELEM (b: its bit pattern, +inf for none) with the 1% hysteresis
// of ns2DComp.ALE.f90:146-156, and the scalars derived from it
__device__ __forceinline__ void dt_finalize_from(StepScal* sc, unsigned long long b) {
    double dtmin = 1.0e20;
    if (b != 0x7ff0000000000000ull) dtmin = __longlong_as_double((long long)b);
    sc->dtmin32_bits = 0x7ff0000000000000ull;
    sc->dtmin_raw = dtmin;
    if (sc->bandera == 1) {
        sc->dtmin1 = dtmin;
        sc->bandera = 2;
    }
    double porc = fabs((dtmin - sc->dtmin1) / dtmin);
    if (100.0 * porc <= 1.0) {
        dtmin = sc->dtmin1;
    } else {
        sc->dtmin1 = dtmin;
        sc->bandera = 2;
    }
    sc->dtmin = dtmin;
    sc->cota = 10.0 * sc->dtmin_raw;
    sc->inv_dtmin = 1.0 / dtmin;
    sc->dtmin_f = (float)dtmin;
}

// normales (subrutinas.f90:21-63) of wall node k: the wall edges touching it in edge order;
// the nodes the reference's compaction keeps (den > 1d-6 and |l| > 0.2) get BC_NORMAL
struct NormalsArgs {
    int nwn;
    const int *wnode, *wptr;
    const int2 *wedge_of, *walls;
    const double *X, *Y;
    unsigned char* bcflag;
    double2* nrm;
};
__device__ __forceinline__ void normales_node(const NormalsArgs& a, int k) {
    const int p = a.wnode[k];
    double nx = 0.0, ny = 0.0, den = 0.0;
    for (int s = a.wptr[k]; s < a.wptr[k + 1]; ++s) {
        const int2 w = a.walls[a.wedge_of[s].x];
        const double lex = a.Y[w.y] - a.Y[w.x];
        const double ley = -(a.X[w.y] - a.X[w.x]);
        const double le = sqrt(lex * lex + ley * ley);
        nx = nx + lex;
        ny = ny + ley;
        den = den + le;
    }
    unsigned char fl = a.bcflag[p] & (unsigned char)~BC_NORMAL;
    if (den > 1.0e-6) {
        const double lx = nx / den, ly = ny / den;
        const double nrmv = sqrt(lx * lx + ly * ly);
        if (nrmv > 0.2) {
            a.nrm[p] = make_double2(lx / nrmv, ly / nrmv);
            fl |= BC_NORMAL;
        }
    }
    a.bcflag[p] = fl;
}

// calcRHS.f90:5 imports: Cv => FCV, lambda_ref => FK, mu_ref => FMU, gamma0 => GAMA, T_inf, CTE
struct GasConst {
    double cv, lambda_ref, mu_ref, gamma, t_inf, cte;
    double fr;  // FR (perfect-gas constant), used by the mixed node kernel
};

// the same constants rounded to FP32 once on the host (the FP32 kernels would otherwise
// convert them per thread, on the FP64 pipe)
struct GasConstF {
    float cv, lambda_ref, mu_ref, gamma, t_inf, cte, fr;
};
inline GasConstF to_float(const GasConst& g) {
    return GasConstF{(float)g.cv, (float)g.lambda_ref, (float)g.mu_ref, (float)g.gamma,
                     (float)g.t_inf, (float)g.cte, (float)g.fr};
}

// Device-side clock and motion increment of the mixed form (the FP64 form keeps them on the
// host, where the oracle computes its sin/cos)
struct MotionScal {
    double time, disn0, disn1;  // TIME, DISN(1:2) (heave, pitch)
    double ca, sa, yposr;       // this step's TRANSF increment
    double dtmin;               // DTMIN of the step
    double veln0, veln1, accn0, accn1;  // CFD_MOTION_NEWMARK: VELN, ACCN
};
// What cfd_step reports, gathered on the device into one record for one copy
struct StepOut {
    StepScal sc;
    MotionScal ms;
    double rz[2], relres[2];
    int it[2], cv[2];
    int bar_err, has_motion;
};
// rz: [|r.z| x 2, ||r||/||ref|| x 2]
__global__ void k_pack_report(const StepScal* sc, const MotionScal* ms, const int* it,
                              const int* cv, const double* rz, const GridBar* bar,
                              const int* wait_err, StepOut* out);

struct MotionTailArgs {
    int do_motion, do_forces;  // the parts this launch runs (Newmark: both)
    int nset;  // FORCES
    const int* set_ptr;
    const int2* set_edges;
    const float* P;
    const double *X, *Y, *xref, *yref;
    int law;  // motion law
    double heave_amp, pitch_amp, freq;
    MotionScal* m;
    int nnmove;  // TRANSF
    const int *fix_node, *fix_set;
    double *xfix_x, *xfix_y;
    int nufix;  // Dirichlet values of the BiCG solves
    const int *ufix_node, *ufix_src;
    double *x0, *x1;
    float *xf0, *xf1;
    double* part;  // [3 * nset][gridDim.x] per-block force sums
    double4_32a* fgeo; // null, or per set edge the step-start geometry (the motion part writes,
                   // the forces part reads: the mesh may have moved in between)
    NormalsArgs nv;    // the forces part also runs normales (nv.nwn = 0: not)
    unsigned* count;
    StepScal* sc;
};
__global__ void k_motion_tail(MotionTailArgs a);
constexpr int kTailBlocks = 64;  // blocks of k_motion_tail at most (<= 256: the fold)

// FORCE_VISC over the force sets' edges: form 0 reads FP64 fields and dNx(j,e) =
// dnx[e*se + j*sj]; form 1 reads float fields and the mixed form's geo8.  terms: 2 per
// edge (scratch); skin: 3 per edge or null; fv[0..9] = F_VX, fv[10..19] = F_VY.
cudaError_t launch_force_visc(cudaStream_t st, int form, int nset, const int* set_ptr,
                              int nedges, const int2* edges, const int* eelem, const int4* elem,
                              const double* dnx, const double* dny, size_t se, size_t sj,
                              const float4* geo8, const void* P, const void* T, const void* VX,
                              const void* VY, const double* X, const double* Y, double u_inf,
                              double v_inf, double rho_inf, double t_inf, double* terms,
                              double* skin, double* fv);

// ------------------------------------------------------------------ mixed precision
__global__ void k_narrow_state(int npoin, const double* U, const double* T, const double* VX,
                               const double* VY, const double* X, const double* Y,
                               const double* WX, const double* WY, float4* Uhi, float4* Ulo,
                               float* Tf, float* VXf, float* VYf, float2* Xhi, float2* Xlo,
                               float2* Wf);
__global__ void k_upload_U(int npoin, const double* hU, double* U, double* VX, double* VY,
                           float4* Uhi, float4* Ulo, float* VXf, float* VYf);
__global__ void k_widen(long n, const float* a, double* b);
__global__ void k_widen_pair(long n, const float* hi, const float* lo, double* out);
__global__ void k_narrow(long n, const double* a, float* b);
__global__ void k_deltat_mixed(int nelem, const int4* elem, const float* T, const float* VX,
                               const float* VY, const float2* W, const float* areaf, float TINF,
                               float fsafe, unsigned long long* dtmin_bits,
                               unsigned long long* block_min, float* DTE);
// ESTAB's constants for the mixed form's stage-1 element kernel (estab_mode as CFD_ESTAB_*)
struct EstabConst {
    float gm, fr, rho_inf, t_inf;
    int mode;
    float eps, dirx, diry;
};
__global__ void k_deltat_refine(int nelem, const int4* elem, const float* T, const float* VX,
                                const float* VY, const float2* W, const float* areaf,
                                const unsigned long long* block_min, int nchunk, float fsafe,
                                float t_inf, StepScal* sc, unsigned* count, int itlocal);
cudaError_t launch_elem_stage1_mixed(bool viscous, cudaStream_t st, int nelem, const int4* elem,
                                     const float4* Uhi, const float4* Ulo, const float4* geo,
                                     const float* VX, const float* VY, EstabConst ec,
                                     const StepScal* sc, GasConstF gc, const float2* W,
                                     const int* slot_pos, const float* T, float4* recInv,
                                     float4* recVisc, float2* mulam, const float* dte);
constexpr int kMulamTB = 128;  // threads per block of k_elem_mulam (128: 0.533 ms, 256: 0.535, 512: 0.538)
__global__ void k_elem_mulam(int nelem, const int4* elem, const float* T, GasConstF gc,
                             float2* mulam);
cudaError_t launch_node_mixed(cudaStream_t st, int npoin, const int* esup_ptr, const int* esup_slot,
                              const float2* mulam, const float4* recInv, const float4* recVisc,
                              float4* invSum, int first_stage, GasConst gc, GasConstF gf,
                              int viscous, const double* U, float4* Uhi, float4* Ulo,
                              const float* invM, float rk_fact, int last_stage,
                              const unsigned char* bcflag, const double* bcval, const double2* nrm,
                              const double* WX, const double* WY, double* U1, float* RHO,
                              float* VX, float* VY, float* E, float* P, float* Tout, float* RMACH,
                              int bulk_smem = 0, int* bulk_err = nullptr);
// dynamic shared memory of the bulk-copy node pass for blocks of `block` nodes (0: the
// variant is not used: its staged slots would not fit)
int node_bulk_smem(const int* esup_ptr_host, int npoin);
__global__ void k_elem_geometry(int nelem, const int4* elem, const double* X, const double* Y,
                                int gcl, int literal, const float2* W, const float2* Wold,
                                int put_area, double* area_old, double* area64, float* areaf,
                                float4* geo, double2* terms, NormalsArgs nv);
constexpr int kGeoNodeBlock = 128;  // block size of k_node_geometry
__global__ void k_elem_grad64(int nelem, const int4* elem, const double* X, const double* Y,
                              const int* slot_pos, float2* k64);
// k_node_geometry (block kGeoNodeBlock); row64 (relative tests): the Laplacian rows summed
// from k64 (element-matrix rows as double-float pairs, written as valf + val_lo), not from geo
cudaError_t launch_node_geometry(bool row64, unsigned grid, cudaStream_t stream, int npoin,
                                 const int* esup_ptr, const int* esup_slot,
                                 const uchar4* lap_pos, const float4* geo, const double2* terms,
                                 const double* dtp, int gcl, const int* rowptr, float* valf,
                                 double* invdiag, float* invdiagf, double* M, float* invM,
                                 const float2* W, float2* Wold, const float2* k64,
                                 float* val_lo);
__global__ void k_widen_geo(int nelem, const float4* geo, double* dN, double* area);
__global__ void k_motion_update_mixed(int npoin, const double* xpos, const double* ypos,
                                      const StepScal* sc, double* X, double* Y, double* WX,
                                      double* WY, float2* Xhi, float2* Xlo, float2* Wf);

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
// gcl main (gcl.f90:8-46): the element terms once per element (scratch: nelem double2),
// then per node M += dt (tot1 + tot2)/2 over them in element order
cudaError_t launch_gcl(cudaStream_t st, int npoin, int nelem, const int4* elem,
                       const int* esup_ptr, const int* esup_slot, const double* geo,
                       const double* area, const double* area_old, const double* Wx,
                       const double* Wy, const double* Wxo, const double* Wyo, const double* dtp,
                       int literal, double2* scratch, double* M);
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
__global__ void k_vel_from_U(int npoin, const double* U, double* VX, double* VY);
// calcRHS split into its stage-invariant part (once per step: the cached addends and
// factors, FUENTE into contribF; with !viscous the final contributions into contrib) and
// the per-stage viscous replay from the cache (kernels_fp64.cu); cache: kInvPlanes x nelem
constexpr int kElemInvPlanes = 100;
cudaError_t launch_elem_inv(bool viscous, cudaStream_t stream, int nelem, const int4* elem,
                            const double* U, const double* geo, const double* area,
                            const double* shoc, const double* dtl_arr, const double* dtl_scalar,
                            const double* ts1, const double* ts2, const double* ts3, GasConst gc,
                            double* cache, double* contrib, const double* WX, const double* WY,
                            double* contribF);
cudaError_t launch_selftest_div3(long long n, unsigned long long seed, unsigned long long* bad);
cudaError_t launch_selftest_divrcp(long long n, unsigned long long seed, unsigned long long* bad);
cudaError_t launch_elem_replay(cudaStream_t stream, int nelem, const int4* elem, const double* T,
                               const double* geo, const double* area, const double* dtl_arr,
                               const double* dtl_scalar, GasConst gc, const double* cache,
                               double* contrib);
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
// laplace (mLaplace.f90:7-58): each element's weight 1/mu^2 once (scratch: nelem
// doubles), then the rows
cudaError_t launch_laplace(cudaStream_t st, int npoin, int nelem, const int4* elem,
                           const int* esup_ptr, const int* esup_slot, const uchar4* lap_pos,
                           const double* geo, const double* X, const double* Y, const int* rowptr,
                           double* scratch, double* vals, double* diag);
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
    double* rdiag;               // FP64 form: RN(1/diag), formed by the first pass and used
                                 // for the iterations' quotients (null: the division)
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
    const float* val_lo;         // relative tests: valf + val_lo = the FP64-assembled matrix
                                 // to 2^-47 (null: valf alone)
    const double* invdiag;
    float* pf[2][2];
    float* zf[2];
    float* xf[2];                // (float)x, kept equal to it on entry and exit
    float2* xs[2];               // relative tests: (hi, lo) = split_bits of the vector the
                                 // precise product reads (k_split_x before each such pass)
    const float* invdiagf;       // (float)(1/diag), with invdiag = (double)invdiagf
    double* part_r;              // [4][nblk_r] per-block partials of the row kernels
    long nblk_r;                 // 256-row blocks of the row kernels
    double* bscal;               // [2 solves][8]: r.r, r.p, p.y, alfa of the first direction,
                                 // the squared reference norm and the threshold on r.r
    unsigned* bcount;            // [3] block counters of the row kernels (zero between uses)
    // learned guess (null: off): the first residual pass sets gflag[0] = (sum r.z >= gate)
    // and clears gflag[1]; a pass with only_if != null runs only when *only_if != 0
    int* gflag;
    double gate;
    int gate_undone;             // 1: the gate opens when a solve's guess fails the stopping
                                 // test (the refined guess's candidate is judged only then)
    const int* only_if;
    GridBar* bar;
    double tol;
    int maxit;
    int tol_mode;                // CFD_BICG_TOL_*: the relative modes also sum r.r per
                                 // iteration, in part[2][s] (part then holds 6 x nchunks)
    int* iters_out;              // [2]
    int accumulate;              // mixed form: a second pass of the same solves (iterations
                                 // add to iters_out, the cap counts both passes)
    int* iterated;               // mixed form (nullable): set to 1 when a solve iterated (x
                                 // moved from the guess whose precise residual was formed)
    double* rz_out;              // [2]
    double* relres_out;          // [2] ||r||/||ref|| (relative modes), may be null
    int* conv_out;               // [2]
};

__global__ void k_pcg_fp64(PcgArgs a);
__global__ void k_pcg_mixed(PcgArgs a);
__global__ void k_selftest_waits(GridBar* gb, int* out, long long limit);
__global__ void k_bicg_fix_mixed(PcgArgs a);
// first pass of a mixed solve (k_bicg_resid_mixed, the variant of a.tol_mode)
cudaError_t launch_bicg_resid_mixed(unsigned grid, cudaStream_t stream, const PcgArgs& a);
// relative tests: a.xs[s] = split_bits(v_s) for the precise product of the next pass; runs
// only when gate is null or *gate != 0
__global__ void k_split_x(PcgArgs a, const double* v0, const double* v1, const int* gate);
__global__ void k_bicg_dir_mixed(PcgArgs a);
// learned-guess judge: r.z of the candidate (cand[s]) per solve when gflag[0] is set
__global__ void k_guess_judge(PcgArgs a, const double* cand0, const double* cand1, double* rr);
__global__ void k_guess_extrapolate(PcgArgs a, const double* dtn_p, double* hist,
                                    double* xprev0, double* xprev1);
__global__ void k_guess_extrapolate_hist(const double* dtn_p, double* hist);
// per solve, the candidate replaces x (and its shadow) when its r.z is the smaller; sets
// gflag[1]; stats[0..3) += (gate open, solve 0 took it, solve 1 took it)
__global__ void k_guess_select(PcgArgs a, const double* cand0, const double* cand1,
                               const double* rr, long long* stats);

}  // namespace cfd

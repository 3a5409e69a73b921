// cfd_context.cuh — the resident context (one mesh, its state and every work array in HBM).
#pragma once
#include <string>
#include <vector>

#include "cfd_kernels.cuh"
#include "host_prep.h"
#include "newmark.h"

struct cfd_mpnn;
struct cfd_mpnn_graph;

namespace cfd {

namespace mpnn {
int graph_build(cfd_mpnn_graph** out, int npoin, const std::vector<int>& rowptr,
                const std::vector<int>& col, const double* x, const double* y, int nb,
                const int* bnode0, const int* bkind, bool training, cudaStream_t st);
int guess_on_stream(cfd_mpnn* net, cfd_mpnn_graph* g, cudaStream_t st, const double* X,
                    const double* Y, const double* bgx, const double* bgy, double* ux,
                    double* uy, const int* gate);
void graph_free(cfd_mpnn_graph* g);
int fields_seed(cfd_mpnn_graph* g, cudaStream_t st);
int fields_guess(cfd_mpnn_graph* g, cudaStream_t st, const double* X, const double* Y,
                 const double* bgx, const double* bgy, const double* x0, const double* x1,
                 double* c0, double* c1);
int fields_update(cfd_mpnn_graph* g, cudaStream_t st, const double* x0, const double* x1);
}  // namespace mpnn

// mesh smoothing (smooth.cu)
__global__ void k_smooth_prep(int n, const double* xpos, const double* ypos, const double* X,
                              const double* Y, double* tol, double* xb, double* yb);
__global__ void k_smooth_w(int n, const double* xpos, const double* ypos, const double* X,
                           const double* Y, const double* xb, const double* yb,
                           const StepScal* sc, double* WX, double* WY, float2* Wf, float2* Xhi,
                           float2* Xlo);
void smoothing_colours(const Adjacency& adj, int npoin, std::vector<int>& order,
                       std::vector<int>& offs);
int smooth_on_device(cudaStream_t st, int npoin, int nelem, const int4* elem,
                     const int* esup_ptr, const int* esup_slot, const int* psup_ptr,
                     const int* psup, const unsigned char* fixed, double* X, double* Y,
                     const double* tol_move, const std::vector<int>& offs, const int* order,
                     unsigned char* smoothable, unsigned long long* scal, int* flags,
                     int* iters_out, double* min_quality_out, int max_star,
                     bool node_order = false);

enum { TM_DELTAT, TM_ESTAB, TM_CALCRHS, TM_FUENTE, TM_UPDATE, TM_FORCES, TM_TRANSF, TM_GRAD,
       TM_NORMALES, TM_DERIV, TM_MASAS, TM_LAPLACE, TM_N };

void set_last_message(const std::string& m);
std::string last_message();

struct Ctx {
    int npoin = 0, nelem = 0, prec = 0;
    long nnz = 0;  // entries of the mesh-motion matrix (CSR, diagonal first in each row)
    cfd_params prm{};
    Adjacency adj;
    BcTables bc;
    cudaStream_t stream = nullptr;
    // mixed form: the mesh-motion solve's stream, forked from and joined to `stream`
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // the refined learned guess's own kernels beside the mesh-motion branch (stream3): the
    // fields' guess beside the first residual pass, their update beside the mesh update
    cudaStream_t stream3 = nullptr;
    cudaEvent_t ev_side[4] = {};
    bool side_join = false;  // the branch still has to wait for ev_side[3]
    cudaEvent_t ev_scal = nullptr;
    StepScal* h_scal = nullptr;  // pinned
    StepOut* h_out = nullptr;    // pinned step report
    StepOut* d_out = nullptr;
    std::vector<void*> allocs;
    // time-loop scalars kept on the host
    int iter = 0;
    int bandera_host = 1;
    double time = 0.0, last_dtmin = 0.0;
    double disn[2] = {0.0, 0.0};
    NewmarkState nm{};  // FP64 form, CFD_MOTION_NEWMARK: velocities and accelerations
    // sizes
    int nwn = 0, nnmove = 0, nufix = 0, pcg_grid = 1, nsm = 1;
    // mesh
    int4* d_elem = nullptr;
    double *d_X = nullptr, *d_Y = nullptr;
    int *d_esup_ptr = nullptr, *d_esup_slot = nullptr;
    uchar4* d_lap_pos = nullptr;
    int *d_rowptr = nullptr, *d_col = nullptr;
    double *d_val = nullptr, *d_diag = nullptr;
    // BC
    unsigned char* d_bcflag = nullptr;
    double* d_bcval = nullptr;
    double2* d_nrm = nullptr;
    int *d_wnode = nullptr, *d_wptr = nullptr;
    int2 *d_wedge = nullptr, *d_walls = nullptr;
    int* d_set_ptr = nullptr;
    int2* d_set_edges = nullptr;
    int* d_set_elem = nullptr;
    // FORCE_VISC: [F_VX(10), F_VY(10)], per-edge terms (scratch) and SKIN.DAT rows
    double *d_fv = nullptr, *d_fv_terms = nullptr, *d_fv_skin = nullptr;
    bool fv_each = false;
    // mesh smoothing: point neighbours, fixed nodes, colour order, scratch
    int *d_psup_ptr = nullptr, *d_psup = nullptr, *d_sm_order = nullptr, *d_sm_flags = nullptr;
    unsigned char *d_sm_fixed = nullptr, *d_sm_flag = nullptr;
    unsigned long long* d_sm_scal = nullptr;
    std::vector<int> sm_offs;
    double *d_xref = nullptr, *d_yref = nullptr;
    int *d_fix_node = nullptr, *d_fix_set = nullptr, *d_ufix_node = nullptr, *d_ufix_src = nullptr;
    unsigned char* d_isfix = nullptr;
    // state
    double *d_U = nullptr, *d_U1 = nullptr, *d_T = nullptr, *d_VX = nullptr, *d_VY = nullptr;
    double *d_RHO = nullptr, *d_E = nullptr, *d_P = nullptr, *d_RMACH = nullptr;
    double *d_WX = nullptr, *d_WY = nullptr, *d_M = nullptr, *d_Wxo = nullptr, *d_Wyo = nullptr;
    double *d_area = nullptr, *d_area_old = nullptr, *d_geo = nullptr, *d_DT = nullptr,
           *d_DTL = nullptr;
    double *d_SHOC = nullptr, *d_TS1 = nullptr, *d_TS2 = nullptr, *d_TS3 = nullptr;
    double *d_contrib = nullptr, *d_contribF = nullptr;
    double* d_einv = nullptr;  // FP64 form: calcRHS's stage-invariant addends (per element)
    // mixed precision: float shadows (FP64 arrays above are widened from them on download)
    float4 *d_Uhi = nullptr, *d_Ulo = nullptr;  // U = hi + lo
    float2 *d_Xhi = nullptr, *d_Xlo = nullptr;  // (X, Y) = hi + lo
    float2 *d_Wf = nullptr, *d_Wof = nullptr;   // W and the gcl's previous W
    float* d_Tf = nullptr;                      // T
    float2* d_mulam = nullptr;                  // per element: mu, lambda of the RK stage
    float *d_VXf = nullptr, *d_VYf = nullptr, *d_RHOf = nullptr, *d_Ef = nullptr, *d_Pf = nullptr,
          *d_RMACHf = nullptr;
    float *d_invMf = nullptr, *d_areaf = nullptr;  // 1/M, element area (FP32 passes)
    float4* d_geo8 = nullptr;  // per element: dNx(1:3), dNy(1:3), area, Laplacian weight
    unsigned long long* d_blockmin = nullptr;  // per-block FP32 DTELEM minima
    double* d_invdiag = nullptr;
    float* d_valf = nullptr;
    float* d_val_lo = nullptr;
    double* d_rdiag = nullptr;   // FP64 form: RN(1/diag) of the BiCG (formed by each solve)
    double* d_lapq = nullptr;    // FP64 form: the Laplacian weight per element
    double2* d_gcl64 = nullptr;  // FP64 form: the gcl element terms   // relative tests: valf + val_lo = the FP64-assembled matrix
    float2* d_k64 = nullptr;     // relative tests: element-matrix rows (hi, lo), per slot (3 each)
    int* d_iterated = nullptr;   // relative tests: a solve iterated (the refinement runs)
    float2* d_xs[2] = {};        // relative tests: split_bits of the precise product's operand
    float2* d_xs_c[2] = {};      // the same for the learned guess's candidates (k_guess_judge)
    float* d_dtef = nullptr;  // mixed form, ITLOCAL != 0: FP32 DT per element
    float* d_pf[2][2] = {};
    float* d_zf[2] = {};
    float* d_posf[2] = {};  // (float) of d_pos, kept by the mixed BiCG kernels
    double* d_part_r = nullptr;  // per-block partials of the mixed BiCG row kernels
    double* d_bscal = nullptr;   // [2][4] first-direction scalars of the mixed BiCG
    unsigned* d_bcount = nullptr;
    float* d_invdiagf = nullptr;
    // learned guess (mixed form, CFD_GUESS_LEARNED): the network (not owned), its graph of
    // this mesh, the candidate guesses, gate flags, judge sums and counters
    cfd_mpnn* net = nullptr;
    cfd_mpnn_graph* lgraph = nullptr;
    double* d_cand[2] = {};
    int* d_gflag = nullptr;
    double* d_grr = nullptr;
    long long* d_gstats = nullptr;
    double guess_gate = 0.0;     // 0: every solve; > 0: iterations of the previous solve
                                 // above which the network runs
    bool guess_first = false;    // the first solve after attaching runs the network
    long long guess_steps = 0;
    // refined learned guess (cfd_ctx_set_guess_refine): per-node basis fields seeded by the
    // network's run and corrected by every solve; each solve between network runs also
    // tries the fields' guess, and keeps the better of it and the previous step's
    bool guess_refine = false;
    bool fields_ready = false;   // the fields were seeded since the network was attached
    // CFD_GUESS_EXTRAPOLATED: the previous step's solutions and the history of DTMIN
    double* d_xprev[2] = {};
    double* d_xhist = nullptr;        // (dt1, dt2, solutions kept)
    int* h_iters = nullptr;      // pinned copy of the last solve's iteration counts
    cudaEvent_t ev_iters = nullptr;  // recorded after that copy
    // mixed form: the clock and the motion increment live on the device
    MotionScal* d_motion = nullptr;
    unsigned* d_tcount = nullptr;  // last-block counters: [0] DTMIN refinement, [1] motion tail
    double* d_tpart = nullptr;     // per-block force sums of the motion tail
    int tail_blocks = 1;
    // mixed form: one step (the network not run) captured as a CUDA graph and replayed;
    // off with the timers or CFD_GRAPHS=0, or when the capture fails
    bool graphs_on = false, capturing = false;
    cudaGraph_t step_graph[2] = {nullptr, nullptr};   // per buffer parity (below)
    cudaGraphExec_t step_exec[2] = {nullptr, nullptr};
    // mixed form: what the mesh-motion branch writes for the next step while the RK stages
    // read the current values; swapped after every step (parity `buf`)
    float4* d_geo8_n = nullptr;
    float* d_invMf_n = nullptr;
    double *d_WX_n = nullptr, *d_WY_n = nullptr;
    float2* d_Wf_n = nullptr;
    double4_32a* d_fgeo = nullptr;  // per force-set edge: the step-start edge geometry
    int buf = 0;
    long long graph_kernels = 0;  // kernels of one replay
    long long mixed_steps = 0;    // steps of this context (the first runs uncaptured)
    long long graph_replays = 0;
    int* d_slot_pos = nullptr;
    float4 *d_recInv = nullptr, *d_recVisc = nullptr;  // slot records, element-around-point order
    float4* d_invSum = nullptr;                         // per node: sum of the recInv slots
    double2* d_gterms = nullptr;  // gcl element terms (FP64)
    double estab_eps = 1.0e-3;  // CFD_ESTAB_REGULARIZED relative gradient scale
    double dir[2] = {1.0, 0.0};  // CFD_ESTAB_REGULARIZED freestream direction
    // mesh motion
    double* d_pos[2] = {nullptr, nullptr};  // xpos, ypos (guess in, solution out)
    double* d_xfix[2] = {nullptr, nullptr};
    double *d_r[2] = {}, *d_z[2] = {}, *d_y[2] = {};
    double* d_p[2][2] = {};
    double* d_part = nullptr;
    GridBar* d_bar = nullptr;
    int *d_pcg_iters = nullptr, *d_pcg_conv = nullptr;
    double* d_pcg_rz = nullptr;
    StepScal* d_scal = nullptr;
    // timers
    bool timers_on = false;
    std::vector<cudaEvent_t> pool;  // event pairs of the timed groups of one step
    size_t pool_next = 0;
    int open_pair[TM_N] = {};
    std::vector<std::pair<int, int>> pending;  // (slot, pair) recorded, not yet read
    cudaEvent_t mark[8] = {};  // caller-requested events (cfd_ctx_mark)
    long long calls[TM_N] = {};
    double seconds[TM_N] = {};

    ~Ctx();
    int create(const cfd_mesh* m, const cfd_params* p, int precision_mode);
    int geometry(bool masas, bool with_laplace);
    int geometry_mixed(bool setup, bool put_area = false, bool to_next = false,
                       cudaStream_t sv = nullptr);
    void swap_mixed_buffers();
    unsigned branch_grid(long n, int threads, cudaStream_t s) const;
    int branch_bpsm = 0;
    int node_bulk = 0;          // dynamic smem of the bulk-copy node pass (0: not used)
    int* d_node_err = nullptr;  // its bounded wait's error flag  // mesh-motion branch: blocks per SM of its grid-stride kernels
    void drop_graphs();
    int narrow_mixed(bool U, bool T, bool VX, bool VY, bool XY, bool W);
    int widen_mixed(int what);
    int run_pcg(int nsolve, bool learned = false, bool fix_done = false,
                cudaStream_t sv = nullptr);
    int set_guess_refine(bool on);
    int guess_buffers();
    bool learned_mode() const {
        return prm.guess_mode == CFD_GUESS_LEARNED || prm.guess_mode == CFD_GUESS_LEARNED_EXTRAPOLATED;
    }
    bool extrap_mode() const {
        return prm.guess_mode == CFD_GUESS_EXTRAPOLATED ||
               prm.guess_mode == CFD_GUESS_LEARNED_EXTRAPOLATED;
    }
    int guess_extrapolate(const PcgArgs& a, cudaStream_t s, unsigned grid);
    int enqueue_mixed(bool learned);
    int launch_step_graph(bool* launched);
    int set_guess_net(cfd_mpnn* n, double gate);
    int force_visc_now();
    int smooth(int* iters, double* min_quality, bool node_order = false);
    int smooth_setup();
    int set_smoothing(int every);
    int smooth_in_step(cudaStream_t s, double* WX, double* WY, float2* Wf);
    int smooth_every = 0;  // smooth the moved mesh every this many steps (0: never)
    double *d_sm_tol = nullptr, *d_sm_xb = nullptr, *d_sm_yb = nullptr;
    long long smooth_steps = 0, smooth_sweeps = 0;
    int smooth_max_star = -1;
    bool smoothing_now = false;
    int set_force_visc_each_step(bool on);
    int step_once();
    int step_once_mixed();
    int step(int nsteps, cfd_step_report* rep);
    int tstart(int slot);
    int tstop(int slot, int ncalls = 1);
    int tcollect();
    template <class T>
    int dalloc(T** p, size_t n);
    template <class T>
    int upload(T** p, const T* h, size_t n);
};

}  // namespace cfd

struct cfd_ctx {
    cfd::Ctx impl;
};

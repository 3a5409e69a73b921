// context.cu — the resident context: device buffers, setup and the time-step loop body
// of ns2DComp.ALE.f90:140-280 as a sequence of sm_103a kernels on one stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "cfd_context.cuh"

namespace cfd {

std::atomic<long long> g_launches{0};
static std::mutex g_err_mu;
static std::string g_last_err;

void set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    char buf[512];
    snprintf(buf, sizeof(buf), "%s: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    g_last_err = buf;
}

void set_last_message(const std::string& m) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_last_err = m;
}

std::string last_message() {
    std::lock_guard<std::mutex> lk(g_err_mu);
    return g_last_err;
}

static const char* kTimerNames[TM_N] = {"deltat_t", "estab_t",  "calcrhs_t", "fuente_t",
                                        "update_t", "forces_t", "transf_t",  "grad_t",
                                        "normales_t", "deriv_t", "masas_t",  "laplace_t"};

// ------------------------------------------------------------------ timers
// Every tstart/tstop pair takes a fresh pair of events from a pool, so a group timed
// several times per step (the 4 RK stages) accumulates every launch.
int Ctx::tstart(int slot) {
    if (!timers_on) return CFD_OK;
    if (2 * (pool_next + 1) > pool.size()) {
        for (int j = 0; j < 2; ++j) {
            cudaEvent_t e;
            CFD_CUDA(cudaEventCreate(&e));
            pool.push_back(e);
        }
    }
    open_pair[slot] = (int)pool_next++;
    CFD_CUDA(cudaEventRecord(pool[2 * open_pair[slot]], stream));
    return CFD_OK;
}
// ncalls: launches of the group the interval covers (one event pair around several)
int Ctx::tstop(int slot, int ncalls) {
    if (!timers_on) return CFD_OK;
    CFD_CUDA(cudaEventRecord(pool[2 * open_pair[slot] + 1], stream));
    pending.push_back(std::make_pair(slot, open_pair[slot]));
    calls[slot] += ncalls;
    return CFD_OK;
}
int Ctx::tcollect() {
    if (!timers_on) return CFD_OK;
    CFD_CUDA(cudaStreamSynchronize(stream));
    for (auto& sp : pending) {
        float ms = 0.f;
        CFD_CUDA(cudaEventElapsedTime(&ms, pool[2 * sp.second], pool[2 * sp.second + 1]));
        seconds[sp.first] += ms * 1e-3;
    }
    pending.clear();
    pool_next = 0;
    return CFD_OK;
}

Ctx::~Ctx() {
    if (stream) cudaStreamSynchronize(stream);
    if (lgraph) mpnn::graph_free(lgraph);
    for (void* p : allocs) cudaFree(p);
    if (h_scal) cudaFreeHost(h_scal);
    if (h_out) cudaFreeHost(h_out);
    if (h_iters) cudaFreeHost(h_iters);
    drop_graphs();
    if (ev_iters) cudaEventDestroy(ev_iters);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (ev_scal) cudaEventDestroy(ev_scal);
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
    for (auto& m : mark)
        if (m) cudaEventDestroy(m);
    for (cudaEvent_t e : ev_side)
        if (e) cudaEventDestroy(e);
    if (stream3) cudaStreamDestroy(stream3);
    if (stream2) cudaStreamDestroy(stream2);
    if (stream) cudaStreamDestroy(stream);
}

// ------------------------------------------------------------------ geometry of the mesh
int Ctx::geometry(bool masas, bool with_laplace) {
    const int N = npoin, E = nelem;
    const int TB = 256;
    tstart(TM_NORMALES);
    if (nwn > 0)
        CFD_LAUNCH(k_normales, blocks_for(nwn, TB), TB, 0, stream, nwn, d_wnode, d_wptr,
                   d_wedge, d_walls, d_X, d_Y, d_bcflag, d_nrm);
    tstop(TM_NORMALES);
    tstart(TM_DERIV);
    CFD_LAUNCH(k_deriv, blocks_for(E, TB), TB, 0, stream, E, d_elem, d_X, d_Y, d_area, d_geo,
               (double*)nullptr, (double*)nullptr, (double*)nullptr);
    tstop(TM_DERIV);
    if (masas) {
        tstart(TM_MASAS);
        CFD_LAUNCH(k_mass, blocks_for(N, TB), TB, 0, stream, N, d_esup_ptr, d_esup_slot, d_area, d_M);
        tstop(TM_MASAS);
    }
    if (with_laplace) {
        tstart(TM_LAPLACE);
        CFD_CUDA(launch_laplace(stream, N, E, d_elem, d_esup_ptr, d_esup_slot, d_lap_pos, d_geo,
                                d_X, d_Y, d_rowptr, d_lapq, d_val, d_diag));
        tstop(TM_LAPLACE);
    }
    return CFD_OK;
}

// ------------------------------------------------------------------ PCG launch
// CFD_GUESS_EXTRAPOLATED: x becomes the last two increments extrapolated to this step's
// DTMIN (k_guess_extrapolate), then the history moves on
int Ctx::guess_extrapolate(const PcgArgs& a, cudaStream_t s, unsigned grid) {
    const double* dtn = &d_scal->dtmin;
    CFD_LAUNCH(k_guess_extrapolate, std::min(grid, (unsigned)(4 * nsm)), 256, 0, s, a, dtn, d_xhist,
               d_xprev[0], d_xprev[1]);
    CFD_LAUNCH(k_guess_extrapolate_hist, 1, 32, 0, s, dtn, d_xhist);
    return CFD_OK;
}

int Ctx::run_pcg(int nsolve, bool learned, bool fix_done, cudaStream_t sv) {
    const cudaStream_t stream = sv ? sv : this->stream;  // the solve's stream
    PcgArgs a{};
    a.n = npoin;
    a.nsolve = nsolve;
    a.rowptr = d_rowptr;
    a.col = d_col;
    a.val = d_val;
    a.diag = d_diag;
    a.rdiag = d_rdiag;  // null in the mixed form
    a.isfix = d_isfix;
    a.nfix = nufix;
    a.fix_node = d_ufix_node;
    a.fix_src = d_ufix_src;
    for (int s = 0; s < 2; ++s) {
        a.fixval[s] = d_xfix[s];
        a.x[s] = d_pos[s];
        a.b[s] = nullptr;
        a.r[s] = d_r[s];
        a.z[s] = d_z[s];
        a.y[s] = d_y[s];
        a.p[s][0] = d_p[s][0];
        a.p[s][1] = d_p[s][1];
    }
    a.part = d_part;
    a.bar = d_bar;
    a.tol = prm.bicg_tol;
    a.maxit = prm.bicg_maxit;
    a.tol_mode = prm.bicg_tol_mode;
    a.iters_out = d_pcg_iters;
    a.rz_out = d_pcg_rz;
    a.relres_out = d_pcg_rz + 2;
    a.conv_out = d_pcg_conv;
    const bool mixed = (prec == CFD_PREC_MIXED);
    if (mixed) {
        a.valf = d_valf;
        a.val_lo = d_val_lo;
        a.invdiag = d_invdiag;
        for (int s = 0; s < 2; ++s) {
            a.pf[s][0] = d_pf[s][0];
            a.pf[s][1] = d_pf[s][1];
            a.zf[s] = d_zf[s];
            a.xf[s] = d_posf[s];
            a.xs[s] = d_xs[s];
        }
        a.invdiagf = d_invdiagf;
        a.part_r = d_part_r;
        a.nblk_r = blocks_for(npoin, 256);
        a.bscal = d_bscal;
        a.bcount = d_bcount;
        // learned guess (decided by the caller): k_guess_judge keeps, per solve, the
        // network's guess or the previous step's, whichever has the smaller r.z.  Between
        // network runs, with the refined guess on, the candidate is the fields' guess.
        const bool with_net = learned_mode() && net && lgraph;
        const bool fields = with_net && guess_refine && !learned && fields_ready;
        a.gflag = (learned || fields) ? d_gflag : nullptr;
        a.gate = 0.0;
        a.gate_undone = fields ? 1 : 0;  // the fields' guess is judged when the first one fails
        a.only_if = nullptr;
        if (nufix > 0 && !fix_done)
            CFD_LAUNCH(k_bicg_fix_mixed, blocks_for(nufix, 256), 256, 0, stream, a);
        // beside the RK stages (sv: the branch stream) the row kernels take a smaller grid
        const unsigned rgrid = (sv && branch_bpsm > 0)
                                   ? (unsigned)std::min<long>(a.nblk_r, (long)branch_bpsm * nsm)
                                   : (unsigned)a.nblk_r;
        if (extrap_mode()) {
            int st = guess_extrapolate(a, stream, rgrid);
            if (st) return st;
        }
        // the relative tests' precise products read x (and the candidates) split in hi + lo
        const bool split = prm.bicg_tol_mode != CFD_BICG_TOL_ABS;
        // on the mesh-motion branch the fields' guess (boundary fit, guess, its split) runs on
        // stream3 beside the first pass: it reads the mesh, the Dirichlet values and the
        // fields, and writes only the candidates and their split
        const bool side = fields && sv != nullptr;
        const unsigned gsz = std::min((unsigned)a.nblk_r, (unsigned)(4 * nsm));
        PcgArgs ac = a;  // the judge's arguments: the candidates' split
        for (int s = 0; s < 2; ++s) ac.xs[s] = d_xs_c[s];
        auto cand_guess = [&](cudaStream_t cs) -> int {
            int st = mpnn::fields_guess(lgraph, cs, d_X, d_Y, d_xfix[0], d_xfix[1], d_pos[0],
                                        d_pos[1], d_cand[0], d_cand[1]);
            if (st) return st;
            if (split)  // ungated: beside the first pass, which sets the gate, on the branch
                CFD_LAUNCH(k_split_x, gsz, 256, 0, cs, ac, (const double*)d_cand[0],
                           (const double*)d_cand[1], (const int*)nullptr);
            return CFD_OK;
        };
        if (side) {
            CFD_CUDA(cudaEventRecord(ev_side[0], stream));
            CFD_CUDA(cudaStreamWaitEvent(stream3, ev_side[0], 0));
            int st = cand_guess(stream3);
            if (st) return st;
            CFD_CUDA(cudaEventRecord(ev_side[1], stream3));
        }
        if (split)
            CFD_LAUNCH(k_split_x, rgrid, 256, 0, stream, a, (const double*)d_pos[0],
                       (const double*)d_pos[1], (const int*)nullptr);
        CFD_CUDA(launch_bicg_resid_mixed(rgrid, stream, a));
        if (fields) {
            if (side) {
                CFD_CUDA(cudaStreamWaitEvent(stream, ev_side[1], 0));
            } else {
                int st = cand_guess(stream);
                if (st) return st;
            }
            CFD_LAUNCH(k_guess_judge, gsz, 256, 0, stream, ac, (const double*)d_cand[0],
                       (const double*)d_cand[1], d_grr);
            CFD_LAUNCH(k_guess_select, gsz, 256, 0, stream, a, (const double*)d_cand[0],
                       (const double*)d_cand[1], (const double*)d_grr, d_gstats + 4);
            PcgArgs b = a;
            b.only_if = d_gflag + 1;
            if (split)
                CFD_LAUNCH(k_split_x, gsz, 256, 0, stream, b, (const double*)d_pos[0],
                           (const double*)d_pos[1], b.only_if);
            CFD_CUDA(launch_bicg_resid_mixed(gsz, stream, b));
        }
        if (learned) {
            // the network runs only when the previous-step guess leaves r.z >= gate; its
            // guess replaces it, per solve, when its r.z is the smaller; the first pass is
            // then redone on the chosen guess
            int st = mpnn::guess_on_stream(net, lgraph, stream, d_X, d_Y, d_xfix[0], d_xfix[1],
                                           d_cand[0], d_cand[1], d_gflag);
            if (st) return st;
            // grid-stride grids of a few waves: a closed gate costs little
            if (split)
                CFD_LAUNCH(k_split_x, gsz, 256, 0, stream, ac, (const double*)d_cand[0],
                           (const double*)d_cand[1], (const int*)d_gflag);
            CFD_LAUNCH(k_guess_judge, gsz, 256, 0, stream, ac, (const double*)d_cand[0],
                       (const double*)d_cand[1], d_grr);
            CFD_LAUNCH(k_guess_select, gsz, 256, 0, stream, a, (const double*)d_cand[0],
                       (const double*)d_cand[1], (const double*)d_grr, d_gstats);
            PcgArgs b = a;
            b.only_if = d_gflag + 1;
            if (split)
                CFD_LAUNCH(k_split_x, gsz, 256, 0, stream, b, (const double*)d_pos[0],
                           (const double*)d_pos[1], b.only_if);
            CFD_CUDA(launch_bicg_resid_mixed(gsz, stream, b));
            if (guess_refine) {
                if ((st = mpnn::fields_seed(lgraph, stream))) return st;
                fields_ready = true;
            }
        }
        CFD_LAUNCH(k_bicg_dir_mixed, rgrid, 256, 0, stream, a);
    }
    if (!mixed && extrap_mode()) {
        int st = guess_extrapolate(a, stream, blocks_for(npoin, 256));
        if (st) return st;
    }
    CFD_CUDA(cudaMemsetAsync(d_bar, 0, sizeof(GridBar), stream));
    if (mixed && prm.bicg_tol_mode == CFD_BICG_TOL_REL) a.iterated = d_iterated;
    void* args[] = {&a};
    CFD_CUDA(cudaLaunchCooperativeKernel(mixed ? (void*)k_pcg_mixed : (void*)k_pcg_fp64, dim3(pcg_grid),
                                         dim3(256), args, 0, stream));
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (mixed && prm.bicg_tol_mode == CFD_BICG_TOL_REL) {
        // refinement: the FP32 iterations meet the test on their recursive residual; the
        // precise residual of the solution (against the FP64-assembled matrix) is formed
        // again, and the solves that it leaves above the test iterate once more
        PcgArgs b = a;
        b.gflag = nullptr;
        b.only_if = d_iterated;  // nothing to refine where no solve moved from its guess
        b.iterated = nullptr;
        b.accumulate = 1;
        const unsigned rgrid = (sv && branch_bpsm > 0)
                                   ? (unsigned)std::min<long>(b.nblk_r, (long)branch_bpsm * nsm)
                                   : (unsigned)b.nblk_r;
        CFD_LAUNCH(k_split_x, rgrid, 256, 0, stream, b, (const double*)d_pos[0],
                   (const double*)d_pos[1], b.only_if);
        CFD_CUDA(launch_bicg_resid_mixed(rgrid, stream, b));
        CFD_LAUNCH(k_bicg_dir_mixed, rgrid, 256, 0, stream, b);
        CFD_CUDA(cudaMemsetAsync(d_bar, 0, sizeof(GridBar), stream));
        void* bargs[] = {&b};
        CFD_CUDA(cudaLaunchCooperativeKernel((void*)k_pcg_mixed, dim3(pcg_grid), dim3(256), bargs, 0,
                                             stream));
        g_launches.fetch_add(1, std::memory_order_relaxed);
    }
    // refined learned guess: the solutions correct the basis fields (on the branch: on
    // stream3 beside the mesh update, which reads the solutions too; the branch waits for it
    // at its end, side_join)
    if (mixed && learned_mode() && net && lgraph && guess_refine &&
        fields_ready) {
        if (sv != nullptr) {
            CFD_CUDA(cudaEventRecord(ev_side[2], stream));
            CFD_CUDA(cudaStreamWaitEvent(stream3, ev_side[2], 0));
            int st = mpnn::fields_update(lgraph, stream3, d_pos[0], d_pos[1]);
            if (st) return st;
            CFD_CUDA(cudaEventRecord(ev_side[3], stream3));
            side_join = true;
        } else {
            int st = mpnn::fields_update(lgraph, stream, d_pos[0], d_pos[1]);
            if (st) return st;
        }
    }
    if (h_iters) {  // the next step's learned-guess decision reads these
        CFD_CUDA(cudaMemcpyAsync(h_iters, d_pcg_iters, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                                 stream));
        // inside a capture the record becomes a node of the graph
        CFD_CUDA(cudaEventRecordWithFlags(ev_iters, stream,
                                          capturing ? cudaEventRecordExternal : cudaEventRecordDefault));
    }
    return CFD_OK;
}

// Attach the learned-guess network (mixed form): builds the network's graph of this mesh
// (neighbours = the Laplacian pattern, boundary = the mesh-motion Dirichlet list: moving
// entries are the body, the others the fixed outer boundary).
int Ctx::set_guess_net(cfd_mpnn* n, double gate) {
    if (prec != CFD_PREC_MIXED) {
        set_last_message("the learned guess runs in the mixed-precision form");
        return CFD_ERR_ARG;
    }
    if (nnmove <= 0) {
        set_last_message("the mesh has no mesh-motion boundary nodes");
        return CFD_ERR_ARG;
    }
    net = n;
    guess_gate = gate;
    guess_first = true;
    guess_steps = 0;
    fields_ready = false;
    drop_graphs();
    if (d_gstats) CFD_CUDA(cudaMemsetAsync(d_gstats, 0, 8 * sizeof(long long), stream));
    if (!n) return CFD_OK;
    if (!lgraph) {
        const int N = npoin;
        std::vector<double> x(N), y(N);
        CFD_CUDA(cudaMemcpyAsync(x.data(), d_X, sizeof(double) * N, cudaMemcpyDeviceToHost, stream));
        CFD_CUDA(cudaMemcpyAsync(y.data(), d_Y, sizeof(double) * N, cudaMemcpyDeviceToHost, stream));
        CFD_CUDA(cudaStreamSynchronize(stream));
        std::vector<int> bkind(nnmove);
        for (int k = 0; k < nnmove; ++k) bkind[k] = bc.fix_set[k] >= 0 ? 1 : 2;
        int st = mpnn::graph_build(&lgraph, N, adj.rowptr, adj.col, x.data(), y.data(), nnmove,
                                   bc.fix_node.data(), bkind.data(), false, stream);
        if (st) return st;
        if ((st = guess_buffers())) return st;
        CFD_CUDA(cudaMallocHost((void**)&h_iters, 2 * sizeof(int)));
        h_iters[0] = h_iters[1] = 0;
        // the captured step has no copy of the counts yet: capture it again
        drop_graphs();
        CFD_CUDA(cudaMemsetAsync(d_gflag, 0, 2 * sizeof(int), stream));
        CFD_CUDA(cudaMemsetAsync(d_gstats, 0, 8 * sizeof(long long), stream));
        CFD_CUDA(cudaStreamSynchronize(stream));
    }
    return CFD_OK;
}

// The candidate buffers, gate flags, judge sums and counters of the guess selection
// (allocated once, by the first of set_guess_net and set_guess_extrapolate)
int Ctx::guess_buffers() {
    if (d_gstats) return CFD_OK;
    int st;
    for (int s = 0; s < 2; ++s)
        if ((st = dalloc(&d_cand[s], npoin))) return st;
    if ((st = dalloc(&d_gflag, 2))) return st;
    if ((st = dalloc(&d_grr, 2))) return st;
    if ((st = dalloc(&d_gstats, 8))) return st;
    CFD_CUDA(cudaMemsetAsync(d_gflag, 0, 2 * sizeof(int), stream));
    CFD_CUDA(cudaMemsetAsync(d_gstats, 0, 8 * sizeof(long long), stream));
    return CFD_OK;
}

// Refined learned guess on or off: the network runs again on the next solve (which seeds
// the fields) and the captured step is captured again with or without the fields' kernels.
int Ctx::set_guess_refine(bool on) {
    guess_refine = on;
    fields_ready = false;
    guess_first = true;
    drop_graphs();
    return CFD_OK;
}

// ------------------------------------------------------------------ FORCE_VISC
// ns2DComp.ALE.f90:819-893 on the current fields, mesh and dNx into d_fv (F_VX, F_VY) and
// d_fv_skin (the SKIN.DAT rows)
int Ctx::force_visc_now() {
    const int ne = (int)bc.set_elem.size();
    if (!d_fv) {
        int st;
        if ((st = dalloc(&d_fv, 20))) return st;
        if ((st = dalloc(&d_fv_terms, 2 * (size_t)ne))) return st;
        if ((st = dalloc(&d_fv_skin, 3 * (size_t)ne))) return st;
    }
    const bool mixed = prec == CFD_PREC_MIXED;
    const size_t E = (size_t)nelem;
    CFD_CUDA(launch_force_visc(
        stream, mixed ? 1 : 0, bc.nset_numb, d_set_ptr, ne, d_set_edges, d_set_elem, d_elem,
        d_geo, d_geo ? d_geo + 3 * E : nullptr, 1, E, d_geo8,
        mixed ? (const void*)d_Pf : (const void*)d_P, mixed ? (const void*)d_Tf : (const void*)d_T,
        mixed ? (const void*)d_VXf : (const void*)d_VX, mixed ? (const void*)d_VYf : (const void*)d_VY,
        d_X, d_Y, prm.u_inf, prm.v_inf, prm.rho_inf, prm.t_inf, d_fv_terms, d_fv_skin, d_fv));
    return CFD_OK;
}

// The smoothing's adjacency, node colours and fixed nodes (the moving and the fixed
// mesh-motion nodes stay), uploaded once
int Ctx::smooth_setup() {
    const int N = npoin;
    int st;
    if (!d_psup_ptr) {
        if ((st = upload(&d_psup_ptr, adj.psup_ptr.data(), adj.psup_ptr.size()))) return st;
        if ((st = upload(&d_psup, adj.psup.data(), adj.psup.size()))) return st;
        std::vector<int> order;
        smoothing_colours(adj, N, order, sm_offs);
        if ((st = upload(&d_sm_order, order.data(), order.size()))) return st;
        std::vector<unsigned char> fx(N, 0);
        for (int p : bc.fix_node) fx[p] = 1;
        if ((st = upload(&d_sm_fixed, fx.data(), fx.size()))) return st;
        if ((st = dalloc(&d_sm_flag, N))) return st;
        if ((st = dalloc(&d_sm_scal, 3))) return st;
        if ((st = dalloc(&d_sm_flags, 2))) return st;
    }
    return CFD_OK;
}

// The setup smoothing of the resident mesh (ns2DComp.ALE.f90:62-72), then the mesh's
// geometry again (normales, deriv, masses, Laplacian) as at setup
int Ctx::smooth(int* iters, double* min_quality, bool node_order) {
    const int N = npoin;
    int st = smooth_setup();
    if (st) return st;
    int max_star = 0;
    for (int p = 0; p < N; ++p) max_star = std::max(max_star, adj.esup_ptr[p + 1] - adj.esup_ptr[p]);
    st = smooth_on_device(stream, N, nelem, d_elem, d_esup_ptr, d_esup_slot, d_psup_ptr, d_psup,
                          d_sm_fixed, d_X, d_Y, nullptr, sm_offs, d_sm_order, d_sm_flag, d_sm_scal,
                          d_sm_flags, iters, min_quality, max_star, node_order);
    if (st) return st;
    if (prec == CFD_PREC_MIXED) {
        if ((st = narrow_mixed(false, false, false, false, true, false))) return st;
        if ((st = geometry_mixed(true, true))) return st;
    } else {
        if ((st = geometry(true, true))) return st;
        CFD_CUDA(cudaMemcpyAsync(d_area_old, d_area, sizeof(double) * nelem,
                                 cudaMemcpyDeviceToDevice, stream));
    }
    CFD_CUDA(cudaStreamSynchronize(stream));
    return tcollect();
}

// The per-step smoothing of the moved mesh (before its geometry): the setTol_move path of
// smoothing.f90:372-386 with the step's displacement, then W of the whole move
int Ctx::set_smoothing(int every) {
    if (every < 0) {
        set_last_message("smoothing interval below 0");
        return CFD_ERR_ARG;
    }
    int st;
    if (every > 0) {
        if ((st = smooth_setup())) return st;
        if (!d_sm_tol) {
            if ((st = dalloc(&d_sm_tol, npoin))) return st;
            if ((st = dalloc(&d_sm_xb, npoin))) return st;
            if ((st = dalloc(&d_sm_yb, npoin))) return st;
        }
        CFD_CUDA(cudaStreamSynchronize(stream));
    }
    smooth_every = every;
    return CFD_OK;
}

int Ctx::smooth_in_step(cudaStream_t s, double* WX, double* WY, float2* Wf) {
    const int N = npoin;
    int st;
    const unsigned g = blocks_for(N, 256);
    CFD_LAUNCH(k_smooth_prep, g, 256, 0, s, N, d_pos[0], d_pos[1], d_X, d_Y, d_sm_tol, d_sm_xb,
               d_sm_yb);
    if (smooth_max_star < 0) {
        smooth_max_star = 0;
        for (int p = 0; p < N; ++p)
            smooth_max_star = std::max(smooth_max_star, adj.esup_ptr[p + 1] - adj.esup_ptr[p]);
    }
    const int max_star = smooth_max_star;
    int iters = 0;
    st = smooth_on_device(s, N, nelem, d_elem, d_esup_ptr, d_esup_slot, d_psup_ptr, d_psup,
                          d_sm_fixed, d_X, d_Y, d_sm_tol, sm_offs, d_sm_order, d_sm_flag,
                          d_sm_scal, d_sm_flags, &iters, nullptr, max_star);
    if (st) return st;
    smooth_steps += 1;
    smooth_sweeps += iters;
    const bool mixed = prec == CFD_PREC_MIXED;
    CFD_LAUNCH(k_smooth_w, g, 256, 0, s, N, d_pos[0], d_pos[1], d_X, d_Y, d_sm_xb, d_sm_yb,
               (const StepScal*)d_scal,
               WX, WY, mixed ? Wf : (float2*)nullptr, mixed ? d_Xhi : (float2*)nullptr,
               mixed ? d_Xlo : (float2*)nullptr);
    return CFD_OK;
}

// Every step computes FORCE_VISC at the reference's print-block point (on), or only
// cfd_ctx_force_visc computes it, on the state and mesh of the call (off).  The captured
// step is captured again.
int Ctx::set_force_visc_each_step(bool on) {
    if (on == fv_each) return CFD_OK;
    fv_each = on;
    drop_graphs();
    if (on && !d_fv) return force_visc_now();  // buffers, and a defined first readout
    return CFD_OK;
}

// ------------------------------------------------------------------ one time step
int Ctx::step_once() {
    const int N = npoin, E = nelem;
    const int TB = 256;
    iter += 1;
    // DELTAT + hysteresis (ns2DComp.ALE.f90:144-156)
    tstart(TM_DELTAT);
    CFD_LAUNCH(k_deltat, blocks_for(E, TB), TB, 0, stream, E, d_elem, d_T, d_VX, d_VY, d_WX, d_WY,
               d_area, prm.fsafe, prm.t_inf, d_DT, &d_scal->dtmin_bits);
    CFD_LAUNCH(k_dt_finalize, 1, 1, 0, stream, d_scal);
    tstop(TM_DELTAT);
    CFD_CUDA(cudaMemcpyAsync(h_scal, d_scal, sizeof(StepScal), cudaMemcpyDeviceToHost, stream));
    CFD_CUDA(cudaEventRecord(ev_scal, stream));
    const double* dtl_arr = nullptr;
    if (prm.itlocal != 0) {  // :159-162
        double dtfact = 1.0 - std::exp(-(iter * 4.6 / prm.itlocal));
        CFD_LAUNCH(k_dtl, blocks_for(E, TB), TB, 0, stream, E, d_DT, d_DTL, d_scal, dtfact);
        dtl_arr = d_DTL;
    }
    const double* dtl_scalar = &d_scal->dtmin;
    // RK (subrutinas.f90:645-849): ESTAB once, then 4 stages of calcRHS+FUENTE and update
    tstart(TM_ESTAB);
    CFD_LAUNCH(k_estab, blocks_for(E, 128), 128, 0, stream, E, d_elem, d_U, d_T, prm.gama,
               (const double*)nullptr, d_VX,
               d_VY, d_WX, d_WY, d_geo, prm.fr, d_scal, prm.rho_inf, prm.t_inf, prm.estab_mode,
               estab_eps, dir[0], dir[1], d_SHOC, d_TS1, d_TS2, d_TS3);
    tstop(TM_ESTAB);
    GasConst gc{prm.fcv, prm.fk, prm.fmu, prm.gama, prm.t_inf, prm.cte, prm.fr};
    const bool viscous = prm.fmu > 2.2250738585072014e-308;
    const int NRK = 4;
    for (int irk = 1; irk <= NRK; ++irk) {
        const double rk_fact = 1.0 / (NRK + 1 - irk);
        // calcRHS and FUENTE see the step-start U in every stage (subrutinas.f90:685,
        // :1064): stage 1 forms FUENTE and calcRHS's stage-invariant addends, and every
        // stage replays the sums with its own viscous terms (bit-identical to evaluating
        // the whole element in each stage; without viscosity the stage-1 result is final)
        tstart(TM_CALCRHS);
        if (irk == 1)
            CFD_CUDA(launch_elem_inv(viscous, stream, E, d_elem, d_U, d_geo, d_area, d_SHOC,
                                     dtl_arr, dtl_scalar, d_TS1, d_TS2, d_TS3, gc, d_einv,
                                     d_contrib, d_WX, d_WY, d_contribF));
        if (viscous)
            CFD_CUDA(launch_elem_replay(stream, E, d_elem, d_T, d_geo, d_area, dtl_arr, dtl_scalar,
                                        gc, d_einv, d_contrib));
        tstop(TM_CALCRHS);
        tstart(TM_UPDATE);
        CFD_LAUNCH(k_node_update, blocks_for(N, TB), TB, 0, stream, N, d_esup_ptr, d_esup_slot,
                   d_contrib, d_contribF, d_U, d_M, rk_fact, prm.gama, prm.fr, d_bcflag,
                   (const double*)d_bcval, d_nrm, d_WX, d_WY, d_U1, d_RHO, d_VX, d_VY, d_E,
                   d_P, d_T, d_RMACH, (const double*)nullptr, (double*)nullptr);
        tstop(TM_UPDATE);
    }
    // fluidStructure (meshMove.f90:28-142) needs TIME: the host reads DTMIN
    CFD_CUDA(cudaEventSynchronize(ev_scal));
    const double dtmin = h_scal->dtmin;
    time = time + dtmin;
    last_dtmin = dtmin;
    tstart(TM_FORCES);
    CFD_LAUNCH(k_forces, 1, 256, 0, stream, bc.nset_numb, d_set_ptr, d_set_edges, d_P, d_X, d_Y,
               d_xref, d_yref, d_scal);
    tstop(TM_FORCES);
    const double PI = std::acos(-1.0);
    double alphav = disn[1], yposrv = disn[0];
    if (prm.motion_law == CFD_MOTION_HARMONIC) {
        double ph = 2.0 * PI * prm.motion_freq * time;
        disn[0] = prm.heave_amp * std::sin(ph);
        disn[1] = prm.pitch_amp * std::sin(ph);
    } else if (prm.motion_law == CFD_MOTION_NEWMARK) {
        // the structural model needs this step's set-1 force and moment
        CFD_CUDA(cudaMemcpyAsync(h_scal, d_scal, sizeof(StepScal), cudaMemcpyDeviceToHost, stream));
        CFD_CUDA(cudaStreamSynchronize(stream));
        double F[2];
        nm.dis[0] = disn[0];
        nm.dis[1] = disn[1];
        newmark_load(nm, h_scal->fx[0], h_scal->fy[0], h_scal->rm[0], F);
        newmark_step(nm, F, dtmin);
        disn[0] = nm.dis[0];
        disn[1] = nm.dis[1];
    } else {
        const double ampli = PI / 8.0;
        disn[1] = ampli * std::sin(10.0 * time);
    }
    const double alpha = disn[1] - alphav, yposr = disn[0] - yposrv;
    const double ca = std::cos(alpha), sa = std::sin(alpha);
    tstart(TM_TRANSF);
    if (nnmove > 0)
        CFD_LAUNCH(k_transf, blocks_for(nnmove, TB), TB, 0, stream, nnmove, d_fix_node, d_fix_set,
                   d_X, d_Y, d_xref, d_yref, ca, sa, yposr, d_xfix[0], d_xfix[1]);
    tstop(TM_TRANSF);
    if (prm.guess_mode == CFD_GUESS_ZERO) {
        CFD_CUDA(cudaMemsetAsync(d_pos[0], 0, sizeof(double) * N, stream));
        CFD_CUDA(cudaMemsetAsync(d_pos[1], 0, sizeof(double) * N, stream));
    }
    tstart(TM_GRAD);
    int st = run_pcg(2);
    if (st) return st;
    tstop(TM_GRAD);
    CFD_LAUNCH(k_motion_update, blocks_for(N, TB), TB, 0, stream, N, d_pos[0], d_pos[1], d_scal,
               d_X, d_Y, d_WX, d_WY);
    if (smooth_every > 0 && iter % smooth_every == 0) {
        st = smooth_in_step(stream, d_WX, d_WY, nullptr);
        if (st) return st;
    }
    if (fv_each) {  // FORCE_VISC at the print block's point: moved mesh, previous dNx
        st = force_visc_now();
        if (st) return st;
    }
    if (prm.moving == 1) {  // ns2DComp.ALE.f90:259-275
        st = geometry(prm.mass_mode == CFD_MASS_MASAS, false);
        if (st) return st;
        if (prm.mass_mode != CFD_MASS_MASAS) {  // gcl main, then putW/putArea
            tstart(TM_MASAS);
            CFD_CUDA(launch_gcl(stream, N, E, d_elem, d_esup_ptr, d_esup_slot, d_geo, d_area,
                                d_area_old, d_WX, d_WY, d_Wxo, d_Wyo, &d_scal->dtmin,
                                prm.mass_mode == CFD_MASS_GCL_LITERAL ? 1 : 0, d_gcl64, d_M));
            CFD_CUDA(cudaMemcpyAsync(d_Wxo, d_WX, sizeof(double) * N, cudaMemcpyDeviceToDevice, stream));
            CFD_CUDA(cudaMemcpyAsync(d_Wyo, d_WY, sizeof(double) * N, cudaMemcpyDeviceToDevice, stream));
            CFD_CUDA(cudaMemcpyAsync(d_area_old, d_area, sizeof(double) * E, cudaMemcpyDeviceToDevice, stream));
            tstop(TM_MASAS);
        }
        tstart(TM_LAPLACE);
        CFD_CUDA(launch_laplace(stream, N, E, d_elem, d_esup_ptr, d_esup_slot, d_lap_pos, d_geo,
                                d_X, d_Y, d_rowptr, d_lapq, d_val, d_diag));
        tstop(TM_LAPLACE);
    }
    std::swap(d_U, d_U1);  // U = U1 (:277-281)
    bandera_host += 1;
    return tcollect();
}

int Ctx::step(int nsteps, cfd_step_report* rep) {
    if (nsteps < 0) return CFD_ERR_ARG;
    for (int s = 0; s < nsteps; ++s) {
        int st = (prec == CFD_PREC_MIXED) ? step_once_mixed() : step_once();
        if (st) return st;
    }
    // the report: one gather on the device, one copy into pinned memory
    CFD_LAUNCH(k_pack_report, 1, 32, 0, stream, (const StepScal*)d_scal,
               (const MotionScal*)d_motion, (const int*)d_pcg_iters, (const int*)d_pcg_conv,
               (const double*)d_pcg_rz, (const GridBar*)d_bar, (const int*)d_node_err, d_out);
    CFD_CUDA(cudaMemcpyAsync(h_out, d_out, sizeof(StepOut), cudaMemcpyDeviceToHost, stream));
    CFD_CUDA(cudaStreamSynchronize(stream));
    *h_scal = h_out->sc;
    const MotionScal ms = h_out->ms;
    const int* it = h_out->it;
    const int* cv = h_out->cv;
    const double* rz = h_out->rz;
    const double* relres = h_out->relres;
    GridBar gb{};
    gb.err = h_out->bar_err;
    if (d_motion && nsteps > 0) {  // the mixed form's clock is kept on the device
        time = ms.time;
        last_dtmin = ms.dtmin;
        disn[0] = ms.disn0;
        disn[1] = ms.disn1;
    }
    if (gb.err) {
        set_last_message("a bounded device wait gave up (BiCG grid barrier or node-pass copy)");
        return CFD_ERR_BARRIER;
    }
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->iter = iter;
        rep->time = time;
        rep->dtmin = last_dtmin;
        for (int s = 0; s < 2; ++s) {
            rep->bicg_iters[s] = it[s];
            rep->bicg_rz[s] = rz[s];
            rep->bicg_relres[s] = relres[s];
            rep->bicg_converged[s] = cv[s];
        }
        rep->nset_numb = bc.nset_numb;
        for (int i = 0; i < 10; ++i) {
            rep->fx[i] = h_scal->fx[i];
            rep->fy[i] = h_scal->fy[i];
            rep->rm[i] = h_scal->rm[i];
        }
    }
    return CFD_OK;
}

// ------------------------------------------------------------------ create
template <class T>
int Ctx::dalloc(T** p, size_t n) {
    if (n == 0) n = 1;
    void* v = nullptr;
    CFD_CUDA(cudaMalloc(&v, n * sizeof(T)));
    allocs.push_back(v);
    *p = (T*)v;
    return CFD_OK;
}

template <class T>
int Ctx::upload(T** p, const T* h, size_t n) {
    int st = dalloc(p, n);
    if (st) return st;
    if (n) CFD_CUDA(cudaMemcpyAsync(*p, h, n * sizeof(T), cudaMemcpyHostToDevice, stream));
    return CFD_OK;
}

int Ctx::create(const cfd_mesh* m, const cfd_params* p, int precision_mode) {
    npoin = m->npoin;
    nelem = m->nelem;
    prm = *p;
    prec = precision_mode;
    if (prm.bicg_maxit <= 0) prm.bicg_maxit = 1000;
    if (!(prm.bicg_tol > 0.0)) prm.bicg_tol = 1.0e-10;
    prm.xref[1] = 1.4;  // meshMove.f90:58 (set before every FORCES/TRANSF)
    prm.yref[1] = 0.0;
    std::string why;
    int st = build_adjacency(npoin, nelem, m->inpoel, adj, &why);
    if (st) { set_last_message(why); return st; }
    st = build_bc_tables(m, bc, &why);
    if (st) { set_last_message(why); return st; }
    const int N = npoin, E = nelem;
    timers_on = getenv("CFD_TIMERS") && atoi(getenv("CFD_TIMERS")) != 0;
    if (getenv("CFD_ESTAB_EPS")) estab_eps = atof(getenv("CFD_ESTAB_EPS"));
    {  // freestream direction (the oracle's or_set_estab_dir, same operations)
        const double n = std::sqrt(prm.u_inf * prm.u_inf + prm.v_inf * prm.v_inf);
        dir[0] = n > 0.0 ? prm.u_inf / n : 1.0;
        dir[1] = n > 0.0 ? prm.v_inf / n : 0.0;
    }
    CFD_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CFD_CUDA(cudaEventCreateWithFlags(&ev_scal, cudaEventDisableTiming));
    CFD_CUDA(cudaEventCreateWithFlags(&ev_iters, cudaEventDisableTiming));
    CFD_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    CFD_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    CFD_CUDA(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking));
    CFD_CUDA(cudaStreamCreateWithFlags(&stream3, cudaStreamNonBlocking));
    for (auto& e : ev_side) CFD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CFD_CUDA(cudaMallocHost((void**)&h_scal, sizeof(StepScal)));
    CFD_CUDA(cudaMallocHost((void**)&h_out, sizeof(StepOut)));
    // mesh
    std::vector<int4> el(E);
    for (int e = 0; e < E; ++e)
        el[e] = make_int4(m->inpoel[3 * e] - 1, m->inpoel[3 * e + 1] - 1, m->inpoel[3 * e + 2] - 1, e);
    if ((st = upload(&d_elem, el.data(), E))) return st;
    if ((st = upload(&d_X, m->x, N))) return st;
    if ((st = upload(&d_Y, m->y, N))) return st;
    if ((st = upload(&d_esup_ptr, adj.esup_ptr.data(), N + 1))) return st;
    {  // padded by 4 ids: the bulk-copy node pass reads whole 16-byte groups of slot ids
        std::vector<int> es(adj.esup_slot);
        es.resize(3 * (size_t)E + 4, 0);
        if ((st = upload(&d_esup_slot, es.data(), es.size()))) return st;
    }
    if ((st = upload(&d_lap_pos, (const uchar4*)adj.lap_pos.data(), 3 * (size_t)E))) return st;
    if ((st = upload(&d_rowptr, adj.rowptr.data(), N + 1))) return st;
    if ((st = upload(&d_col, adj.col.data(), adj.col.size()))) return st;
    if ((st = dalloc(&d_val, adj.col.size()))) return st;
    nnz = (long)adj.col.size();
    if ((st = dalloc(&d_diag, N))) return st;
    if (prec == CFD_PREC_FP64 && (st = dalloc(&d_rdiag, N))) return st;
    if (prec == CFD_PREC_FP64 && (st = dalloc(&d_lapq, E))) return st;
    if (prec == CFD_PREC_FP64 && (st = dalloc(&d_gcl64, E))) return st;
    // BC tables
    std::vector<uint8_t> fl = bc.flag;
    for (auto& f : fl) {  // host bits -> device bits (same values, normals set on device)
        uint8_t d = 0;
        if (f & 1) d |= BC_FIXV;
        if (f & 4) d |= BC_FIXRHO;
        if (f & 8) d |= BC_FIXT;
        f = d;
    }
    if ((st = upload(&d_bcflag, fl.data(), N))) return st;
    if ((st = upload(&d_bcval, bc.val.data(), 4 * (size_t)N))) return st;
    if ((st = dalloc(&d_nrm, N))) return st;
    CFD_CUDA(cudaMemsetAsync(d_nrm, 0, sizeof(double2) * N, stream));
    nwn = (int)bc.wnode.size();
    if ((st = upload(&d_wnode, bc.wnode.data(), bc.wnode.size()))) return st;
    if ((st = upload(&d_wptr, bc.wptr.data(), bc.wptr.size()))) return st;
    std::vector<int2> wo(bc.wedge.size());
    for (size_t i = 0; i < wo.size(); ++i) wo[i] = make_int2(bc.wedge[i], 0);
    if ((st = upload(&d_wedge, wo.data(), wo.size()))) return st;
    if ((st = upload(&d_walls, (const int2*)bc.walls.data(), bc.walls.size() / 2))) return st;
    if ((st = upload(&d_set_ptr, bc.set_ptr.data(), bc.set_ptr.size()))) return st;
    if ((st = upload(&d_set_edges, (const int2*)bc.set_edges.data(), bc.set_edges.size() / 2))) return st;
    if ((st = upload(&d_set_elem, bc.set_elem.data(), bc.set_elem.size()))) return st;
    if ((st = upload(&d_xref, prm.xref, 10))) return st;
    if ((st = upload(&d_yref, prm.yref, 10))) return st;
    nnmove = (int)bc.fix_node.size();
    if ((st = upload(&d_fix_node, bc.fix_node.data(), bc.fix_node.size()))) return st;
    if ((st = upload(&d_fix_set, bc.fix_set.data(), bc.fix_set.size()))) return st;
    nufix = (int)bc.ufix_node.size();
    if ((st = upload(&d_ufix_node, bc.ufix_node.data(), bc.ufix_node.size()))) return st;
    if ((st = upload(&d_ufix_src, bc.ufix_src.data(), bc.ufix_src.size()))) return st;
    if ((st = upload(&d_isfix, bc.isfix.data(), N))) return st;
    // state and work arrays
    for (double** q : {&d_U, &d_U1}) if ((st = dalloc(q, 4 * (size_t)N))) return st;
    for (double** q : {&d_T, &d_VX, &d_VY, &d_RHO, &d_E, &d_P, &d_RMACH, &d_WX, &d_WY, &d_M,
                       &d_Wxo, &d_Wyo})
        if ((st = dalloc(q, N))) return st;
    for (double** q : {&d_area, &d_area_old, &d_DT, &d_DTL, &d_SHOC, &d_TS1, &d_TS2, &d_TS3})
        if ((st = dalloc(q, E))) return st;
    if ((st = dalloc(&d_geo, 6 * (size_t)E))) return st;
    if ((st = dalloc(&d_contrib, 12 * (size_t)E))) return st;
    if ((st = dalloc(&d_contribF, 12 * (size_t)E))) return st;
    if (prec == CFD_PREC_FP64 && (st = dalloc(&d_einv, (size_t)kElemInvPlanes * E))) return st;
    for (int s = 0; s < 2; ++s) {
        for (double** q : {&d_pos[s], &d_r[s], &d_z[s], &d_y[s], &d_p[s][0], &d_p[s][1]})
            if ((st = dalloc(q, N))) return st;
        if ((st = dalloc(&d_xfix[s], nnmove))) return st;
        CFD_CUDA(cudaMemsetAsync(d_pos[s], 0, sizeof(double) * N, stream));
        CFD_CUDA(cudaMemsetAsync(d_xfix[s], 0, sizeof(double) * (nnmove ? nnmove : 1), stream));
        if (extrap_mode()) {
            if ((st = dalloc(&d_xprev[s], N))) return st;
            CFD_CUDA(cudaMemsetAsync(d_xprev[s], 0, sizeof(double) * N, stream));
        }
    }
    if (extrap_mode()) {
        if ((st = dalloc(&d_xhist, 3))) return st;
        CFD_CUDA(cudaMemsetAsync(d_xhist, 0, 3 * sizeof(double), stream));
    }
    const long nc = ((long)N + kChunk - 1) / kChunk;
    if ((st = dalloc(&d_part, 6 * (size_t)(nc > 0 ? nc : 1)))) return st;
    if ((st = dalloc(&d_bar, 1))) return st;
    if ((st = dalloc(&d_pcg_iters, 2))) return st;
    if ((st = dalloc(&d_pcg_conv, 2))) return st;
    if ((st = dalloc(&d_pcg_rz, 4))) return st;  // |r.z| and ||r||/||ref|| per solve
    CFD_CUDA(cudaMemsetAsync(d_pcg_iters, 0, 2 * sizeof(int), stream));
    CFD_CUDA(cudaMemsetAsync(d_pcg_conv, 0, 2 * sizeof(int), stream));
    CFD_CUDA(cudaMemsetAsync(d_pcg_rz, 0, 4 * sizeof(double), stream));
    if ((st = dalloc(&d_scal, 1))) return st;
    if ((st = dalloc(&d_out, 1))) return st;
    StepScal sc0{};
    sc0.dtmin_bits = 0x7ff0000000000000ull;
    sc0.dtmin32_bits = 0x7ff0000000000000ull;
    sc0.bandera = 1;
    std::memcpy(h_scal, &sc0, sizeof(sc0));
    CFD_CUDA(cudaMemcpyAsync(d_scal, h_scal, sizeof(StepScal), cudaMemcpyHostToDevice, stream));
    CFD_CUDA(cudaStreamSynchronize(stream));
    // persistent BiCG grid: co-resident blocks only
    int dev = 0, per_sm = 0;
    CFD_CUDA(cudaGetDevice(&dev));
    CFD_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    CFD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, prec == CFD_PREC_MIXED ? k_pcg_mixed : k_pcg_fp64, 256, 0));
    long g = (long)nsm * (per_sm > 0 ? per_sm : 1);
    if (g > nc) g = nc;
    pcg_grid = (int)(g > 0 ? g : 1);
    // RESTART: freestream (ns2DComp.ALE.f90:59-60, :404-420)
    std::vector<double> U(4 * (size_t)N), T(N), VX(N), VY(N), zero(N, 0.0);
    for (int i = 0; i < N; ++i) {
        const double rhoamb = prm.rho_inf, uamb = prm.u_inf, vamb = prm.v_inf;
        const double pamb = prm.rho_inf * prm.fr * prm.t_inf;
        U[4 * i] = rhoamb;
        U[4 * i + 1] = rhoamb * uamb;
        U[4 * i + 2] = rhoamb * vamb;
        double energia = pamb / ((prm.gama - 1.0) * rhoamb) + 0.5 * (uamb * uamb + vamb * vamb);
        U[4 * i + 3] = energia * rhoamb;
        VX[i] = uamb;
        VY[i] = vamb;
        T[i] = prm.t_inf;
    }
    CFD_CUDA(cudaMemcpyAsync(d_U, U.data(), sizeof(double) * 4 * N, cudaMemcpyHostToDevice, stream));
    CFD_CUDA(cudaMemcpyAsync(d_T, T.data(), sizeof(double) * N, cudaMemcpyHostToDevice, stream));
    CFD_CUDA(cudaMemcpyAsync(d_VX, VX.data(), sizeof(double) * N, cudaMemcpyHostToDevice, stream));
    CFD_CUDA(cudaMemcpyAsync(d_VY, VY.data(), sizeof(double) * N, cudaMemcpyHostToDevice, stream));
    for (double* q : {d_WX, d_WY, d_Wxo, d_Wyo, d_RHO, d_E, d_P, d_RMACH})
        CFD_CUDA(cudaMemsetAsync(q, 0, sizeof(double) * N, stream));
    if (prec == CFD_PREC_MIXED) {
        if (prm.itlocal != 0 && (st = dalloc(&d_dtef, E))) return st;  // DT per element
        if ((st = dalloc(&d_invdiag, N))) return st;
        for (float** q : {&d_Tf, &d_VXf, &d_VYf, &d_RHOf, &d_Ef, &d_Pf, &d_RMACHf,
                          &d_invMf})
            if ((st = dalloc(q, N))) return st;
        for (float2** q : {&d_Xhi, &d_Xlo, &d_Wf, &d_Wof})
            if ((st = dalloc(q, N))) return st;
        for (float4** q : {&d_Uhi, &d_Ulo})
            if ((st = dalloc(q, N))) return st;
        if ((st = dalloc(&d_areaf, E))) return st;
        if ((st = dalloc(&d_blockmin, blocks_for(E, 256)))) return st;
        if ((st = dalloc(&d_geo8, 2 * (size_t)E))) return st;
        if ((st = dalloc(&d_mulam, E))) return st;
        for (float* q : {d_RHOf, d_Ef, d_Pf, d_RMACHf})
            CFD_CUDA(cudaMemsetAsync(q, 0, sizeof(float) * N, stream));
        CFD_CUDA(cudaMemsetAsync(d_Wof, 0, sizeof(float2) * N, stream));
        for (int s = 0; s < 2; ++s) {
            for (float** q : {&d_pf[s][0], &d_pf[s][1], &d_zf[s], &d_posf[s]})
                if ((st = dalloc(q, N))) return st;
            CFD_CUDA(cudaMemsetAsync(d_posf[s], 0, sizeof(float) * N, stream));
        }
        if ((st = dalloc(&d_part_r, 6 * (size_t)blocks_for(N, 256)))) return st;
        if ((st = dalloc(&d_bscal, 16))) return st;
        if ((st = dalloc(&d_bcount, 3))) return st;
        if ((st = dalloc(&d_invdiagf, N))) return st;
        CFD_CUDA(cudaMemsetAsync(d_bscal, 0, 16 * sizeof(double), stream));
        CFD_CUDA(cudaMemsetAsync(d_bcount, 0, 3 * sizeof(unsigned), stream));
        if ((st = dalloc(&d_valf, adj.col.size()))) return st;
        if (prm.bicg_tol_mode != CFD_BICG_TOL_ABS) {  // the FP64-assembled operator
            if ((st = dalloc(&d_val_lo, adj.col.size()))) return st;
            if ((st = dalloc(&d_k64, 9 * (size_t)E))) return st;
            if ((st = dalloc(&d_iterated, 1))) return st;
            for (int k = 0; k < 2; ++k) {
                if ((st = dalloc(&d_xs[k], (size_t)N))) return st;
                if ((st = dalloc(&d_xs_c[k], (size_t)N))) return st;
            }
            CFD_CUDA(cudaMemsetAsync(d_iterated, 0, sizeof(int), stream));
        }
        if ((st = dalloc(&d_gterms, E))) return st;
        // slot (e, i) -> its position in element-around-point order
        std::vector<int> pos(3 * (size_t)E);
        for (size_t s = 0; s < adj.esup_slot.size(); ++s) pos[adj.esup_slot[s]] = (int)s;
        if ((st = upload(&d_slot_pos, pos.data(), pos.size()))) return st;
        if ((st = dalloc(&d_recInv, 3 * (size_t)E))) return st;
        if ((st = dalloc(&d_recVisc, 3 * (size_t)E))) return st;
        if ((st = dalloc(&d_invSum, N))) return st;
        if ((st = dalloc(&d_motion, 1))) return st;
        if ((st = dalloc(&d_geo8_n, 2 * (size_t)E))) return st;
        if ((st = dalloc(&d_invMf_n, N))) return st;
        if ((st = dalloc(&d_WX_n, N))) return st;
        if ((st = dalloc(&d_WY_n, N))) return st;
        if ((st = dalloc(&d_Wf_n, N))) return st;
        if ((st = dalloc(&d_fgeo, std::max<size_t>(1, bc.set_elem.size())))) return st;
        if ((st = dalloc(&d_tcount, 4))) return st;
        if ((st = dalloc(&d_node_err, 1))) return st;
        CFD_CUDA(cudaMemsetAsync(d_node_err, 0, sizeof(int), stream));
        if (!(getenv("CFD_NODE_BULK") && atoi(getenv("CFD_NODE_BULK")) == 0))
            node_bulk = node_bulk_smem(adj.esup_ptr.data(), N);
        {  // blocks of the motion tail: a block per 32 edges, moving nodes or fixed values
            // (the items interleave over the blocks), at most kTailBlocks (64 measured
            // better than 128 at 16 items, 0.574 vs 0.576 ms at 1M nodes)
            int w = std::max(std::max(nnmove, nufix), nwn);
            for (int s = 0; s < bc.nset_numb; ++s) w = std::max(w, bc.set_ptr[s + 1] - bc.set_ptr[s]);
            tail_blocks = std::min(kTailBlocks, std::max(1, (int)blocks_for(w, 32)));
        }
        if ((st = dalloc(&d_tpart, 3 * 10 * kTailBlocks))) return st;
        CFD_CUDA(cudaMemsetAsync(d_tcount, 0, 4 * sizeof(unsigned), stream));
        CFD_CUDA(cudaMemsetAsync(d_motion, 0, sizeof(MotionScal), stream));
        graphs_on = !timers_on && !(getenv("CFD_GRAPHS") && atoi(getenv("CFD_GRAPHS")) == 0);
        // 5 blocks per SM measured best at 1M nodes with the current passes (the FP64 gcl
        // areas on the branch; 1000-step runs: 5: 0.557-0.559 ms, 6: 0.561-0.562; 600-step
        // runs, 4, 8, 12: 0.579, 0.568, 0.586); 0 = full grids
        branch_bpsm = getenv("CFD_BRANCH_BLOCKS_PER_SM") ? atoi(getenv("CFD_BRANCH_BLOCKS_PER_SM"))
                                                         : 5;
        if ((st = narrow_mixed(true, true, true, true, true, true))) return st;
    }
    // setup geometry: NORMALES, DERIV, MASAS, laplace (ns2DComp.ALE.f90:88-100)
    st = (prec == CFD_PREC_MIXED) ? geometry_mixed(true, true) : geometry(true, true);
    if (st) return st;
    if (prec != CFD_PREC_MIXED)
        CFD_CUDA(cudaMemcpyAsync(d_area_old, d_area, sizeof(double) * E, cudaMemcpyDeviceToDevice, stream));
    CFD_CUDA(cudaStreamSynchronize(stream));
    return tcollect();
}

// ------------------------------------------------------------------ mixed precision
// FP64 arrays -> float shadows, for the arrays the caller replaced (uploads, setup)
int Ctx::narrow_mixed(bool U, bool T, bool VX, bool VY, bool XY, bool W) {
    const int N = npoin;
    CFD_LAUNCH(k_narrow_state, blocks_for(N, 256), 256, 0, stream, N, U ? d_U : nullptr,
               T ? d_T : nullptr, VX ? d_VX : nullptr, VY ? d_VY : nullptr, XY ? d_X : nullptr,
               XY ? d_Y : nullptr, W ? d_WX : nullptr, W ? d_WY : nullptr, d_Uhi, d_Ulo, d_Tf,
               d_VXf, d_VYf, d_Xhi, d_Xlo, d_Wf);
    return CFD_OK;
}

// float fields -> the FP64 arrays the download entries read
// what: 1 = T only, 2 = the seven node fields, 4 = the geometry (bits may combine)
int Ctx::widen_mixed(int what) {
    const long N = npoin, E = nelem;
    const float* src[7] = {d_Tf, d_VXf, d_VYf, d_RHOf, d_Ef, d_Pf, d_RMACHf};
    double* dst[7] = {d_T, d_VX, d_VY, d_RHO, d_E, d_P, d_RMACH};
    const int nf = (what & 2) ? 7 : ((what & 1) ? 1 : 0);
    for (int i = 0; i < nf; ++i)
        CFD_LAUNCH(k_widen, blocks_for(N, 256), 256, 0, stream, N, src[i], dst[i]);
    if (what & 4)  // d_area is the FP64 area the element pass keeps
        CFD_LAUNCH(k_widen_geo, blocks_for(E, 256), 256, 0, stream, (int)E, (const float4*)d_geo8,
                   d_geo, (double*)nullptr);
    return CFD_OK;
}

// Geometry of the current mesh for the mixed form: normales, then one element pass
// (deriv, Laplacian weights, gcl element terms, putArea) and one node pass (Laplacian rows,
// 1/diag, MASAS at setup or per step, or the gcl mass update and putW).
int Ctx::geometry_mixed(bool setup, bool put_area, bool to_next, cudaStream_t sv) {
    const cudaStream_t stream = sv ? sv : this->stream;
    const int N = npoin, E = nelem;
    const int TB = 256;
    const bool gcl = !setup && prm.mass_mode != CFD_MASS_MASAS;
    // to_next (the step's mesh-motion branch): the next step's geo8, 1/M, with W the next
    // and W_old the current W (putW by the buffer swap); normales are left to the caller
    // (the RK stages still read this step's).  Otherwise normales ride on the element pass
    // (its own blocks after the elements').
    float4* geo8 = to_next ? d_geo8_n : d_geo8;
    float* invMf = to_next ? d_invMf_n : d_invMf;
    const float2* Wn = to_next ? d_Wf_n : d_Wf;
    const float2* Wo = to_next ? d_Wf : d_Wof;
    tstart(TM_DERIV);
    const NormalsArgs nv{to_next ? 0 : nwn, d_wnode, d_wptr, d_wedge, d_walls, d_X, d_Y, d_bcflag,
                         d_nrm};
    CFD_LAUNCH(k_elem_geometry,
               nv.nwn > 0 ? blocks_for(E, TB) + blocks_for(nv.nwn, TB) : branch_grid(E, TB, sv), TB,
               0, stream, E, d_elem, d_X, d_Y, gcl ? 1 : 0,
               prm.mass_mode == CFD_MASS_GCL_LITERAL ? 1 : 0, Wn, Wo,
               (gcl || put_area) ? 1 : 0, d_area_old, d_area, d_areaf, geo8, d_gterms, nv);
    tstop(TM_DERIV);
    tstart(TM_LAPLACE);
    if (d_val_lo)  // relative tests: the mesh-motion operator to FP64-class accuracy
        CFD_LAUNCH(k_elem_grad64, branch_grid(E, TB, sv), TB, 0, stream, E, d_elem, d_X, d_Y,
                   (const int*)d_slot_pos, d_k64);
    CFD_CUDA(launch_node_geometry(d_val_lo != nullptr, branch_grid(N, kGeoNodeBlock, sv), stream,
                                  N, d_esup_ptr, d_esup_slot, d_lap_pos, geo8, d_gterms,
                                  &d_scal->dtmin, gcl ? 1 : 0, d_rowptr, d_valf, d_invdiag,
                                  d_invdiagf, d_M, invMf, Wn, to_next ? (float2*)nullptr : d_Wof,
                                  (const float2*)d_k64, d_val_lo));
    tstop(TM_LAPLACE);
    return CFD_OK;
}

// The device work of one mixed step, in order.  No host wait: DTMIN, the clock and the
// motion increment stay on the device, so the sequence can be captured as a graph.
int Ctx::enqueue_mixed(bool learned) {
    const int N = npoin, E = nelem;
    const int TB = 256;
    // deltat alone (a light pass, so that the mesh motion forks early); the FP64 refinement
    // of the elements near the FP32 minimum, whose last block forms DTMIN.  ESTAB is formed
    // in the stage-1 element pass.
    tstart(TM_DELTAT);
    CFD_LAUNCH(k_deltat_mixed, blocks_for(E, TB), TB, 0, stream, E, d_elem, d_Tf, d_VXf, d_VYf,
               d_Wf, d_areaf, (float)prm.t_inf, (float)prm.fsafe, &d_scal->dtmin32_bits,
               d_blockmin, d_dtef);
    {
        const int nchunk = (int)blocks_for(E, TB);
        CFD_LAUNCH(k_deltat_refine, blocks_for(nchunk, TB), TB, 0, stream, E, d_elem, d_Tf, d_VXf,
                   d_VYf, d_Wf, d_areaf, (const unsigned long long*)d_blockmin, nchunk,
                   (float)prm.fsafe, (float)prm.t_inf, d_scal, d_tcount, prm.itlocal);
    }
    tstop(TM_DELTAT);
    // The mesh motion of a prescribed law needs DTMIN and the step-start mesh only, and
    // what it produces (the moved mesh, W, the new geometry) is the next step's: it runs
    // on its own stream beside the RK stages, writing the next-step buffers (swapped after
    // the step), and joins before FORCES.  The Newmark law needs this step's forces: its
    // motion follows them on the main stream.
    const bool structural = prm.motion_law == CFD_MOTION_NEWMARK;
    const bool fork = !timers_on && !structural;
    MotionTailArgs t{};
    t.nset = bc.nset_numb;
    t.set_ptr = d_set_ptr;
    t.set_edges = d_set_edges;
    t.P = d_Pf;
    t.X = d_X;
    t.Y = d_Y;
    t.xref = d_xref;
    t.yref = d_yref;
    t.law = prm.motion_law;
    t.heave_amp = prm.heave_amp;
    t.pitch_amp = prm.pitch_amp;
    t.freq = prm.motion_freq;
    t.m = d_motion;
    t.nnmove = nnmove;
    t.fix_node = d_fix_node;
    t.fix_set = d_fix_set;
    t.xfix_x = d_xfix[0];
    t.xfix_y = d_xfix[1];
    t.nufix = nufix;
    t.ufix_node = d_ufix_node;
    t.ufix_src = d_ufix_src;
    t.x0 = d_pos[0];
    t.x1 = d_pos[1];
    t.xf0 = d_posf[0];
    t.xf1 = d_posf[1];
    t.part = d_tpart;
    t.sc = d_scal;
    t.fgeo = structural ? nullptr : d_fgeo;
    // clock and motion law, TRANSF, the solves' Dirichlet values (and with the Newmark law
    // FORCES first), the two solves, the mesh update and the next step's geometry
    auto motion = [&](cudaStream_t s) -> int {
        if (prm.guess_mode == CFD_GUESS_ZERO)
            for (int c = 0; c < 2; ++c) {
                CFD_CUDA(cudaMemsetAsync(d_pos[c], 0, sizeof(double) * N, s));
                CFD_CUDA(cudaMemsetAsync(d_posf[c], 0, sizeof(float) * N, s));
            }
        MotionTailArgs m = t;
        m.do_motion = 1;
        m.do_forces = structural ? 1 : 0;
        m.count = d_tcount + 1;
        tstart(TM_FORCES);
        CFD_LAUNCH(k_motion_tail, (unsigned)tail_blocks, 256, 0, s, m);
        tstop(TM_FORCES);
        tstart(TM_GRAD);
        int st = run_pcg(2, learned, true, s);
        if (st) return st;
        tstop(TM_GRAD);
        CFD_LAUNCH(k_motion_update_mixed, branch_grid(N, TB, s), TB, 0, s, N, d_pos[0], d_pos[1],
                   d_scal, d_X, d_Y, d_WX_n, d_WY_n, d_Xhi, d_Xlo, d_Wf_n);
        if (smoothing_now && (st = smooth_in_step(s, d_WX_n, d_WY_n, d_Wf_n))) return st;
        if (prm.moving == 1 && (st = geometry_mixed(false, false, true, s))) return st;
        if (side_join) {  // the fields' update on stream3 (it reads this step's solutions)
            CFD_CUDA(cudaStreamWaitEvent(s, ev_side[3], 0));
            side_join = false;
        }
        return CFD_OK;
    };
    if (fork) {
        CFD_CUDA(cudaEventRecord(ev_fork, stream));
        CFD_CUDA(cudaStreamWaitEvent(stream2, ev_fork, 0));
        int st = motion(stream2);
        if (st) return st;
        CFD_CUDA(cudaEventRecord(ev_join, stream2));
    } else if (!structural) {
        int st = motion(stream);
        if (st) return st;
    }
    GasConst gc{prm.fcv, prm.fk, prm.fmu, prm.gama, prm.t_inf, prm.cte, prm.fr};
    const GasConstF gf = to_float(gc);
    const bool viscous = prm.fmu > 2.2250738585072014e-308;
    tstart(TM_CALCRHS);
    const EstabConst ec{(float)((prm.gama + prm.gama + prm.gama) / 3.0), (float)prm.fr,
                        (float)prm.rho_inf, (float)prm.t_inf, prm.estab_mode, (float)estab_eps,
                        (float)dir[0], (float)dir[1]};
    CFD_CUDA(launch_elem_stage1_mixed(viscous, stream, E, d_elem, d_Uhi, d_Ulo, d_geo8, d_VXf,
                                      d_VYf, ec, d_scal, gf, d_Wf, d_slot_pos, d_Tf, d_recInv,
                                      d_recVisc, d_mulam, (const float*)d_dtef));
    tstop(TM_CALCRHS);
    // stage s uses mu, lambda from the T of stage s-1 (the reference's module T): stage 1's
    // come from the element kernel above, the others from k_elem_mulam before the node pass.
    // The last stage updates U in place.
    const int NRK = 4;
    // one event pair around the four stages (no event between their kernels), counted as
    // four launches of the group
    tstart(TM_UPDATE);
    for (int irk = 1; irk <= NRK; ++irk) {
        const float rk_fact = 1.f / (float)(NRK + 1 - irk);
        if (irk > 1 && viscous)
            CFD_LAUNCH(k_elem_mulam, blocks_for(E, kMulamTB), kMulamTB, 0, stream, E, d_elem,
                       (const float*)d_Tf, gf, d_mulam);
        CFD_CUDA(launch_node_mixed(stream, N, d_esup_ptr, d_esup_slot, d_mulam, d_recInv, d_recVisc,
                                   d_invSum, irk == 1 ? 1 : 0, gc, gf, viscous ? 1 : 0, d_U, d_Uhi,
                                   d_Ulo, d_invMf, rk_fact, irk == NRK ? 1 : 0, d_bcflag, d_bcval,
                                   d_nrm, d_WX, d_WY, d_U, d_RHOf, d_VXf, d_VYf, d_Ef, d_Pf, d_Tf,
                                   d_RMACHf, node_bulk, d_node_err));
    }
    tstop(TM_UPDATE, NRK);
    int st = CFD_OK;
    if (structural) {
        if ((st = motion(stream))) return st;
    } else {
        // FORCES on the step's pressure and the step-start edge geometry
        if (fork) CFD_CUDA(cudaStreamWaitEvent(stream, ev_join, 0));
        MotionTailArgs f = t;
        f.do_motion = 0;
        f.do_forces = 1;
        f.count = d_tcount + 2;
        if (prm.moving == 1)  // normales of the moved mesh ride on this launch
            f.nv = NormalsArgs{nwn, d_wnode, d_wptr, d_wedge, d_walls, d_X, d_Y, d_bcflag, d_nrm};
        tstart(TM_FORCES);
        CFD_LAUNCH(k_motion_tail, (unsigned)tail_blocks, 256, 0, stream, f);
        tstop(TM_FORCES);
    }
    if (prm.moving == 1 && structural) {  // normales of the moved mesh (the Newmark path)
        tstart(TM_NORMALES);
        if (nwn > 0)
            CFD_LAUNCH(k_normales, blocks_for(nwn, TB), TB, 0, stream, nwn, d_wnode, d_wptr, d_wedge,
                       d_walls, d_X, d_Y, d_bcflag, d_nrm);
        tstop(TM_NORMALES);
    }
    if (fv_each) {  // FORCE_VISC at the print block's point: moved mesh, this step's dNx
        st = force_visc_now();
        if (st) return st;
    }
    return CFD_OK;
}

// Grid of a kernel over n items with `threads` per block: full, or on the mesh-motion
// branch's stream (running beside the RK stages) at most branch_bpsm blocks per SM
unsigned Ctx::branch_grid(long n, int threads, cudaStream_t s) const {
    const unsigned full = blocks_for(n, threads);
    if (!s || s != stream2 || branch_bpsm <= 0) return full;
    return std::min<unsigned>(full, (unsigned)(branch_bpsm * nsm));
}

// The next-step buffers become the current ones (after each mixed step)
void Ctx::swap_mixed_buffers() {
    std::swap(d_WX, d_WX_n);
    std::swap(d_WY, d_WY_n);
    std::swap(d_Wf, d_Wf_n);
    if (prm.moving == 1) {
        std::swap(d_geo8, d_geo8_n);
        std::swap(d_invMf, d_invMf_n);
    }
    buf ^= 1;
}

void Ctx::drop_graphs() {
    for (int p = 0; p < 2; ++p) {
        if (step_exec[p]) cudaGraphExecDestroy(step_exec[p]);
        if (step_graph[p]) cudaGraphDestroy(step_graph[p]);
        step_exec[p] = nullptr;
        step_graph[p] = nullptr;
    }
}

// Replay the captured step, capturing it first.  *launched = false when the capture is
// not possible here (the caller then enqueues the step launch by launch, and stays so).
int Ctx::launch_step_graph(bool* launched) {
    *launched = false;
    // one graph per buffer parity: the captured pointers are the parity's
    cudaGraph_t& step_graph = this->step_graph[buf];
    cudaGraphExec_t& step_exec = this->step_exec[buf];
    if (!step_exec) {
        const long long k0 = g_launches.load();
        CFD_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        capturing = true;
        const int st = enqueue_mixed(false);
        capturing = false;
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(stream, &g);
        const long long nk = g_launches.load() - k0;
        g_launches.fetch_sub(nk);  // captured, not run
        cudaGraphExec_t ex = nullptr;
        if (st == CFD_OK && ce == cudaSuccess && g &&
            cudaGraphInstantiate(&ex, g, 0) == cudaSuccess) {
            step_graph = g;
            step_exec = ex;
            graph_kernels = nk;
        } else {
            if (g) cudaGraphDestroy(g);
            (void)cudaGetLastError();
            graphs_on = false;
            return CFD_OK;
        }
    }
    CFD_CUDA(cudaGraphLaunch(step_exec, stream));
    g_launches.fetch_add(graph_kernels, std::memory_order_relaxed);
    graph_replays += 1;
    *launched = true;
    return CFD_OK;
}

// One mixed step.  The learned guess runs on the first solve after the network was
// attached, and when the previous solve took more than guess_gate iterations (every solve
// when guess_gate is 0): the host reads the previous solve's counts once they are in
// pinned memory (mid previous step, while the device finishes its mesh update).  The
// steps without the network replay a captured graph from the second step on.
int Ctx::step_once_mixed() {
    iter += 1;
    bool learned = false;
    if (learned_mode() && net && lgraph) {
        guess_steps += 1;
        if (!guess_first && guess_gate > 0.0) CFD_CUDA(cudaEventSynchronize(ev_iters));
        learned = guess_first || guess_gate <= 0.0 ||
                  (double)std::max(h_iters[0], h_iters[1]) > guess_gate;
        guess_first = false;
    }
    bandera_host += 1;
    // a step that smooths its moved mesh waits on the host for the sweeps' convergence
    // flags: it is enqueued launch by launch
    smoothing_now = smooth_every > 0 && iter % smooth_every == 0;
    if (graphs_on && !learned && !smoothing_now && mixed_steps > 0) {
        bool launched = false;
        int st = launch_step_graph(&launched);
        if (st) return st;
        if (launched) {
            mixed_steps += 1;
            swap_mixed_buffers();
            return CFD_OK;
        }
    }
    int st = enqueue_mixed(learned);
    if (st) return st;
    mixed_steps += 1;
    swap_mixed_buffers();
    return tcollect();
}

}  // namespace cfd

// abi.cu — the extern "C" entry points of include/cfd_gpu.h.
//
// Drop-in routines stage host arrays (reference layout, 1-based) to the device, run the
// same kernels the resident context uses and copy the results back.  Every call checks
// its arguments and returns a status; nothing here falls back to the CPU.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "cfd_context.cuh"

using namespace cfd;

namespace {

// device buffers freed at scope exit
struct Scratch {
    std::vector<void*> ptrs;
    cudaStream_t stream = nullptr;
    ~Scratch() {
        if (stream) {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
        for (void* p : ptrs) cudaFree(p);
    }
    int init() {
        CFD_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        return CFD_OK;
    }
    template <class T>
    int alloc(T** p, size_t n) {
        void* v = nullptr;
        CFD_CUDA(cudaMalloc(&v, (n ? n : 1) * sizeof(T)));
        ptrs.push_back(v);
        *p = (T*)v;
        return CFD_OK;
    }
    template <class T>
    int put(T** p, const T* h, size_t n) {
        int st = alloc(p, n);
        if (st) return st;
        if (n) CFD_CUDA(cudaMemcpyAsync(*p, h, n * sizeof(T), cudaMemcpyHostToDevice, stream));
        return CFD_OK;
    }
    template <class T>
    int get(T* h, const T* d, size_t n) {
        if (n) CFD_CUDA(cudaMemcpyAsync(h, d, n * sizeof(T), cudaMemcpyDeviceToHost, stream));
        return CFD_OK;
    }
    int sync() {
        CFD_CUDA(cudaStreamSynchronize(stream));
        return CFD_OK;
    }
};

#define TRY(x)                 \
    do {                       \
        int st_ = (x);         \
        if (st_) return st_;   \
    } while (0)

int arg_error(const char* what) {
    set_last_message(std::string("invalid argument: ") + what);
    return CFD_ERR_ARG;
}

// The device's view of a pointer into pinned (page-locked, mapped) host memory, 16-B
// aligned; nullptr for pageable or device memory, which then take cudaMemcpyAsync.
const double* pinned_device_view(const double* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr) return nullptr;
    if (reinterpret_cast<uintptr_t>(a.devicePointer) & 15) return nullptr;
    return static_cast<const double*>(a.devicePointer);
}

// inpoel(3,nelem) 1-based -> int4 0-based, with range checks
int make_elems(const int* inpoel, int nelem, int npoin, std::vector<int4>& el) {
    el.resize(nelem);
    for (int e = 0; e < nelem; ++e) {
        int a = inpoel[3 * e], b = inpoel[3 * e + 1], c = inpoel[3 * e + 2];
        if (a < 1 || a > npoin || b < 1 || b > npoin || c < 1 || c > npoin) {
            set_last_message("inpoel(:," + std::to_string(e + 1) + ") outside 1..npoin");
            return CFD_ERR_MESH;
        }
        el[e] = make_int4(a - 1, b - 1, c - 1, e);
    }
    return CFD_OK;
}

// esup of pointNeighbor.f90:5-43, 0-based slots (3*e + local)
void make_esup(const int* inpoel, int nelem, int npoin, std::vector<int>& ptr, std::vector<int>& slot) {
    ptr.assign(npoin + 1, 0);
    for (long e = 0; e < nelem; ++e)
        for (int i = 0; i < 3; ++i) ptr[inpoel[3 * e + i]] += 1;
    for (int p = 1; p <= npoin; ++p) ptr[p] += ptr[p - 1];
    slot.assign(3 * (size_t)nelem, 0);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (long e = 0; e < nelem; ++e)
        for (int i = 0; i < 3; ++i) slot[fill[inpoel[3 * e + i] - 1]++] = (int)(3 * e + i);
}

// dNx(3,nelem), dNy(3,nelem) -> [dNx1|dNx2|dNx3|dNy1|dNy2|dNy3]
std::vector<double> to_geo(const double* dNx, const double* dNy, int nelem) {
    std::vector<double> g(6 * (size_t)nelem);
    for (int e = 0; e < nelem; ++e)
        for (int i = 0; i < 3; ++i) {
            g[i * (size_t)nelem + e] = dNx[3 * e + i];
            g[(3 + i) * (size_t)nelem + e] = dNy[3 * e + i];
        }
    return g;
}

bool bad_sizes(const int* nelem, const int* npoin) {
    return !nelem || !npoin || *nelem <= 0 || *npoin <= 0;
}

}  // namespace

extern "C" {

const char* cfd_strerror(int status) {
    static thread_local std::string msg;
    const char* base = "unknown status";
    switch (status) {
        case CFD_OK: base = "ok"; break;
        case CFD_ERR_ARG: base = "invalid argument"; break;
        case CFD_ERR_MESH: base = "invalid mesh"; break;
        case CFD_ERR_CUDA: base = "CUDA runtime error"; break;
        case CFD_ERR_NOMEM: base = "device allocation failed"; break;
        case CFD_ERR_NOT_CONVERGED: base = "BiCG did not converge"; break;
        case CFD_ERR_NONFINITE: base = "non-finite value in the state"; break;
        case CFD_ERR_BARRIER: base = "device-side wait gave up"; break;
        case CFD_ERR_LIMIT: base = "size above the documented maximum"; break;
        case CFD_ERR_STATE: base = "call out of order"; break;
    }
    std::string last = last_message();
    msg = last.empty() || status == CFD_OK ? std::string(base) : std::string(base) + ": " + last;
    return msg.c_str();
}

int cfd_device_available(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n > 0 ? 1 : 0;
}

long long cfd_kernel_launches(void) { return g_launches.load(); }

int cfd_selftest_div3(long long n, unsigned long long seed, unsigned long long* mismatches) {
    if (n < 1 || n > (1LL << 36) || !mismatches)
        return arg_error("n in [1, 2^36] and a mismatch counter");
    unsigned long long* bad = nullptr;
    CFD_CUDA(cudaMalloc(&bad, sizeof(unsigned long long)));
    unsigned long long h = ~0ull;
    cudaError_t e = cudaMemset(bad, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = launch_selftest_div3(n, seed, bad);
    if (e == cudaSuccess) e = cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(bad);
    CFD_CUDA(e);
    *mismatches = h;
    return CFD_OK;
}

int cfd_selftest_div_rcp(long long n, unsigned long long seed, unsigned long long* mismatches) {
    if (n < 1 || n > (1LL << 36) || !mismatches)
        return arg_error("n in [1, 2^36] and a mismatch counter");
    unsigned long long* bad = nullptr;
    CFD_CUDA(cudaMalloc(&bad, sizeof(unsigned long long)));
    unsigned long long h = ~0ull;
    cudaError_t e = cudaMemset(bad, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = launch_selftest_divrcp(n, seed, bad);
    if (e == cudaSuccess) e = cudaMemcpy(&h, bad, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(bad);
    CFD_CUDA(e);
    *mismatches = h;
    return CFD_OK;
}

int cfd_selftest_waits(long long polls, int* barrier_status, int* mbarrier_status) {
    if (polls < 1 || polls > (1LL << 24) || !barrier_status || !mbarrier_status)
        return arg_error("polls in [1, 2^24] and two status pointers");
    GridBar* gb = nullptr;
    int* out = nullptr;
    CFD_CUDA(cudaMalloc(&gb, sizeof(GridBar)));
    const cudaError_t e1 = cudaMalloc(&out, 2 * sizeof(int));
    if (e1 != cudaSuccess) {
        cudaFree(gb);
        CFD_CUDA(e1);
    }
    int h[2] = {-1, -1};
    cudaError_t e = cudaMemset(gb, 0, sizeof(GridBar));
    if (e == cudaSuccess) e = cudaMemset(out, 0xff, 2 * sizeof(int));
    if (e == cudaSuccess) {
        k_selftest_waits<<<1, 32>>>(gb, out, polls);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(h, out, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(gb);
    cudaFree(out);
    CFD_CUDA(e);
    *barrier_status = h[0];
    *mbarrier_status = h[1];
    return CFD_OK;
}

void* cfd_ctx_stream(cfd_ctx* ctx) { return ctx ? (void*)ctx->impl.stream : nullptr; }

int cfd_ctx_mark(cfd_ctx* ctx, int slot) {
    if (!ctx || slot < 0 || slot >= 8) return arg_error("ctx/slot");
    Ctx& c = ctx->impl;
    if (!c.mark[slot]) CFD_CUDA(cudaEventCreate(&c.mark[slot]));
    CFD_CUDA(cudaEventRecord(c.mark[slot], c.stream));
    return CFD_OK;
}

int cfd_ctx_elapsed(cfd_ctx* ctx, int a, int b, double* ms) {
    if (!ctx || !ms || a < 0 || a >= 8 || b < 0 || b >= 8) return arg_error("ctx/slot");
    Ctx& c = ctx->impl;
    if (!c.mark[a] || !c.mark[b]) return CFD_ERR_STATE;
    CFD_CUDA(cudaEventSynchronize(c.mark[b]));
    float f = 0.f;
    CFD_CUDA(cudaEventElapsedTime(&f, c.mark[a], c.mark[b]));
    *ms = f;
    return CFD_OK;
}

int cfd_set_device(int ordinal) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        set_last_message("no CUDA device");
        return CFD_ERR_CUDA;
    }
    if (ordinal < 0 || ordinal >= n) return arg_error("device ordinal");
    CFD_CUDA(cudaSetDevice(ordinal));
    return CFD_OK;
}

const char* cfd_timer_name(int slot) {
    static const char* names[TM_N] = {"deltat_t", "estab_t",    "calcrhs_t", "fuente_t",
                                      "update_t", "forces_t",   "transf_t",  "grad_t",
                                      "normales_t", "deriv_t",  "masas_t",   "laplace_t"};
    return (slot >= 0 && slot < TM_N) ? names[slot] : nullptr;
}

// ------------------------------------------------------------------ resident context
int cfd_ctx_create(cfd_ctx** out, const cfd_mesh* mesh, const cfd_params* p, int precision_mode) {
    if (!out || !mesh || !p) return arg_error("null pointer");
    *out = nullptr;
    if (precision_mode != CFD_PREC_FP64 && precision_mode != CFD_PREC_MIXED)
        return arg_error("precision_mode");
    if (p->estab_mode < CFD_ESTAB_REFERENCE || p->estab_mode > CFD_ESTAB_REGULARIZED)
        return arg_error("estab_mode");
    if (p->bicg_tol_mode < CFD_BICG_TOL_ABS || p->bicg_tol_mode > CFD_BICG_TOL_REL_R0)
        return arg_error("bicg_tol_mode");
    if (p->guess_mode < CFD_GUESS_PREVIOUS || p->guess_mode > CFD_GUESS_LEARNED_EXTRAPOLATED)
        return arg_error("guess_mode");
    if (p->ngas != 0) {
        set_last_message("only the perfect-gas path (NGAS = 0) is implemented");
        return CFD_ERR_ARG;
    }
    if (!cfd_device_available()) {
        set_last_message("no CUDA device");
        return CFD_ERR_CUDA;
    }
    std::unique_ptr<cfd_ctx> c(new cfd_ctx());
    int st = c->impl.create(mesh, p, precision_mode);
    if (st) return st;
    *out = c.release();
    return CFD_OK;
}

void cfd_ctx_destroy(cfd_ctx* ctx) { delete ctx; }

int cfd_ctx_upload_state(cfd_ctx* ctx, const double* U, const double* T, const double* VEL_X,
                         const double* VEL_Y) {
    if (!ctx) return arg_error("ctx");
    Ctx& c = ctx->impl;
    const size_t N = c.npoin;
    // U in pinned host memory with the velocities left out: one kernel reads it over the
    // host link and writes U, the velocities and the mixed form's shadows (k_upload_U)
    const double* hU = (U && !VEL_X && !VEL_Y) ? pinned_device_view(U) : nullptr;
    if (hU) {
        const bool mx = c.prec == CFD_PREC_MIXED;
        CFD_LAUNCH(k_upload_U, blocks_for((long)N, 256), 256, 0, c.stream, (int)N, hU, c.d_U,
                   c.d_VX, c.d_VY, mx ? c.d_Uhi : nullptr, mx ? c.d_Ulo : nullptr,
                   mx ? c.d_VXf : nullptr, mx ? c.d_VYf : nullptr);
        if (T) {
            CFD_CUDA(cudaMemcpyAsync(c.d_T, T, 8 * N, cudaMemcpyHostToDevice, c.stream));
            if (mx) TRY(c.narrow_mixed(false, true, false, false, false, false));
        }
        CFD_CUDA(cudaStreamSynchronize(c.stream));
        return CFD_OK;
    }
    if (U) CFD_CUDA(cudaMemcpyAsync(c.d_U, U, 32 * N, cudaMemcpyHostToDevice, c.stream));
    if (T) CFD_CUDA(cudaMemcpyAsync(c.d_T, T, 8 * N, cudaMemcpyHostToDevice, c.stream));
    if (VEL_X) CFD_CUDA(cudaMemcpyAsync(c.d_VX, VEL_X, 8 * N, cudaMemcpyHostToDevice, c.stream));
    if (VEL_Y) CFD_CUDA(cudaMemcpyAsync(c.d_VY, VEL_Y, 8 * N, cudaMemcpyHostToDevice, c.stream));
    if (U && (!VEL_X || !VEL_Y))  // the velocities the caller left out, from U on the device
        CFD_LAUNCH(k_vel_from_U, blocks_for((long)N, 256), 256, 0, c.stream, (int)N, c.d_U,
                   VEL_X ? nullptr : c.d_VX, VEL_Y ? nullptr : c.d_VY);
    if (c.prec == CFD_PREC_MIXED)
        TRY(c.narrow_mixed(U != nullptr, T != nullptr, VEL_X || U, VEL_Y || U, false, false));
    CFD_CUDA(cudaStreamSynchronize(c.stream));
    return CFD_OK;
}

int cfd_ctx_upload_mesh(cfd_ctx* ctx, const double* X, const double* Y, const double* W_X,
                        const double* W_Y, const double* xpos, const double* ypos) {
    if (!ctx) return arg_error("ctx");
    Ctx& c = ctx->impl;
    const size_t n8 = 8 * (size_t)c.npoin;
    if (X) CFD_CUDA(cudaMemcpyAsync(c.d_X, X, n8, cudaMemcpyHostToDevice, c.stream));
    if (Y) CFD_CUDA(cudaMemcpyAsync(c.d_Y, Y, n8, cudaMemcpyHostToDevice, c.stream));
    if (W_X) CFD_CUDA(cudaMemcpyAsync(c.d_WX, W_X, n8, cudaMemcpyHostToDevice, c.stream));
    if (W_Y) CFD_CUDA(cudaMemcpyAsync(c.d_WY, W_Y, n8, cudaMemcpyHostToDevice, c.stream));
    if (xpos) CFD_CUDA(cudaMemcpyAsync(c.d_pos[0], xpos, n8, cudaMemcpyHostToDevice, c.stream));
    if (ypos) CFD_CUDA(cudaMemcpyAsync(c.d_pos[1], ypos, n8, cudaMemcpyHostToDevice, c.stream));
    if (c.prec == CFD_PREC_MIXED)
        for (int k = 0; k < 2; ++k)
            if (k == 0 ? xpos != nullptr : ypos != nullptr)
                CFD_LAUNCH(k_narrow, blocks_for(c.npoin, 256), 256, 0, c.stream, (long)c.npoin,
                           (const double*)c.d_pos[k], c.d_posf[k]);
    if (c.prec == CFD_PREC_MIXED && (X || Y || W_X || W_Y))
        TRY(c.narrow_mixed(false, false, false, false, X || Y, W_X || W_Y));
    if (X || Y) TRY(c.prec == CFD_PREC_MIXED ? c.geometry_mixed(true) : c.geometry(true, true));
    CFD_CUDA(cudaStreamSynchronize(c.stream));
    return c.tcollect();
}

int cfd_ctx_set_clock(cfd_ctx* ctx, int iter, double time, double dtmin1, int bandera,
                      double disn1, double disn2) {
    if (!ctx) return arg_error("ctx");
    Ctx& c = ctx->impl;
    c.iter = iter;
    c.time = time;
    c.disn[0] = disn1;
    c.disn[1] = disn2;
    c.bandera_host = bandera;
    StepScal sc{};
    CFD_CUDA(cudaMemcpyAsync(&sc, c.d_scal, sizeof(sc), cudaMemcpyDeviceToHost, c.stream));
    CFD_CUDA(cudaStreamSynchronize(c.stream));
    sc.dtmin1 = dtmin1;
    sc.bandera = bandera;
    sc.iter = iter;
    CFD_CUDA(cudaMemcpyAsync(c.d_scal, &sc, sizeof(sc), cudaMemcpyHostToDevice, c.stream));
    if (c.d_motion) {  // the structural model's velocities and accelerations are kept
        MotionScal ms{};
        CFD_CUDA(cudaMemcpyAsync(&ms, c.d_motion, sizeof(ms), cudaMemcpyDeviceToHost, c.stream));
        CFD_CUDA(cudaStreamSynchronize(c.stream));
        ms.time = time;
        ms.disn0 = disn1;
        ms.disn1 = disn2;
        CFD_CUDA(cudaMemcpyAsync(c.d_motion, &ms, sizeof(ms), cudaMemcpyHostToDevice, c.stream));
    }
    CFD_CUDA(cudaStreamSynchronize(c.stream));
    return CFD_OK;
}

int cfd_ctx_set_guess_net(cfd_ctx* ctx, cfd_mpnn* net, double gate) {
    if (!ctx) return arg_error("ctx");
    if (!(gate >= 0.0)) return arg_error("gate");
    return ctx->impl.set_guess_net(net, gate);
}

int cfd_ctx_set_guess_refine(cfd_ctx* ctx, int on) {
    if (!ctx) return arg_error("ctx");
    return ctx->impl.set_guess_refine(on != 0);
}

int cfd_ctx_guess_stats_ex(cfd_ctx* ctx, long long* out8) {
    if (!ctx || !out8) return arg_error("null pointer");
    Ctx& c = ctx->impl;
    for (int k = 0; k < 8; ++k) out8[k] = 0;
    if (!c.d_gstats) return CFD_OK;
    CFD_CUDA(cudaMemcpyAsync(out8, c.d_gstats, 8 * sizeof(long long), cudaMemcpyDeviceToHost,
                             c.stream));
    CFD_CUDA(cudaStreamSynchronize(c.stream));
    out8[3] = c.guess_steps;
    out8[7] = 0;
    return CFD_OK;
}

int cfd_ctx_guess_stats(cfd_ctx* ctx, long long* out4) {
    if (!ctx || !out4) return arg_error("null pointer");
    Ctx& c = ctx->impl;
    if (!c.d_gstats) {
        for (int k = 0; k < 4; ++k) out4[k] = 0;
        return CFD_OK;
    }
    CFD_CUDA(cudaMemcpyAsync(out4, c.d_gstats, 3 * sizeof(long long), cudaMemcpyDeviceToHost,
                             c.stream));
    CFD_CUDA(cudaStreamSynchronize(c.stream));
    out4[3] = c.guess_steps;
    return CFD_OK;
}

int cfd_ctx_set_force_visc(cfd_ctx* ctx, int each_step) {
    if (!ctx) return arg_error("ctx");
    Ctx& c = ctx->impl;
    TRY(c.set_force_visc_each_step(each_step != 0));
    CFD_CUDA(cudaStreamSynchronize(c.stream));
    return CFD_OK;
}

int cfd_ctx_set_smoothing(cfd_ctx* ctx, int every) {
    if (!ctx) return arg_error("ctx");
    TRY(ctx->impl.set_smoothing(every));
    return CFD_OK;
}

int cfd_ctx_smoothing_stats(cfd_ctx* ctx, long long* out2) {
    if (!ctx || !out2) return arg_error("null pointer");
    out2[0] = ctx->impl.smooth_steps;
    out2[1] = ctx->impl.smooth_sweeps;
    return CFD_OK;
}

int cfd_ctx_force_visc(cfd_ctx* ctx, double* F_VX, double* F_VY, double* skin) {
    if (!ctx || !F_VX || !F_VY) return arg_error("null pointer");
    Ctx& c = ctx->impl;
    if (!c.fv_each) TRY(c.force_visc_now());
    double fv[20];
    CFD_CUDA(cudaMemcpyAsync(fv, c.d_fv, sizeof(fv), cudaMemcpyDeviceToHost, c.stream));
    const size_t ne = c.bc.set_elem.size();
    if (skin && ne)
        CFD_CUDA(cudaMemcpyAsync(skin, c.d_fv_skin, 3 * ne * sizeof(double),
                                 cudaMemcpyDeviceToHost, c.stream));
    CFD_CUDA(cudaStreamSynchronize(c.stream));
    for (int s = 0; s < 10; ++s) {
        F_VX[s] = fv[s];
        F_VY[s] = fv[10 + s];
    }
    return CFD_OK;
}

int cfd_ctx_smooth(cfd_ctx* ctx, int* iters, double* min_quality) {
    if (!ctx) return arg_error("ctx");
    return ctx->impl.smooth(iters, min_quality);
}

int cfd_ctx_smooth_ex(cfd_ctx* ctx, int visit, int* iters, double* min_quality) {
    if (!ctx) return arg_error("ctx");
    if (visit != CFD_SMOOTH_COLOUR && visit != CFD_SMOOTH_NODE_ORDER) return arg_error("order");
    return ctx->impl.smooth(iters, min_quality, visit == CFD_SMOOTH_NODE_ORDER);
}

int cfd_ctx_graph_state(cfd_ctx* ctx, long long* out3) {
    if (!ctx || !out3) return arg_error("null pointer");
    const Ctx& c = ctx->impl;
    out3[0] = c.graphs_on ? 1 : 0;
    out3[1] = c.graph_replays;
    out3[2] = c.graph_kernels;
    return CFD_OK;
}

int cfd_step(cfd_ctx* ctx, int nsteps, cfd_step_report* rep) {
    if (!ctx) return arg_error("ctx");
    return ctx->impl.step(nsteps, rep);
}

int cfd_ctx_download_state(cfd_ctx* ctx, double* U, double* T, double* X, double* Y) {
    if (!ctx) return arg_error("ctx");
    Ctx& c = ctx->impl;
    const size_t N = c.npoin;
    if (T && c.prec == CFD_PREC_MIXED) TRY(c.widen_mixed(1));
    if (U) CFD_CUDA(cudaMemcpyAsync(U, c.d_U, 32 * N, cudaMemcpyDeviceToHost, c.stream));
    if (T) CFD_CUDA(cudaMemcpyAsync(T, c.d_T, 8 * N, cudaMemcpyDeviceToHost, c.stream));
    if (X) CFD_CUDA(cudaMemcpyAsync(X, c.d_X, 8 * N, cudaMemcpyDeviceToHost, c.stream));
    if (Y) CFD_CUDA(cudaMemcpyAsync(Y, c.d_Y, 8 * N, cudaMemcpyDeviceToHost, c.stream));
    CFD_CUDA(cudaStreamSynchronize(c.stream));
    return CFD_OK;
}

int cfd_ctx_download_fields(cfd_ctx* ctx, double* RHO, double* VEL_X, double* VEL_Y, double* E,
                            double* P, double* RMACH, double* W_X, double* W_Y) {
    if (!ctx) return arg_error("ctx");
    Ctx& c = ctx->impl;
    const size_t n8 = 8 * (size_t)c.npoin;
    if (c.prec == CFD_PREC_MIXED) TRY(c.widen_mixed(2));
    const double* src[8] = {c.d_RHO, c.d_VX, c.d_VY, c.d_E, c.d_P, c.d_RMACH, c.d_WX, c.d_WY};
    double* dst[8] = {RHO, VEL_X, VEL_Y, E, P, RMACH, W_X, W_Y};
    for (int i = 0; i < 8; ++i)
        if (dst[i]) CFD_CUDA(cudaMemcpyAsync(dst[i], src[i], n8, cudaMemcpyDeviceToHost, c.stream));
    CFD_CUDA(cudaStreamSynchronize(c.stream));
    return CFD_OK;
}

int cfd_ctx_download_motion(cfd_ctx* ctx, double* xpos, double* ypos) {
    if (!ctx) return arg_error("ctx");
    Ctx& c = ctx->impl;
    const size_t n8 = 8 * (size_t)c.npoin;
    if (xpos) CFD_CUDA(cudaMemcpyAsync(xpos, c.d_pos[0], n8, cudaMemcpyDeviceToHost, c.stream));
    if (ypos) CFD_CUDA(cudaMemcpyAsync(ypos, c.d_pos[1], n8, cudaMemcpyDeviceToHost, c.stream));
    CFD_CUDA(cudaStreamSynchronize(c.stream));
    return CFD_OK;
}

int cfd_ctx_download_geometry(cfd_ctx* ctx, double* area, double* dNx, double* dNy, double* M) {
    if (!ctx) return arg_error("ctx");
    Ctx& c = ctx->impl;
    const size_t E = c.nelem;
    if ((dNx || dNy || area) && c.prec == CFD_PREC_MIXED) TRY(c.widen_mixed(4));
    if (area) CFD_CUDA(cudaMemcpyAsync(area, c.d_area, 8 * E, cudaMemcpyDeviceToHost, c.stream));
    if (M) CFD_CUDA(cudaMemcpyAsync(M, c.d_M, 8 * (size_t)c.npoin, cudaMemcpyDeviceToHost, c.stream));
    std::vector<double> g;
    if (dNx || dNy) {
        g.resize(6 * E);
        CFD_CUDA(cudaMemcpyAsync(g.data(), c.d_geo, 48 * E, cudaMemcpyDeviceToHost, c.stream));
    }
    CFD_CUDA(cudaStreamSynchronize(c.stream));
    for (size_t e = 0; e < E && !g.empty(); ++e)
        for (int i = 0; i < 3; ++i) {
            if (dNx) dNx[3 * e + i] = g[i * E + e];
            if (dNy) dNy[3 * e + i] = g[(3 + i) * E + e];
        }
    return CFD_OK;
}

int cfd_ctx_download_laplace(cfd_ctx* ctx, double* val) {
    if (!ctx || !val) return arg_error("ctx/val");
    Ctx& c = ctx->impl;
    const size_t n = (size_t)c.nnz;
    if (c.prec != CFD_PREC_MIXED) {
        CFD_CUDA(cudaMemcpyAsync(val, c.d_val, 8 * n, cudaMemcpyDeviceToHost, c.stream));
        CFD_CUDA(cudaStreamSynchronize(c.stream));
        return CFD_OK;
    }
    double* tmp = nullptr;  // an inspection call: its own scratch
    CFD_CUDA(cudaMalloc(&tmp, 8 * n));
    k_widen_pair<<<blocks_for((long)n, 256), 256, 0, c.stream>>>(
        (long)n, (const float*)c.d_valf, (const float*)c.d_val_lo, tmp);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(val, tmp, 8 * n, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    cudaFree(tmp);
    CFD_CUDA(e);
    return CFD_OK;
}

int cfd_ctx_timers(cfd_ctx* ctx, double* seconds, int max, int* n) {
    if (!ctx || !seconds) return arg_error("ctx/seconds");
    int k = max < TM_N ? max : TM_N;
    for (int i = 0; i < k; ++i) seconds[i] = ctx->impl.seconds[i];
    if (n) *n = k;
    return CFD_OK;
}

int cfd_ctx_timer_calls(cfd_ctx* ctx, long long* calls, int max, int* n) {
    if (!ctx || !calls) return arg_error("ctx/calls");
    int k = max < TM_N ? max : TM_N;
    for (int i = 0; i < k; ++i) calls[i] = ctx->impl.calls[i];
    if (n) *n = k;
    return CFD_OK;
}

// ------------------------------------------------------------------ host-side adjacency
int cfd_get_esup(const int* inpoel, const int* nelem, const int* npoin, int* esup1, int* esup2) {
    if (!inpoel || bad_sizes(nelem, npoin) || !esup1 || !esup2) return arg_error("esup args");
    std::vector<int4> el;
    TRY(make_elems(inpoel, *nelem, *npoin, el));
    std::vector<int> ptr, slot;
    make_esup(inpoel, *nelem, *npoin, ptr, slot);
    for (int p = 0; p <= *npoin; ++p) esup2[p] = ptr[p];
    for (size_t s = 0; s < slot.size(); ++s) esup1[s] = slot[s] / 3 + 1;
    return CFD_OK;
}

int cfd_get_psup(const int* inpoel, const int* nelem, const int* npoin, int* psup1, int* psup2,
                 int* npsup) {
    if (!inpoel || bad_sizes(nelem, npoin)) return arg_error("psup args");
    Adjacency a;
    std::string why;
    int st = build_adjacency(*npoin, *nelem, inpoel, a, &why);
    if (st) { set_last_message(why); return st; }
    if (npsup) *npsup = (int)a.psup.size();
    if (psup2) for (int p = 0; p <= *npoin; ++p) psup2[p] = a.psup_ptr[p];
    if (psup1) for (size_t k = 0; k < a.psup.size(); ++k) psup1[k] = a.psup[k] + 1;
    return CFD_OK;
}

int cfd_laplace_pattern(const int* inpoel, const int* nelem, const int* npoin, int* lap_rowptr,
                        int* lap_idx, int* nnz) {
    if (!inpoel || bad_sizes(nelem, npoin)) return arg_error("pattern args");
    Adjacency a;
    std::string why;
    int st = build_adjacency(*npoin, *nelem, inpoel, a, &why);
    if (st) { set_last_message(why); return st; }
    if (nnz) *nnz = (int)a.col.size();
    if (!lap_idx) return CFD_OK;
    if (!lap_rowptr) return arg_error("lap_rowptr");
    for (int p = 0; p <= *npoin; ++p) lap_rowptr[p] = a.rowptr[p];
    for (size_t k = 0; k < a.col.size(); ++k) lap_idx[k] = a.col[k] + 1;
    return CFD_OK;
}

// ------------------------------------------------------------------ drop-in routines
int cfd_calcrhs(double* rhs, const double* U, const double* theta, const double* dNx,
                const double* dNy, const double* area, const double* shoc, const double* dtl,
                const double* t_sugn1, const double* t_sugn2, const double* t_sugn3,
                const int* inpoel, const int* nelem, const int* npoin, const double* T,
                const double* gas6) {
    if (!rhs || !U || !dNx || !dNy || !area || !shoc || !dtl || !t_sugn1 || !t_sugn2 ||
        !t_sugn3 || !inpoel || !T || !gas6 || bad_sizes(nelem, npoin))
        return arg_error("cfd_calcrhs");
    const int E = *nelem, N = *npoin;
    std::vector<int4> el;
    TRY(make_elems(inpoel, E, N, el));
    std::vector<int> ptr, slot;
    make_esup(inpoel, E, N, ptr, slot);
    std::vector<double> geo = to_geo(dNx, dNy, E);
    Scratch s;
    TRY(s.init());
    int4* d_el; int *d_ptr, *d_slot;
    double *d_U, *d_th = nullptr, *d_geo, *d_area, *d_shoc, *d_dtl, *d_t1, *d_t2, *d_t3, *d_T,
           *d_rhs, *d_c;
    TRY(s.put(&d_el, el.data(), E));
    TRY(s.put(&d_ptr, ptr.data(), N + 1));
    TRY(s.put(&d_slot, slot.data(), 3 * (size_t)E));
    TRY(s.put(&d_U, U, 4 * (size_t)N));
    if (theta) TRY(s.put(&d_th, theta, 4 * (size_t)N));
    TRY(s.put(&d_geo, geo.data(), 6 * (size_t)E));
    TRY(s.put(&d_area, area, E));
    TRY(s.put(&d_shoc, shoc, E));
    TRY(s.put(&d_dtl, dtl, E));
    TRY(s.put(&d_t1, t_sugn1, E));
    TRY(s.put(&d_t2, t_sugn2, E));
    TRY(s.put(&d_t3, t_sugn3, E));
    TRY(s.put(&d_T, T, N));
    TRY(s.put(&d_rhs, rhs, 4 * (size_t)N));
    TRY(s.alloc(&d_c, 12 * (size_t)E));
    GasConst gc{gas6[0], gas6[1], gas6[2], gas6[3], gas6[4], gas6[5]};
    const bool visc = gc.mu_ref > 2.2250738585072014e-308;
    const double* nd = nullptr;
    double* ndo = nullptr;
    CFD_CUDA(launch_elem_rhs(visc, theta != nullptr, s.stream, E, d_el, d_U, d_th, d_T, d_geo,
                             d_area, d_shoc, d_dtl, nd, d_t1, d_t2, d_t3, gc, d_c, nd, nd, ndo));
    CFD_LAUNCH(k_node_update, blocks_for(N, 256), 256, 0, s.stream, N, d_ptr, d_slot, d_c, nd, nd,
               nd, 0.0, 0.0, 0.0, (const unsigned char*)nullptr, (const double*)nullptr,
               (const double2*)nullptr, nd, nd, ndo, ndo, ndo, ndo, ndo, ndo, ndo, ndo, d_rhs, d_rhs);
    TRY(s.get(rhs, d_rhs, 4 * (size_t)N));
    return s.sync();
}

int cfd_fuente(double* rhs, const double* U, const double* W_X, const double* W_Y,
               const double* dNx, const double* dNy, const double* area, const double* dtl,
               const int* inpoel, const int* nelem, const int* npoin) {
    if (!rhs || !U || !W_X || !W_Y || !dNx || !dNy || !area || !dtl || !inpoel ||
        bad_sizes(nelem, npoin))
        return arg_error("cfd_fuente");
    const int E = *nelem, N = *npoin;
    std::vector<int4> el;
    TRY(make_elems(inpoel, E, N, el));
    std::vector<int> ptr, slot;
    make_esup(inpoel, E, N, ptr, slot);
    std::vector<double> geo = to_geo(dNx, dNy, E);
    Scratch s;
    TRY(s.init());
    int4* d_el; int *d_ptr, *d_slot;
    double *d_U, *d_wx, *d_wy, *d_geo, *d_area, *d_dtl, *d_rhs, *d_f;
    TRY(s.put(&d_el, el.data(), E));
    TRY(s.put(&d_ptr, ptr.data(), N + 1));
    TRY(s.put(&d_slot, slot.data(), 3 * (size_t)E));
    TRY(s.put(&d_U, U, 4 * (size_t)N));
    TRY(s.put(&d_wx, W_X, N));
    TRY(s.put(&d_wy, W_Y, N));
    TRY(s.put(&d_geo, geo.data(), 6 * (size_t)E));
    TRY(s.put(&d_area, area, E));
    TRY(s.put(&d_dtl, dtl, E));
    TRY(s.put(&d_rhs, rhs, 4 * (size_t)N));
    TRY(s.alloc(&d_f, 12 * (size_t)E));
    GasConst gc{};
    const double* nd = nullptr;
    double* ndo = nullptr;
    CFD_CUDA(launch_elem_rhs(false, false, s.stream, E, d_el, d_U, nd, nd, d_geo, d_area, nd, d_dtl,
                             nd, nd, nd, nd, gc, ndo, d_wx, d_wy, d_f));
    CFD_LAUNCH(k_node_update, blocks_for(N, 256), 256, 0, s.stream, N, d_ptr, d_slot, d_f, nd, nd,
               nd, 0.0, 0.0, 0.0, (const unsigned char*)nullptr, (const double*)nullptr,
               (const double2*)nullptr, nd, nd, ndo, ndo, ndo, ndo, ndo, ndo, ndo, ndo, d_rhs, d_rhs);
    TRY(s.get(rhs, d_rhs, 4 * (size_t)N));
    return s.sync();
}

int cfd_estab(const double* U, const double* T, const double* GAMM, const double* VEL_X,
              const double* VEL_Y, const double* W_X, const double* W_Y, const double* dNx,
              const double* dNy, const int* inpoel, const int* nelem, const int* npoin,
              const double* scal5, double* SHOC, double* T_SUGN1, double* T_SUGN2,
              double* T_SUGN3) {
    if (!U || !T || !GAMM || !VEL_X || !VEL_Y || !W_X || !W_Y || !dNx || !dNy || !inpoel ||
        !scal5 || !SHOC || !T_SUGN1 || !T_SUGN2 || !T_SUGN3 || bad_sizes(nelem, npoin))
        return arg_error("cfd_estab");
    const int E = *nelem, N = *npoin;
    std::vector<int4> el;
    TRY(make_elems(inpoel, E, N, el));
    std::vector<double> geo = to_geo(dNx, dNy, E);
    Scratch s;
    TRY(s.init());
    int4* d_el;
    double *d_U, *d_T, *d_G, *d_vx, *d_vy, *d_wx, *d_wy, *d_geo, *o[4];
    StepScal* d_sc;
    TRY(s.put(&d_el, el.data(), E));
    TRY(s.put(&d_U, U, 4 * (size_t)N));
    TRY(s.put(&d_T, T, N));
    TRY(s.put(&d_G, GAMM, N));
    TRY(s.put(&d_vx, VEL_X, N));
    TRY(s.put(&d_vy, VEL_Y, N));
    TRY(s.put(&d_wx, W_X, N));
    TRY(s.put(&d_wy, W_Y, N));
    TRY(s.put(&d_geo, geo.data(), 6 * (size_t)E));
    for (int i = 0; i < 4; ++i) TRY(s.alloc(&o[i], E));
    StepScal sc{};
    sc.dtmin = scal5[2];
    TRY(s.put(&d_sc, &sc, 1));
    CFD_LAUNCH(k_estab, blocks_for(E, 128), 128, 0, s.stream, E, d_el, d_U, d_T, scal5[0], d_G, d_vx,
               d_vy, d_wx, d_wy, d_geo, scal5[1], d_sc, scal5[3], scal5[4], (int)CFD_ESTAB_REFERENCE,
               0.0, 1.0, 0.0, o[0], o[1], o[2], o[3]);
    TRY(s.get(SHOC, o[0], E));
    TRY(s.get(T_SUGN1, o[1], E));
    TRY(s.get(T_SUGN2, o[2], E));
    TRY(s.get(T_SUGN3, o[3], E));
    return s.sync();
}

int cfd_deltat(const double* T, const double* VEL_X, const double* VEL_Y, const double* W_X,
               const double* W_Y, const double* area, const int* inpoel, const int* nelem,
               const int* npoin, const double* scal4, double* DT, double* DTMIN) {
    if (!T || !VEL_X || !VEL_Y || !W_X || !W_Y || !area || !inpoel || !scal4 || !DT || !DTMIN ||
        bad_sizes(nelem, npoin))
        return arg_error("cfd_deltat");
    const int E = *nelem, N = *npoin;
    std::vector<int4> el;
    TRY(make_elems(inpoel, E, N, el));
    Scratch s;
    TRY(s.init());
    int4* d_el;
    double *d_T, *d_vx, *d_vy, *d_wx, *d_wy, *d_a, *d_DT;
    StepScal* d_sc;
    TRY(s.put(&d_el, el.data(), E));
    TRY(s.put(&d_T, T, N));
    TRY(s.put(&d_vx, VEL_X, N));
    TRY(s.put(&d_vy, VEL_Y, N));
    TRY(s.put(&d_wx, W_X, N));
    TRY(s.put(&d_wy, W_Y, N));
    TRY(s.put(&d_a, area, E));
    TRY(s.alloc(&d_DT, E));
    StepScal sc{};
    sc.dtmin_bits = 0x7ff0000000000000ull;
    sc.bandera = 1;
    TRY(s.put(&d_sc, &sc, 1));
    CFD_LAUNCH(k_deltat, blocks_for(E, 256), 256, 0, s.stream, E, d_el, d_T, d_vx, d_vy, d_wx, d_wy, d_a,
               scal4[0], scal4[3], d_DT, &d_sc->dtmin_bits);
    CFD_LAUNCH(k_dt_finalize, 1, 1, 0, s.stream, d_sc);
    CFD_LAUNCH(k_dt_clamp, blocks_for(E, 256), 256, 0, s.stream, E, d_DT, d_sc);
    TRY(s.get(DT, d_DT, E));
    TRY(s.get(&sc, d_sc, 1));
    TRY(s.sync());
    *DTMIN = sc.dtmin_raw;
    return CFD_OK;
}

int cfd_force_visc(const int* NELEM, const int* npoin, const int* nsets, const int* IELEM_SETS,
                   const int* ISET, const int* inpoel, const int* NSET_NUMB, const double* U_inf,
                   const double* V_inf, const double* RHO_inf, const double* T_inf,
                   const double* X, const double* Y, const double* P, const double* T,
                   const double* VEL_X, const double* VEL_Y, const double* DNX,
                   const double* DNY, const double* RMU, const double* RHO, double* F_VX,
                   double* F_VY, double* skin) {
    (void)RMU;
    (void)RHO;
    if (!NELEM || !npoin || !nsets || !IELEM_SETS || !ISET || !inpoel || !NSET_NUMB || !U_inf ||
        !V_inf || !RHO_inf || !T_inf || !X || !Y || !P || !T || !VEL_X || !VEL_Y || !DNX ||
        !DNY || !F_VX || !F_VY || bad_sizes(NELEM, npoin))
        return arg_error("cfd_force_visc");
    const int E = *NELEM, N = *npoin, NS = *nsets, nset = *NSET_NUMB;
    if (nset < 0 || nset > 10) return arg_error("NSET_NUMB");
    std::vector<int> ptr(11, 0), eel;
    std::vector<int2> edges;
    for (int s = 0; s < nset; ++s) {
        if (IELEM_SETS[s] < 0 || IELEM_SETS[s] > NS) return arg_error("IELEM_SETS");
        for (int ii = 0; ii < IELEM_SETS[s]; ++ii) {
            const int* e = ISET + 3 * (s + 10 * (size_t)ii);
            if (e[0] < 1 || e[0] > N || e[1] < 1 || e[1] > N || e[2] < 1 || e[2] > E)
                return arg_error("ISET");
            edges.push_back(make_int2(e[0] - 1, e[1] - 1));
            eel.push_back(e[2] - 1);
        }
        ptr[s + 1] = (int)edges.size();
    }
    for (int s = nset; s < 10; ++s) ptr[s + 1] = ptr[s];
    std::vector<int4> el;
    TRY(make_elems(inpoel, E, N, el));
    const int ne = (int)edges.size();
    Scratch s;
    TRY(s.init());
    int4* d_el;
    int2* d_ed;
    int *d_ptr, *d_eel;
    double *d_X, *d_Y, *d_P, *d_T, *d_vx, *d_vy, *d_dnx, *d_dny, *d_terms, *d_skin, *d_fv;
    TRY(s.put(&d_el, el.data(), E));
    TRY(s.put(&d_ed, edges.data(), edges.size()));
    TRY(s.put(&d_ptr, ptr.data(), ptr.size()));
    TRY(s.put(&d_eel, eel.data(), eel.size()));
    TRY(s.put(&d_X, X, N));
    TRY(s.put(&d_Y, Y, N));
    TRY(s.put(&d_P, P, N));
    TRY(s.put(&d_T, T, N));
    TRY(s.put(&d_vx, VEL_X, N));
    TRY(s.put(&d_vy, VEL_Y, N));
    TRY(s.put(&d_dnx, DNX, 3 * (size_t)E));
    TRY(s.put(&d_dny, DNY, 3 * (size_t)E));
    TRY(s.alloc(&d_terms, 2 * (size_t)ne));
    TRY(s.alloc(&d_skin, 3 * (size_t)ne));
    TRY(s.alloc(&d_fv, 20));
    CFD_CUDA(launch_force_visc(s.stream, 0, nset, d_ptr, ne, d_ed, d_eel, d_el, d_dnx, d_dny, 3, 1,
                               nullptr, d_P, d_T, d_vx, d_vy, d_X, d_Y, *U_inf, *V_inf, *RHO_inf,
                               *T_inf, d_terms, skin ? d_skin : nullptr, d_fv));
    double fv[20];
    TRY(s.get(fv, d_fv, 20));
    if (skin) TRY(s.get(skin, d_skin, 3 * (size_t)ne));
    TRY(s.sync());
    for (int k = 0; k < 10; ++k) {
        F_VX[k] = fv[k];
        F_VY[k] = fv[10 + k];
    }
    return CFD_OK;
}

int cfd_smoothing(double* X, double* Y, const int* inpoel, const int* fixed, const int* npoin,
                  const int* nelem, const double* dX, const double* dY, int* iters,
                  double* min_quality) {
    return cfd_smoothing_ex(X, Y, inpoel, fixed, npoin, nelem, dX, dY, iters, min_quality,
                            CFD_SMOOTH_COLOUR);
}

int cfd_smoothing_ex(double* X, double* Y, const int* inpoel, const int* fixed, const int* npoin,
                     const int* nelem, const double* dX, const double* dY, int* iters,
                     double* min_quality, int visit) {
    if (!X || !Y || !inpoel || !fixed || bad_sizes(nelem, npoin) || (!dX != !dY) ||
        (visit != CFD_SMOOTH_COLOUR && visit != CFD_SMOOTH_NODE_ORDER))
        return arg_error("cfd_smoothing");
    const int E = *nelem, N = *npoin;
    std::vector<int4> el;
    TRY(make_elems(inpoel, E, N, el));
    Adjacency adj;
    std::string why;
    if (int st = build_adjacency(N, E, inpoel, adj, &why)) {
        set_last_message(why);
        return st;
    }
    std::vector<int> order, offs;
    smoothing_colours(adj, N, order, offs);
    std::vector<unsigned char> fx(N);
    for (int p = 0; p < N; ++p) fx[p] = fixed[p] ? 1 : 0;
    std::vector<double> tol;
    if (dX) {  // setTol_move (smoothing.f90:372-386)
        tol.resize(N);
        for (int p = 0; p < N; ++p) tol[p] = std::fabs(dX[p]) + std::fabs(dY[p]);
    }
    int max_star = 0;
    for (int p = 0; p < N; ++p) max_star = std::max(max_star, adj.esup_ptr[p + 1] - adj.esup_ptr[p]);
    Scratch s;
    TRY(s.init());
    int4* d_el;
    int *d_ep, *d_es, *d_pp, *d_ps, *d_ord, *d_flags;
    unsigned char *d_fx, *d_sm;
    double *d_X, *d_Y, *d_tol = nullptr;
    unsigned long long* d_scal;
    TRY(s.put(&d_el, el.data(), E));
    TRY(s.put(&d_ep, adj.esup_ptr.data(), adj.esup_ptr.size()));
    TRY(s.put(&d_es, adj.esup_slot.data(), adj.esup_slot.size()));
    TRY(s.put(&d_pp, adj.psup_ptr.data(), adj.psup_ptr.size()));
    TRY(s.put(&d_ps, adj.psup.data(), adj.psup.size()));
    TRY(s.put(&d_ord, order.data(), order.size()));
    TRY(s.put(&d_fx, fx.data(), fx.size()));
    TRY(s.put(&d_X, X, N));
    TRY(s.put(&d_Y, Y, N));
    if (dX) TRY(s.put(&d_tol, tol.data(), tol.size()));
    TRY(s.alloc(&d_sm, N));
    TRY(s.alloc(&d_scal, 3));
    TRY(s.alloc(&d_flags, 2));
    TRY(smooth_on_device(s.stream, N, E, d_el, d_ep, d_es, d_pp, d_ps, d_fx, d_X, d_Y, d_tol,
                         offs, d_ord, d_sm, d_scal, d_flags, iters, min_quality, max_star,
                         visit == CFD_SMOOTH_NODE_ORDER));
    TRY(s.get(X, d_X, N));
    TRY(s.get(Y, d_Y, N));
    return s.sync();
}

int cfd_deriv(const double* X, const double* Y, const int* inpoel, const int* nelem,
              const int* npoin, double* area, double* dNx, double* dNy, double* HH, double* HHX,
              double* HHY, double* hmin) {
    if (!X || !Y || !inpoel || !area || !dNx || !dNy || !HH || !HHX || !HHY || !hmin ||
        bad_sizes(nelem, npoin))
        return arg_error("cfd_deriv");
    const int E = *nelem, N = *npoin;
    std::vector<int4> el;
    TRY(make_elems(inpoel, E, N, el));
    Scratch s;
    TRY(s.init());
    int4* d_el;
    double *d_X, *d_Y, *d_a, *d_geo, *d_hh, *d_hx, *d_hy;
    unsigned long long* d_bits;
    TRY(s.put(&d_el, el.data(), E));
    TRY(s.put(&d_X, X, N));
    TRY(s.put(&d_Y, Y, N));
    TRY(s.alloc(&d_a, E));
    TRY(s.alloc(&d_geo, 6 * (size_t)E));
    TRY(s.alloc(&d_hh, E));
    TRY(s.alloc(&d_hx, E));
    TRY(s.alloc(&d_hy, E));
    unsigned long long inf = 0x7ff0000000000000ull;
    TRY(s.put(&d_bits, &inf, 1));
    CFD_LAUNCH(k_deriv, blocks_for(E, 256), 256, 0, s.stream, E, d_el, d_X, d_Y, d_a, d_geo, d_hh, d_hx, d_hy);
    CFD_LAUNCH(k_min_positive, 152, 256, 0, s.stream, (long)E, d_hh, d_bits);
    std::vector<double> geo(6 * (size_t)E);
    TRY(s.get(area, d_a, E));
    TRY(s.get(geo.data(), d_geo, 6 * (size_t)E));
    TRY(s.get(HH, d_hh, E));
    TRY(s.get(HHX, d_hx, E));
    TRY(s.get(HHY, d_hy, E));
    unsigned long long bits = 0;
    TRY(s.get(&bits, d_bits, 1));
    TRY(s.sync());
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < 3; ++i) {
            dNx[3 * e + i] = geo[i * (size_t)E + e];
            dNy[3 * e + i] = geo[(3 + i) * (size_t)E + e];
        }
    double h;
    std::memcpy(&h, &bits, sizeof(h));
    if (h > 1.0e10) h = 1.0e10;  // subrutinas.f90:125 (also when no element is positive)
    *hmin = h;
    return CFD_OK;
}

int cfd_masas(const double* area, const int* inpoel, const int* nelem, const int* npoin, double* M) {
    if (!area || !inpoel || !M || bad_sizes(nelem, npoin)) return arg_error("cfd_masas");
    const int E = *nelem, N = *npoin;
    std::vector<int4> el;
    TRY(make_elems(inpoel, E, N, el));
    std::vector<int> ptr, slot;
    make_esup(inpoel, E, N, ptr, slot);
    Scratch s;
    TRY(s.init());
    int *d_ptr, *d_slot;
    double *d_a, *d_M;
    TRY(s.put(&d_ptr, ptr.data(), N + 1));
    TRY(s.put(&d_slot, slot.data(), 3 * (size_t)E));
    TRY(s.put(&d_a, area, E));
    TRY(s.alloc(&d_M, N));
    CFD_LAUNCH(k_mass, blocks_for(N, 256), 256, 0, s.stream, N, d_ptr, d_slot, d_a, d_M);
    TRY(s.get(M, d_M, N));
    return s.sync();
}

int cfd_gcl(double* M, const double* W_x, const double* W_y, const double* W_x_old,
            const double* W_y_old, const double* dNx, const double* dNy, const double* area,
            const double* area_old, const int* inpoel, const int* nelem, const int* npoin,
            const double* dt, int mode) {
    if (!M || !W_x || !W_y || !W_x_old || !W_y_old || !dNx || !dNy || !area || !area_old ||
        !inpoel || !dt || bad_sizes(nelem, npoin))
        return arg_error("cfd_gcl");
    if (mode != CFD_MASS_GCL_LITERAL && mode != CFD_MASS_GCL_CORRECTED) return arg_error("mode");
    const int E = *nelem, N = *npoin;
    std::vector<int4> el;
    TRY(make_elems(inpoel, E, N, el));
    std::vector<int> ptr, slot;
    make_esup(inpoel, E, N, ptr, slot);
    std::vector<double> geo = to_geo(dNx, dNy, E);
    Scratch s;
    TRY(s.init());
    int4* d_el; int *d_ptr, *d_slot;
    double *d_M, *d_wx, *d_wy, *d_wxo, *d_wyo, *d_geo, *d_a, *d_ao, *d_dt;
    TRY(s.put(&d_el, el.data(), E));
    TRY(s.put(&d_ptr, ptr.data(), N + 1));
    TRY(s.put(&d_slot, slot.data(), 3 * (size_t)E));
    TRY(s.put(&d_M, M, N));
    TRY(s.put(&d_wx, W_x, N));
    TRY(s.put(&d_wy, W_y, N));
    TRY(s.put(&d_wxo, W_x_old, N));
    TRY(s.put(&d_wyo, W_y_old, N));
    TRY(s.put(&d_geo, geo.data(), 6 * (size_t)E));
    TRY(s.put(&d_a, area, E));
    TRY(s.put(&d_ao, area_old, E));
    TRY(s.put(&d_dt, dt, 1));
    double2* d_terms;
    TRY(s.alloc(&d_terms, E));
    CFD_CUDA(launch_gcl(s.stream, N, E, d_el, d_ptr, d_slot, d_geo, d_a, d_ao, d_wx, d_wy, d_wxo,
                        d_wyo, d_dt, mode == CFD_MASS_GCL_LITERAL ? 1 : 0, d_terms, d_M));
    TRY(s.get(M, d_M, N));
    return s.sync();
}

int cfd_laplace(const int* inpoel, const double* area, const double* dNx, const double* dNy,
                const int* nelem, const int* npoin, const double* X, const double* Y,
                double* lap_sparse, const int* lap_idx, const int* lap_rowptr, double* lap_diag) {
    (void)area;  // accepted and unused, as mLaplace.f90:16
    if (!inpoel || !dNx || !dNy || !X || !Y || !lap_sparse || !lap_idx || !lap_rowptr ||
        !lap_diag || bad_sizes(nelem, npoin))
        return arg_error("cfd_laplace");
    const int E = *nelem, N = *npoin;
    std::vector<int4> el;
    TRY(make_elems(inpoel, E, N, el));
    std::vector<int> ptr, slot;
    make_esup(inpoel, E, N, ptr, slot);
    // positions by the reference's linear search (mLaplace.f90:46-50) in the caller's pattern
    std::vector<uchar4> pos(3 * (size_t)E);
    for (int p = 0; p < N; ++p) {
        const int r0 = lap_rowptr[p], r1 = lap_rowptr[p + 1];
        if (r1 - r0 > 255 || r1 < r0) return arg_error("lap_rowptr");
        for (int s2 = ptr[p]; s2 < ptr[p + 1]; ++s2) {
            int e = slot[s2] / 3;
            unsigned char o[3];
            for (int j = 0; j < 3; ++j) {
                int q = inpoel[3 * e + j];
                int off = -1;
                for (int k = r0; k < r1; ++k)
                    if (lap_idx[k] == q) { off = k - r0; break; }
                if (off < 0) {
                    set_last_message("lap_idx misses a node of an element around row " + std::to_string(p + 1));
                    return CFD_ERR_MESH;
                }
                o[j] = (unsigned char)off;
            }
            pos[s2] = make_uchar4(o[0], o[1], o[2], 0);
        }
    }
    std::vector<double> geo = to_geo(dNx, dNy, E);
    const int nnz = lap_rowptr[N];
    Scratch s;
    TRY(s.init());
    int4* d_el; int *d_ptr, *d_slot, *d_rp;
    uchar4* d_pos;
    double *d_geo, *d_X, *d_Y, *d_v, *d_d;
    TRY(s.put(&d_el, el.data(), E));
    TRY(s.put(&d_ptr, ptr.data(), N + 1));
    TRY(s.put(&d_slot, slot.data(), 3 * (size_t)E));
    TRY(s.put(&d_pos, pos.data(), 3 * (size_t)E));
    TRY(s.put(&d_rp, lap_rowptr, N + 1));
    TRY(s.put(&d_geo, geo.data(), 6 * (size_t)E));
    TRY(s.put(&d_X, X, N));
    TRY(s.put(&d_Y, Y, N));
    TRY(s.alloc(&d_v, nnz));
    TRY(s.alloc(&d_d, N));
    double* d_q;
    TRY(s.alloc(&d_q, E));
    CFD_CUDA(launch_laplace(s.stream, N, E, d_el, d_ptr, d_slot, d_pos, d_geo, d_X, d_Y, d_rp, d_q,
                            d_v, d_d));
    TRY(s.get(lap_sparse, d_v, nnz));
    TRY(s.get(lap_diag, d_d, N));
    return s.sync();
}

int cfd_bicg_mode(const double* spMtx, const int* spIdx, const int* spRowptr,
                  const double* diagMtx, double* x, const double* b, const double* x_fix,
                  const int* x_fixIdx, const int* npoin, const int* nfix, double tol, int maxit,
                  int tol_mode, cfd_solve_info* info) {
    if (!spMtx || !spIdx || !spRowptr || !diagMtx || !x || !b || !npoin || !nfix || *npoin <= 0 ||
        *nfix < 0 || (*nfix > 0 && (!x_fix || !x_fixIdx)) || maxit < 0 ||
        tol_mode < CFD_BICG_TOL_ABS || tol_mode > CFD_BICG_TOL_REL_R0)
        return arg_error("cfd_bicg");
    const int N = *npoin, NF = *nfix;
    const int nnz = spRowptr[N];
    if (spRowptr[0] != 0 || nnz < 0) return arg_error("spRowptr");
    std::vector<int> col(nnz);
    for (int k = 0; k < nnz; ++k) {
        if (spIdx[k] < 1 || spIdx[k] > N) {
            set_last_message("spIdx outside 1..npoin");
            return CFD_ERR_MESH;
        }
        col[k] = spIdx[k] - 1;
    }
    std::vector<unsigned char> isfix(N, 0);
    std::vector<int> last(N, -1);
    for (int k = 0; k < NF; ++k) {
        if (x_fixIdx[k] < 1 || x_fixIdx[k] > N) {
            set_last_message("x_fixIdx outside 1..npoin");
            return CFD_ERR_MESH;
        }
        last[x_fixIdx[k] - 1] = k;
    }
    std::vector<int> unode, usrc;
    for (int p = 0; p < N; ++p)
        if (last[p] >= 0) {
            isfix[p] = 1;
            unode.push_back(p);
            usrc.push_back(last[p]);
        }
    Scratch s;
    TRY(s.init());
    int *d_rp, *d_col, *d_un, *d_us, *d_it, *d_cv;
    unsigned char* d_isfix;
    double *d_val, *d_diag, *d_x, *d_b, *d_fv, *d_r, *d_z, *d_y, *d_p0, *d_p1, *d_part, *d_rz;
    GridBar* d_bar;
    TRY(s.put(&d_rp, spRowptr, N + 1));
    TRY(s.put(&d_col, col.data(), nnz));
    TRY(s.put(&d_val, spMtx, nnz));
    TRY(s.put(&d_diag, diagMtx, N));
    TRY(s.put(&d_isfix, isfix.data(), N));
    TRY(s.put(&d_un, unode.data(), unode.size()));
    TRY(s.put(&d_us, usrc.data(), usrc.size()));
    TRY(s.put(&d_fv, NF ? x_fix : (const double*)&tol, NF ? NF : 1));
    TRY(s.put(&d_x, x, N));
    TRY(s.put(&d_b, b, N));
    for (double** q : {&d_r, &d_z, &d_y, &d_p0, &d_p1}) TRY(s.alloc(q, N));
    const long nc = ((long)N + kChunk - 1) / kChunk;
    TRY(s.alloc(&d_part, 6 * (size_t)nc));
    TRY(s.alloc(&d_bar, 1));
    TRY(s.alloc(&d_it, 2));
    TRY(s.alloc(&d_cv, 2));
    TRY(s.alloc(&d_rz, 4));
    CFD_CUDA(cudaMemsetAsync(d_bar, 0, sizeof(GridBar), s.stream));
    PcgArgs a{};
    a.n = N;
    a.nsolve = 1;
    a.rowptr = d_rp;
    a.col = d_col;
    a.val = d_val;
    a.diag = d_diag;
    a.isfix = d_isfix;
    a.nfix = (int)unode.size();
    a.fix_node = d_un;
    a.fix_src = d_us;
    a.fixval[0] = a.fixval[1] = d_fv;
    a.x[0] = a.x[1] = d_x;
    a.b[0] = a.b[1] = d_b;
    a.r[0] = a.r[1] = d_r;
    a.z[0] = a.z[1] = d_z;
    a.y[0] = a.y[1] = d_y;
    a.p[0][0] = a.p[1][0] = d_p0;
    a.p[0][1] = a.p[1][1] = d_p1;
    a.part = d_part;
    a.bar = d_bar;
    a.tol = tol;
    a.maxit = maxit;
    a.tol_mode = tol_mode;
    a.iters_out = d_it;
    a.rz_out = d_rz;
    a.relres_out = d_rz + 2;
    a.conv_out = d_cv;
    int dev = 0, nsm = 0, per_sm = 0;
    CFD_CUDA(cudaGetDevice(&dev));
    CFD_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    CFD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_fp64, 256, 0));
    long g = (long)nsm * (per_sm > 0 ? per_sm : 1);
    if (g > nc) g = nc;
    if (g < 1) g = 1;
    void* args[] = {&a};
    CFD_CUDA(cudaLaunchCooperativeKernel((void*)k_pcg_fp64, dim3((unsigned)g), dim3(256), args, 0, s.stream));
    g_launches.fetch_add(1, std::memory_order_relaxed);
    int it = 0, cv = 0;
    double rz[4] = {0.0, 0.0, 0.0, 0.0};
    GridBar gb{};
    TRY(s.get(x, d_x, N));
    TRY(s.get(&it, d_it, 1));
    TRY(s.get(&cv, d_cv, 1));
    TRY(s.get(rz, d_rz, 4));
    TRY(s.get(&gb, d_bar, 1));
    TRY(s.sync());
    if (gb.err) {
        set_last_message("a grid barrier of the BiCG kernel gave up waiting");
        return CFD_ERR_BARRIER;
    }
    if (info) {
        info->iters = it;
        info->converged = cv;
        info->rz = rz[0];
        info->relres = rz[2];
    }
    return CFD_OK;
}

int cfd_bicg_ex(const double* spMtx, const int* spIdx, const int* spRowptr, const double* diagMtx,
                double* x, const double* b, const double* x_fix, const int* x_fixIdx,
                const int* npoin, const int* nfix, double tol, int maxit, cfd_solve_info* info) {
    return cfd_bicg_mode(spMtx, spIdx, spRowptr, diagMtx, x, b, x_fix, x_fixIdx, npoin, nfix, tol,
                         maxit, CFD_BICG_TOL_ABS, info);
}

int cfd_bicg(const double* spMtx, const int* spIdx, const int* spRowptr, const double* diagMtx,
             double* x, const double* b, const double* x_fix, const int* x_fixIdx, const int* npoin,
             const int* nfix, cfd_solve_info* info) {
    return cfd_bicg_ex(spMtx, spIdx, spRowptr, diagMtx, x, b, x_fix, x_fixIdx, npoin, nfix, 1.0e-10,
                       1000, info);
}

}  // extern "C"

// noalloc.cu — a BiCG entry point that performs no device allocation.
//
// Some callers cannot call cudaMalloc at the point where they need a mesh-motion solve:
// a host that owns all of the device memory itself (a CUDA Fortran / OpenACC code whose
// arrays are already resident, or a framework with its own memory pool and a fixed
// budget), or a time loop that must not allocate once it is running.  For them
// cfd_bicg_device_noalloc solves on arrays that are already in device memory and keeps
// its work vectors in one file-scope static device array of fixed size.  The CUDA runtime
// creates that array when it loads this file's module on a device; with lazy module
// loading (the default since CUDA 12.2, CUDA_MODULE_LOADING=LAZY) that happens inside the
// first call on each device, at its cudaGetSymbolAddress, so a caller whose own pool will
// take all free device memory makes that first call during its set-up.  Later calls on the
// device use the address found then and allocate nothing.
#include <cuda_runtime.h>

#include <mutex>

#include "cfd_context.cuh"

namespace cfd {
namespace {

// Work space: r, z, y and the two search directions (5 vectors of npoin doubles), the
// chunk partial sums of the dots (4 x npoin/1024), then a 256-byte control block with the
// grid barrier and the solve's outputs.
constexpr int kNoallocMaxN = CFD_NOALLOC_MAX_NPOIN;
constexpr long kVecBytes = 5L * kNoallocMaxN * 8;
constexpr long kPartBytes = 4L * ((kNoallocMaxN + kChunk - 1) / kChunk) * 8;
constexpr long kCtlBytes = 256;
constexpr long kScratchBytes = kVecBytes + kPartBytes + kCtlBytes;

static __device__ __align__(256) unsigned char g_bicg_scratch[kScratchBytes];

struct NoallocCtl {
    GridBar bar;
    int iters[2];
    int conv[2];
    double rz[2];
};
static_assert(sizeof(NoallocCtl) <= kCtlBytes, "control block");

// device address of g_bicg_scratch, looked up once per device
constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {};
int g_grid[kMaxDevices] = {};

int scratch_for_current_device(unsigned char** addr, int* grid) {
    int dev = 0;
    CFD_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_last_message("device ordinal above the no-allocation table");
        return CFD_ERR_LIMIT;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        CFD_CUDA(cudaGetSymbolAddress(&p, g_bicg_scratch));
        int nsm = 0, per_sm = 0;
        CFD_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        CFD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_fp64, 256, 0));
        g_grid[dev] = nsm * (per_sm > 0 ? per_sm : 1);
        g_addr[dev] = (unsigned char*)p;
    }
    *addr = g_addr[dev];
    *grid = g_grid[dev];
    return CFD_OK;
}

}  // namespace
}  // namespace cfd

using namespace cfd;

extern "C" int cfd_bicg_device_noalloc(const double* spMtx, const int* col, const int* rowptr,
                                       const double* diag, const unsigned char* isfix, double* x,
                                       const double* b, int npoin, double tol, int maxit,
                                       void* stream, cfd_solve_info* info) {
    if (!spMtx || !col || !rowptr || !diag || !isfix || !x || npoin <= 0 || maxit < 0) {
        set_last_message("invalid argument: cfd_bicg_device_noalloc");
        return CFD_ERR_ARG;
    }
    if (npoin > kNoallocMaxN) {
        set_last_message("npoin above CFD_NOALLOC_MAX_NPOIN of cfd_bicg_device_noalloc");
        return CFD_ERR_LIMIT;
    }
    unsigned char* base = nullptr;
    int maxgrid = 1;
    int st = scratch_for_current_device(&base, &maxgrid);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const long N = npoin;
    double* v = (double*)base;
    NoallocCtl* ctl = (NoallocCtl*)(base + kVecBytes + kPartBytes);
    const long nc = (N + kChunk - 1) / kChunk;
    PcgArgs a{};
    a.n = npoin;
    a.nsolve = 1;
    a.rowptr = rowptr;
    a.col = col;
    a.val = spMtx;
    a.diag = diag;
    a.isfix = isfix;
    a.nfix = 0;  // Dirichlet values are already in x at the isfix rows
    a.x[0] = a.x[1] = x;
    a.b[0] = a.b[1] = b;
    a.r[0] = a.r[1] = v;
    a.z[0] = a.z[1] = v + N;
    a.y[0] = a.y[1] = v + 2 * N;
    a.p[0][0] = a.p[1][0] = v + 3 * N;
    a.p[0][1] = a.p[1][1] = v + 4 * N;
    a.part = (double*)(base + kVecBytes);
    a.bar = &ctl->bar;
    a.tol = tol;
    a.maxit = maxit;
    a.iters_out = ctl->iters;
    a.rz_out = ctl->rz;
    a.conv_out = ctl->conv;
    // the barrier starts at zero; every other word is written before it is read
    CFD_CUDA(cudaMemsetAsync(&ctl->bar, 0, sizeof(GridBar), s));
    long g = maxgrid < nc ? maxgrid : nc;
    if (g < 1) g = 1;
    void* args[] = {&a};
    CFD_CUDA(cudaLaunchCooperativeKernel((void*)k_pcg_fp64, dim3((unsigned)g), dim3(256), args, 0, s));
    g_launches.fetch_add(1, std::memory_order_relaxed);
    NoallocCtl h{};
    CFD_CUDA(cudaMemcpyAsync(&h, ctl, sizeof(h), cudaMemcpyDeviceToHost, s));
    CFD_CUDA(cudaStreamSynchronize(s));
    if (h.bar.err) {
        set_last_message("a grid barrier of the BiCG kernel gave up waiting");
        return CFD_ERR_BARRIER;
    }
    if (info) {
        info->iters = h.iters[0];
        info->converged = h.conv[0];
        info->rz = h.rz[0];
        info->relres = 0.0;
    }
    return CFD_OK;
}

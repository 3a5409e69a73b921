// smooth.cu — the mesh smoothing of smoothing.f90 (module smoothing_mod), GPU variant.
//
// The reference visits the nodes one after another, in node order, and every move is seen
// by the nodes after it (smoothing.f90:55-67, :80-114).  Here the nodes are coloured so that
// no two nodes of a colour share an element (a greedy colouring of the point-neighbour
// graph): the nodes of one colour move at the same time, each seeing the moves of the
// colours before it.  Per node the operations are the reference's: the quality metric mu
// (:351-362) and the length h (:364-377), two Laplacian sweeps that keep a move only when
// the node's worst element does not get worse (:74-114), then up to NITER worklist sweeps
// of finite-difference gradient ascent on the node's worst element with the reference's
// step rule and halving line search (:116-272), a moved node putting its neighbours back on
// the worklist (:300-309), until the largest squared move of a sweep is below
// FACTOR_TOL_DIST * H_MIN_GLOBAL (:58-66).  With tol_move (setTol_move, :372-386) the
// moves are limited by each node's own displacement of the step.
#include <cstring>
#include <vector>

#include "cfd_context.cuh"

namespace cfd {
namespace {

constexpr double TWOSQRT3 = 3.46410161513775;
constexpr int kMaxStar = 32;  // elements around a node (the reference's array holds 20)
constexpr int NITER = 100, MITER = 2, NTRY = 8;
constexpr double TOL_METRIC = .85, FACTOR_TOL_DIST = 1e-2, FACTOR_DELTA = 1e-2;
constexpr double FACTOR_PLUS = 1.0, FACTOR_STEP = 3.0;
constexpr double TINY = 2.2250738585072014e-308;  // tiny(1.d0)

struct SmArgs {
    int npoin, nelem;
    const int4* elem;                   // 0-based nodes
    const int *esup_ptr, *esup_slot;    // element-around-point slots (3*e + local index)
    const int *psup_ptr, *psup;         // point neighbours
    const unsigned char* fixed;
    unsigned char* smoothable;
    double *X, *Y;
    const double* tol_move;             // null: SWITCH_TOL_MOVE off
    const unsigned long long* hmin_bits;  // H_MIN_GLOBAL
    unsigned long long* dmax_bits;      // d_max of the sweep
    const int* order;                   // nodes grouped by colour
    int begin, end;                     // this colour's range of order
};

// mu (smoothing.f90:351-362)
__device__ double sm_mu(const double x[3], const double y[3]) {
    const double area = x[1] * y[2] + x[2] * y[0] + x[0] * y[1] -
                        (x[1] * y[0] + x[2] * y[1] + x[0] * y[2]);
    const double l1 = (x[2] - x[1]) * (x[2] - x[1]) + (y[2] - y[1]) * (y[2] - y[1]);
    const double l2 = (x[0] - x[2]) * (x[0] - x[2]) + (y[0] - y[2]) * (y[0] - y[2]);
    const double l3 = (x[1] - x[0]) * (x[1] - x[0]) + (y[1] - y[0]) * (y[1] - y[0]);
    const double l = l1 + l2 + l3;
    return TWOSQRT3 * area / l;
}

// h (smoothing.f90:364-377)
__device__ double sm_h(const double x[3], const double y[3]) {
    const double area = x[1] * y[2] + x[2] * y[0] + x[0] * y[1] -
                        (x[1] * y[0] + x[2] * y[1] + x[0] * y[2]);
    const double d1 = fabs(x[2] - x[1]) + fabs(y[2] - y[1]);
    const double d2 = fabs(x[0] - x[2]) + fabs(y[0] - y[2]);
    const double d3 = fabs(x[1] - x[0]) + fabs(y[1] - y[0]);
    const double d = d1 + d2 + d3;
    return fabs(area) / d;
}

// coordinates of element e with node p at (xp, yp)
__device__ __forceinline__ void sm_elem(const SmArgs& a, int e, int p, double xp, double yp,
                                        double x[3], double y[3]) {
    const int4 n = a.elem[e];
    const int nn[3] = {n.x, n.y, n.z};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        x[j] = nn[j] == p ? xp : a.X[nn[j]];
        y[j] = nn[j] == p ? yp : a.Y[nn[j]];
    }
}

// getMu_vec (:190-213); returns the star size
__device__ int sm_mu_vec(const SmArgs& a, int p, double xp, double yp, double* mu, int* min_idx) {
    const int s0 = a.esup_ptr[p], s1 = a.esup_ptr[p + 1];
    double mu_min = 1.0;
    if (min_idx) *min_idx = 0;
    for (int s = s0; s < s1; ++s) {
        double x[3], y[3];
        sm_elem(a, a.esup_slot[s] / 3, p, xp, yp, x, y);
        const double mu1 = sm_mu(x, y);
        mu[s - s0] = mu1;
        if (min_idx && mu1 < mu_min) {
            mu_min = mu1;
            *min_idx = s - s0;
        }
    }
    return s1 - s0;
}

// getMu_min (:215-230)
__device__ double sm_mu_min(const SmArgs& a, int p, double xp, double yp) {
    double m = 1.0;
    for (int s = a.esup_ptr[p]; s < a.esup_ptr[p + 1]; ++s) {
        double x[3], y[3];
        sm_elem(a, a.esup_slot[s] / 3, p, xp, yp, x, y);
        const double mu1 = sm_mu(x, y);
        if (mu1 <= m) m = mu1;
    }
    return m;
}

// getH_min (:280-298)
__device__ double sm_h_min(const SmArgs& a, int p, double xp, double yp) {
    double m = 1.0;
    for (int s = a.esup_ptr[p]; s < a.esup_ptr[p + 1]; ++s) {
        double x[3], y[3];
        sm_elem(a, a.esup_slot[s] / 3, p, xp, yp, x, y);
        const double h1 = sm_h(x, y);
        if (h1 < m) m = h1;
    }
    return m;
}

__device__ __forceinline__ double hmin_global(const SmArgs& a) {
    return __longlong_as_double((long long)*a.hmin_bits);
}

// checkMesh (:388-404): smoothable nodes and H_MIN_GLOBAL; any != 0 when a node is marked
__global__ void k_sm_check(SmArgs a, unsigned long long* hmin_bits, int* any) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.nelem) return;
    const int4 n = a.elem[e];
    const double x[3] = {a.X[n.x], a.X[n.y], a.X[n.z]}, y[3] = {a.Y[n.x], a.Y[n.y], a.Y[n.z]};
    if (sm_mu(x, y) < TOL_METRIC) {
        a.smoothable[n.x] = 1;
        a.smoothable[n.y] = 1;
        a.smoothable[n.z] = 1;
        *any = 1;
    }
    const double h1 = sm_h(x, y);
    if (h1 >= 0.0) atomicMin(hmin_bits, (unsigned long long)__double_as_longlong(h1));
}

// laplacianSmoothing (:74-114) of node p
__device__ void sm_laplace_node(const SmArgs& a, int p) {
    if (!a.smoothable[p] || a.fixed[p]) return;
    const double xo = a.X[p], yo = a.Y[p];
    const double mu_old = sm_mu_min(a, p, xo, yo);
    double xn = 0.0, yn = 0.0;
    const int q0 = a.psup_ptr[p], q1 = a.psup_ptr[p + 1];
    for (int q = q0; q < q1; ++q) {
        xn = xn + a.X[a.psup[q]];
        yn = yn + a.Y[a.psup[q]];
    }
    const double n = (double)(q1 - q0);
    xn = xn / n;
    yn = yn / n;
    if (a.tol_move) {
        const double dx = xn - xo, dy = yn - yo;
        const double t = a.tol_move[p];
        xn = xo + dx / (fabs(dx) + fabs(dy)) * t / 2 * FACTOR_STEP;
        yn = yo + dy / (fabs(dx) + fabs(dy)) * t / 2 * FACTOR_STEP;
    }
    if (sm_mu_min(a, p, xn, yn) < mu_old) return;  // if worse, restore
    a.X[p] = xn;
    a.Y[p] = yn;
}

// laplacianSmoothing over one colour
__global__ void k_sm_laplace(SmArgs a) {
    const int k = a.begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.end) return;
    sm_laplace_node(a, a.order[k]);
}

// one visit of the worklist sweep (:58-66) to node p: moveIpoin (:116-188) with getG
// (:232-255) and getStep (:257-278)
__device__ void sm_sweep_node(const SmArgs& a, int p) {
    if (!a.smoothable[p] || a.fixed[p]) return;
    a.smoothable[p] = 0;
    double mu[kMaxStar], gx[kMaxStar], gy[kMaxStar];
    int min_idx;
    const double x0 = a.X[p], y0 = a.Y[p];
    const int ns = sm_mu_vec(a, p, x0, y0, mu, &min_idx);
    if (!(mu[min_idx] < TOL_METRIC)) return;
    const double DELTA = hmin_global(a) * FACTOR_DELTA;
    double xc = x0, yc = y0;
    for (int i = 0; i < MITER; ++i) {
        const double mu_min = mu[min_idx];
        const double x_old = xc, y_old = yc;
        sm_mu_vec(a, p, xc + DELTA, yc, gx, nullptr);
        for (int s = 0; s < ns; ++s) gx[s] = (gx[s] - mu[s]) / DELTA;
        sm_mu_vec(a, p, xc, yc + DELTA, gy, nullptr);
        for (int s = 0; s < ns; ++s) gy[s] = (gy[s] - mu[s]) / DELTA;
        const double gx_min = gx[min_idx], gy_min = gy[min_idx];
        const double g2 = gx_min * gx_min + gy_min * gy_min;
        double step;
        if (a.tol_move)
            step = a.tol_move[p] / ((fabs(gx_min) + fabs(gy_min)) * NITER);
        else
            step = sm_h_min(a, p, xc, yc) * FACTOR_STEP / (fabs(gx_min) + fabs(gy_min));
        for (int s = 0; s < ns; ++s) {
            const double gg = gx_min * gx[s] + gy_min * gy[s];
            if (gg < 0) {
                const double step1 = (mu[s] - mu_min) / (g2 - gg);
                if (step1 < step) step = step1;
            }
        }
        bool accepted = false;
        for (int j = 0; j < NTRY; ++j) {  // the trial moves accumulate, as in the reference
            xc = xc + step * gx_min;
            yc = yc + step * gy_min;
            int min_new;
            sm_mu_vec(a, p, xc, yc, mu, &min_new);
            if (mu[min_new] > mu_min * FACTOR_PLUS) {
                min_idx = min_new;
                accepted = true;
                break;
            }
            step = .5 * step;
        }
        if (!accepted) {
            xc = x_old;
            yc = y_old;
            break;
        }
    }
    a.X[p] = xc;
    a.Y[p] = yc;
    const double d_move = (xc - x0) * (xc - x0) + (yc - y0) * (yc - y0);
    atomicMax(a.dmax_bits, (unsigned long long)__double_as_longlong(d_move));
    if (d_move > TINY)
        for (int q = a.psup_ptr[p]; q < a.psup_ptr[p + 1]; ++q) a.smoothable[a.psup[q]] = 1;
}

// one worklist sweep over one colour
__global__ void __launch_bounds__(128) k_sm_sweep(SmArgs a) {
    const int k = a.begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.end) return;
    sm_sweep_node(a, a.order[k]);
}

// The reference's own order: one thread visits every node in node order, each visit seeing
// every move before it (smoothing.f90:55-67 and :80-114 as written).  The chain of
// dependences runs through the whole mesh (on the O-grids every ring's first node follows
// the previous ring's last), so this order has no parallel form; it is the setup-time
// parity variant, the colour kernels above the parallel one.
__global__ void k_sm_laplace_seq(SmArgs a) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int p = 0; p < a.npoin; ++p) sm_laplace_node(a, p);
}

__global__ void k_sm_sweep_seq(SmArgs a) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int p = 0; p < a.npoin; ++p) sm_sweep_node(a, p);
}

// doubles as unsigned integers in the same order (for atomicMin of any sign)
__host__ __device__ inline unsigned long long ordered_bits(unsigned long long u) {
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__host__ __device__ inline unsigned long long unordered_bits(unsigned long long o) {
    return (o >> 63) ? (o & 0x7fffffffffffffffull) : ~o;
}

// getMeshQuality (:379-386): the minimum mu, starting from 1, in ordered bits
__global__ void k_sm_quality(SmArgs a, unsigned long long* qbits) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.nelem) return;
    const int4 n = a.elem[e];
    const double x[3] = {a.X[n.x], a.X[n.y], a.X[n.z]}, y[3] = {a.Y[n.x], a.Y[n.y], a.Y[n.z]};
    const double m = sm_mu(x, y);
    atomicMin(qbits, ordered_bits((unsigned long long)__double_as_longlong(m)));
}

}  // namespace

// Per-step smoothing inside the time loop (the setTol_move path): tol = |xpos| + |ypos|,
// the step's displacement, and the mesh before smoothing
__global__ void k_smooth_prep(int n, const double* __restrict__ xpos,
                              const double* __restrict__ ypos, const double* __restrict__ X,
                              const double* __restrict__ Y, double* __restrict__ tol,
                              double* __restrict__ xb, double* __restrict__ yb) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        tol[p] = fabs(xpos[p]) + fabs(ypos[p]);
        xb[p] = X[p];
        yb[p] = Y[p];
    }
}

// ... and after it: W is the whole move of the step over DTMIN (the prescribed displacement
// plus the smoothing's), so that the geometric conservation law sees the mesh that is
// used; the mixed form also refreshes its float shadows of W and of (X, Y)
__global__ void k_smooth_w(int n, const double* __restrict__ xpos, const double* __restrict__ ypos,
                           const double* __restrict__ X, const double* __restrict__ Y,
                           const double* __restrict__ xb, const double* __restrict__ yb,
                           const StepScal* __restrict__ sc, double* __restrict__ WX,
                           double* __restrict__ WY, float2* __restrict__ Wf,
                           float2* __restrict__ Xhi, float2* __restrict__ Xlo) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const double x = X[p], y = Y[p];
        const double dx = x - xb[p], dy = y - yb[p];
        if (dx == 0.0 && dy == 0.0) continue;
        const double mx = xpos[p] + dx, my = ypos[p] + dy;
        if (Wf) {
            const double wx = mx * sc->inv_dtmin, wy = my * sc->inv_dtmin;
            WX[p] = wx;
            WY[p] = wy;
            Wf[p] = make_float2(d2f_trunc(wx), d2f_trunc(wy));
            float hx, lx, hy, ly;
            split_bits(x, hx, lx);
            split_bits(y, hy, ly);
            Xhi[p] = make_float2(hx, hy);
            Xlo[p] = make_float2(lx, ly);
        } else {
            WX[p] = mx / sc->dtmin;
            WY[p] = my / sc->dtmin;
        }
    }
}

// Greedy colouring of the point-neighbour graph in node order; returns the nodes grouped by
// colour (node order within a colour) and the colour offsets.
void smoothing_colours(const Adjacency& adj, int npoin, std::vector<int>& order,
                       std::vector<int>& offs) {
    std::vector<int> col(npoin, -1), mark;
    int ncol = 0;
    for (int p = 0; p < npoin; ++p) {
        mark.assign(ncol + 1, 0);
        for (int q = adj.psup_ptr[p]; q < adj.psup_ptr[p + 1]; ++q)
            if (col[adj.psup[q]] >= 0) mark[col[adj.psup[q]]] = 1;
        int c = 0;
        while (mark[c]) ++c;
        col[p] = c;
        if (c == ncol) ++ncol;
    }
    offs.assign(ncol + 1, 0);
    for (int p = 0; p < npoin; ++p) offs[col[p] + 1] += 1;
    for (int c = 0; c < ncol; ++c) offs[c + 1] += offs[c];
    order.resize(npoin);
    std::vector<int> fill(offs.begin(), offs.end() - 1);
    for (int p = 0; p < npoin; ++p) order[fill[col[p]]++] = p;
}

// The whole smoothing (the reference's `smoothing` subroutine) on device arrays.  scratch:
// the device copies of the colour order; iters: the reference's loop counter at exit
// (NITER + 1 when the sweeps did not settle, 0 when no element was below TOL_METRIC).
int smooth_on_device(cudaStream_t st, int npoin, int nelem, const int4* elem,
                     const int* esup_ptr, const int* esup_slot, const int* psup_ptr,
                     const int* psup, const unsigned char* fixed, double* X, double* Y,
                     const double* tol_move, const std::vector<int>& offs, const int* order,
                     unsigned char* smoothable, unsigned long long* scal, int* flags,
                     int* iters_out, double* min_quality_out, int max_star, bool node_order) {
    if (max_star > kMaxStar) {
        set_last_message("a node has more elements around it than the smoothing handles (32)");
        return CFD_ERR_LIMIT;
    }
    SmArgs a{};
    a.npoin = npoin;
    a.nelem = nelem;
    a.elem = elem;
    a.esup_ptr = esup_ptr;
    a.esup_slot = esup_slot;
    a.psup_ptr = psup_ptr;
    a.psup = psup;
    a.fixed = fixed;
    a.smoothable = smoothable;
    a.X = X;
    a.Y = Y;
    a.tol_move = tol_move;
    a.hmin_bits = scal;
    a.dmax_bits = scal + 1;
    a.order = order;
    // checkMesh: H_MIN_GLOBAL starts at 1 (:395)
    unsigned long long h0[3];
    const double one = 1.0;
    std::memcpy(&h0[0], &one, 8);
    h0[1] = 0ull;
    h0[2] = ordered_bits(h0[0]);
    CFD_CUDA(cudaMemcpyAsync(scal, h0, sizeof(h0), cudaMemcpyHostToDevice, st));
    CFD_CUDA(cudaMemsetAsync(smoothable, 0, (size_t)npoin, st));
    CFD_CUDA(cudaMemsetAsync(flags, 0, 2 * sizeof(int), st));
    const unsigned ge = blocks_for(nelem, 256);
    CFD_LAUNCH(k_sm_check, ge, 256, 0, st, a, scal, flags);
    int any = 0;
    CFD_CUDA(cudaMemcpyAsync(&any, flags, sizeof(int), cudaMemcpyDeviceToHost, st));
    CFD_CUDA(cudaStreamSynchronize(st));
    int iter = 0;
    if (any) {
        const int ncol = (int)offs.size() - 1;
        for (int it = 0; it < 2; ++it) {
            if (node_order) {
                CFD_LAUNCH(k_sm_laplace_seq, 1, 1, 0, st, a);
                continue;
            }
            for (int c = 0; c < ncol; ++c) {
                a.begin = offs[c];
                a.end = offs[c + 1];
                CFD_LAUNCH(k_sm_laplace, blocks_for(a.end - a.begin, 128), 128, 0, st, a);
            }
        }
        unsigned long long hb = 0;
        CFD_CUDA(cudaMemcpyAsync(&hb, scal, 8, cudaMemcpyDeviceToHost, st));
        CFD_CUDA(cudaStreamSynchronize(st));
        double hmin;
        std::memcpy(&hmin, &hb, 8);
        const double TOL_DIST = FACTOR_TOL_DIST * hmin;
        for (iter = 1; iter <= NITER; ++iter) {
            CFD_CUDA(cudaMemsetAsync(scal + 1, 0, 8, st));  // d_max = 0
            if (node_order) {
                CFD_LAUNCH(k_sm_sweep_seq, 1, 1, 0, st, a);
            } else {
                for (int c = 0; c < ncol; ++c) {
                    a.begin = offs[c];
                    a.end = offs[c + 1];
                    CFD_LAUNCH(k_sm_sweep, blocks_for(a.end - a.begin, 128), 128, 0, st, a);
                }
            }
            unsigned long long db = 0;
            CFD_CUDA(cudaMemcpyAsync(&db, scal + 1, 8, cudaMemcpyDeviceToHost, st));
            CFD_CUDA(cudaStreamSynchronize(st));
            double d_max;
            std::memcpy(&d_max, &db, 8);
            if (d_max < TOL_DIST) break;
        }
    }
    if (iters_out) *iters_out = iter;
    if (min_quality_out) {
        CFD_LAUNCH(k_sm_quality, ge, 256, 0, st, a, scal + 2);
        unsigned long long qb = 0;
        CFD_CUDA(cudaMemcpyAsync(&qb, scal + 2, 8, cudaMemcpyDeviceToHost, st));
        CFD_CUDA(cudaStreamSynchronize(st));
        qb = unordered_bits(qb);
        double q;
        std::memcpy(&q, &qb, 8);
        *min_quality_out = q;
    }
    return CFD_OK;
}

}  // namespace cfd

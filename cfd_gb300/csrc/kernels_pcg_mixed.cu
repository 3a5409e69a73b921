// kernels_pcg_mixed.cu — biCG (biconjGrad.f90:117-171) for the mixed-precision form.
//
// Same persistent two-phase iteration as k_pcg_fp64 (kernels_pcg.cu) with the matrix in
// FP32 and the SpMV accumulated in FP32 over FP32 shadows of the search direction p and of
// z; the vectors x, r, z, p, y, the Jacobi scaling (as a multiply by 1/diag), the dots (in
// the fixed tree of cfd_common.cuh) and the scalars alfa, beta stay FP64.
#include "cfd_kernels.cuh"

namespace cfd {

__device__ __forceinline__ double spmv_row_f(const PcgArgs& a, int i, const double* v) {
    float dot = 0.f;
    const int j1 = a.rowptr[i + 1];
    for (int j = a.rowptr[i]; j < j1; ++j) dot += a.valf[j] * (float)v[a.col[j]];
    return (double)dot;
}

__device__ __forceinline__ double spmv_row_dir_f(const PcgArgs& a, int i, const float* pf,
                                                 const float* zf, float beta) {
    float dot = 0.f;
    const int j1 = a.rowptr[i + 1];
    for (int j = a.rowptr[i]; j < j1; ++j) {
        const int c = a.col[j];
        dot += a.valf[j] * (beta * pf[c] + zf[c]);
    }
    return (double)dot;
}

__device__ __forceinline__ bool bar_failed_m(GridBar* gb) {
    return *((volatile int*)&gb->err) != 0;
}

__global__ void __launch_bounds__(256) k_pcg_mixed(PcgArgs a) {
    __shared__ double red[9];
    const int t = threadIdx.x;
    const int n = a.n;
    const int ns = a.nsolve;
    const long nc = ((long)n + kChunk - 1) / kChunk;
    const unsigned nb = gridDim.x;
    auto part = [&](int buf, int s) { return a.part + ((long)buf * 2 + s) * nc; };

    for (int k = blockIdx.x * blockDim.x + t; k < a.nfix; k += gridDim.x * blockDim.x)
        for (int s = 0; s < ns; ++s) a.x[s][a.fix_node[k]] = a.fixval[s][a.fix_src[k]];
    grid_barrier(a.bar, nb);
    if (bar_failed_m(a.bar)) return;

    // y = A.x; y(fix) = 1e30 x(fix); r = b - y; r(fix) = 0; r.r
    for (long c = blockIdx.x; c < nc; c += gridDim.x) {
        double acc[2] = {0.0, 0.0};
        for (int k = 0; k < 4; ++k) {
            const long i = c * kChunk + t + 256L * k;
            if (i >= n) break;
            const bool fx = a.isfix[i];
            for (int s = 0; s < ns; ++s) {
                const double yi = fx ? 1.0e30 * a.x[s][i] : spmv_row_f(a, (int)i, a.x[s]);
                a.y[s][i] = yi;
                const double ri = fx ? 0.0 : (a.b[s] ? a.b[s][i] : 0.0) - yi;
                a.r[s][i] = ri;
                acc[s] = (k == 0) ? ri * ri : acc[s] + ri * ri;
            }
        }
        for (int s = 0; s < ns; ++s) {
            const double v = block_tree256(acc[s], red);
            if (t == 0) part(0, s)[c] = v;
        }
    }
    grid_barrier(a.bar, nb);
    if (bar_failed_m(a.bar)) return;
    bool done[2] = {true, true};
    double err_old[2] = {0.0, 0.0}, alfa[2] = {0.0, 0.0};
    for (int s = 0; s < ns; ++s) {
        const double rr = fold_partials(part(0, s), nc, red);
        done[s] = rr < a.tol;
        if (done[s] && blockIdx.x == 0 && t == 0) {
            a.iters_out[s] = 0;
            a.rz_out[s] = rr;
            a.conv_out[s] = 1;
        }
    }
    if (done[0] && (ns < 2 || done[1])) return;

    // p = r/diag; err = r.p
    for (long c = blockIdx.x; c < nc; c += gridDim.x) {
        double acc[2] = {0.0, 0.0};
        for (int k = 0; k < 4; ++k) {
            const long i = c * kChunk + t + 256L * k;
            if (i >= n) break;
            const double id = a.invdiag[i];
            for (int s = 0; s < ns; ++s) {
                if (done[s]) continue;
                const double ri = a.r[s][i];
                const double pi = ri * id;
                a.p[s][0][i] = pi;
                a.pf[s][0][i] = (float)pi;
                acc[s] = (k == 0) ? ri * pi : acc[s] + ri * pi;
            }
        }
        for (int s = 0; s < ns; ++s) {
            if (done[s]) continue;
            const double v = block_tree256(acc[s], red);
            if (t == 0) part(1, s)[c] = v;
        }
    }
    grid_barrier(a.bar, nb);
    if (bar_failed_m(a.bar)) return;
    double err_new[2] = {0.0, 0.0};
    for (int s = 0; s < ns; ++s)
        if (!done[s]) err_new[s] = fold_partials(part(1, s), nc, red);

    // y = A.p (FP32 over the shadow); py = p.y
    for (long c = blockIdx.x; c < nc; c += gridDim.x) {
        double acc[2] = {0.0, 0.0};
        for (int k = 0; k < 4; ++k) {
            const long i = c * kChunk + t + 256L * k;
            if (i >= n) break;
            const bool fx = a.isfix[i];
            for (int s = 0; s < ns; ++s) {
                if (done[s]) continue;
                const double pi = a.p[s][0][i];
                const double yi = fx ? 1.0e30 * pi : spmv_row_dir_f(a, (int)i, a.pf[s][0], a.pf[s][0], 0.f);
                a.y[s][i] = yi;
                acc[s] = (k == 0) ? pi * yi : acc[s] + pi * yi;
            }
        }
        for (int s = 0; s < ns; ++s) {
            if (done[s]) continue;
            const double v = block_tree256(acc[s], red);
            if (t == 0) part(0, s)[c] = v;
        }
    }
    grid_barrier(a.bar, nb);
    if (bar_failed_m(a.bar)) return;
    bool pend[2] = {false, false};
    int cur[2] = {0, 0};
    for (int s = 0; s < ns; ++s) {
        if (done[s]) continue;
        const double py = fold_partials(part(0, s), nc, red);
        alfa[s] = err_new[s] / py;
        err_old[s] = err_new[s];
        pend[s] = true;
    }

    int k = 0;
    int last_iter[2] = {0, 0};
    while (true) {
        bool act[2] = {false, false};
        for (int s = 0; s < ns; ++s) act[s] = !done[s] && fabs(err_old[s]) > a.tol && k < a.maxit;
        if (!act[0] && !act[1]) break;
        k = k + 1;
        // phase 1: x += alfa p; r -= alfa y; z = r/diag; r.z
        for (long c = blockIdx.x; c < nc; c += gridDim.x) {
            double acc[2] = {0.0, 0.0};
            for (int kk = 0; kk < 4; ++kk) {
                const long i = c * kChunk + t + 256L * kk;
                if (i >= n) break;
                const double id = a.invdiag[i];
                for (int s = 0; s < ns; ++s) {
                    if (pend[s]) a.x[s][i] += alfa[s] * a.p[s][cur[s]][i];
                    if (!act[s]) continue;
                    const double ri = a.r[s][i] - alfa[s] * a.y[s][i];
                    const double zi = ri * id;
                    a.r[s][i] = ri;
                    a.z[s][i] = zi;
                    a.zf[s][i] = (float)zi;
                    acc[s] = (kk == 0) ? ri * zi : acc[s] + ri * zi;
                }
            }
            for (int s = 0; s < ns; ++s) {
                if (!act[s]) continue;
                const double v = block_tree256(acc[s], red);
                if (t == 0) part(1, s)[c] = v;
            }
        }
        for (int s = 0; s < ns; ++s) pend[s] = false;
        grid_barrier(a.bar, nb);
        if (bar_failed_m(a.bar)) return;
        double beta[2] = {0.0, 0.0};
        for (int s = 0; s < ns; ++s) {
            if (!act[s]) continue;
            err_new[s] = fold_partials(part(1, s), nc, red);
            beta[s] = err_new[s] / err_old[s];
        }
        // phase 2: p_new = beta p + z (FP64 for the row, FP32 shadow for the SpMV); y = A p_new
        for (long c = blockIdx.x; c < nc; c += gridDim.x) {
            double acc[2] = {0.0, 0.0};
            for (int kk = 0; kk < 4; ++kk) {
                const long i = c * kChunk + t + 256L * kk;
                if (i >= n) break;
                const bool fx = a.isfix[i];
                for (int s = 0; s < ns; ++s) {
                    if (!act[s]) continue;
                    const double pn = beta[s] * a.p[s][cur[s]][i] + a.z[s][i];
                    const double yi = fx ? 1.0e30 * pn
                                         : spmv_row_dir_f(a, (int)i, a.pf[s][cur[s]], a.zf[s], (float)beta[s]);
                    a.p[s][cur[s] ^ 1][i] = pn;
                    a.pf[s][cur[s] ^ 1][i] = (float)pn;
                    a.y[s][i] = yi;
                    acc[s] = (kk == 0) ? pn * yi : acc[s] + pn * yi;
                }
            }
            for (int s = 0; s < ns; ++s) {
                if (!act[s]) continue;
                const double v = block_tree256(acc[s], red);
                if (t == 0) part(0, s)[c] = v;
            }
        }
        grid_barrier(a.bar, nb);
        if (bar_failed_m(a.bar)) return;
        for (int s = 0; s < ns; ++s) {
            if (!act[s]) continue;
            const double py = fold_partials(part(0, s), nc, red);
            alfa[s] = err_new[s] / py;
            err_old[s] = err_new[s];
            cur[s] ^= 1;
            pend[s] = true;
            last_iter[s] = k;
        }
    }
    for (long c = blockIdx.x; c < nc; c += gridDim.x)
        for (int kk = 0; kk < 4; ++kk) {
            const long i = c * kChunk + t + 256L * kk;
            if (i >= n) break;
            for (int s = 0; s < ns; ++s)
                if (pend[s]) a.x[s][i] += alfa[s] * a.p[s][cur[s]][i];
        }
    if (blockIdx.x == 0 && t == 0)
        for (int s = 0; s < ns; ++s) {
            if (done[s]) continue;
            a.iters_out[s] = last_iter[s];
            a.rz_out[s] = fabs(err_old[s]);
            a.conv_out[s] = fabs(err_old[s]) > a.tol ? 0 : 1;
        }
}

}  // namespace cfd

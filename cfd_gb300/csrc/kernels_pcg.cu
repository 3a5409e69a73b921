// kernels_pcg.cu — biCG (biconjGrad.f90:8-62) as one persistent cooperative kernel.
//
// The reference's solver is Jacobi-preconditioned CG with Dirichlet rows handled by
// overwrite and a 1e30 penalty; every vector operation is a separate OpenMP loop and the
// dots are OpenMP reductions.  Here the whole solve (both mesh-motion right-hand sides at
// once, sharing the matrix reads) is one launch: each iteration is three grid-wide passes
// separated by bounded grid barriers.
//   phase 1: x += alfa*p (deferred from the previous iteration), r -= alfa*y, z = r/diag,
//            partial sums of r.z (and of r.r under a relative stopping test)
//   phase 2: p_new = beta*p + z per row (biconjGrad.f90's vector update), a grid barrier,
//            then y = A.p_new, y(fix) = 1e30*p_new(fix), partial p.y
//   (the quotients z = r/diag use a reciprocal formed once per solve and two FMA
//   corrections, which give the division's bits: div_rcp)
// Every block folds the chunk partials itself in the fixed order of cfd_common.cuh, so
// all blocks hold bit-identical scalars and take the same branch.  With --fmad=false the
// iterates equal the CPU restatement's bit for bit.
#include "cfd_kernels.cuh"

namespace cfd {

__device__ __forceinline__ double spmv_row(const PcgArgs& a, int i, const double* v) {
    double dot = 0.0;
    const int j1 = a.rowptr[i + 1];
    for (int j = a.rowptr[i]; j < j1; ++j) dot = dot + a.val[j] * v[a.col[j]];
    return dot;
}

// Row i of A.v and, in the same column order, the sum over the Dirichlet columns only
// (the product with x_D, the vector that is v on the Dirichlet rows and 0 elsewhere; a
// skipped term adds +0, which leaves a sum that starts at +0 unchanged)
__device__ __forceinline__ double spmv_row_fixcols(const PcgArgs& a, int i, const double* v,
                                                   double& dfix) {
    double dot = 0.0, df = 0.0;
    const int j1 = a.rowptr[i + 1];
    for (int j = a.rowptr[i]; j < j1; ++j) {
        const int c = a.col[j];
        const double t = a.val[j] * v[c];
        dot = dot + t;
        if (a.isfix[c]) df = df + t;
    }
    dfix = df;
    return dot;
}

__device__ __forceinline__ bool bar_failed(GridBar* gb) {
    return *((volatile int*)&gb->err) != 0;
}

__global__ void __launch_bounds__(256, 3) k_pcg_fp64(PcgArgs a) {
    __shared__ double red[9];
    __shared__ double s_thr[2], s_ref2[2];  // relative modes: threshold on r.r, ref.ref
    const int t = threadIdx.x;
    const int n = a.n;
    const int ns = a.nsolve;
    const long nc = ((long)n + kChunk - 1) / kChunk;
    const unsigned nb = gridDim.x;
    auto part = [&](int buf, int s) { return a.part + ((long)buf * 2 + s) * nc; };
    const bool rel = a.tol_mode != CFD_BICG_TOL_ABS;      // r.r per iteration
    const bool relb = a.tol_mode == CFD_BICG_TOL_REL;     // ||b - A.x_D|| as reference

    // copy1 (biconjGrad.f90:28): x(fix) = x_fix
    for (int k = blockIdx.x * blockDim.x + t; k < a.nfix; k += gridDim.x * blockDim.x)
        for (int s = 0; s < ns; ++s) a.x[s][a.fix_node[k]] = 1.0 * a.fixval[s][a.fix_src[k]];
    grid_barrier(a.bar, nb);
    if (bar_failed(a.bar)) return;

    // y = A.x; y(fix) = 1e30*x(fix); r = -1*y + b; r(fix) = 0; r.r   (:138-144)
    // CFD_BICG_TOL_REL also forms b - A.x_D (0 on the Dirichlet rows) and its square sum
    for (long c = blockIdx.x; c < nc; c += gridDim.x) {
        double acc[2] = {0.0, 0.0}, accb[2] = {0.0, 0.0};
        for (int k = 0; k < 4; ++k) {
            const long i = c * kChunk + t + 256L * k;
            if (i >= n) break;
            const bool fx = a.isfix[i];
            for (int s = 0; s < ns; ++s) {
                double dfix = 0.0;
                double yi = fx ? 1.0e30 * a.x[s][i]
                               : (relb ? spmv_row_fixcols(a, (int)i, a.x[s], dfix)
                                       : spmv_row(a, (int)i, a.x[s]));
                a.y[s][i] = yi;
                const double bi = a.b[s] ? a.b[s][i] : 0.0;
                double ri = -1.0 * yi + bi;
                if (fx) ri = 0.0;
                a.r[s][i] = ri;
                acc[s] = (k == 0) ? ri * ri : acc[s] + ri * ri;
                if (relb) {
                    double ei = -1.0 * dfix + bi;
                    if (fx) ei = 0.0;
                    accb[s] = (k == 0) ? ei * ei : accb[s] + ei * ei;
                }
            }
        }
        for (int s = 0; s < ns; ++s) {
            double v = block_tree256(acc[s], red);
            if (t == 0) part(0, s)[c] = v;
            if (relb) {
                v = block_tree256(accb[s], red);
                if (t == 0) part(2, s)[c] = v;
            }
        }
    }
    grid_barrier(a.bar, nb);
    if (bar_failed(a.bar)) return;
    bool done[2] = {true, true};
    double err_old[2] = {0.0, 0.0}, alfa[2] = {0.0, 0.0};
    // relative modes: r.r of the current residual (rrc), and in shared memory the squared
    // reference norm and the threshold r.r <= tol^2 * ref.ref
    double rrc[2] = {0.0, 0.0};
    for (int s = 0; s < ns; ++s) {
        double rr = fold_partials(part(0, s), nc, red);
        if (rel) {
            const double ref2 = relb ? fold_partials(part(2, s), nc, red) : rr;
            if (t == 0) {
                s_ref2[s] = ref2;
                s_thr[s] = (a.tol * a.tol) * ref2;
            }
            __syncthreads();
            rrc[s] = rr;
            done[s] = rr <= s_thr[s];
        } else {
            done[s] = rr < a.tol;
        }
        if (done[s] && blockIdx.x == 0 && t == 0) {
            a.iters_out[s] = 0;
            a.rz_out[s] = rr;
            a.conv_out[s] = 1;
            if (a.relres_out)
                a.relres_out[s] = (rel && s_ref2[s] > 0.0) ? sqrt(rr / s_ref2[s]) : 0.0;
        }
    }
    if (done[0] && (ns < 2 || done[1])) return;

    // p = r/diag; err_new = r.p   (:146-147)
    for (long c = blockIdx.x; c < nc; c += gridDim.x) {
        double acc[2] = {0.0, 0.0};
        for (int k = 0; k < 4; ++k) {
            const long i = c * kChunk + t + 256L * k;
            if (i >= n) break;
            const double d = a.diag[i];
            if (a.rdiag) a.rdiag[i] = 1.0 / d;
            for (int s = 0; s < ns; ++s) {
                if (done[s]) continue;
                double ri = a.r[s][i];
                double pi = ri / d;
                a.p[s][0][i] = pi;
                acc[s] = (k == 0) ? ri * pi : acc[s] + ri * pi;
            }
        }
        for (int s = 0; s < ns; ++s) {
            if (done[s]) continue;
            double v = block_tree256(acc[s], red);
            if (t == 0) part(1, s)[c] = v;
        }
    }
    grid_barrier(a.bar, nb);
    if (bar_failed(a.bar)) return;
    double err_new[2] = {0.0, 0.0};
    for (int s = 0; s < ns; ++s)
        if (!done[s]) err_new[s] = fold_partials(part(1, s), nc, red);

    // y = A.p; y(fix) = 1e30*p(fix); py = p.y   (:148-151)
    for (long c = blockIdx.x; c < nc; c += gridDim.x) {
        double acc[2] = {0.0, 0.0};
        for (int k = 0; k < 4; ++k) {
            const long i = c * kChunk + t + 256L * k;
            if (i >= n) break;
            const bool fx = a.isfix[i];
            for (int s = 0; s < ns; ++s) {
                if (done[s]) continue;
                const double* p = a.p[s][0];
                double yi = fx ? 1.0e30 * p[i] : spmv_row(a, (int)i, p);
                a.y[s][i] = yi;
                acc[s] = (k == 0) ? p[i] * yi : acc[s] + p[i] * yi;
            }
        }
        for (int s = 0; s < ns; ++s) {
            if (done[s]) continue;
            double v = block_tree256(acc[s], red);
            if (t == 0) part(0, s)[c] = v;
        }
    }
    grid_barrier(a.bar, nb);
    if (bar_failed(a.bar)) return;
    bool pend[2] = {false, false};
    int cur[2] = {0, 0};
    for (int s = 0; s < ns; ++s) {
        if (done[s]) continue;
        double py = fold_partials(part(0, s), nc, red);
        alfa[s] = err_new[s] / py;  // :152
        err_old[s] = err_new[s];
        pend[s] = true;  // x = alfa*p + x (:153), applied in the next pass
    }

    int k = 0;
    int last_iter[2] = {0, 0};
    while (true) {  // :156-170
        bool act[2] = {false, false};
        for (int s = 0; s < ns; ++s)
            act[s] = !done[s] && (rel ? rrc[s] > s_thr[s] : fabs(err_old[s]) > a.tol) &&
                     k < a.maxit;
        if (!act[0] && !act[1]) break;
        k = k + 1;
        // phase 1
        for (long c = blockIdx.x; c < nc; c += gridDim.x) {
            double acc[2] = {0.0, 0.0}, accr[2] = {0.0, 0.0};
            for (int kk = 0; kk < 4; ++kk) {
                const long i = c * kChunk + t + 256L * kk;
                if (i >= n) break;
                const double d = a.diag[i];
                const double rd = a.rdiag ? a.rdiag[i] : 0.0;
                for (int s = 0; s < ns; ++s) {
                    if (pend[s]) a.x[s][i] = alfa[s] * a.p[s][cur[s]][i] + a.x[s][i];
                    if (!act[s]) continue;
                    double ri = (-alfa[s]) * a.y[s][i] + a.r[s][i];
                    double zi = a.rdiag ? div_rcp(ri, d, rd) : ri / d;
                    a.r[s][i] = ri;
                    a.z[s][i] = zi;
                    acc[s] = (kk == 0) ? ri * zi : acc[s] + ri * zi;
                    if (rel) accr[s] = (kk == 0) ? ri * ri : accr[s] + ri * ri;
                }
            }
            for (int s = 0; s < ns; ++s) {
                if (!act[s]) continue;
                double v = block_tree256(acc[s], red);
                if (t == 0) part(1, s)[c] = v;
                if (rel) {
                    v = block_tree256(accr[s], red);
                    if (t == 0) part(2, s)[c] = v;
                }
            }
        }
        for (int s = 0; s < ns; ++s) pend[s] = false;
        grid_barrier(a.bar, nb);
        if (bar_failed(a.bar)) return;
        double beta[2] = {0.0, 0.0};
        for (int s = 0; s < ns; ++s) {
            if (!act[s]) continue;
            err_new[s] = fold_partials(part(1, s), nc, red);
            if (rel) rrc[s] = fold_partials(part(2, s), nc, red);
            beta[s] = err_new[s] / err_old[s];
        }
        // phase 2a: p_new = beta p + z, once per row (the SpMV below reads it; forming it
        // inside every row's column loop would cost two FP64 operations per entry)
        for (long c = blockIdx.x; c < nc; c += gridDim.x)
            for (int kk = 0; kk < 4; ++kk) {
                const long i = c * kChunk + t + 256L * kk;
                if (i >= n) break;
                for (int s = 0; s < ns; ++s)
                    if (act[s]) a.p[s][cur[s] ^ 1][i] = beta[s] * a.p[s][cur[s]][i] + a.z[s][i];
            }
        grid_barrier(a.bar, nb);
        if (bar_failed(a.bar)) return;
        // phase 2b: y = A p_new, y(fix) = 1e30 p_new(fix), partial p.y
        for (long c = blockIdx.x; c < nc; c += gridDim.x) {
            double acc[2] = {0.0, 0.0};
            for (int kk = 0; kk < 4; ++kk) {
                const long i = c * kChunk + t + 256L * kk;
                if (i >= n) break;
                const bool fx = a.isfix[i];
                for (int s = 0; s < ns; ++s) {
                    if (!act[s]) continue;
                    const double* pn_v = a.p[s][cur[s] ^ 1];
                    const double pn = pn_v[i];
                    double yi = fx ? 1.0e30 * pn : spmv_row(a, (int)i, pn_v);
                    a.y[s][i] = yi;
                    acc[s] = (kk == 0) ? pn * yi : acc[s] + pn * yi;
                }
            }
            for (int s = 0; s < ns; ++s) {
                if (!act[s]) continue;
                double v = block_tree256(acc[s], red);
                if (t == 0) part(0, s)[c] = v;
            }
        }
        grid_barrier(a.bar, nb);
        if (bar_failed(a.bar)) return;
        for (int s = 0; s < ns; ++s) {
            if (!act[s]) continue;
            double py = fold_partials(part(0, s), nc, red);
            alfa[s] = err_new[s] / py;
            err_old[s] = err_new[s];
            cur[s] ^= 1;
            pend[s] = true;
            last_iter[s] = k;
        }
    }
    // the last deferred x update
    for (long c = blockIdx.x; c < nc; c += gridDim.x)
        for (int kk = 0; kk < 4; ++kk) {
            const long i = c * kChunk + t + 256L * kk;
            if (i >= n) break;
            for (int s = 0; s < ns; ++s)
                if (pend[s]) a.x[s][i] = alfa[s] * a.p[s][cur[s]][i] + a.x[s][i];
        }
    if (blockIdx.x == 0 && t == 0)
        for (int s = 0; s < ns; ++s) {
            if (done[s]) continue;
            a.iters_out[s] = last_iter[s];
            a.rz_out[s] = fabs(err_old[s]);
            a.conv_out[s] = (rel ? rrc[s] > s_thr[s] : fabs(err_old[s]) > a.tol) ? 0 : 1;
            if (a.relres_out)
                a.relres_out[s] = (rel && s_ref2[s] > 0.0) ? sqrt(rrc[s] / s_ref2[s]) : 0.0;
        }
}

// Failure-detection self-test of the two bounded waits (one block): a grid barrier that
// expects a second block that never comes, and an mbarrier nothing arrives on.  Both give
// up after `limit` polls; out[0] = the barrier's error word, out[1] = CFD_ERR_BARRIER when
// the mbarrier wait gave up (0 if it completed).
// CFD_GUESS_EXTRAPOLATED: the solves start from the last two increments extrapolated to
// this step.  A solve's unknown is the step's mesh increment, the mean mesh velocity over the
// step times DTMIN; with that velocity linear in time through the last two steps' midpoints,
//     x = c1 x_{n-1} + c2 x_{n-2},  h = (dt_n + dt1) / (dt1 + dt2),
//     c1 = dt_n / dt1 (1 + h),  c2 = -(dt_n / dt2) h
// on the free rows (x_{n-1} is the previous solution, still in x), in the oracle's operation
// order (--fmad=false: the same bits); x_{n-1} is kept as the next step's x_{n-2}.  hist =
// (dt1, dt2, solutions kept); with fewer than two kept the guess stays x_{n-1}.  The fixed
// rows are left to the Dirichlet values (set before, or by the solve).  The float shadow
// (mixed form) follows x.
__global__ void k_guess_extrapolate(PcgArgs a, const double* __restrict__ dtn_p,
                                    double* __restrict__ hist, double* __restrict__ xprev0,
                                    double* __restrict__ xprev1) {
    const double dtn = *dtn_p, dt1 = hist[0], dt2 = hist[1];
    const bool two = hist[2] >= 2.0;
    double c1 = 1.0, c2 = 0.0;
    if (two) {
        const double h = (dtn + dt1) / (dt1 + dt2);
        c1 = dtn / dt1 * (1.0 + h);
        c2 = -(dtn / dt2) * h;
    }
    double* xprev[2] = {xprev0, xprev1};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < a.n;
         i += (long)gridDim.x * blockDim.x) {
        if (a.isfix[i]) continue;
        for (int s = 0; s < a.nsolve; ++s) {
            const double x1 = a.x[s][i];
            const double xn = two ? c1 * x1 + c2 * xprev[s][i] : x1;
            xprev[s][i] = x1;
            if (two) {
                a.x[s][i] = xn;
                if (a.xf[s]) a.xf[s][i] = d2f_trunc(xn);
            }
        }
    }
}

// after k_guess_extrapolate: hist = (dt_n, dt1, solutions kept + 1)
__global__ void k_guess_extrapolate_hist(const double* __restrict__ dtn_p,
                                         double* __restrict__ hist) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        hist[1] = hist[0];
        hist[0] = *dtn_p;
        hist[2] = hist[2] + 1.0;
    }
}

// div_rcp against the division x / d over n input pairs: a third raw 64-bit patterns for
// both (splitmix64: every exponent and sign, zeros, subnormals, infinities, NaNs), a third
// with both of magnitude 2^-60 .. 2^60, a third with x = d * m for a random significand m
// moved by up to +-2^12 ulps (quotients next to binade edges and to halfway cases).  Counts
// the pairs whose results differ in any bit (two NaNs count as equal).
__device__ __forceinline__ unsigned long long splitmix(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__global__ void k_selftest_divrcp(long long n, unsigned long long seed,
                                  unsigned long long* __restrict__ bad) {
    unsigned long long local = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned long long z1 = splitmix(seed + (unsigned long long)i * 0x9e3779b97f4a7c15ull);
        const unsigned long long z2 = splitmix(z1 + 0x632be59bd9b4e019ull);
        unsigned long long bx = z1, bd = z2;
        const int kind = (int)(i % 3);
        if (kind == 1) {
            bx = (z1 & 0x800fffffffffffffull) | ((963ull + (z1 >> 52) % 121ull) << 52);
            bd = (z2 & 0x800fffffffffffffull) | ((963ull + (z2 >> 52) % 121ull) << 52);
        } else if (kind == 2) {
            bd = (z2 & 0x800fffffffffffffull) | ((993ull + (z2 >> 52) % 61ull) << 52);
            const double m = __longlong_as_double((long long)((z1 & 0x000fffffffffffffull) |
                                                              (1023ull << 52)));
            const long long b = __double_as_longlong(__longlong_as_double((long long)bd) * m);
            bx = (unsigned long long)(b + ((long long)(z1 >> 52 & 0x1fffull) - 4096));
        }
        const double x = __longlong_as_double((long long)bx), d = __longlong_as_double((long long)bd);
        const double y = 1.0 / d;
        const double a = div_rcp(x, d, y), b = x / d;
        if (__double_as_longlong(a) != __double_as_longlong(b) && !(a != a && b != b)) ++local;
    }
    if (local) atomicAdd(bad, local);
}

cudaError_t launch_selftest_divrcp(long long n, unsigned long long seed, unsigned long long* bad) {
    k_selftest_divrcp<<<152 * 8, 256>>>(n, seed, bad);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

__global__ void k_selftest_waits(GridBar* gb, int* out, long long limit) {
    __shared__ __align__(8) unsigned long long bar;
    grid_barrier(gb, 2u, limit);
    if (threadIdx.x == 0) {
        const unsigned ubar = (unsigned)__cvta_generic_to_shared(&bar);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ubar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        out[1] = mbar_wait_bounded(ubar, 0u, limit) ? 0 : (int)CFD_ERR_BARRIER;
        out[0] = gb->err;
    }
}

}  // namespace cfd

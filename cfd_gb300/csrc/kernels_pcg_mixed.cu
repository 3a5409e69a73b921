// kernels_pcg_mixed.cu — biCG (biconjGrad.f90:8-62) for the mixed-precision form.
//
// The matrix is FP32 and every SpMV accumulates in FP32 over FP32 shadows (of x for the
// first residual, of the search direction p and of z in the iterations); the vectors x, r,
// z, p, y, the Jacobi scaling (as a multiply by 1/diag), the dots and the scalars alfa,
// beta stay FP64.
//
// A solve is four launches: k_bicg_fix_mixed (Dirichlet values into x and its shadow),
// k_bicg_resid_mixed (r = b - A.x, p = r/diag, r.r and r.p), k_bicg_dir_mixed (y = A.p,
// p.y, alfa) — row kernels with one row per thread whose last block folds the per-block
// sums — and the persistent cooperative k_pcg_mixed (convergence test and iterations).
// The shadow xf of x (d2f_trunc of cfd_common.cuh) must match x on entry; the kernels keep
// it so on exit (the Dirichlet scatter writes both, and a solve that iterated refreshes xf
// from the final x).
#include "cfd_kernels.cuh"

namespace cfd {

// The SpMV rows gather in batches of B entries (8 in the FP32 residual kernel, 4 in the
// register-limited persistent kernel and in the precise residual, whose 4-entry batches
// measured 1.29 -> 1.25 ms per 1M-node step against 8): the column indices and values of a batch are loaded
// together, then the gathered vector entries, so each batch costs two dependent memory
// latencies instead of two per entry.  The products are still summed in column order.

// row i of A times (v0, v1): one pass over the row's columns for both right-hand sides;
// with FIXC also the sums over the Dirichlet columns only (f0, f1: the row of A.x_D)
template <int NS, bool FIXC = false, int kRowBatch = 8>
__device__ __forceinline__ void spmv_row2_f(const PcgArgs& a, int i, const float* v0,
                                            const float* v1, float& d0, float& d1,
                                            float* f0 = nullptr, float* f1 = nullptr) {
    float s0 = 0.f, s1 = 0.f, g0 = 0.f, g1 = 0.f;
    const int j0 = a.rowptr[i], j1 = a.rowptr[i + 1];
    for (int jb = j0; jb < j1; jb += kRowBatch) {
        int c[kRowBatch];
        float m[kRowBatch], x0[kRowBatch], x1[kRowBatch];
        bool fx[kRowBatch];
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u)
            if (jb + u < j1) {
                c[u] = a.col[jb + u];
                m[u] = a.valf[jb + u];
            }
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u)
            if (jb + u < j1) {
                x0[u] = v0[c[u]];
                if (NS == 2) x1[u] = v1[c[u]];
                if (FIXC) fx[u] = a.isfix[c[u]] != 0;
            }
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u)
            if (jb + u < j1) {
                s0 += m[u] * x0[u];
                if (NS == 2) s1 += m[u] * x1[u];
                if (FIXC && fx[u]) {
                    g0 += m[u] * x0[u];
                    if (NS == 2) g1 += m[u] * x1[u];
                }
            }
    }
    d0 = s0;
    d1 = s1;
    if (FIXC) {
        *f0 = g0;
        *f1 = g1;
    }
}

// Row i of A times the FP64 vectors (x0, x1), as accurately as FP64 arithmetic: each x_j
// comes split into FP32 hi + lo (split_bits, exact to 2^-47; k_split_x forms the split once
// per node, so a row gathers 8 B per entry as the FP64 vector would), a_ij*hi is formed
// exactly as a float pair (product + fmaf remainder), the products are summed with a
// compensated FP32 sum (TwoSum: the exact error of every add, without a branch) and the
// remainders and a_ij*lo terms with a plain one, and the three partial sums are added in
// FP64; with val_lo (the relative tests: the matrix assembled in FP64 and held as valf +
// val_lo) the a_lo*hi terms join the plain sum.  The first residual of a solve, r = b - A.x,
// takes this product under the relative stopping tests: it is the one SpMV of the solve
// whose operand is the whole displacement rather than a correction, so an FP32 product's
// error there (~1e-7 of |A||x|) would be a floor under the starting residual of any good
// initial guess.  The reference's absolute test, loose against that floor, keeps the FP32
// product.  With FIXC also the FP32 sums over the Dirichlet columns (the row of A.x_D).
struct Acc2 {
    float s, c, t;  // compensated sum s + c of the exact products' leading parts; tail sum t
    __device__ __forceinline__ void init() { s = c = t = 0.f; }
    __device__ __forceinline__ void add(float m, float2 x, float mlo = 0.f) {
        const float p = m * x.x;
        const float e = fmaf(m, x.x, -p);
        const float u = s + p;
        const float bp = u - s;
        c += (s - (u - bp)) + (p - bp);
        s = u;
        t += e + m * x.y + mlo * x.x;
    }
    __device__ __forceinline__ double value() const {
        return (f2d_bits(s) + f2d_bits(c)) + f2d_bits(t);
    }
};

template <int NS, bool FIXC = false, int kRowBatch = 8>
__device__ __forceinline__ void spmv_row2_x(const PcgArgs& a, int i, const float2* v0,
                                            const float2* v1, double& d0, double& d1,
                                            float* f0 = nullptr, float* f1 = nullptr) {
    Acc2 s0, s1;
    s0.init();
    s1.init();
    float g0 = 0.f, g1 = 0.f;
    const int j0 = a.rowptr[i], j1 = a.rowptr[i + 1];
    for (int jb = j0; jb < j1; jb += kRowBatch) {
        int c[kRowBatch];
        float m[kRowBatch], ml[kRowBatch];
        float2 x0[kRowBatch], x1[kRowBatch];
        bool fx[kRowBatch];
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u)
            if (jb + u < j1) {
                c[u] = a.col[jb + u];
                m[u] = a.valf[jb + u];
                ml[u] = a.val_lo ? a.val_lo[jb + u] : 0.f;
            }
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u)
            if (jb + u < j1) {
                x0[u] = v0[c[u]];
                if (NS == 2) x1[u] = v1[c[u]];
                if (FIXC) fx[u] = a.isfix[c[u]] != 0;
            }
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u)
            if (jb + u < j1) {
                s0.add(m[u], x0[u], ml[u]);
                if (NS == 2) s1.add(m[u], x1[u], ml[u]);
                if (FIXC && fx[u]) {  // hi = d2f_trunc(x), the FP32 shadow's value
                    g0 += m[u] * x0[u].x;
                    if (NS == 2) g1 += m[u] * x1[u].x;
                }
            }
    }
    d0 = s0.value();
    d1 = (NS == 2) ? s1.value() : 0.0;
    if (FIXC) {
        *f0 = g0;
        *f1 = g1;
    }
}

// a.xs[s] = split_bits(v_s) (the precise product's operand; relative tests)
__global__ void k_split_x(PcgArgs a, const double* __restrict__ v0, const double* __restrict__ v1,
                          const int* __restrict__ gate) {
    if (gate && !*gate) return;  // the same in every block
    const double* v[2] = {v0, v1};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < a.n;
         i += (long)gridDim.x * blockDim.x)
#pragma unroll
        for (int s = 0; s < 2; ++s)
            if (s < a.nsolve) {
                float hi, lo;
                split_bits(v[s][i], hi, lo);
                a.xs[s][i] = make_float2(hi, lo);
            }
}

template <int kRowBatch = 4>
__device__ __forceinline__ float spmv_row_dir_f(const PcgArgs& a, int i, const float* pf,
                                                const float* zf, float beta) {
    float dot = 0.f;
    const int j0 = a.rowptr[i], j1 = a.rowptr[i + 1];
    for (int jb = j0; jb < j1; jb += kRowBatch) {
        int c[kRowBatch];
        float m[kRowBatch], pv[kRowBatch], zv[kRowBatch];
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u)
            if (jb + u < j1) {
                c[u] = a.col[jb + u];
                m[u] = a.valf[jb + u];
            }
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u)
            if (jb + u < j1) {
                pv[u] = pf[c[u]];
                zv[u] = zf[c[u]];
            }
#pragma unroll
        for (int u = 0; u < kRowBatch; ++u)
            if (jb + u < j1) dot += m[u] * (beta * pv[u] + zv[u]);
    }
    return dot;
}

__device__ __forceinline__ bool bar_failed_m(GridBar* gb) {
    return *((volatile int*)&gb->err) != 0;
}

// x(fix) = x_fix (biconjGrad.f90:28), in x and in its shadow
__global__ void k_bicg_fix_mixed(PcgArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.nfix) return;
    const int i = a.fix_node[k];
#pragma unroll
    for (int s = 0; s < 2; ++s)
        if (s < a.nsolve) {
            const double v = a.fixval[s][a.fix_src[k]];
            a.x[s][i] = v;
            a.xf[s][i] = d2f_trunc(v);
        }
}

// Sums of 256 doubles per block for the row kernels: nsum arrays of 256 values in shared
// memory; warp w sums array w, lane l the values l, l+32, ..., l+224 in that order, then a
// shuffle-down tree.  (One warp per sum keeps the FP64 adds few: FP64 runs at 1/64 of the
// FP32 rate here.)  Result in lane 0 of warp w.
__device__ __forceinline__ double warp_sum256(const double* v) {
    const int l = threadIdx.x & 31;
    double acc = v[l];
#pragma unroll
    for (int k = 1; k < 8; ++k) acc = acc + v[l + 32 * k];
    return warp_tree32(acc);
}

// The last block to finish (block counter) folds the nb per-block partials of each of the
// nsum sums in a fixed order: lane t of the block sums partials t, t+256, ..., then the
// 256-value sum above.  Returns true in the last block, with the sums in out[0..nsum).
__device__ bool last_block_fold(unsigned* count, const double* part, long nb, int nsum,
                                double (*sh)[256], double* out) {
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = atomicAdd(count, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    const int t = threadIdx.x;
    for (int w = 0; w < nsum; ++w) {
        double acc = 0.0;
        for (long c = t; c < nb; c += 256) acc = acc + __ldcg(part + w * nb + c);
        sh[w][t] = acc;
    }
    __syncthreads();
    if ((t >> 5) < nsum) {
        const double v = warp_sum256(sh[t >> 5]);
        if ((t & 31) == 0) out[t >> 5] = v;
    }
    __syncthreads();
    if (t == 0) *count = 0u;
    return true;
}

// First pass of a solve, one row per thread: y = A.x (FP32 SpMV over the shadow of x),
// r = b - y with r(fix) = 0, p = r/diag (as r*(1/diag)); per-block partials of r.r and r.p
// (biconjGrad.f90:29-38), and with RELB of e.e, e = b - A.x_D (0 on the Dirichlet rows),
// the reference norm of CFD_BICG_TOL_REL.  y itself is not kept: the next pass overwrites
// it.  A block visits the 256-row groups blockIdx.x, blockIdx.x + gridDim.x, ... (one
// group when the grid has a block per group); there is one partial per block.
template <int NS, bool RELB, bool PRECISE>
__device__ __forceinline__ void first_rows(const PcgArgs& a, double (*sh)[256]) {
    const int t = threadIdx.x;
    double rr[2] = {0.0, 0.0}, rp[2] = {0.0, 0.0}, ee[2] = {0.0, 0.0};
    for (long rb = blockIdx.x; rb < a.nblk_r; rb += gridDim.x) {
    const long i = rb * 256 + t;
    if (i < a.n) {
        const bool fx = a.isfix[i];
        double d[2] = {0.0, 0.0};
        float f[2] = {0.f, 0.f};
        if (!fx) {
            if (PRECISE) {
                spmv_row2_x<NS, RELB, 4>(a, (int)i, a.xs[0], a.xs[1], d[0], d[1], &f[0], &f[1]);
            } else {
                float d32[2];
                spmv_row2_f<NS, RELB>(a, (int)i, a.xf[0], a.xf[1], d32[0], d32[1], &f[0], &f[1]);
                d[0] = f2d_bits(d32[0]);
                d[1] = f2d_bits(d32[1]);
            }
        }
        const double id = a.invdiag[i];
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            double r, p, e = 0.0;
            float pf;
            if (fx) {
                r = 0.0;
                p = 0.0;
                pf = 0.f;
            } else {
                r = a.b[s] ? a.b[s][i] - d[s] : -d[s];
                p = r * id;
                pf = d2f_trunc(p);
                if (RELB) e = a.b[s] ? a.b[s][i] - f2d_bits(f[s]) : f2d_bits(-f[s]);
            }
            a.r[s][i] = r;
            a.p[s][0][i] = p;
            a.pf[s][0][i] = pf;
            rr[s] += r * r;
            rp[s] += r * p;
            if (RELB) ee[s] += e * e;
        }
    }
    }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        sh[s][t] = rr[s];
        sh[2 + s][t] = rp[s];
        if (RELB) sh[4 + s][t] = ee[s];
    }
    __syncthreads();
    if ((t >> 5) < (RELB ? 6 : 4)) {
        const double v = warp_sum256(sh[t >> 5]);
        if ((t & 31) == 0) a.part_r[(t >> 5) * gridDim.x + blockIdx.x] = v;
    }
}

// The first pass's convergence test of solve s (biconjGrad.f90:35, or the relative test)
__device__ __forceinline__ bool first_done(const PcgArgs& a, int s) {
    const double rr = a.bscal[8 * s];
    return a.tol_mode == CFD_BICG_TOL_ABS ? rr < a.tol : rr <= a.bscal[8 * s + 5];
}

// REL: the relative tests' variant (accurate product, reference norm of CFD_BICG_TOL_REL
// when tol_mode asks for it); the absolute test's variant keeps the FP32 product
template <bool REL>
__global__ void __launch_bounds__(256) k_bicg_resid_mixed(PcgArgs a) {
    __shared__ double sh[6][256];
    __shared__ double out[6];
    if (a.only_if && !*a.only_if) return;  // the same in every block
    const bool relb = a.tol_mode == CFD_BICG_TOL_REL;
    if (!REL) {
        if (a.nsolve == 2) first_rows<2, false, false>(a, sh);
        else first_rows<1, false, false>(a, sh);
    } else if (a.nsolve == 2) {
        relb ? first_rows<2, true, true>(a, sh) : first_rows<2, false, true>(a, sh);
    } else {
        relb ? first_rows<1, true, true>(a, sh) : first_rows<1, false, true>(a, sh);
    }
    if (last_block_fold(&a.bcount[0], a.part_r, gridDim.x, relb ? 6 : 4, sh, out) &&
        threadIdx.x == 0) {
        for (int s = 0; s < 2; ++s) {
            a.bscal[8 * s + 0] = out[s];      // r.r
            a.bscal[8 * s + 1] = out[2 + s];  // r.p
            if (a.tol_mode != CFD_BICG_TOL_ABS) {
                const double ref2 = relb ? out[4 + s] : out[s];
                a.bscal[8 * s + 4] = ref2;
                a.bscal[8 * s + 5] = (a.tol * a.tol) * ref2;
            }
        }
        if (a.gflag && !a.only_if) {  // gate on r.z, the convergence measure of the solve,
            bool open = out[2] + out[3] >= a.gate;  // or on the stopping test itself
            if (a.gate_undone) {
                open = false;
                for (int s = 0; s < a.nsolve; ++s) open = open || !first_done(a, s);
            }
            a.gflag[0] = open ? 1 : 0;
            a.gflag[1] = 0;
        }
    }
}

cudaError_t launch_bicg_resid_mixed(unsigned grid, cudaStream_t stream, const PcgArgs& a) {
    if (a.tol_mode == CFD_BICG_TOL_ABS) k_bicg_resid_mixed<false><<<grid, 256, 0, stream>>>(a);
    else k_bicg_resid_mixed<true><<<grid, 256, 0, stream>>>(a);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

// r.z = r.r/diag of the candidate guesses (with the first pass's SpMV), per 256-row block,
// folded by the last block; fixed rows contribute 0 as in the first pass
__global__ void __launch_bounds__(256) k_guess_judge(PcgArgs a, const double* __restrict__ cand0,
                                                     const double* __restrict__ cand1,
                                                     double* __restrict__ rr) {
    __shared__ double sh[4][256];
    __shared__ double out[4];
    if (!a.gflag[0]) return;  // the same in every block
    const int t = threadIdx.x;
    const double* cand[2] = {cand0, cand1};
    double q[2] = {0.0, 0.0};
    for (long i = blockIdx.x * (long)blockDim.x + t; i < a.n; i += (long)gridDim.x * blockDim.x) {
        if (a.isfix[i]) continue;
        double d[2] = {0.0, 0.0};
        if (a.tol_mode == CFD_BICG_TOL_ABS) {  // the first pass's FP32 product
            for (int s = 0; s < a.nsolve; ++s) {
                float q32 = 0.f;
                for (int j = a.rowptr[i]; j < a.rowptr[i + 1]; ++j)
                    q32 += a.valf[j] * d2f_trunc(cand[s][a.col[j]]);
                d[s] = f2d_bits(q32);
            }
        } else if (a.nsolve == 2) {  // the candidates' split (k_split_x)
            spmv_row2_x<2, false, 4>(a, (int)i, a.xs[0], a.xs[1], d[0], d[1]);
        } else {
            spmv_row2_x<1, false, 4>(a, (int)i, a.xs[0], a.xs[1], d[0], d[1]);
        }
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (s >= a.nsolve) continue;
            const double r = -d[s];
            q[s] += r * r * a.invdiag[i];
        }
    }
    sh[0][t] = q[0];
    sh[1][t] = q[1];
    __syncthreads();
    if ((t >> 5) < 2) {
        const double v = warp_sum256(sh[t >> 5]);
        if ((t & 31) == 0) a.part_r[(t >> 5) * gridDim.x + blockIdx.x] = v;
    }
    if (last_block_fold(&a.bcount[2], a.part_r, gridDim.x, 2, sh, out) && t == 0) {
        rr[0] = out[0];
        rr[1] = out[1];
    }
}

__global__ void k_guess_select(PcgArgs a, const double* __restrict__ cand0,
                               const double* __restrict__ cand1, const double* __restrict__ rr,
                               long long* __restrict__ stats) {
    const bool open = a.gflag[0] != 0;
    bool use[2] = {false, false};
    if (open)
#pragma unroll
        for (int s = 0; s < 2; ++s) use[s] = s < a.nsolve && rr[s] < a.bscal[8 * s + 1];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        stats[0] += open ? 1 : 0;
        stats[1] += use[0] ? 1 : 0;
        stats[2] += use[1] ? 1 : 0;
        a.gflag[1] = (use[0] || use[1]) ? 1 : 0;
    }
    if (!use[0] && !use[1]) return;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < a.n;
         i += (long)gridDim.x * blockDim.x) {
        if (use[0]) {
            a.x[0][i] = cand0[i];
            a.xf[0][i] = d2f_trunc(cand0[i]);
        }
        if (use[1]) {
            a.x[1][i] = cand1[i];
            a.xf[1][i] = d2f_trunc(cand1[i]);
        }
    }
}

// Second pass, for the solves with r.r >= tol: y = A.p (FP32 over the shadow), y(fix) =
// 1e30 p(fix); per-block partials of p.y; the last block forms alfa = r.p / p.y
// (biconjGrad.f90:39-43)
__global__ void __launch_bounds__(256) k_bicg_dir_mixed(PcgArgs a) {
    __shared__ double sh[4][256];
    __shared__ double out[4];
    const int t = threadIdx.x;
    bool act[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) act[s] = s < a.nsolve && !first_done(a, s);
    if (!act[0] && !act[1]) return;  // the same in every block
    // 256-row groups blockIdx.x, blockIdx.x + gridDim.x, ...; one partial per block
    double py[2] = {0.0, 0.0};
    for (long rb = blockIdx.x; rb < a.nblk_r; rb += gridDim.x) {
        const long i = rb * 256 + t;
        if (i >= a.n) continue;
        const bool fx = a.isfix[i];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (!act[s]) continue;
            const double pi = a.p[s][0][i];
            const double yi =
                fx ? 1.0e30 * pi : f2d_bits(spmv_row_dir_f<8>(a, (int)i, a.pf[s][0], a.pf[s][0], 0.f));
            a.y[s][i] = yi;
            py[s] += pi * yi;
        }
    }
    sh[0][t] = py[0];
    sh[1][t] = py[1];
    __syncthreads();
    if ((t >> 5) < 2) {
        const double v = warp_sum256(sh[t >> 5]);
        if ((t & 31) == 0) a.part_r[(t >> 5) * gridDim.x + blockIdx.x] = v;
    }
    if (last_block_fold(&a.bcount[1], a.part_r, gridDim.x, 2, sh, out) && t == 0)
        for (int s = 0; s < 2; ++s)
            if (act[s]) {
                a.bscal[8 * s + 2] = out[s];
                a.bscal[8 * s + 3] = a.bscal[8 * s + 1] / out[s];
            }
}

// The iteration kernel's block sums and folds (FP64, in an order of the mixed solve's own;
// the FP64 solve keeps the oracle's tree).  Up to four sums ("slots") at once, one warp
// each: a block sum puts the threads' values in shared memory and warp j adds slot j's 256
// entries (warp_sum256: 7 adds, then the shuffle tree); a fold of nc chunk partials gives
// each slot 256/m threads (m = the slot count rounded up to 1, 2 or 4) that add the
// partials with that stride before warp j finishes.  A sum costs 12 FP64 warp instructions
// instead of the 43 of block_tree256, and the slots' sums run side by side.
__device__ __forceinline__ void block_sums_m(double (&v)[4], int m, double (*sh)[256],
                                             double* res) {
    const int t = threadIdx.x;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (j < m) sh[j][t] = v[j];
    __syncthreads();
    if ((t >> 5) < m) {
        const double r = warp_sum256(sh[t >> 5]);
        if ((t & 31) == 0) res[t >> 5] = r;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (j < m) v[j] = res[j];
}

__device__ __forceinline__ void fold_m(const double* const (&src)[4], int m, long nc,
                                       double (*sh)[256], double* res, double (&out)[4]) {
    const int t = threadIdx.x;
    const int lg = m > 2 ? 2 : (m > 1 ? 1 : 0);  // m rounded up to 2^lg
    const int g = 256 >> lg;                     // threads per slot
    const int j = t >> (8 - lg), u = t & (g - 1);
    double acc = 0.0;
    if (j < m) {
        const double* pj = j == 0 ? src[0] : (j == 1 ? src[1] : (j == 2 ? src[2] : src[3]));
        for (long c = u; c < nc; c += g) acc = acc + __ldcg(pj + c);
    }
    double* flat = &sh[0][0];
    flat[t] = acc;
    __syncthreads();
    if ((t >> 5) < m) {
        const double* v = flat + (t >> 5) * g;
        const int l = t & 31;
        double s = v[l];
        for (int q = 1; q < (g >> 5); ++q) s = s + v[l + 32 * q];
        s = warp_tree32(s);
        if (l == 0) res[t >> 5] = s;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k < m) out[k] = res[k];
}

__global__ void __launch_bounds__(256, 2) k_pcg_mixed(PcgArgs a) {
    __shared__ double sh[4][256];
    __shared__ double res[4];
    __shared__ double s_thr[2], s_ref2[2];  // relative modes: threshold on r.r, ref.ref
    const int t = threadIdx.x;
    const int n = a.n;
    const int ns = a.nsolve;
    const long nc = ((long)n + kChunk - 1) / kChunk;
    const unsigned nb = gridDim.x;
    auto part = [&](int buf, int s) { return a.part + ((long)buf * 2 + s) * nc; };
    // each block owns one contiguous range of rows (a multiple of 256, so the ranges differ
    // by at most 256 rows between blocks) and leaves one partial per sum
    const long R = (((long)n + nb - 1) / nb + 255) / 256 * 256;
    const long rb = blockIdx.x * R, re = min((long)n, rb + R);

    // x(fix), r, p, err = r.p, y = A.p and alfa come from k_bicg_fix_mixed,
    // k_bicg_resid_mixed and k_bicg_dir_mixed
    const bool rel = a.tol_mode != CFD_BICG_TOL_ABS;  // r.r per iteration
    bool done[2] = {true, true};
    double err_old[2] = {0.0, 0.0}, alfa[2] = {0.0, 0.0};
    bool pend[2] = {false, false};
    int cur[2] = {0, 0};
    double err_new[2] = {0.0, 0.0};
    double rrc[2] = {0.0, 0.0};
    if (t < 2) {
        s_ref2[t] = a.bscal[8 * t + 4];
        s_thr[t] = a.bscal[8 * t + 5];
    }
    __syncthreads();
    int prev[2] = {0, 0};  // a second pass: the first pass's iterations
#pragma unroll
    for (int s = 0; s < 2; ++s)
        if (s < ns) {
            const double rr = a.bscal[8 * s];
            done[s] = first_done(a, s);
            if (a.accumulate) prev[s] = *((volatile const int*)&a.iters_out[s]);
            if (rel) rrc[s] = rr;
            if (done[s]) {
                if (blockIdx.x == 0 && t == 0) {
                    if (!a.accumulate) a.iters_out[s] = 0;
                    a.rz_out[s] = rr;
                    a.conv_out[s] = 1;
                    if (a.relres_out)
                        a.relres_out[s] = (rel && s_ref2[s] > 0.0) ? sqrt(rr / s_ref2[s]) : 0.0;
                }
            } else {
                err_new[s] = a.bscal[8 * s + 1];
                alfa[s] = a.bscal[8 * s + 3];
                err_old[s] = err_new[s];
                pend[s] = true;
            }
        }
    if (done[0] && done[1]) {
        if (a.iterated && blockIdx.x == 0 && t == 0) *a.iterated = 0;
        return;
    }

    int k = 0;
    int last_iter[2] = {0, 0};
    while (true) {
        bool act[2] = {false, false};
#pragma unroll
        for (int s = 0; s < 2; ++s)
            act[s] = !done[s] && (rel ? rrc[s] > s_thr[s] : fabs(err_old[s]) > a.tol) &&
                     k + prev[s] < a.maxit;
        if (!act[0] && !act[1]) break;
        k = k + 1;
        // phase 1: x += alfa p; r -= alfa y; z = r/diag; r.z (and r.r, relative modes).
        // A thread's four rows of a chunk are loaded together, then updated, so that their
        // loads are in flight at once.
        {
        double acc[2] = {0.0, 0.0}, accr[2] = {0.0, 0.0};
        for (long i0 = rb + t; i0 < re; i0 += kChunk) {
            double id[4];
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) id[kk] = (i0 + 256L * kk < re) ? a.invdiag[i0 + 256L * kk] : 0.0;
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                if (!pend[s] && !act[s]) continue;
                double* __restrict__ xs = a.x[s];
                const double* __restrict__ ps = a.p[s][cur[s]];
                double* __restrict__ rs = a.r[s];
                const double* __restrict__ ys = a.y[s];
                double* __restrict__ zs = a.z[s];
                float* __restrict__ zfs = a.zf[s];
                double xv[4], pv[4], rv[4], yv[4];
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const long i = i0 + 256L * kk;
                    const bool in = i < re;
                    xv[kk] = (in && pend[s]) ? xs[i] : 0.0;
                    pv[kk] = (in && pend[s]) ? ps[i] : 0.0;
                    rv[kk] = (in && act[s]) ? rs[i] : 0.0;
                    yv[kk] = (in && act[s]) ? ys[i] : 0.0;
                }
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const long i = i0 + 256L * kk;
                    if (i >= re) break;
                    if (pend[s]) xs[i] = xv[kk] + alfa[s] * pv[kk];
                    if (!act[s]) continue;
                    const double ri = rv[kk] - alfa[s] * yv[kk];
                    const double zi = ri * id[kk];
                    rs[i] = ri;
                    zs[i] = zi;
                    zfs[i] = d2f_trunc(zi);
                    acc[s] = acc[s] + ri * zi;
                    if (rel) accr[s] = accr[s] + ri * ri;
                }
            }
        }
            double v[4] = {0.0, 0.0, 0.0, 0.0};
            int m = 0;
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                if (!act[s]) continue;
                v[m++] = acc[s];
                if (rel) v[m++] = accr[s];
            }
            block_sums_m(v, m, sh, res);
            if (t == 0) {
                int j = 0;
#pragma unroll
                for (int s = 0; s < 2; ++s) {
                    if (!act[s]) continue;
                    part(1, s)[blockIdx.x] = v[j++];
                    if (rel) part(2, s)[blockIdx.x] = v[j++];
                }
            }
        }
#pragma unroll
        for (int s = 0; s < 2; ++s) pend[s] = false;
        grid_barrier(a.bar, nb);
        if (bar_failed_m(a.bar)) return;
        double beta[2] = {0.0, 0.0};
        float betaf[2] = {0.f, 0.f};
        {
            const double* src[4] = {nullptr, nullptr, nullptr, nullptr};
            double out[4] = {0.0, 0.0, 0.0, 0.0};
            int m = 0;
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                if (!act[s]) continue;
                src[m++] = part(1, s);
                if (rel) src[m++] = part(2, s);
            }
            fold_m(src, m, (long)nb, sh, res, out);
            int j = 0;
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                if (!act[s]) continue;
                err_new[s] = out[j++];
                if (rel) rrc[s] = out[j++];
            }
        }
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (!act[s]) continue;
            beta[s] = err_new[s] / err_old[s];
            betaf[s] = d2f_trunc(beta[s]);
        }
        // phase 2: p_new = beta p + z (FP64 for the row, FP32 shadow for the SpMV); y = A p_new.
        // Per solve, a thread's rows go in pairs: the two rows' pointers, p and z, then their
        // column batches and gathers are issued together.
        {
        double acc[2] = {0.0, 0.0};
        for (long i0 = rb + t; i0 < re; i0 += kChunk) {
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                if (!act[s]) continue;
                const double* __restrict__ ps = a.p[s][cur[s]];
                const double* __restrict__ zs = a.z[s];
                const float* __restrict__ pfs = a.pf[s][cur[s]];
                const float* __restrict__ zfs = a.zf[s];
                double* __restrict__ pn_out = a.p[s][cur[s] ^ 1];
                float* __restrict__ pfn_out = a.pf[s][cur[s] ^ 1];
                double* __restrict__ ys = a.y[s];
#pragma unroll
                for (int kp = 0; kp < 4; kp += 2) {
                    long ii[2];
                    bool in[2], fx[2];
                    int j0[2], j1[2];
                    double pv[2], zv[2];
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        ii[q] = i0 + 256L * (kp + q);
                        in[q] = ii[q] < re;
                        fx[q] = in[q] ? a.isfix[ii[q]] != 0 : true;
                        j0[q] = (in[q] && !fx[q]) ? a.rowptr[ii[q]] : 0;
                        j1[q] = (in[q] && !fx[q]) ? a.rowptr[ii[q] + 1] : 0;
                        pv[q] = in[q] ? ps[ii[q]] : 0.0;
                        zv[q] = in[q] ? zs[ii[q]] : 0.0;
                    }
                    float dot[2] = {0.f, 0.f};
                    const int len = max(j1[0] - j0[0], j1[1] - j0[1]);
                    constexpr int B = 3;
                    for (int u0 = 0; u0 < len; u0 += B) {
                        int cc[2][B];
                        float mm[2][B], pp[2][B], zz[2][B];
#pragma unroll
                        for (int q = 0; q < 2; ++q)
#pragma unroll
                            for (int u = 0; u < B; ++u)
                                if (j0[q] + u0 + u < j1[q]) {
                                    cc[q][u] = a.col[j0[q] + u0 + u];
                                    mm[q][u] = a.valf[j0[q] + u0 + u];
                                }
#pragma unroll
                        for (int q = 0; q < 2; ++q)
#pragma unroll
                            for (int u = 0; u < B; ++u)
                                if (j0[q] + u0 + u < j1[q]) {
                                    pp[q][u] = pfs[cc[q][u]];
                                    zz[q][u] = zfs[cc[q][u]];
                                }
#pragma unroll
                        for (int q = 0; q < 2; ++q)
#pragma unroll
                            for (int u = 0; u < B; ++u)
                                if (j0[q] + u0 + u < j1[q])
                                    dot[q] += mm[q][u] * (betaf[s] * pp[q][u] + zz[q][u]);
                    }
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        if (!in[q]) continue;
                        const double pn = beta[s] * pv[q] + zv[q];
                        const double yi = fx[q] ? 1.0e30 * pn : f2d_bits(dot[q]);
                        pn_out[ii[q]] = pn;
                        pfn_out[ii[q]] = d2f_trunc(pn);
                        ys[ii[q]] = yi;
                        acc[s] = acc[s] + pn * yi;
                    }
                }
            }
        }
            double v[4] = {0.0, 0.0, 0.0, 0.0};
            int m = 0;
#pragma unroll
            for (int s = 0; s < 2; ++s)
                if (act[s]) v[m++] = acc[s];
            block_sums_m(v, m, sh, res);
            if (t == 0) {
                int j = 0;
#pragma unroll
                for (int s = 0; s < 2; ++s)
                    if (act[s]) part(0, s)[blockIdx.x] = v[j++];
            }
        }
        grid_barrier(a.bar, nb);
        if (bar_failed_m(a.bar)) return;
        double pyv[4] = {0.0, 0.0, 0.0, 0.0};
        {
            const double* src[4] = {nullptr, nullptr, nullptr, nullptr};
            int m = 0;
#pragma unroll
            for (int s = 0; s < 2; ++s)
                if (act[s]) src[m++] = part(0, s);
            fold_m(src, m, (long)nb, sh, res, pyv);
        }
        int jpy = 0;
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (!act[s]) continue;
            const double py = pyv[jpy++];
            alfa[s] = err_new[s] / py;
            err_old[s] = err_new[s];
            cur[s] ^= 1;
            pend[s] = true;
            last_iter[s] = k;
        }
    }
    // last deferred x update; the shadow follows x for the solves that iterated
    for (long c = blockIdx.x; c < nc; c += gridDim.x)
        for (int kk = 0; kk < 4; ++kk) {
            const long i = c * kChunk + t + 256L * kk;
            if (i >= n) break;
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                if (done[s]) continue;
                double xi = a.x[s][i];
                if (pend[s]) {
                    xi += alfa[s] * a.p[s][cur[s]][i];
                    a.x[s][i] = xi;
                }
                a.xf[s][i] = d2f_trunc(xi);
            }
        }
    if (blockIdx.x == 0 && t == 0 && a.iterated) *a.iterated = (last_iter[0] + last_iter[1]) > 0;
    if (blockIdx.x == 0 && t == 0)
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (done[s]) continue;
            a.iters_out[s] = prev[s] + last_iter[s];
            a.rz_out[s] = fabs(err_old[s]);
            a.conv_out[s] = (rel ? rrc[s] > s_thr[s] : fabs(err_old[s]) > a.tol) ? 0 : 1;
            if (a.relres_out)
                a.relres_out[s] = (rel && s_ref2[s] > 0.0) ? sqrt(rrc[s] / s_ref2[s]) : 0.0;
        }
}

}  // namespace cfd

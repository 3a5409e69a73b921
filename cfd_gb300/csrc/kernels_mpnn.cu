// kernels_mpnn.cu — kernels of the learned mesh-motion guess (mpnn.cuh): boundary
// statistics and features, the FP32 training forward and backward passes, Adam, and the
// BF16 tensor-core inference pass.
//
// Graph arrays: ptr/nbr = CSR point neighbours (0-based, symmetric); src[k] = the source
// node of edge k = (src[k] -> nbr[k]); rev[k] = the index of the reverse edge.
// Reductions over nodes or edges (weight gradients, loss) go through per-block partials
// folded in a fixed order, so a training step is deterministic.
#include <algorithm>

#include "mpnn_kernels.cuh"

namespace cfd {
namespace mpnn {

// ------------------------------------------------------------------ globals and features
__device__ __forceinline__ double block_max256(double v, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, off));
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double w = lane < 8 ? red[lane] : 0.0;
#pragma unroll
        for (int off = 4; off > 0; off >>= 1) w = fmax(w, __shfl_down_sync(0xffffffffu, w, off));
        if (lane == 0) red[8] = w;
    }
    __syncthreads();
    const double r = red[8];
    __syncthreads();
    return r;
}

// One block of 256 threads.  Boundary nodes are listed in bnode[0..nb) with their kind and
// prescribed displacement (gx, gy).  Body geometry (c, L, R) and the least-squares affine
// fit g = t + M d, d = p - c, over the body nodes: since sum d = 0, t = mean g and each row
// of M solves [Sxx Sxy; Sxy Syy] m = [sum g d_x; sum g d_y].
__global__ void k_globals(int nb, const int* __restrict__ bnode, const int* __restrict__ bkind,
                          const double* __restrict__ gx, const double* __restrict__ gy,
                          const double* __restrict__ X, const double* __restrict__ Y,
                          Globals* __restrict__ G, const int* __restrict__ gate) {
    if (gate && !*gate) return;
    __shared__ double red[9];
    const int t = threadIdx.x;
    double nbody = 0, sx = 0, sy = 0, sgx = 0, sgy = 0, nout = 0;
    for (int k = t; k < nb; k += 256) {
        const int p = bnode[k];
        if (bkind[k] == KIND_BODY) {
            nbody += 1.0;
            sx += X[p];
            sy += Y[p];
            sgx += gx[k];
            sgy += gy[k];
        } else {
            nout += 1.0;
        }
    }
    nbody = block_tree256(nbody, red);
    sx = block_tree256(sx, red);
    sy = block_tree256(sy, red);
    sgx = block_tree256(sgx, red);
    sgy = block_tree256(sgy, red);
    nout = block_tree256(nout, red);
    const double inb = nbody > 0 ? 1.0 / nbody : 0.0;
    const double cx = sx * inb, cy = sy * inb;
    double rmax = 0, rsum = 0, sxx = 0, sxy = 0, syy = 0, gxdx = 0, gxdy = 0, gydx = 0, gydy = 0;
    for (int k = t; k < nb; k += 256) {
        const int p = bnode[k];
        const double dx = X[p] - cx, dy = Y[p] - cy;
        const double r = sqrt(dx * dx + dy * dy);
        if (bkind[k] == KIND_BODY) {
            rmax = fmax(rmax, r);
            sxx += dx * dx;
            sxy += dx * dy;
            syy += dy * dy;
            gxdx += gx[k] * dx;
            gxdy += gx[k] * dy;
            gydx += gy[k] * dx;
            gydy += gy[k] * dy;
        } else {
            rsum += r;
        }
    }
    rmax = block_max256(rmax, red);
    rsum = block_tree256(rsum, red);
    sxx = block_tree256(sxx, red);
    sxy = block_tree256(sxy, red);
    syy = block_tree256(syy, red);
    gxdx = block_tree256(gxdx, red);
    gxdy = block_tree256(gxdy, red);
    gydx = block_tree256(gydx, red);
    gydy = block_tree256(gydy, red);
    if (t == 0) {
        Globals g;
        g.cx = cx;
        g.cy = cy;
        g.L = rmax > 0 ? 2.0 * rmax : 1.0;
        g.R = nout > 0 ? rsum / nout : g.L;
        g.tx = sgx * inb;
        g.ty = sgy * inb;
        const double det = sxx * syy - sxy * sxy;
        const double id = det > 0 ? 1.0 / det : 0.0;
        g.m11 = (syy * gxdx - sxy * gxdy) * id;
        g.m12 = (sxx * gxdy - sxy * gxdx) * id;
        g.m21 = (syy * gydx - sxy * gydy) * id;
        g.m22 = (sxx * gydy - sxy * gydx) * id;
        // second-moment ellipse: eigenvalues of [sxx sxy; sxy syy] / nbody
        const double hx = 0.5 * (sxx - syy) * inb, mxy = sxy * inb, tr = 0.5 * (sxx + syy) * inb;
        const double rt = sqrt(hx * hx + mxy * mxy);
        g.ea = sqrt(2.0 * (tr + rt));
        g.eb = sqrt(fmax(2.0 * (tr - rt), 0.0));
        const double al = 0.5 * atan2(2.0 * mxy, 2.0 * hx);
        g.ec = cos(al);
        g.es = sin(al);
        *G = g;
    }
}

// Basis fields kept per node in FP64 (planes F[0..2] = Phi, Psi_x, Psi_y in length units)
// for the refined learned guess: seeded from a network run, combined with each solve's
// affine fit (G) into its guess, and corrected by each solve's solution.
// Seed: F = (y0, L y1, L y2) at the free nodes, 0 elsewhere.
__global__ void k_fields_seed(int n, const float* __restrict__ y, const int* __restrict__ kind,
                              const Globals* __restrict__ G, double* __restrict__ F) {
    const double L = G->L;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const bool f = kind[i] == KIND_FREE;
        F[i] = f ? (double)y[OUT * i] : 0.0;
        F[n + i] = f ? L * (double)y[OUT * i + 1] : 0.0;
        F[2 * (size_t)n + i] = f ? L * (double)y[OUT * i + 2] : 0.0;
    }
}

// Guess: c = t Phi + M (Psi_x, Psi_y) at the free nodes (x: (tx, m11, m12), y: (ty, m21,
// m22)); the boundary nodes keep x, which already holds this solve's Dirichlet values.
__global__ void k_fields_guess(int n, const int* __restrict__ kind, const Globals* __restrict__ G,
                               const double* __restrict__ F, const double* __restrict__ x0,
                               const double* __restrict__ x1, double* __restrict__ c0,
                               double* __restrict__ c1) {
    const Globals g = *G;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double a = x0[i], b = x1[i];
        if (kind[i] == KIND_FREE) {
            const double f0 = F[i], f1 = F[n + i], f2 = F[2 * (size_t)n + i];
            a = g.tx * f0 + g.m11 * f1 + g.m12 * f2;
            b = g.ty * f0 + g.m21 * f1 + g.m22 * f2;
        }
        c0[i] = a;
        c1[i] = b;
    }
}

// Correction after the solves: each solve s with coefficients a_s (its affine fit) and
// solution x_s gives one equation a_s . F_i = x_s(i) per node; F_i moves to the nearest
// point that satisfies it (a Kaczmarz step per node: the x solve's, then the y solve's;
// solves with no prescribed motion are skipped).
__global__ void k_fields_update(int n, const int* __restrict__ kind, const Globals* __restrict__ G,
                                const double* __restrict__ x0, const double* __restrict__ x1,
                                double* __restrict__ F) {
    const Globals g = *G;
    const double a[2][3] = {{g.tx, g.m11, g.m12}, {g.ty, g.m21, g.m22}};
    double iq[2];  // 1/|a_s|^2 (0: the solve has no prescribed motion), once per launch
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        const double q = a[s][0] * a[s][0] + a[s][1] * a[s][1] + a[s][2] * a[s][2];
        iq[s] = q > 0.0 ? 1.0 / q : 0.0;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (kind[i] != KIND_FREE) continue;
        double f[3] = {F[i], F[n + i], F[2 * (size_t)n + i]};
        const double x[2] = {x0[i], x1[i]};
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (iq[s] == 0.0) continue;
            const double r = (x[s] - (a[s][0] * f[0] + a[s][1] * f[1] + a[s][2] * f[2])) * iq[s];
#pragma unroll
            for (int c = 0; c < 3; ++c) f[c] += a[s][c] * r;
        }
        F[i] = f[0];
        F[n + i] = f[1];
        F[2 * (size_t)n + i] = f[2];
    }
}

// per-node prescribed displacement (0 at free nodes) from the boundary list
__global__ void k_scatter_bc(int nb, const int* __restrict__ bnode, const double* __restrict__ gx,
                             const double* __restrict__ gy, double* __restrict__ gnx,
                             double* __restrict__ gny, const int* __restrict__ gate) {
    if (gate && !*gate) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nb) return;
    gnx[bnode[k]] = gx[k];
    gny[bnode[k]] = gy[k];
}

// Geometry-only node features: position, log-radius, boundary kinds, and the three fields
// of a continuum model of the mesh-motion operator, which the network corrects.  The
// operator's entries grad N_i . grad N_j q carry no area factor (mLaplace.f90:40, 48), so in
// the continuum it is div(k grad u) with k ~ 1/(element area), k ~ 1/r^2 on O-grids whose
// spacing grows with r.  For a circular body of radius a = L/2 inside a circle of radius R:
// Phi = (R^2 - r^2)/(R^2 - a^2) (clamped to [0, 1]) and Psi = psi(rho) d / rho with
// psi(r) = a ((r/R)^p - (r/R)^q) / ((a/R)^p - (a/R)^q), p, q = 1 +- sqrt(2), over L, where
// rho = r a / r_b(theta) stretches the body's second-moment ellipse (radius r_b along the
// node's direction) onto the circle of radius a, so that Psi = d on the body.  Feature 9 is
// the ellipse's aspect ratio.
__global__ void k_features(int n, const double* __restrict__ X, const double* __restrict__ Y,
                           const int* __restrict__ kind, const Globals* __restrict__ G,
                           float* __restrict__ f, const int* __restrict__ gate) {
    if (gate && !*gate) return;
    // per-graph constants (FP32 arithmetic below; positions are differenced in FP64)
    const Globals g = *G;
    const float L = (float)g.L, iL = 1.f / L, a = 0.5f * L, R = (float)g.R;
    const float ea = (float)g.ea, eb = (float)g.eb, ec = (float)g.ec, es = (float)g.es;
    const float p = 2.41421356f, q = -0.41421356f;
    const float ar = a / R, den = powf(ar, p) - powf(ar, q);
    const float logRL = logf(R * iL), aspect = ea > 0.f ? eb / ea : 1.f;
    const bool annulus = R > a;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float dx = (float)(X[i] - g.cx), dy = (float)(Y[i] - g.cy);
        const float r2 = dx * dx + dy * dy, r = sqrtf(r2);
        float* o = f + (size_t)i * F_IN;
        o[0] = dx * iL;
        o[1] = dy * iL;
        o[2] = logf(r * iL + 1e-6f);
        o[3] = logRL;
        o[4] = kind[i] == KIND_BODY ? 1.f : 0.f;
        o[5] = kind[i] == KIND_OUTER ? 1.f : 0.f;
        float phi = 0.f, c = 0.f;
        if (annulus && r < R) {
            phi = (R * R - r2) / (R * R - a * a);
            const float rs = fmaxf(r, 1e-6f * L);
            // body radius along the node's direction (frame of the ellipse's axes)
            const float u = (dx * ec + dy * es) / rs, v = (-dx * es + dy * ec) / rs;
            const float rb = ea * eb / fmaxf(sqrtf(eb * eb * u * u + ea * ea * v * v), 1e-30f);
            const float rho = fminf(rs * a / fmaxf(rb, 1e-6f * L), 0.999999f * R);
            const float rr = rho / R;
            c = a * (powf(rr, p) - powf(rr, q)) / den / rho;
        }
        o[6] = fminf(fmaxf(phi, 0.f), 1.f);
        o[7] = c * dx * iL;
        o[8] = c * dy * iL;
        o[9] = aspect;
    }
}

__global__ void k_edge_features(int m, const int* __restrict__ src, const int* __restrict__ nbr,
                                const double* __restrict__ X, const double* __restrict__ Y,
                                const Globals* __restrict__ G, float* __restrict__ e,
                                const int* __restrict__ gate) {
    if (gate && !*gate) return;
    const float iL = (float)(1.0 / G->L);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        const int i = src[k], j = nbr[k];
        const float dx = (float)(X[j] - X[i]), dy = (float)(Y[j] - Y[i]);
        const float ln = sqrtf(dx * dx + dy * dy), il = 1.f / ln;
        e[3 * (size_t)k] = dx * il;
        e[3 * (size_t)k + 1] = dy * il;
        e[3 * (size_t)k + 2] = logf(ln * iL);
    }
}

// ------------------------------------------------------------------ FP32 dense layers
// Y[n][O] = [X1 | X2][n][I1 + I2] . W^T + b   (W: O x (I1+I2) row-major; b may be null)
__global__ void __launch_bounds__(128) k_dense(int n, const float* __restrict__ X1, int I1,
                                               const float* __restrict__ X2, int I2,
                                               const float* __restrict__ W,
                                               const float* __restrict__ b, int O,
                                               float* __restrict__ Y) {
    __shared__ float xs[DT][2 * HID + 1];
    const int I = I1 + I2;
    const int base = blockIdx.x * DT;
    for (int q = threadIdx.x; q < DT * I; q += blockDim.x) {
        const int r = q / I, k = q - r * I, node = base + r;
        float v = 0.f;
        if (node < n) v = (k < I1) ? X1[(size_t)node * I1 + k] : X2[(size_t)node * I2 + (k - I1)];
        xs[r][k] = v;
    }
    __syncthreads();
    for (int o = threadIdx.x; o < O; o += blockDim.x) {
        float acc[DT];
        const float bo = b ? b[o] : 0.f;
#pragma unroll
        for (int r = 0; r < DT; ++r) acc[r] = bo;
        for (int k = 0; k < I; ++k) {
            const float wv = W[(size_t)o * I + k];
#pragma unroll
            for (int r = 0; r < DT; ++r) acc[r] += wv * xs[r][k];
        }
#pragma unroll
        for (int r = 0; r < DT; ++r)
            if (base + r < n) Y[(size_t)(base + r) * O + o] = acc[r];
    }
}

// dX[n][I] = dY[n][O] . W   (W: O x I row-major)
__global__ void __launch_bounds__(128) k_dense_t(int n, const float* __restrict__ dY, int O,
                                                 const float* __restrict__ W, int I,
                                                 float* __restrict__ dX) {
    __shared__ float ys[DT][2 * HID + 1];
    const int base = blockIdx.x * DT;
    for (int q = threadIdx.x; q < DT * O; q += blockDim.x) {
        const int r = q / O, o = q - r * O, node = base + r;
        ys[r][o] = node < n ? dY[(size_t)node * O + o] : 0.f;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < I; k += blockDim.x) {
        float acc[DT];
#pragma unroll
        for (int r = 0; r < DT; ++r) acc[r] = 0.f;
        for (int o = 0; o < O; ++o) {
            const float wv = W[(size_t)o * I + k];
#pragma unroll
            for (int r = 0; r < DT; ++r) acc[r] += wv * ys[r][o];
        }
#pragma unroll
        for (int r = 0; r < DT; ++r)
            if (base + r < n) dX[(size_t)(base + r) * I + k] = acc[r];
    }
}

// Weight gradient partials over chunks of WG rows: part[chunk][O*I (+O)] =
// sum_r dY[r][o] X[r][k] (and sum_r dY[r][o] for the bias)
__global__ void __launch_bounds__(256) k_wgrad(int n, const float* __restrict__ dY, int O,
                                               const float* __restrict__ X1, int I1,
                                               const float* __restrict__ X2, int I2, int with_bias,
                                               float* __restrict__ part) {
    extern __shared__ float sm[];
    const int I = I1 + I2;
    float* ys = sm;              // WG x O
    float* xs = sm + WG * O;     // WG x I
    const int base = blockIdx.x * WG;
    for (int q = threadIdx.x; q < WG * O; q += blockDim.x) {
        const int r = q / O, o = q - r * O, row = base + r;
        ys[q] = row < n ? dY[(size_t)row * O + o] : 0.f;
    }
    for (int q = threadIdx.x; q < WG * I; q += blockDim.x) {
        const int r = q / I, k = q - r * I, row = base + r;
        float v = 0.f;
        if (row < n) v = (k < I1) ? X1[(size_t)row * I1 + k] : X2[(size_t)row * I2 + (k - I1)];
        xs[q] = v;
    }
    __syncthreads();
    const int stride = O * I + (with_bias ? O : 0);
    float* out = part + (size_t)blockIdx.x * stride;
    for (int q = threadIdx.x; q < O * I; q += blockDim.x) {
        const int o = q / I, k = q - o * I;
        float acc = 0.f;
        for (int r = 0; r < WG; ++r) acc += ys[r * O + o] * xs[r * I + k];
        out[q] = acc;
    }
    if (with_bias)
        for (int o = threadIdx.x; o < O; o += blockDim.x) {
            float acc = 0.f;
            for (int r = 0; r < WG; ++r) acc += ys[r * O + o];
            out[O * I + o] = acc;
        }
}

// out[q] (+)= sum over chunks c (in order) of part[c][q]
__global__ void k_fold(int nchunk, int stride, const float* __restrict__ part, int accumulate,
                       float* __restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= stride) return;
    float acc = 0.f;
    for (int c = 0; c < nchunk; ++c) acc += part[(size_t)c * stride + q];
    out[q] = accumulate ? out[q] + acc : acc;
}

// ------------------------------------------------------------------ elementwise
__global__ void k_relu(long n, const float* __restrict__ a, float* __restrict__ h) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) h[i] = fmaxf(a[i], 0.f);
}

// h1 = h0 + relu(v)
__global__ void k_residual(long n, const float* __restrict__ h0, const float* __restrict__ v,
                           float* __restrict__ h1) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) h1[i] = h0[i] + fmaxf(v[i], 0.f);
}

// d = g * (a > 0)
__global__ void k_relu_bwd(long n, const float* __restrict__ g, const float* __restrict__ a,
                           float* __restrict__ d) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) d[i] = a[i] > 0.f ? g[i] : 0.f;
}

// dh[i][o] = dh[i][o] + dhc[i][o] (first HID of the 2*HID row) + dpq[i][o]
__global__ void k_add_dh(int n, const float* __restrict__ dhc, const float* __restrict__ dpqh,
                         float* __restrict__ dh) {
    const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)n * HID) return;
    const long i = q / HID, o = q - i * HID;
    dh[q] = dh[q] + dhc[i * 2 * HID + o] + dpqh[q];
}

// ------------------------------------------------------------------ message passing
// z[k][o] = PQ[i][o] + PQ[j][HID+o] + C[o] . e[k] + c[o]   for edge k = (i -> j)
__global__ void k_edge_fwd(int m, const int* __restrict__ src, const int* __restrict__ nbr,
                           const float* __restrict__ PQ, const float* __restrict__ e,
                           const float* __restrict__ C, const float* __restrict__ c,
                           float* __restrict__ z) {
    const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)m * HID) return;
    const long k = q / HID;
    const int o = (int)(q - k * HID);
    const int i = src[k], j = nbr[k];
    const float* ek = e + 3 * k;
    z[q] = PQ[(size_t)i * 2 * HID + o] + PQ[(size_t)j * 2 * HID + HID + o] +
           (C[o * 3] * ek[0] + C[o * 3 + 1] * ek[1] + C[o * 3 + 2] * ek[2]) + c[o];
}

// agg[i][o] = sum over the edges k of i of relu(z[k][o]) / max(deg_i, 1)
__global__ void k_node_agg(int n, const int* __restrict__ ptr, const float* __restrict__ z,
                           float* __restrict__ agg) {
    const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)n * HID) return;
    const long i = q / HID;
    const int o = (int)(q - i * HID);
    const int k0 = ptr[i], k1 = ptr[i + 1];
    float s = 0.f;
    for (int k = k0; k < k1; ++k) s += fmaxf(z[(size_t)k * HID + o], 0.f);
    agg[q] = s / (float)max(k1 - k0, 1);
}

// dz[k][o] = dhc[i][HID+o] / max(deg_i, 1) * (z[k][o] > 0)  (dhc holds d[h; agg])
__global__ void k_edge_bwd(int m, const int* __restrict__ src, const int* __restrict__ ptr,
                           const float* __restrict__ dhc, const float* __restrict__ z,
                           float* __restrict__ dz) {
    const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)m * HID) return;
    const long k = q / HID;
    const int o = (int)(q - k * HID);
    const int i = src[k];
    const int deg = max(ptr[i + 1] - ptr[i], 1);
    dz[q] = z[q] > 0.f ? dhc[(size_t)i * 2 * HID + HID + o] / (float)deg : 0.f;
}

// dPQ[i][o] = sum_{k in edges(i)} dz[k][o];  dPQ[i][HID+o] = sum_{k in edges(i)} dz[rev[k]][o]
__global__ void k_node_dpq(int n, const int* __restrict__ ptr, const int* __restrict__ rev,
                           const float* __restrict__ dz, float* __restrict__ dPQ) {
    const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= (long)n * HID) return;
    const long i = q / HID;
    const int o = (int)(q - i * HID);
    float sp = 0.f, sq = 0.f;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
        sp += dz[(size_t)k * HID + o];
        sq += dz[(size_t)rev[k] * HID + o];
    }
    dPQ[(size_t)i * 2 * HID + o] = sp;
    dPQ[(size_t)i * 2 * HID + HID + o] = sq;
}

// ------------------------------------------------------------------ loss and Adam
// dy = 2 (y - t) / nfree at free nodes; per-block partial sums of |y - t|^2 (256 threads)
__global__ void __launch_bounds__(256) k_loss(int n, const float* __restrict__ y,
                                              const float* __restrict__ t,
                                              const int* __restrict__ kind, float inv_nfree,
                                              float* __restrict__ dy, float* __restrict__ part) {
    __shared__ float red[256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < n) {
        const bool fr = kind[i] == KIND_FREE;
#pragma unroll
        for (int q = 0; q < OUT; ++q) {
            const float d = fr ? y[OUT * i + q] - t[OUT * i + q] : 0.f;
            l += d * d;
            dy[OUT * i + q] = 2.f * d * inv_nfree;
        }
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_adam(int np, float* __restrict__ w, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2,
                       float eps, float bc1, float bc2) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const float gq = g[q];
    const float mq = b1 * m[q] + (1.f - b1) * gq;
    const float vq = b2 * v[q] + (1.f - b2) * gq * gq;
    m[q] = mq;
    v[q] = vq;
    const float mh = mq / bc1, vh = vq / bc2;
    w[q] = w[q] - lr * mh / (sqrtf(vh) + eps);
}

// training targets: the fields (Phi, Psi_x, Psi_y) of the plain solve, stored as
// (Phi, Psi_x / L, Psi_y / L)
__global__ void k_targets(int n, const double* __restrict__ phi, const double* __restrict__ psx,
                          const double* __restrict__ psy, const Globals* __restrict__ G,
                          float* __restrict__ t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double iL = 1.0 / G->L;
    t[OUT * i] = (float)phi[i];
    t[OUT * i + 1] = (float)(psx[i] * iL);
    t[OUT * i + 2] = (float)(psy[i] * iL);
}

// guess at free nodes: u = t Phi + L M (Psi_x/L, Psi_y/L); boundary nodes keep their
// prescribed values
__global__ void k_guess(int n, const float* __restrict__ y, const int* __restrict__ kind,
                        const double* __restrict__ gnx, const double* __restrict__ gny,
                        const Globals* __restrict__ G, double* __restrict__ ux,
                        double* __restrict__ uy, const int* __restrict__ gate) {
    if (gate && !*gate) return;
    const Globals g = *G;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (kind[i] != KIND_FREE) {
            ux[i] = gnx[i];
            uy[i] = gny[i];
            continue;
        }
        const double phi = y[OUT * i], px = g.L * (double)y[OUT * i + 1],
                     py = g.L * (double)y[OUT * i + 2];
        ux[i] = g.tx * phi + g.m11 * px + g.m12 * py;
        uy[i] = g.ty * phi + g.m21 * px + g.m22 * py;
    }
}

}  // namespace mpnn
}  // namespace cfd

namespace cfd {
namespace mpnn {

// ------------------------------------------------------------------ BF16 inference
// Tensor-core pass (mma.sync m16n8k16, BF16 operands, FP32 accumulation).  A warp owns 16
// nodes, a block of IW warps a tile of 16*IW nodes; blocks loop over tiles so that each
// loads the layer's weights into shared memory once.  Per layer one kernel: the message
// aggregation of the layer (FP32 arithmetic on the BF16 P, Q of the previous kernel), the
// update GEMM U [h; agg], the residual, then the next layer's P|Q GEMM or, after the last
// layer, the decoder.  P|Q alternates between two buffers.
constexpr int IW = 8;
constexpr int TILE = 16 * IW;
constexpr int XS = 2 * HID + 8;  // shared row stride (bf16) of 128-wide tiles
constexpr int HS = HID + 8;      // of 64-wide tiles (the +8 keeps fragment loads
                                 // free of bank conflicts)
typedef __nv_bfloat16 bf16;

__device__ __forceinline__ unsigned ld_b32(const bf16* p) {
    return *reinterpret_cast<const unsigned*>(p);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], unsigned a0, unsigned a1, unsigned a2,
                                         unsigned a3, unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// acc[nt] += X[16][K] . W[nt*8 .. nt*8+8)[K]^T, X and W in shared memory (row strides xs,
// ws in elements).  Fragment layout of m16n8k16: lane = 4 g + t; A rows g and g+8, columns
// 2t, 2t+1 (+8); B column g, rows 2t, 2t+1 (+8); D rows g and g+8, columns 2t, 2t+1.
template <int K, int NT>
__device__ __forceinline__ void warp_gemm(const bf16* X, int xs, const bf16* W, int ws,
                                          float (&acc)[NT][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int kk = 0; kk < K / 16; ++kk) {
        const int k0 = kk * 16 + 2 * t;
        const unsigned a0 = ld_b32(X + g * xs + k0);
        const unsigned a1 = ld_b32(X + (g + 8) * xs + k0);
        const unsigned a2 = ld_b32(X + g * xs + k0 + 8);
        const unsigned a3 = ld_b32(X + (g + 8) * xs + k0 + 8);
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const bf16* wr = W + (nt * 8 + g) * ws + k0;
            mma_bf16(acc[nt], a0, a1, a2, a3, ld_b32(wr), ld_b32(wr + 8));
        }
    }
}

// D (16 x NT*8, FP32 fragments) -> global rows base.. (row stride ld), BF16
template <int NT>
__device__ __forceinline__ void store_tile_bf16(const float (&acc)[NT][4], int base, int n, bf16* out,
                                                int ld) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const int col = nt * 8 + 2 * t;
        if (base + g < n)
            *reinterpret_cast<__nv_bfloat162*>(out + (size_t)(base + g) * ld + col) =
                __floats2bfloat162_rn(acc[nt][0], acc[nt][1]);
        if (base + g + 8 < n)
            *reinterpret_cast<__nv_bfloat162*>(out + (size_t)(base + g + 8) * ld + col) =
                __floats2bfloat162_rn(acc[nt][2], acc[nt][3]);
    }
}

__global__ void k_to_bf16(int np, const float* __restrict__ w, bf16* __restrict__ wb) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < np) wb[q] = __float2bfloat16_rn(w[q]);
}

// rows x cols of a row-major BF16 matrix into shared memory with row stride ld
__device__ __forceinline__ void load_mat(bf16* dst, int ld, const bf16* src, int rows, int cols) {
    for (int q = threadIdx.x; q < rows * cols / 2; q += blockDim.x) {
        const int r = (2 * q) / cols, c = 2 * q - r * cols;
        *reinterpret_cast<unsigned*>(dst + r * ld + c) =
            *reinterpret_cast<const unsigned*>(src + (size_t)r * cols + c);
    }
}

// h0 = relu(W_in f + b_in) (FP32), then P|Q of layer 0
__global__ void __launch_bounds__(32 * IW) k_infer_encode(int n, const float* __restrict__ f,
                                                          const float* __restrict__ w,
                                                          const bf16* __restrict__ wb,
                                                          bf16* __restrict__ hb,
                                                          bf16* __restrict__ pq_out,
                                                          const int* __restrict__ gate) {
    if (gate && !*gate) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    bf16* Ws = reinterpret_cast<bf16*>(smem_raw);   // 128 x HS: [A0; B0]
    bf16* Hs = Ws + 2 * HID * HS;                    // IW x 16 x HS
    float* Wi = reinterpret_cast<float*>(Hs + IW * 16 * HS);  // HID x F_IN, then b_in
    load_mat(Ws, HS, wb + layer_off(0) + L_A, 2 * HID, HID);
    for (int q = threadIdx.x; q < HID * F_IN + HID; q += blockDim.x) Wi[q] = w[OFF_W_IN + q];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    bf16* H = Hs + warp * 16 * HS;
    const int ntile = (n + TILE - 1) / TILE;
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const int base = tile * TILE + warp * 16;
        {  // all 16 nodes at once: lane l owns node l/2 and the outputs [32 (l%2), +32)
            const int r = lane >> 1, o0 = 32 * (lane & 1), node = base + r;
            float fi[F_IN];
#pragma unroll
            for (int k = 0; k < F_IN; ++k) fi[k] = node < n ? f[(size_t)node * F_IN + k] : 0.f;
            unsigned w16[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                float hv[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int o = o0 + 2 * q + u;
                    float a = Wi[HID * F_IN + o];
#pragma unroll
                    for (int k = 0; k < F_IN; ++k) a += Wi[o * F_IN + k] * fi[k];
                    hv[u] = node < n ? fmaxf(a, 0.f) : 0.f;
                }
                const __nv_bfloat162 h2 = __floats2bfloat162_rn(hv[0], hv[1]);
                w16[q] = *reinterpret_cast<const unsigned*>(&h2);
            }
            uint4* hs = reinterpret_cast<uint4*>(H + r * HS + o0);
            uint4* hg = reinterpret_cast<uint4*>(hb + (size_t)node * HID + o0);
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                const uint4 w = make_uint4(w16[4 * v], w16[4 * v + 1], w16[4 * v + 2], w16[4 * v + 3]);
                hs[v] = w;
                if (node < n) hg[v] = w;
            }
        }
        __syncwarp();
        float acc[16][4];
#pragma unroll
        for (int nt = 0; nt < 16; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
        warp_gemm<HID, 16>(H, HS, Ws, HS, acc);
        store_tile_bf16<16>(acc, base, n, pq_out, 2 * HID);
        __syncwarp();
    }
}

// layer l: aggregation, update GEMM, residual; then P|Q of layer l+1 (wb_next) or the
// decoder (wb_next == null)
__global__ void __launch_bounds__(32 * IW, 2) k_infer_layer(
    int n, int l, const int* __restrict__ ptr, const int* __restrict__ nbr,
    const float* __restrict__ e, const float* __restrict__ w, const bf16* __restrict__ wb,
    int has_next, const bf16* __restrict__ pq_in, bf16* __restrict__ hb,
    bf16* __restrict__ pq_out, float* __restrict__ y, const int* __restrict__ gate) {
    if (gate && !*gate) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    bf16* Us = reinterpret_cast<bf16*>(smem_raw);  // HID x XS
    bf16* Ws = Us + HID * XS;                       // 128 x HS: [A; B] of layer l+1
    bf16* Xs = Ws + 2 * HID * HS;                   // IW x 16 x XS
    float* Cs = reinterpret_cast<float*>(Xs + IW * 16 * XS);  // C (HID x 3), c, u
    float* cs = Cs + HID * E_F;
    float* us = cs + HID;
    const float* W = w + layer_off(l);
    load_mat(Us, XS, wb + layer_off(l) + L_U, HID, 2 * HID);
    if (has_next) load_mat(Ws, HS, wb + layer_off(l + 1) + L_A, 2 * HID, HID);
    for (int q = threadIdx.x; q < HID * E_F; q += blockDim.x) Cs[q] = W[L_C + q];
    for (int q = threadIdx.x; q < HID; q += blockDim.x) {
        cs[q] = W[L_c + q];
        us[q] = W[L_u + q];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    bf16* X = Xs + warp * 16 * XS;
    const int o0 = 2 * lane;
    const int ntile = (n + TILE - 1) / TILE;
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const int base = tile * TILE + warp * 16;
        // [h; agg] rows of the warp's 16 nodes, 8 at a time: lane l owns node l/4 (+8) and
        // the 16 features [16 (l%4), 16 (l%4) + 16); rows are read as 16-byte vectors
        for (int pass = 0; pass < 2; ++pass) {
            const int r = (lane >> 2) + 8 * pass, f0 = 16 * (lane & 3), node = base + r;
            float acc16[16], pz[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) acc16[q] = 0.f;
            uint4 hv4[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
            if (node < n) {
                const uint4* hp = reinterpret_cast<const uint4*>(hb + (size_t)node * HID + f0);
                const uint4* pp = reinterpret_cast<const uint4*>(pq_in + (size_t)node * 2 * HID + f0);
#pragma unroll
                for (int v = 0; v < 2; ++v) {
                    hv4[v] = hp[v];
                    const uint4 pv = pp[v];
                    const unsigned w4[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const float2 f2 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w4[u]));
                        pz[8 * v + 2 * u] = f2.x + cs[f0 + 8 * v + 2 * u];  // P_i + c
                        pz[8 * v + 2 * u + 1] = f2.y + cs[f0 + 8 * v + 2 * u + 1];
                    }
                }
                const int k0 = ptr[node], k1 = ptr[node + 1];
                for (int k = k0; k < k1; ++k) {
                    const int j = nbr[k];
                    const float e0 = e[3 * (size_t)k], e1 = e[3 * (size_t)k + 1],
                                e2 = e[3 * (size_t)k + 2];
                    const uint4* qp =
                        reinterpret_cast<const uint4*>(pq_in + (size_t)j * 2 * HID + HID + f0);
                    const uint4 qa = qp[0], qb = qp[1];
                    const unsigned w8[8] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y, qb.z, qb.w};
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const float2 q2 =
                            __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w8[u]));
                        const int o = f0 + 2 * u;
                        const float z0 = pz[2 * u] + q2.x +
                                         (Cs[o * 3] * e0 + Cs[o * 3 + 1] * e1 + Cs[o * 3 + 2] * e2);
                        const float z1 = pz[2 * u + 1] + q2.y +
                                         (Cs[o * 3 + 3] * e0 + Cs[o * 3 + 4] * e1 + Cs[o * 3 + 5] * e2);
                        acc16[2 * u] += fmaxf(z0, 0.f);
                        acc16[2 * u + 1] += fmaxf(z1, 0.f);
                    }
                }
                const float inv = 1.f / (float)max(k1 - k0, 1);
#pragma unroll
                for (int q = 0; q < 16; ++q) acc16[q] *= inv;
            }
            uint4* xh = reinterpret_cast<uint4*>(X + r * XS + f0);
            uint4* xa = reinterpret_cast<uint4*>(X + r * XS + HID + f0);
#pragma unroll
            for (int v = 0; v < 2; ++v) {
                xh[v] = hv4[v];
                unsigned w4[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const __nv_bfloat162 b2 =
                        __floats2bfloat162_rn(acc16[8 * v + 2 * u], acc16[8 * v + 2 * u + 1]);
                    w4[u] = *reinterpret_cast<const unsigned*>(&b2);
                }
                xa[v] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
            }
        }
        __syncwarp();
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
        warp_gemm<2 * HID, 8>(X, XS, Us, XS, acc);
        __syncwarp();
        // h <- h + relu(v + u), written back over the h half of the tile and to hb
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int col = nt * 8 + 2 * t;
#pragma unroll
            for (int hlf = 0; hlf < 2; ++hlf) {
                const int row = g + 8 * hlf;
                const float2 hv = __bfloat1622float2(
                    *reinterpret_cast<const __nv_bfloat162*>(X + row * XS + col));
                const float n0 = hv.x + fmaxf(acc[nt][2 * hlf] + us[col], 0.f);
                const float n1 = hv.y + fmaxf(acc[nt][2 * hlf + 1] + us[col + 1], 0.f);
                const __nv_bfloat162 nh = __floats2bfloat162_rn(n0, n1);
                *reinterpret_cast<__nv_bfloat162*>(X + row * XS + col) = nh;
                if (base + row < n)
                    *reinterpret_cast<__nv_bfloat162*>(hb + (size_t)(base + row) * HID + col) = nh;
            }
        }
        __syncwarp();
        if (has_next) {
            float acc2[16][4];
#pragma unroll
            for (int nt = 0; nt < 16; ++nt)
                acc2[nt][0] = acc2[nt][1] = acc2[nt][2] = acc2[nt][3] = 0.f;
            warp_gemm<HID, 16>(X, XS, Ws, HS, acc2);
            store_tile_bf16<16>(acc2, base, n, pq_out, 2 * HID);
        } else {
            // decoder: 16 nodes x OUT outputs over the warp's lanes
            for (int q = lane; q < 16 * OUT; q += 32) {
                const int r = q / OUT, o = q - r * OUT, node = base + r;
                float a = w[OFF_B_OUT + o];
                for (int k = 0; k < HID; ++k)
                    a += w[OFF_W_OUT + o * HID + k] * __bfloat162float(X[r * XS + k]);
                if (node < n) y[(size_t)OUT * node + o] = a;
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------ BF16 inference, tcgen05
// The same passes with the GEMMs on the 5th-generation tensor cores.  A block of 8 warps
// owns a tile of 128 nodes (the MMA's M): the warps gather the tile's [h; agg] rows (16
// nodes each, the arithmetic of the mma.sync pass) into shared memory, one thread issues
// tcgen05.mma (BF16 operands from shared memory, FP32 accumulators in tensor memory) and
// commits it to an mbarrier, and after the bounded wait every warp reads its 32 rows of
// the accumulator with tcgen05.ld for the epilogue.  The update GEMM (N = 64, K = 128) and
// the next layer's P|Q GEMM (N = 128, K = 64) use the same 128 tensor-memory columns one
// after the other.
namespace tc {
constexpr int TM = 128;          // nodes per tile
constexpr int NTHR = 256;        // 8 warps
constexpr unsigned TMEM_COLS = 128;
// K-major operands in the no-swizzle core-matrix layout: a core matrix is 8 rows x 16
// bytes (128 contiguous bytes); the core matrices of one 8-row group lie along K, 128 B
// apart (the descriptor's leading byte offset); the 8-row groups lie SBO bytes apart.
constexpr int LBO = 128;
constexpr int SBO_X = 16 * 2 * HID;  // the tile, 128 rows x K = 128 (h, then agg)
constexpr int SBO_U = 16 * 2 * HID;  // U: N = 64 rows x K = 128
constexpr int SBO_W = 16 * HID;      // [A; B]: N = 128 rows x K = 64
constexpr int X_BYTES = TM * 2 * HID * 2;
constexpr int U_BYTES = HID * 2 * HID * 2;
constexpr int W_BYTES = 2 * HID * HID * 2;
constexpr int F_FLOATS = HID * F_IN + HID;  // the largest float table (W_in, b_in)
static_assert(HID * E_F + 2 * HID + OUT * HID + OUT <= F_FLOATS, "float tables");
constexpr int SMEM = X_BYTES + U_BYTES + W_BYTES + 4 * F_FLOATS + 16;

__host__ __device__ constexpr int cm_off(int r, int k, int sbo) {
    return (r >> 3) * sbo + (k >> 3) * LBO + (r & 7) * 16 + (k & 7) * 2;
}

// shared-memory matrix descriptor: start address, leading and stride byte offsets (all
// >> 4), the descriptor version 1 at bit 46, base offset 0, no swizzle
__device__ __forceinline__ unsigned long long sdesc(unsigned saddr, unsigned sbo) {
    return (unsigned long long)((saddr & 0x3FFFFu) >> 4) |
           ((unsigned long long)(LBO >> 4) << 16) | ((unsigned long long)(sbo >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator (bit 4), A and B BF16 (bits 7,
// 10), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr unsigned idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(n >> 3) << 17) |
           ((unsigned)(m >> 4) << 24);
}

__device__ __forceinline__ unsigned su32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// this thread's st.shared become visible to the tensor cores' reads
__device__ __forceinline__ void fence_smem_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mma(unsigned d, unsigned long long a, unsigned long long b,
                                    unsigned idesc, unsigned accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        :
        : "r"(d), "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void commit(unsigned mbar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
        : "memory");
}

// bounded wait on the mbarrier's phase of the given parity (mbar_wait_bounded)
__device__ __forceinline__ bool wait_parity(unsigned mbar, unsigned parity) {
    return mbar_wait_bounded(mbar, parity);
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane; the wait is tied to
// the registers so that no use moves above it
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float (&v)[16]) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                   "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                   "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
                 :
                 : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// rows x cols of a row-major BF16 matrix into the core-matrix layout (16-byte chunks)
__device__ __forceinline__ void load_cm(unsigned char* dst, int sbo, const bf16* src, int rows,
                                        int cols) {
    const int per_row = cols / 8;
    for (int q = threadIdx.x; q < rows * per_row; q += blockDim.x) {
        const int r = q / per_row, k = (q - r * per_row) * 8;
        *reinterpret_cast<uint4*>(dst + cm_off(r, k, sbo)) =
            *reinterpret_cast<const uint4*>(src + (size_t)r * cols + k);
    }
}

__device__ __forceinline__ unsigned pack2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const unsigned*>(&h);
}

// ENC: h0 = relu(W_in f + b_in), then P|Q of layer 0.  Otherwise layer l: aggregation,
// update GEMM, residual, then P|Q of layer l+1 (has_next) or the decoder.
template <bool ENC>
__global__ void __launch_bounds__(NTHR, 2) k_infer_tc(
    int n, int l, const int* __restrict__ ptr, const int* __restrict__ nbr,
    const float* __restrict__ e, const float* __restrict__ f, const float* __restrict__ w,
    const bf16* __restrict__ wb, int has_next, const bf16* __restrict__ pq_in,
    bf16* __restrict__ hb, bf16* __restrict__ pq_out, float* __restrict__ y,
    const int* __restrict__ gate, int* __restrict__ err) {
    if (gate && !*gate) return;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* Xs = smem_raw;
    unsigned char* Us = Xs + X_BYTES;
    unsigned char* Ws = Us + U_BYTES;
    float* fl = reinterpret_cast<float*>(Ws + W_BYTES);
    unsigned long long* mbar = reinterpret_cast<unsigned long long*>(fl + F_FLOATS);
    unsigned* tslot = reinterpret_cast<unsigned*>(mbar + 1);
    int* abort_flag = reinterpret_cast<int*>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // float tables: ENC W_in, b_in; layers C, c, u, W_out, b_out
    float *Cs = fl, *cs = fl + HID * E_F, *us = cs + HID, *wo = us + HID;
    const int has_pq = ENC || has_next;
    if (ENC) {
        for (int q = tid; q < F_FLOATS; q += NTHR) fl[q] = w[OFF_W_IN + q];
    } else {
        const float* W = w + layer_off(l);
        load_cm(Us, SBO_U, wb + layer_off(l) + L_U, HID, 2 * HID);
        for (int q = tid; q < HID * E_F; q += NTHR) Cs[q] = W[L_C + q];
        for (int q = tid; q < HID; q += NTHR) {
            cs[q] = W[L_c + q];
            us[q] = W[L_u + q];
        }
        if (!has_next)
            for (int q = tid; q < OUT * HID + OUT; q += NTHR) wo[q] = w[OFF_W_OUT + q];
    }
    if (has_pq) load_cm(Ws, SBO_W, wb + layer_off(ENC ? 0 : l + 1) + L_A, 2 * HID, HID);
    const unsigned ubar = su32(mbar);
    if (tid == 0) {
        *abort_flag = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ubar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        __syncwarp();
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         su32(tslot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_smem_async();
    fence_before();
    __syncthreads();
    fence_after();
    const unsigned tbase = *tslot;
    const unsigned xa = su32(Xs), ua = su32(Us), wa = su32(Ws);
    // epilogue geometry: warp w reads tensor-memory lanes 32 (w % 4) .. (its 32 rows) and
    // half w / 4 of the accumulator's columns
    const int q4 = warp & 3, half = warp >> 2;
    const int erow = 32 * q4 + lane;
    const unsigned tlane = tbase + ((unsigned)(32 * q4) << 16);
    unsigned phase = 0;
    bool pending = false;  // a commit that this block has not seen arrive
    float acc_hi[8];
    const int ntile = (n + TM - 1) / TM;
    for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
        const int tb = tile * TM;
        if (ENC) {
            // lane l of warp w owns row 16 w + l / 2 and the outputs [32 (l % 2), +32)
            const int r = 16 * warp + (lane >> 1), o0 = 32 * (lane & 1), node = tb + r;
            float fi[F_IN];
#pragma unroll
            for (int k = 0; k < F_IN; ++k) fi[k] = node < n ? f[(size_t)node * F_IN + k] : 0.f;
            unsigned w16[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                float hv[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int o = o0 + 2 * q + u;
                    float a = fl[HID * F_IN + o];
#pragma unroll
                    for (int k = 0; k < F_IN; ++k) a += fl[o * F_IN + k] * fi[k];
                    hv[u] = node < n ? fmaxf(a, 0.f) : 0.f;
                }
                w16[q] = pack2(hv[0], hv[1]);
            }
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                const uint4 wv = make_uint4(w16[4 * v], w16[4 * v + 1], w16[4 * v + 2], w16[4 * v + 3]);
                *reinterpret_cast<uint4*>(Xs + cm_off(r, o0 + 8 * v, SBO_X)) = wv;
                if (node < n)
                    *reinterpret_cast<uint4*>(hb + (size_t)node * HID + o0 + 8 * v) = wv;
            }
        } else {
            // [h; agg] rows, 8 nodes per pass: lane l owns row 16 w + l / 4 (+8) and the 16
            // features [16 (l % 4), +16)
            for (int pass = 0; pass < 2; ++pass) {
                const int r = 16 * warp + (lane >> 2) + 8 * pass, f0 = 16 * (lane & 3),
                          node = tb + r;
                float acc16[16], pz[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) acc16[q] = 0.f;
                uint4 hv4[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
                if (node < n) {
                    const uint4* hp = reinterpret_cast<const uint4*>(hb + (size_t)node * HID + f0);
                    const uint4* pp =
                        reinterpret_cast<const uint4*>(pq_in + (size_t)node * 2 * HID + f0);
#pragma unroll
                    for (int v = 0; v < 2; ++v) {
                        hv4[v] = hp[v];
                        const uint4 pv = pp[v];
                        const unsigned w4[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const float2 f2 =
                                __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w4[u]));
                            pz[8 * v + 2 * u] = f2.x + cs[f0 + 8 * v + 2 * u];
                            pz[8 * v + 2 * u + 1] = f2.y + cs[f0 + 8 * v + 2 * u + 1];
                        }
                    }
                    const int k0 = ptr[node], k1 = ptr[node + 1];
                    for (int k = k0; k < k1; ++k) {
                        const int j = nbr[k];
                        const float e0 = e[3 * (size_t)k], e1 = e[3 * (size_t)k + 1],
                                    e2 = e[3 * (size_t)k + 2];
                        const uint4* qp = reinterpret_cast<const uint4*>(
                            pq_in + (size_t)j * 2 * HID + HID + f0);
                        const uint4 qa = qp[0], qb = qp[1];
                        const unsigned w8[8] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y, qb.z, qb.w};
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const float2 q2 = __bfloat1622float2(
                                *reinterpret_cast<const __nv_bfloat162*>(&w8[u]));
                            const int o = f0 + 2 * u;
                            const float z0 = pz[2 * u] + q2.x +
                                             (Cs[o * 3] * e0 + Cs[o * 3 + 1] * e1 + Cs[o * 3 + 2] * e2);
                            const float z1 =
                                pz[2 * u + 1] + q2.y +
                                (Cs[o * 3 + 3] * e0 + Cs[o * 3 + 4] * e1 + Cs[o * 3 + 5] * e2);
                            acc16[2 * u] += fmaxf(z0, 0.f);
                            acc16[2 * u + 1] += fmaxf(z1, 0.f);
                        }
                    }
                    const float inv = 1.f / (float)max(k1 - k0, 1);
#pragma unroll
                    for (int q = 0; q < 16; ++q) acc16[q] *= inv;
                }
#pragma unroll
                for (int v = 0; v < 2; ++v) {
                    *reinterpret_cast<uint4*>(Xs + cm_off(r, f0 + 8 * v, SBO_X)) = hv4[v];
                    *reinterpret_cast<uint4*>(Xs + cm_off(r, HID + f0 + 8 * v, SBO_X)) =
                        make_uint4(pack2(acc16[8 * v], acc16[8 * v + 1]),
                                   pack2(acc16[8 * v + 2], acc16[8 * v + 3]),
                                   pack2(acc16[8 * v + 4], acc16[8 * v + 5]),
                                   pack2(acc16[8 * v + 6], acc16[8 * v + 7]));
                }
            }
        }
        fence_smem_async();
        fence_before();
        __syncthreads();
        if (*abort_flag) break;
        if (!ENC) {
            // v = U [h; agg]: 8 MMAs of K = 16 into columns 0..63
            if (tid == 0) {
                fence_after();
#pragma unroll
                for (int kk = 0; kk < 2 * HID / 16; ++kk)
                    mma(tbase, sdesc(xa + kk * 2 * LBO, SBO_X), sdesc(ua + kk * 2 * LBO, SBO_U),
                        idesc_bf16(TM, HID), kk > 0 ? 1u : 0u);
                commit(ubar);
            }
            pending = true;
            // the warp goes on only as a whole (tcgen05.ld is warp-collective)
            if (!__all_sync(0xffffffffu, wait_parity(ubar, phase & 1))) {
                atomicExch(err, (int)CFD_ERR_BARRIER);
                *abort_flag = 1;
            } else {
                pending = false;
                phase += 1;
                fence_after();
                // h <- h + relu(v + u) on this thread's row, columns [32 half, +32)
                const int node = tb + erow;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float acc[8];
                    if (c % 2 == 0) {
                        float a16[16];
                        tmem_ld16(tlane + 32 * half + 8 * c, a16);
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            acc[i] = a16[i];
                            acc_hi[i] = a16[8 + i];
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < 8; ++i) acc[i] = acc_hi[i];
                    }
                    const int k0 = 32 * half + 8 * c;
                    uint4* xp = reinterpret_cast<uint4*>(Xs + cm_off(erow, k0, SBO_X));
                    const uint4 hv = *xp;
                    const unsigned hw[4] = {hv.x, hv.y, hv.z, hv.w};
                    unsigned nw[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const float2 h2 =
                            __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&hw[u]));
                        const int col = k0 + 2 * u;
                        nw[u] = pack2(h2.x + fmaxf(acc[2 * u] + us[col], 0.f),
                                      h2.y + fmaxf(acc[2 * u + 1] + us[col + 1], 0.f));
                    }
                    const uint4 nv = make_uint4(nw[0], nw[1], nw[2], nw[3]);
                    *xp = nv;
                    if (node < n) *reinterpret_cast<uint4*>(hb + (size_t)node * HID + k0) = nv;
                }
            }
            fence_smem_async();
            fence_before();
            __syncthreads();
            if (*abort_flag) break;
        }
        if (has_pq) {
            // P|Q = [A; B] h: 4 MMAs of K = 16 into columns 0..127
            if (tid == 0) {
                fence_after();
#pragma unroll
                for (int kk = 0; kk < HID / 16; ++kk)
                    mma(tbase, sdesc(xa + kk * 2 * LBO, SBO_X), sdesc(wa + kk * 2 * LBO, SBO_W),
                        idesc_bf16(TM, 2 * HID), kk > 0 ? 1u : 0u);
                commit(ubar);
            }
            pending = true;
            if (!__all_sync(0xffffffffu, wait_parity(ubar, phase & 1))) {
                atomicExch(err, (int)CFD_ERR_BARRIER);
                *abort_flag = 1;
            } else {
                pending = false;
                phase += 1;
                fence_after();
                const int node = tb + erow;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    float v[16];
                    tmem_ld16(tlane + 64 * half + 16 * c, v);
                    if (node < n) {
                        uint4* op = reinterpret_cast<uint4*>(pq_out + (size_t)node * 2 * HID +
                                                             64 * half + 16 * c);
                        op[0] = make_uint4(pack2(v[0], v[1]), pack2(v[2], v[3]),
                                           pack2(v[4], v[5]), pack2(v[6], v[7]));
                        op[1] = make_uint4(pack2(v[8], v[9]), pack2(v[10], v[11]),
                                           pack2(v[12], v[13]), pack2(v[14], v[15]));
                    }
                }
            }
        } else if (half == 0) {
            // decoder: y = W_out h + b_out on this thread's row
            const int node = tb + erow;
            float hrow[HID];
#pragma unroll
            for (int c = 0; c < HID / 8; ++c) {
                const uint4 hv = *reinterpret_cast<const uint4*>(Xs + cm_off(erow, 8 * c, SBO_X));
                const unsigned hw[4] = {hv.x, hv.y, hv.z, hv.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float2 h2 =
                        __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&hw[u]));
                    hrow[8 * c + 2 * u] = h2.x;
                    hrow[8 * c + 2 * u + 1] = h2.y;
                }
            }
            if (node < n)
                for (int o = 0; o < OUT; ++o) {
                    float a = wo[OUT * HID + o];
                    for (int k = 0; k < HID; ++k) a += wo[o * HID + k] * hrow[k];
                    y[(size_t)OUT * node + o] = a;
                }
        }
        fence_before();
        __syncthreads();
        if (*abort_flag) break;
    }
    // a commit that timed out may still land: wait for it (bounded) before the columns go
    if (tid == 0 && pending) wait_parity(ubar, phase & 1);
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase),
                     "r"(TMEM_COLS)
                     : "memory");
    }
}
}  // namespace tc

int infer_bf16(cudaStream_t st, const float* w, bf16* wb, bool* wb_valid, int n, const int* ptr,
               const int* nbr, const float* f, const float* e, bf16* hb, bf16* pqb, float* y,
               const int* gate, int* err) {
    if (!*wb_valid) {
        CFD_LAUNCH(k_to_bf16, blocks_for(N_PARAMS, 256), 256, 0, st, N_PARAMS, w, wb);
        *wb_valid = true;
    }
    int dev = 0, nsm = 1;
    CFD_CUDA(cudaGetDevice(&dev));
    CFD_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    bf16* pq[2] = {pqb, pqb + (size_t)n * 2 * HID};
    // tensor-core generation: tcgen05 unless CFD_MPNN_TC=0 (the mma.sync passes)
    const char* tce = getenv("CFD_MPNN_TC");
    if (!(tce && atoi(tce) == 0)) {
        static bool tc_attr = false;
        if (!tc_attr) {
            CFD_CUDA(cudaFuncSetAttribute(tc::k_infer_tc<true>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM));
            CFD_CUDA(cudaFuncSetAttribute(tc::k_infer_tc<false>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM));
            tc_attr = true;
        }
        const int ntile = (n + tc::TM - 1) / tc::TM;
        const int grid = std::max(1, std::min(ntile, 2 * nsm));
        CFD_LAUNCH(tc::k_infer_tc<true>, grid, tc::NTHR, tc::SMEM, st, n, 0, ptr, nbr, e, f, w,
                   (const bf16*)wb, 1, (const bf16*)nullptr, hb, pq[0], y, gate, err);
        for (int l = 0; l < LAYERS; ++l) {
            const int next = l + 1 < LAYERS ? 1 : 0;
            CFD_LAUNCH(tc::k_infer_tc<false>, grid, tc::NTHR, tc::SMEM, st, n, l, ptr, nbr, e, f,
                       w, (const bf16*)wb, next, (const bf16*)pq[l & 1], hb, pq[(l + 1) & 1], y,
                       gate, err);
        }
        return CFD_OK;
    }
    const size_t smem_enc = sizeof(bf16) * (2 * HID * HS + IW * 16 * HS) +
                            sizeof(float) * (HID * F_IN + HID);
    const size_t smem_layer = sizeof(bf16) * (HID * XS + 2 * HID * HS + IW * 16 * XS) +
                              sizeof(float) * (HID * E_F + 2 * HID);
    static bool attr_set = false;
    if (!attr_set) {
        CFD_CUDA(cudaFuncSetAttribute(k_infer_encode, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem_enc));
        CFD_CUDA(cudaFuncSetAttribute(k_infer_layer, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem_layer));
        attr_set = true;
    }
    const int ntile = (n + TILE - 1) / TILE;
    const int grid = std::min(ntile, 2 * nsm);  // resident blocks (registers, shared memory)
    CFD_LAUNCH(k_infer_encode, grid, 32 * IW, smem_enc, st, n, f, w, (const bf16*)wb, hb, pq[0],
               gate);
    for (int l = 0; l < LAYERS; ++l) {
        const int next = l + 1 < LAYERS ? 1 : 0;
        CFD_LAUNCH(k_infer_layer, grid, 32 * IW, smem_layer, st, n, l, ptr, nbr, e, w,
                   (const bf16*)wb, next, (const bf16*)pq[l & 1], hb, pq[(l + 1) & 1], y, gate);
    }
    return CFD_OK;
}

}  // namespace mpnn
}  // namespace cfd

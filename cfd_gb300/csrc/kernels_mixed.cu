// kernels_mixed.cu — the mixed-precision form of the step (CFD_PREC_MIXED), sm_103a.
//
// FP32 for calcRHS, FUENTE, ESTAB, deltat and the Laplacian values; FP64 for the
// conserved-state update U1 = U - rk_fact/M*RHS, the areas and the gcl mass update, DTMIN,
// and (in the BiCG kernel) the vectors, dots and scalars.  Per-node sums of the FP32
// contributions are compensated (Neumaier).
//
// GB300's FP64 pipe runs 2 thread-ops per clock per SM, 64x fewer than FP32, and it also
// executes every double<->float conversion.  So the FP32 kernels read FP32 data only:
// float shadows of the primitives, of the geometry and of W, and float hi/lo splits of U
// and of (X, Y) (value = hi + lo), whose differences give gradients as accurate as FP64
// differences rounded to FP32.  FP64 arithmetic is left to the few places that need it.
//
// Stage invariance (calcRHS/FUENTE see the step-start U in all four RK stages,
// subrutinas.f90:685, :1064; only the module T changes, through mu and lambda,
// calcRHS.f90:49-51): stage 1 evaluates each element once and stores, per (element, local
// node) slot, the stage-invariant part Inv(0:3) (Galerkin, SUPG, shock capturing, FUENTE)
// and the coefficients of the viscous part, which is linear in (mu, lambda): Vmu(1:3),
// Vlam(3).  Slots are stored in element-around-point order, so each RK stage is one node
// kernel that streams its slots and forms Inv + mu*Vmu + lambda*Vlam with the stage's T.
#include "cfd_kernels.cuh"
#include "newmark.h"

namespace cfd {

__device__ __forceinline__ float pow15f(float x) { return x * sqrtf(x); }

// FP32 quotients of the stabilisation, time-step, Sutherland and RHS element kernels:
// __fdividef (within 2 ulp), several times fewer instructions than the IEEE quotient in
// kernels that are instruction-issue bound.  The node update keeps IEEE quotients.
__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }

// Neumaier-compensated float accumulator
struct Acc {
    float s, c;
    __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
    __device__ __forceinline__ void add(float x) {
        float t = s + x;
        if (fabsf(s) >= fabsf(x)) c += (s - t) + x;
        else c += (x - t) + s;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s + c; }
};

// hi/lo split of a double (split_bits of cfd_common.cuh)
__device__ __forceinline__ void split(double v, float& hi, float& lo) { split_bits(v, hi, lo); }

// ------------------------------------------------------------------ float shadows
// U -> (Uhi, Ulo); T, VX, VY -> float; (X, Y) -> (Xhi, Xlo); W -> Wf.  Any input may be NULL.
__global__ void k_narrow_state(int npoin, const double* __restrict__ U, const double* __restrict__ T,
                               const double* __restrict__ VX, const double* __restrict__ VY,
                               const double* __restrict__ X, const double* __restrict__ Y,
                               const double* __restrict__ WX, const double* __restrict__ WY,
                               float4* __restrict__ Uhi, float4* __restrict__ Ulo,
                               float* __restrict__ Tf, float* __restrict__ VXf,
                               float* __restrict__ VYf, float2* __restrict__ Xhi,
                               float2* __restrict__ Xlo, float2* __restrict__ Wf) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoin) return;
    if (U) {
        float h[4], l[4];
        for (int q = 0; q < 4; ++q) split(U[4 * (size_t)p + q], h[q], l[q]);
        Uhi[p] = make_float4(h[0], h[1], h[2], h[3]);
        Ulo[p] = make_float4(l[0], l[1], l[2], l[3]);
    }
    if (T) Tf[p] = (float)T[p];
    if (VX) VXf[p] = (float)VX[p];
    if (VY) VYf[p] = (float)VY[p];
    if (X) {
        float hx, lx, hy, ly;
        split(X[p], hx, lx);
        split(Y[p], hy, ly);
        Xhi[p] = make_float2(hx, hy);
        Xlo[p] = make_float2(lx, ly);
    }
    if (WX) Wf[p] = make_float2((float)WX[p], (float)WY[p]);
}

// Upload of U straight from pinned host memory (read by the kernel over the host link): the
// FP64 copy, the velocities ρu/ρ, ρv/ρ (k_vel_from_U's quotients) and, when Uhi is given,
// the mixed form's hi/lo split and float velocities (k_narrow_state's) in one pass, so
// the HBM writes ride under the link's transfer instead of following it.  hU is 16-B
// aligned (the caller checks).
__global__ void k_upload_U(int npoin, const double* __restrict__ hU, double* __restrict__ U,
                           double* __restrict__ VX, double* __restrict__ VY,
                           float4* __restrict__ Uhi, float4* __restrict__ Ulo,
                           float* __restrict__ VXf, float* __restrict__ VYf) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoin) return;
    const double2 a = reinterpret_cast<const double2*>(hU)[2 * (size_t)p];
    const double2 b = reinterpret_cast<const double2*>(hU)[2 * (size_t)p + 1];
    reinterpret_cast<double2*>(U)[2 * (size_t)p] = a;
    reinterpret_cast<double2*>(U)[2 * (size_t)p + 1] = b;
    const double vx = a.y / a.x, vy = b.x / a.x;
    VX[p] = vx;
    VY[p] = vy;
    if (Uhi) {
        float h[4], l[4];
        split(a.x, h[0], l[0]);
        split(a.y, h[1], l[1]);
        split(b.x, h[2], l[2]);
        split(b.y, h[3], l[3]);
        Uhi[p] = make_float4(h[0], h[1], h[2], h[3]);
        Ulo[p] = make_float4(l[0], l[1], l[2], l[3]);
        VXf[p] = (float)vx;
        VYf[p] = (float)vy;
    }
}

// double -> float
__global__ void k_narrow(long n, const double* __restrict__ a, float* __restrict__ b) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// hi + lo -> double (exact: lo starts below hi's last bit); lo may be null
__global__ void k_widen_pair(long n, const float* __restrict__ hi, const float* __restrict__ lo,
                             double* __restrict__ out) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = lo ? f2d_bits(hi[i]) + f2d_bits(lo[i]) : f2d_bits(hi[i]);
}

// float -> double (downloads of the mixed form's float fields)
__global__ void k_widen(long n, const float* __restrict__ a, double* __restrict__ b) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (double)a[i];
}

// ------------------------------------------------------------------ deltat
__device__ __forceinline__ float dtelem_f32(const int4 n, const float* __restrict__ T,
                                            const float* __restrict__ VX, const float* __restrict__ VY,
                                            const float2* __restrict__ W, float area, float fsafe,
                                            float t_inf) {
    const int nn[3] = {n.x, n.y, n.z};
    float vumax = 0.f, vvmax = 0.f;
    const float T_iel = (T[nn[0]] + T[nn[1]] + T[nn[2]]) * (1.f / 3.f);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float2 w = W[nn[i]];
        vumax = fmaxf(vumax, fabsf(VX[nn[i]] - w.x));
        vvmax = fmaxf(vvmax, fabsf(VY[nn[i]] - w.y));
    }
    const float hh = sqrtf(2.f * area);
    const float vel = sqrtf(vumax * vumax + vvmax * vvmax);
    const float et = 0.017f * pow15f(fdiv(T_iel, t_inf)) * fdiv(t_inf + 110.f, T_iel + 110.f);
    const float alpha = fminf(fdiv(vel * hh, 2.f * et) * (1.f / 3.f), 1.f);
    const float a = fdiv(4.f * et, hh * hh);
    // FSAFE/(1/DELTATC + 1/DELTATU) with 1/DELTATC = a, 1/DELTATU = a + alpha*vel/hh
    return fdiv(fsafe, a + (a + fdiv(alpha * vel, hh)));
}

// Second pass: elements whose FP32 DTELEM is within 1e-4 of the FP32 minimum get their
// DTELEM in FP64 (subrutinas.f90:172-206); the FP64 minimum over them is DTMIN, so the 1%
// hysteresis of ns2DComp.ALE.f90:146-156 sees an FP64-accurate value.  Only the
// 256-element chunks of k_deltat_mixed whose FP32 minimum lies in the band are visited.
__device__ __forceinline__ void refine_one(int e, const int4* __restrict__ elem,
                                           const float* __restrict__ T, const float* __restrict__ VX,
                                           const float* __restrict__ VY, const float2* __restrict__ W,
                                           const float* __restrict__ areaf, float fsafe, float t_inf,
                                           double m32, StepScal* __restrict__ sc) {
    const int4 n = elem[e];
    const float d32 = dtelem_f32(n, T, VX, VY, W, areaf[e], fsafe, t_inf);
    if ((double)d32 > m32 * (1.0 + 1.0e-4)) return;
    const int nn[3] = {n.x, n.y, n.z};
    double vumax = 0.0, vvmax = 0.0;
    const double T_iel = ((double)T[nn[0]] + (double)T[nn[1]] + (double)T[nn[2]]) / 3.0;
    for (int i = 0; i < 3; ++i) {
        const float2 w = W[nn[i]];
        const double vu = fabs((double)VX[nn[i]] - (double)w.x), vv = fabs((double)VY[nn[i]] - (double)w.y);
        if (vu > vumax) vumax = vu;
        if (vv > vvmax) vvmax = vv;
    }
    const double tinf = (double)t_inf;
    const double hh = sqrt(2.0 * (double)areaf[e]);
    const double vel = sqrt(vumax * vumax + vvmax * vvmax);
    const double et = 0.017 * (T_iel / tinf) * sqrt(T_iel / tinf) * (tinf + 110.0) / (T_iel + 110.0);
    const double alpha = fmin((vel * hh) / (2.0 * et) / 3.0, 1.0);
    const double deltatu = 1.0 / (4.0 * et / (hh * hh) + alpha * vel / hh);
    const double deltatc = 1.0 / (4.0 * et / (hh * hh));
    const double d = (double)fsafe / (1.0 / deltatc + 1.0 / deltatu);
    if (d > 0.0 && d < 1.0e20) atomicMin(&sc->dtmin_bits, (unsigned long long)__double_as_longlong(d));
}

__global__ void k_deltat_refine(int nelem, const int4* __restrict__ elem, const float* __restrict__ T,
                                const float* __restrict__ VX, const float* __restrict__ VY,
                                const float2* __restrict__ W, const float* __restrict__ areaf,
                                const unsigned long long* __restrict__ block_min, int nchunk,
                                float fsafe, float t_inf, StepScal* __restrict__ sc,
                                unsigned* __restrict__ count, int itlocal) {
    // thread t tests chunk blockIdx.x*256 + t; the block then refines the listed chunks
    __shared__ int list[256];
    __shared__ int nlist;
    const double m32 = __longlong_as_double((long long)sc->dtmin32_bits);
    const double band = m32 * (1.0 + 1.0e-4);
    if (threadIdx.x == 0) nlist = 0;
    __syncthreads();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nchunk && !(__longlong_as_double((long long)block_min[c]) > band))
        list[atomicAdd(&nlist, 1)] = c;
    __syncthreads();
    for (int k = 0; k < nlist; ++k) {
        const int e = list[k] * 256 + threadIdx.x;
        if (e < nelem) refine_one(e, elem, T, VX, VY, W, areaf, fsafe, t_inf, m32, sc);
    }
    // the last block to finish forms DTMIN (k_dt_finalize of the FP64 form)
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(count, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        *count = 0u;
        dt_finalize_from(sc, atomicExch(&sc->dtmin_bits, 0x7ff0000000000000ull));
        sc->iter += 1;
        if (itlocal) {  // DTFACT of ns2DComp.ALE.f90:160 for this ITER; COTA = 10*DTMIN raw
            sc->dtfact_f = (float)(1.0 - exp(-(sc->iter * 4.6 / itlocal)));
            sc->cota_f = (float)sc->cota;
        }
    }
}

// ------------------------------------------------------------------ deltat + ESTAB (FP32)
// ESTAB (subrutinas.f90:346-443; estab_mode as CFD_ESTAB_*) up to, not including, its use
// of DTMIN: SHOC, 1/tau^2 and the squared viscous terms (k4/h^2)^2 of the two lengths
// h_rgn, h_rgne (-1 where h = 0, whose TS is 0).  The stage-1 element kernel forms
// TS1 = (1/tau^2 + (2/DTMIN)^2)^(-1/2), TS2, TS3 = (1/tau^2 + (2/DTMIN)^2 + (k4/h^2)^2)^(-1/2).
struct EstabPre {
    float shoc, inv_tau2, v_rgn, v_rgne;
};

__device__ __forceinline__ EstabPre estab_pre(const float DX[3], const float DY[3], float rh1,
                                              float rh2, float rh3, float rl1, float rl2,
                                              float rl3, float vx, float vy, float t1, float t2,
                                              float t3, float gm, float FR, float RHOINF,
                                              float TINF, int estab_mode, float eps_dir,
                                              float dirx, float diry) {
    const float rho_elem = ((rh1 + rh2 + rh3) + (rl1 + rl2 + rl3)) * (1.f / 3.f);
    const float vel2 = sqrtf(vx * vx + vy * vy);
    // gradients from differences to node 1 (the shape-function gradients sum to 0)
    const float d2 = (rh2 - rh1) + (rl2 - rl1), d3 = (rh3 - rh1) + (rl3 - rl1);
    const float drx = d2 * DX[1] + d3 * DX[2], dry = d2 * DY[1] + d3 * DY[2];
    const float e2 = t2 - t1, e3 = t3 - t1;
    const float dtx = e2 * DX[1] + e3 * DX[2], dty = e2 * DY[1] + e3 * DY[2];
    const float temp = (t1 + t2 + t3) * (1.f / 3.f);
    const float dr2 = sqrtf(drx * drx + dry * dry) + 1.0e-20f;
    const float dt2 = sqrtf(dtx * dtx + dty * dty) + 1.0e-20f;
    float dux = 0.f, duy = 0.f;
    if (estab_mode == CFD_ESTAB_REFERENCE) {
        dux = vel2 * DX[0] + vel2 * DX[1] + vel2 * DX[2];
        duy = vel2 * DY[0] + vel2 * DY[1] + vel2 * DY[2];
    }
    const float du2 = sqrtf(dux * dux + duy * duy) + 1.0e-20f;
    const float idt2 = fdiv(1.f, dt2), idr2 = fdiv(1.f, dr2), idu2 = fdiv(1.f, du2);
    float rtx = dtx * idt2, rty = dty * idt2;
    float rjx = drx * idr2, rjy = dry * idr2;
    float rux = dux * idu2, ruy = duy * idu2;
    if (estab_mode == CFD_ESTAB_REGULARIZED) {
        float ge = 0.f;
#pragma unroll
        for (int i = 0; i < 3; ++i) ge += sqrtf(DX[i] * DX[i] + DY[i] * DY[i]);
        const float sr = eps_dir * rho_elem * ge, st = eps_dir * temp * ge;
        const float gx = drx + sr * dirx, gy = dry + sr * diry;
        const float hx = dtx + st * dirx, hy = dty + st * diry;
        const float ig = rsqrtf(gx * gx + gy * gy), ih = rsqrtf(hx * hx + hy * hy);
        rjx = gx * ig;
        rjy = gy * ig;
        rtx = hx * ih;
        rty = hy * ih;
        rux = dirx;
        ruy = diry;
    }
    const float c = sqrtf(gm * FR * temp);
    const float fmu = 0.017f * pow15f(fdiv(temp, TINF)) * fdiv(TINF + 110.f, temp + 110.f);
    float tau = 0.f, h_rgne = 0.f, h_rgn = 0.f, h_jgn = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float term1 = fabsf(vx * DX[i] + vy * DY[i]);
        const float term2 = fabsf(rjx * DX[i] + rjy * DY[i]);
        tau += term1 + term2 * c;
        h_rgne += fabsf(rtx * DX[i] + rty * DY[i]);
        h_rgn += fabsf(rux * DX[i] + ruy * DY[i]);
        h_jgn += term2;
    }
    tau = fdiv(1.f, tau);
    h_rgne = fdiv(2.f, h_rgne);
    h_rgn = fdiv(2.f, h_rgn);
    if (!(h_rgn <= 10.f)) h_rgn = 0.f;  // > 10 (and inf from 2/0) -> 0
    h_jgn = fdiv(2.f, h_jgn);
    if (!(h_jgn <= 10.f)) h_jgn = 0.f;
    const float tr1 = fdiv(dr2 * h_jgn, rho_elem);
    const float zzz = fdiv(h_jgn, 2.f * c);
    EstabPre o;
    o.shoc = (tr1 + tr1 * tr1) * 0.5f * (c * c) * zzz;
    o.inv_tau2 = fdiv(1.f, tau * tau);
    const float k4 = fdiv(4.f * fmu, RHOINF);
    // (resumen + 1/tau_s^2)^(-1/2), tau_s = h^2/k4, is (resumen + k4^2/h^4)^(-1/2); h = 0 -> 0
    const float hr2 = h_rgn * h_rgn, he2 = h_rgne * h_rgne;
    o.v_rgn = (hr2 > 0.f) ? fdiv(k4 * k4, hr2 * hr2) : -1.f;
    o.v_rgne = (he2 > 0.f) ? fdiv(k4 * k4, he2 * he2) : -1.f;
    return o;
}

// The step's first pass: deltat (subrutinas.f90:170-210) per element in FP32, per-block
// minima and the FP32 minimum as the bit pattern of a positive double, for the FP64
// refinement that forms DTMIN.  It gathers T, the velocities and W only, so that the mesh
// motion, which needs DTMIN, can start early; ESTAB's DTMIN-free part is formed by the
// stage-1 element kernel from the node data it gathers anyway.
__global__ void __launch_bounds__(256)
k_deltat_mixed(int nelem, const int4* __restrict__ elem, const float* __restrict__ T,
               const float* __restrict__ VX, const float* __restrict__ VY,
               const float2* __restrict__ W, const float* __restrict__ areaf, float TINF,
               float fsafe, unsigned long long* __restrict__ dtmin_bits,
               unsigned long long* __restrict__ block_min, float* __restrict__ DTE) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long mybits = 0x7ff0000000000000ull;
    if (e < nelem) {
        const float d32 = dtelem_f32(elem[e], T, VX, VY, W, areaf[e], fsafe, TINF);
        // 0 < d < 1e20 in FP64 as integer tests on the float's bits (positive normal,
        // below 0x60ad78ec = 1e20f, the least float >= 1e20): no FP64 compare per element
        const unsigned ub = __float_as_uint(d32);
        if (ub >= 0x00800000u && ub < 0x60ad78ecu)
            mybits = (unsigned long long)__double_as_longlong(f2d_bits(d32));
        if (DTE) DTE[e] = d32;  // DT of the element, for ITLOCAL's DTL
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long q = __shfl_down_sync(0xffffffffu, mybits, off);
        mybits = q < mybits ? q : mybits;
    }
    __shared__ unsigned long long wmin[32];
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = mybits;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = wmin[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = wmin[w] < m ? wmin[w] : m;
        block_min[blockIdx.x] = m;
        atomicMin(dtmin_bits, m);
    }
}

// ------------------------------------------------------------------ element mu, lambda
// calcRHS.f90:49-51: Sutherland mu and lambda at the element's mean T, in FP32
__device__ __forceinline__ float2 elem_mu_lambda(const int4 n, const float* __restrict__ T,
                                                 const GasConstF& gc) {
    const float t_inf = gc.t_inf;
    const float Ta = (T[n.x] + T[n.y] + T[n.z]) * (1.f / 3.f);
    const float r15 = pow15f(fdiv(Ta, t_inf));
    return make_float2(gc.mu_ref * r15 * fdiv(t_inf + 110.f, Ta + 110.f),
                       gc.lambda_ref * r15 * fdiv(t_inf + 194.f, Ta + 194.f));
}

// mu, lambda of every element from the T of the previous RK stage (stages 2-4)
__global__ void k_elem_mulam(int nelem, const int4* __restrict__ elem, const float* __restrict__ T,
                             GasConstF gc, float2* __restrict__ mulam) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    mulam[e] = elem_mu_lambda(elem[e], T, gc);
}

// ------------------------------------------------------------------ stage-1 element kernel
// ESTAB (subrutinas.f90:346-443, its DTMIN-free part by estab_pre, then TS1-3 with the step's
// DTMIN) and calcRHS.f90:36-141 + FUENTE (subrutinas.f90:1060-1078) in FP32, folded with
// the step's area*dtl/3, written as slot records in element-around-point order: recInv
// holds the stage-invariant contributions to the 4 equations, recVisc Vmu(1), Vmu(2),
// Vmu(3), Vlam(3).

template <bool VISCOUS>
__global__ void __launch_bounds__(128, 6)
k_elem_stage1_mixed(int nelem, const int4* __restrict__ elem, const float4* __restrict__ Uhi,
                    const float4* __restrict__ Ulo, const float4* __restrict__ geo,
                    const float* __restrict__ VX, const float* __restrict__ VY, EstabConst ec,
                    const StepScal* __restrict__ sc, GasConstF gc,
                    const float2* __restrict__ W, const int* __restrict__ slot_pos,
                    const float* __restrict__ T, float4* __restrict__ recInv,
                    float4* __restrict__ recVisc, float2* __restrict__ mulam,
                    const float* __restrict__ dte) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    const float g = gc.gamma, Cv = gc.cv;
    const int4 n = elem[e];
    if (VISCOUS) mulam[e] = elem_mu_lambda(n, T, gc);  // for the first RK stage
    const int p[3] = {n.x, n.y, n.z};
    const float4 ga = geo[2 * (size_t)e], gb = geo[2 * (size_t)e + 1];
    const float Nx[3] = {ga.x, ga.y, ga.z};
    const float Ny[3] = {ga.w, gb.x, gb.y};
    float Un[3][4], Ul[3][4];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float4 h = Uhi[p[i]], l = Ulo[p[i]];
        Un[i][0] = h.x; Un[i][1] = h.y; Un[i][2] = h.z; Un[i][3] = h.w;
        Ul[i][0] = l.x; Ul[i][1] = l.y; Ul[i][2] = l.z; Ul[i][3] = l.w;
    }
    float Ux[4], Uy[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float d1 = (Un[1][q] - Un[0][q]) + (Ul[1][q] - Ul[0][q]);
        const float d2 = (Un[2][q] - Un[0][q]) + (Ul[2][q] - Ul[0][q]);
        Ux[q] = d1 * Nx[1] + d2 * Nx[2];
        Uy[q] = d1 * Ny[1] + d2 * Ny[2];
    }
    const float2 w0 = W[p[0]], w1 = W[p[1]], w2 = W[p[2]];
    // ESTAB: the DTMIN-free part from the gathered rho (hi, lo), relative velocity and T,
    // then TS1-3 with this step's DTMIN
    float tau[3], nu;
    {
        const float t1 = T[p[0]], t2 = T[p[1]], t3 = T[p[2]];
        const float vx = ((VX[p[0]] + VX[p[1]] + VX[p[2]]) - (w0.x + w1.x + w2.x)) * (1.f / 3.f);
        const float vy = ((VY[p[0]] + VY[p[1]] + VY[p[2]]) - (w0.y + w1.y + w2.y)) * (1.f / 3.f);
        const EstabPre o = estab_pre(Nx, Ny, Un[0][0], Un[1][0], Un[2][0], Ul[0][0], Ul[1][0],
                                     Ul[2][0], vx, vy, t1, t2, t3, ec.gm, ec.fr, ec.rho_inf,
                                     ec.t_inf, ec.mode, ec.eps, ec.dirx, ec.diry);
        const float two_dt = fdiv(2.f, sc->dtmin_f);
        const float resumen = o.inv_tau2 + two_dt * two_dt;
        tau[0] = rsqrtf(resumen);
        tau[1] = (o.v_rgn >= 0.f) ? rsqrtf(resumen + o.v_rgn) : 0.f;
        tau[2] = (o.v_rgne >= 0.f) ? rsqrtf(resumen + o.v_rgne) : 0.f;
        nu = o.shoc * gc.cte;
    }
    // area*dtl/3 with dtl = DTMIN, or under ITLOCAL DTL = DTMIN*DTFACT + min(DT, COTA)*(1-DTFACT)
    // (ns2DComp.ALE.f90:159-162, subrutinas.f90:211-215)
    float dtl = sc->dtmin_f;
    if (dte) {
        const float f = sc->dtfact_f;
        dtl = sc->dtmin_f * f + fminf(dte[e], sc->cota_f) * (1.f - f);
    }
    const float scale = gb.z * dtl * (1.f / 3.f);
    // Over the three edge-midpoint quadrature points k, only A (the Galerkin flux
    // divergence, to the two nodes other than k), B1, B2 and the viscous coefficients
    // depend on k; the test-function gradients and tau do not.  So the k-loop sums A per
    // node, B1, B2 and the seven viscous coefficients, and the products with Nx, Ny, tau
    // and the shock-capturing term (the same at every k) are formed once.
    float r[3][4], SB1[4], SB2[4];
    float Sm11 = 0.f, Sm12 = 0.f, Sm22 = 0.f, Sm13 = 0.f, Sm23 = 0.f, Sl13 = 0.f, Sl23 = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        SB1[q] = 0.f;
        SB2[q] = 0.f;
#pragma unroll
        for (int i = 0; i < 3; ++i) r[i][q] = 0.f;
    }
    const float gm1 = g - 1.f, gm3 = g - 3.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int ia = (k == 0) ? 1 : 0;
        const int ib = (k == 2) ? 1 : 2;
        float Uk[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) Uk[q] = 0.5f * (Un[ia][q] + Un[ib][q]);
        const float rho = Uk[0];
        const float irho = fdiv(1.f, rho);
        const float v1 = Uk[1] * irho, v2 = Uk[2] * irho, ev = Uk[3] * irho;
        const float V_sq = v1 * v1 + v2 * v2;
        const float W0 = V_sq * gm1 - ev * g;
        float A[4];
        A[0] = Ux[1] + Uy[2];
        A[1] = 0.5f * Ux[0] * (V_sq * gm1 - 2.f * v1 * v1) - Ux[1] * v1 * gm3 - Ux[2] * v2 * gm1 +
               Ux[3] * gm1 - Uy[0] * v1 * v2 + Uy[1] * v2 + Uy[2] * v1;
        A[2] = -Ux[0] * v1 * v2 + Ux[1] * v2 + Ux[2] * v1 + 0.5f * Uy[0] * (V_sq * gm1 - 2.f * v2 * v2) -
               Uy[1] * v1 * gm1 - Uy[2] * v2 * gm3 + Uy[3] * gm1;
        A[3] = Ux[0] * v1 * W0 - 0.5f * Ux[1] * (V_sq * gm1 - 2.f * ev * g + 2.f * v1 * v1 * gm1) -
               Ux[2] * v1 * v2 * gm1 + Ux[3] * g * v1 + Uy[0] * v2 * W0 - Uy[1] * v1 * v2 * gm1 -
               0.5f * Uy[2] * (V_sq * gm1 - 2.f * ev * g + 2.f * v2 * v2 * gm1) + Uy[3] * g * v2;
        float B1[4], B2[4];
        const float h0 = 0.5f * V_sq * gm1;
        B1[0] = A[1];
        B1[1] = v1 * (3.f - g) * A[1] - v2 * gm1 * A[2] + gm1 * A[3] + (h0 - v1 * v1) * A[0];
        B1[2] = -v1 * v2 * A[0] + v1 * A[2] + v2 * A[1];
        B1[3] = g * v1 * A[3] - v1 * v2 * gm1 * A[2] + v1 * W0 * A[0] + (-h0 + ev * g - v1 * v1 * gm1) * A[1];
        B2[0] = A[2];
        B2[1] = B1[2];
        B2[2] = -v1 * gm1 * A[1] + v2 * (3.f - g) * A[2] + gm1 * A[3] + (h0 - v2 * v2) * A[0];
        B2[3] = g * v2 * A[3] - v1 * v2 * gm1 * A[1] + v2 * W0 * A[0] + (-h0 + ev * g - v2 * v2 * gm1) * A[2];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            SB1[q] += B1[q];
            SB2[q] += B2[q];
            r[ia][q] += 0.5f * A[q];
            r[ib][q] += 0.5f * A[q];
        }
        if (VISCOUS) {
            // K1, K2 of calcRHS.f90:121-132 split as mu*(...) + lambda*(...)
            const float icv = irho * fdiv(1.f, Cv);
            const float m11 = (2.f / 3.f) * (-2.f * Ux[0] * v1 + 2.f * Ux[1] + Uy[0] * v2 - Uy[2]) * irho;
            const float m12 = (-Ux[0] * v2 + Ux[2] - Uy[0] * v1 + Uy[1]) * irho;
            const float m22 = (2.f / 3.f) * (Ux[0] * v1 - Ux[1] - 2.f * Uy[0] * v2 + 2.f * Uy[2]) * irho;
            const float m13 = (1.f / 3.f) * Cv *
                              ((-Uy[0] * v1 * v2 + 3.f * Uy[1] * v2 - 2.f * Uy[2] * v1) -
                               Ux[0] * (3.f * V_sq + v1 * v1) + 4.f * Ux[1] * v1 + 3.f * Ux[2] * v2) * icv;
            const float l13 = (1.f / 3.f) *
                              (3.f * Ux[0] * (V_sq - ev) - 3.f * Ux[1] * v1 - 3.f * Ux[2] * v2 + 3.f * Ux[3]) * icv;
            const float m23 = (1.f / 3.f) * Cv *
                              ((-Ux[0] * v1 * v2 - 2.f * Ux[1] * v2 + 3.f * Ux[2] * v1) -
                               Uy[0] * (3.f * V_sq + v2 * v2) + 3.f * Uy[1] * v1 + 4.f * Uy[2] * v2) * icv;
            const float l23 = (1.f / 3.f) *
                              (3.f * Uy[0] * (V_sq - ev) - 3.f * Uy[1] * v1 - 3.f * Uy[2] * v2 + 3.f * Uy[3]) * icv;
            Sm11 += m11;
            Sm12 += m12;
            Sm22 += m22;
            Sm13 += m13;
            Sm23 += m23;
            Sl13 += l13;
            Sl23 += l23;
        }
    }
    // SUPG (tau) and shock capturing (nu, three quadrature points of the same value)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q)
            r[i][q] += tau[i] * (Nx[i] * SB1[q] + Ny[i] * SB2[q]) +
                       3.f * nu * (Nx[i] * Ux[q] + Ny[i] * Uy[q]);
    {  // FUENTE: -AR*sum_k sp(i,k)*(Ux*wx_k + Uy*wy_k), AR = area*dtl/3 = scale
        const float wx[3] = {0.5f * (w0.x + w1.x), 0.5f * (w1.x + w2.x), 0.5f * (w0.x + w2.x)};
        const float wy[3] = {0.5f * (w0.y + w1.y), 0.5f * (w1.y + w2.y), 0.5f * (w0.y + w2.y)};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float q0 = Ux[q] * wx[0] + Uy[q] * wy[0];
            const float q1 = Ux[q] * wx[1] + Uy[q] * wy[1];
            const float q2 = Ux[q] * wx[2] + Uy[q] * wy[2];
            r[0][q] -= 0.5f * (q0 + q2);
            r[1][q] -= 0.5f * (q0 + q1);
            r[2][q] -= 0.5f * (q1 + q2);
        }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int pos = slot_pos[3 * (size_t)e + i];
        recInv[pos] = make_float4(r[i][0] * scale, r[i][1] * scale, r[i][2] * scale, r[i][3] * scale);
        if (VISCOUS) {
            const float vm0 = Nx[i] * Sm11 + Ny[i] * Sm12, vm1 = Nx[i] * Sm12 + Ny[i] * Sm22;
            const float vm2 = Nx[i] * Sm13 + Ny[i] * Sm23, vl = Nx[i] * Sl13 + Ny[i] * Sl23;
            recVisc[pos] = make_float4(vm0 * scale, vm1 * scale, vm2 * scale, vl * scale);
        }
    }
}

// ------------------------------------------------------------------ RK stage, node side
// subrutinas.f90:680-825 for one stage.  The node's RHS is the compensated sum over its
// slots of Inv, formed in the first stage and kept per node, plus the compensated sum of
// mu_e*Vmu + lambda_e*Vlam (mu, lambda from the stage's element T, calcRHS.f90:49-51);
// delta = rk_fact/M*RHS in FP32; U1 = U - delta in FP64.  Nodes
// without a boundary condition keep U1 as updated and get FP32 primitives; boundary nodes
// follow the reference's FP64 primitive round trip and BC order.
// Only T of stages 1-3 is read later (through mu, lambda of the next stage; U1 and the
// other primitives are rewritten by stage 4), so stages 1-3 write T alone at nodes without
// a boundary condition.  The last stage writes U1, every primitive and the hi/lo split of
// U1 (the next step's U).  Node p alone reads U[p] and writes U1[p], so U1 may be U (the
// update in place, U = U1 of ns2DComp.ALE.f90:277-281 without a copy).
constexpr int kNodeTB = 128;  // threads per block of the node passes
// The node's update once its slot sums are known (inv: the stage-invariant sum in the first
// stage, read back from invSum in the others; sv1..3: the viscous sums)
// The node's own inputs of node_finish, loaded ahead of its slot sums so that they are in
// flight together with the slot loads (the stage-invariant sum of the first stage is formed
// from the slots, not loaded)
struct NodePre {
    float4 inv, h;
    float im;
    unsigned char fl;
};
template <bool FIRST>
__device__ __forceinline__ NodePre node_pre(int p, const float4* __restrict__ invSum,
                                            const float* __restrict__ invM,
                                            const unsigned char* __restrict__ bcflag,
                                            const float4* __restrict__ Uhi) {
    NodePre q;
    q.inv = FIRST ? make_float4(0.f, 0.f, 0.f, 0.f) : invSum[p];
    q.im = invM[p];
    q.fl = bcflag[p];
    q.h = Uhi[p];
    return q;
}

template <bool FIRST, bool LAST>
__device__ __forceinline__ void node_finish(
    int p, const NodePre& pre, float4 inv, float sv1, float sv2, float sv3,
    float4* __restrict__ invSum, GasConst gc,
    GasConstF gf, const double* U, float4* __restrict__ Uhi, float4* __restrict__ Ulo,
    const float* __restrict__ invM, float rk_fact, const unsigned char* __restrict__ bcflag,
    const double* __restrict__ bcval, const double2* __restrict__ nrm,
    const double* __restrict__ WX, const double* __restrict__ WY, double* U1,
    float* __restrict__ RHO, float* __restrict__ VX, float* __restrict__ VY,
    float* __restrict__ Eo, float* __restrict__ Po, float* __restrict__ Tout,
    float* __restrict__ RMACH) {
    if (FIRST) invSum[p] = inv;
    else inv = pre.inv;
    const float f = rk_fact * pre.im;
    const float d0 = f * inv.x, d1 = f * (inv.y + sv1), d2 = f * (inv.z + sv2),
                d3 = f * (inv.w + sv3);
    const float g = gf.gamma;
    const unsigned char fl = pre.fl;
    if (!fl) {
        const float4 h = pre.h;
        const float rho = h.x - d0, ir = 1.f / rho;
        const float vx = (h.y - d1) * ir, vy = (h.z - d2) * ir, ee = (h.w - d3) * ir;
        const float vel2 = vx * vx + vy * vy;
        const float pp = rho * (g - 1.f) * (ee - 0.5f * vel2);
        const float tt = pp / (rho * gf.fr);
        Tout[p] = tt;
        if (!LAST) return;
        RHO[p] = rho; VX[p] = vx; VY[p] = vy; Eo[p] = ee; Po[p] = pp;
        RMACH[p] = sqrtf(fdiv(vel2, tt * g * gf.fr));
    }
    const double2* u2 = reinterpret_cast<const double2*>(U + 4 * (size_t)p);
    const double2 ua = u2[0], ub = u2[1];
    double u1_0 = ua.x - f2d_bits(d0), u1_1 = ua.y - f2d_bits(d1), u1_2 = ub.x - f2d_bits(d2),
           u1_3 = ub.y - f2d_bits(d3);
    if (fl) {
        const double gd = gc.gamma, FR = gc.fr;
        double rho = u1_0;
        double vx = u1_1 / rho, vy = u1_2 / rho, ee = u1_3 / rho;
        const double vel2 = vx * vx + vy * vy;
        const double pp = rho * (gd - 1.0) * (ee - 0.5 * vel2);
        double tt = pp / (rho * FR);
        RMACH[p] = (float)sqrt(vel2 / (tt * gd * FR));
        Po[p] = (float)pp;
        const double2* b2 = reinterpret_cast<const double2*>(bcval + 4 * (size_t)p);
        const double2 bva = b2[0], bvb = b2[1];
        if (fl & BC_FIXV) { vx = bva.x; vy = bva.y; }
        if (fl & BC_NORMAL) {
            const double2 nn = nrm[p];
            const double wx = WX[p], wy = WY[p];
            const double q = -(nn.y * (vx - wx)) + nn.x * (vy - wy);
            vx = -(nn.y * q) + wx;
            vy = nn.x * q + wy;
        }
        if (fl & BC_FIXRHO) rho = bvb.x;
        if (fl & BC_FIXT) {
            tt = bvb.y;
            ee = tt * FR / (gd - 1.0) + 0.5 * (vx * vx + vy * vy);
        }
        RHO[p] = (float)rho; VX[p] = (float)vx; VY[p] = (float)vy; Eo[p] = (float)ee;
        Tout[p] = (float)tt;
        u1_0 = rho; u1_1 = vx * rho; u1_2 = vy * rho; u1_3 = ee * rho;
    }
    if (LAST) {  // U1 of stages 1-3 is never read (only their T is), so it is not written
        double2* o = reinterpret_cast<double2*>(U1 + 4 * (size_t)p);
        o[0] = make_double2(u1_0, u1_1);
        o[1] = make_double2(u1_2, u1_3);
        float h[4], l[4];
        split(u1_0, h[0], l[0]);
        split(u1_1, h[1], l[1]);
        split(u1_2, h[2], l[2]);
        split(u1_3, h[3], l[3]);
        Uhi[p] = make_float4(h[0], h[1], h[2], h[3]);
        Ulo[p] = make_float4(l[0], l[1], l[2], l[3]);
    }
}

constexpr int kSlotBatch = 4, kSlotBatchFirst = 4;  // slots whose loads go out together
template <bool FIRST, bool LAST>
__global__ void __launch_bounds__(kNodeTB)
k_node_mixed(int npoin, const int* __restrict__ esup_ptr, const int* __restrict__ esup_slot,
             const float2* __restrict__ mulam, const float4* __restrict__ recInv,
             const float4* __restrict__ recVisc, float4* __restrict__ invSum, GasConst gc,
             GasConstF gf, int viscous,
             const double* U, float4* __restrict__ Uhi, float4* __restrict__ Ulo,
             const float* __restrict__ invM, float rk_fact,
             const unsigned char* __restrict__ bcflag, const double* __restrict__ bcval,
             const double2* __restrict__ nrm, const double* __restrict__ WX,
             const double* __restrict__ WY, double* U1, float* __restrict__ RHO, float* __restrict__ VX,
             float* __restrict__ VY, float* __restrict__ Eo, float* __restrict__ Po,
             float* __restrict__ Tout, float* __restrict__ RMACH) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoin) return;
    const NodePre pre = node_pre<FIRST>(p, invSum, invM, bcflag, Uhi);
    Acc a0, a1, a2, a3, v1, v2, v3;
    a0.init(); a1.init(); a2.init(); a3.init();
    v1.init(); v2.init(); v3.init();
    const int s0 = esup_ptr[p], s1 = esup_ptr[p + 1];
    // B slots per pass: their loads are issued together, the sums stay in slot order
    constexpr int B = FIRST ? kSlotBatchFirst : kSlotBatch;
    for (int s = s0; s < s1; s += B) {
        float4 ri[B], rv[B];
        int e[B];
        float2 ml[B];
#pragma unroll
        for (int j = 0; j < B; ++j) {
            if (s + j < s1) {
                if (FIRST) ri[j] = recInv[s + j];
                if (viscous) {
                    rv[j] = recVisc[s + j];
                    e[j] = esup_slot[s + j] / 3;
                }
            }
        }
        if (viscous) {
#pragma unroll
            for (int j = 0; j < B; ++j)
                if (s + j < s1) ml[j] = mulam[e[j]];
        }
#pragma unroll
        for (int j = 0; j < B; ++j) {
            if (s + j < s1) {
                if (FIRST) {
                    a0.add(ri[j].x);
                    a1.add(ri[j].y);
                    a2.add(ri[j].z);
                    a3.add(ri[j].w);
                }
                if (viscous) {
                    v1.add(ml[j].x * rv[j].x);
                    v2.add(ml[j].x * rv[j].y);
                    v3.add(ml[j].x * rv[j].z + ml[j].y * rv[j].w);
                }
            }
        }
    }
    const float4 inv =
        FIRST ? make_float4(a0.value(), a1.value(), a2.value(), a3.value()) : make_float4(0.f, 0.f, 0.f, 0.f);
    node_finish<FIRST, LAST>(p, pre, inv, v1.value(), v2.value(), v3.value(), invSum, gc, gf, U, Uhi, Ulo,
                             invM, rk_fact, bcflag, bcval, nrm, WX, WY, U1, RHO, VX, VY, Eo, Po,
                             Tout, RMACH);
}

// ------------------------------------------------------------------ geometry (mixed)
// Per element, 8 floats (two float4): geo[2e] = (dNx1, dNx2, dNx3, dNy1),
// geo[2e+1] = (dNy2, dNy3, area, q) with q the mesh-Laplacian weight of the element.
//
// Element pass: the edge vectors and the signed area 2a = x1*y2 - x2*y1 (deriv,
// subrutinas.f90:102-115) in FP64 from the FP64 coordinates; the area is kept in FP64 for
// the gcl (area, putArea's area_old), the gradients and the Laplacian weight in FP32 from
// the edge vectors truncated to FP32.  The Laplacian weight of mLaplace.f90:28-56: with
// |grad N_i|^2 = l_i^2/(2a)^2 the quality mu = 2*sqrt(3)*(2a)/sum(l_i^2) of
// mLaplace.f90:96-108 is sqrt(3)/(a*sum|grad N_i|^2), so q = 1/mu^2 = (a*sum|grad N_i|^2)^2/3;
// with gcl, the element terms of gcl main (gcl.f90:27-45) divW*area and divW_old*area_old
// in FP64 (divW itself from the FP32 gradients and W; the node pass applies the 1/3), then
// putArea.
__global__ void k_elem_geometry(int nelem, const int4* __restrict__ elem,
                                const double* __restrict__ X, const double* __restrict__ Y,
                                int gcl, int literal, const float2* __restrict__ W,
                                const float2* __restrict__ Wold, int put_area,
                                double* __restrict__ area_old, double* __restrict__ area64,
                                float* __restrict__ areaf, float4* __restrict__ geo,
                                double2* __restrict__ terms, NormalsArgs nv) {
    // the blocks after the elements' do normales (one wall node per thread)
    const int eblocks = (nelem + blockDim.x - 1) / blockDim.x;
    if (nv.nwn > 0 && (int)blockIdx.x >= eblocks) {
        const int k = ((int)blockIdx.x - eblocks) * blockDim.x + threadIdx.x;
        if (k < nv.nwn) normales_node(nv, k);
        return;
    }
    // grid-stride over the elements (the normales blocks, when any, follow eblocks blocks)
    const int estride = (nv.nwn > 0 ? eblocks : (int)gridDim.x) * blockDim.x;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nelem; e += estride) {
    const int4 n = elem[e];
    const double X0 = X[n.x], Y0 = Y[n.x];
    const double dx1 = X[n.y] - X0, dy1 = Y[n.y] - Y0;
    const double dx2 = X[n.z] - X0, dy2 = Y[n.z] - Y0;
    // 2a = x1*y2 - x2*y1 (the reference's signed area from differences to node 1), FP64
    const double a64 = 0.5 * (dx1 * dy2 - dx2 * dy1);
    const float x1 = d2f_trunc(dx1), y1 = d2f_trunc(dy1);
    const float x2 = d2f_trunc(dx2), y2 = d2f_trunc(dy2);
    const float a2f = fmaf(x1, y2, -(x2 * y1));
    const float area = 0.5f * a2f;
    const float ia = fdiv(1.f, a2f);
    const float gx[3] = {(y1 - y2) * ia, y2 * ia, -y1 * ia};  // (y_2 - y_3)/(2a), ... with y_1 = 0
    const float gy[3] = {(x2 - x1) * ia, -x2 * ia, x1 * ia};
    const float s2 = gx[0] * gx[0] + gy[0] * gy[0] + gx[1] * gx[1] + gy[1] * gy[1] +
                     gx[2] * gx[2] + gy[2] * gy[2];
    const float am = area * s2;
    const float q = am * am * (1.f / 3.f);
    geo[2 * (size_t)e] = make_float4(gx[0], gx[1], gx[2], gy[0]);
    geo[2 * (size_t)e + 1] = make_float4(gy[1], gy[2], area, q);
    areaf[e] = area;
    area64[e] = a64;
    if (gcl) {
        const int nn[3] = {n.x, n.y, n.z};
        float divW = 0.f, divWo = 0.f;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float2 w = W[nn[i]], wo = Wold[nn[i]];
            divW += gx[i] * w.x + gy[i] * (literal ? w.x : w.y);
            divWo += gx[i] * wo.x + gy[i] * (literal ? wo.x : wo.y);
        }
        terms[e] = make_double2(f2d_bits(divW) * a64, f2d_bits(divWo) * area_old[e]);
    }
    if (put_area) area_old[e] = a64;
    }
}

// Double-float arithmetic (a value as an unevaluated FP32 pair h + l, |l| <= ulp(h)): the
// relative tests' element matrices and their row sums in ~2^-46 relative accuracy on the
// FP32 pipe, which runs 64 times the FP64 pipe's operations on this GPU.  TwoSum, Fast2Sum (|a| >= |b|) and the exact
// product by fmaf are the error-free transformations; the quotient takes two remainder
// corrections.
struct DF {
    float h, l;
};
__device__ __forceinline__ DF df_fast2(float a, float b) {
    const float s = a + b;
    return DF{s, b - (s - a)};
}
__device__ __forceinline__ DF df_two(float a, float b) {
    const float s = a + b, bb = s - a;
    return DF{s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DF df_add(DF x, DF y) {
    const DF s = df_two(x.h, y.h);
    return df_fast2(s.h, s.l + (x.l + y.l));
}
__device__ __forceinline__ DF df_sub(DF x, DF y) { return df_add(x, DF{-y.h, -y.l}); }
// a += b for pairs held as float2 (x = h, y = l)
__device__ __forceinline__ void df_acc(float2& a, float2 b) {
    const DF s = df_add(DF{a.x, a.y}, DF{b.x, b.y});
    a = make_float2(s.h, s.l);
}
__device__ __forceinline__ DF df_mul(DF x, DF y) {
    const float p = x.h * y.h;
    float e = fmaf(x.h, y.h, -p);
    e = fmaf(x.h, y.l, e);
    e = fmaf(x.l, y.h, e);
    return df_fast2(p, e);
}
__device__ __forceinline__ DF df_div(DF x, DF y) {
    const float q1 = x.h / y.h;
    const DF r1 = df_sub(x, df_mul(y, DF{q1, 0.f}));
    const DF s = df_fast2(q1, r1.h / y.h);
    const DF r2 = df_sub(x, df_mul(y, s));
    return df_add(s, DF{r2.h / y.h, 0.f});
}
__device__ __forceinline__ DF df_of(double v) {
    DF r;
    split_bits(v, r.h, r.l);
    return r;
}

// Node pass: the row of the mesh Laplacian (mLaplace.f90:28-56; rows of up to 16 entries
// are summed in shared memory, longer ones in place), 1/diag, and the lumped mass: MASAS
// (subrutinas.f90:128-153) as a compensated FP32 sum of area/3, or the gcl update
// M += dt*(tot1+tot2)/2 in FP64 from FP64 sums (slot order) of the FP64 element terms,
// followed by putW (W_old = W).  ROW64 (the relative stopping tests): the row is the sum, in
// double-float and slot order, of the slots' rows of the element matrices (k_elem_grad64),
// written as valf + val_lo (the pair's h and l); the FP32 geometry is then read only for
// MASAS.
constexpr int kLapRow = 16;
constexpr int kGeoBatch = 2;  // slots per pass of k_node_geometry
constexpr int kGeoBlock = kGeoNodeBlock;


template <bool ROW64>
__global__ void __launch_bounds__(kGeoBlock)
k_node_geometry(int npoin, const int* __restrict__ esup_ptr, const int* __restrict__ esup_slot,
                const uchar4* __restrict__ lap_pos, const float4* __restrict__ geo,
                const double2* __restrict__ terms, const double* __restrict__ dtp, int gcl,
                const int* __restrict__ rowptr, float* __restrict__ valf,
                double* __restrict__ invdiag, float* __restrict__ invdiagf,
                double* __restrict__ M, float* __restrict__ invM,
                const float2* __restrict__ W, float2* __restrict__ Wold,
                const float2* __restrict__ k64, float* __restrict__ val_lo) {
    __shared__ float row[ROW64 ? 1 : kGeoBlock][kLapRow + 1];
    __shared__ float2 row64[ROW64 ? kGeoBlock : 1][kLapRow + 1];
    const bool need_geo = !ROW64 || !gcl;
    // grid-stride (a smaller grid leaves room for kernels running beside it)
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npoin; p += gridDim.x * blockDim.x) {
    float* acc = row[ROW64 ? 0 : threadIdx.x];
    float2* acc64 = row64[ROW64 ? threadIdx.x : 0];
    const int r0 = rowptr[p], r1 = rowptr[p + 1];
    const int len = r1 - r0;
    const bool in_smem = len <= kLapRow;
    if (ROW64) {
        if (in_smem)
            for (int k = 0; k < len; ++k) acc64[k] = make_float2(0.f, 0.f);
    } else if (in_smem) {
#pragma unroll
        for (int k = 0; k < kLapRow; ++k) acc[k] = 0.f;
    } else {
        for (int k = r0; k < r1; ++k) valf[k] = 0.f;
    }
    Acc m1;
    m1.init();
    double t1 = 0.0, t2 = 0.0;  // gcl: tot1, tot2 (times 3)
    // kGeoBatch slots per pass: their loads go out together, the sums stay in slot order
    const int s0 = esup_ptr[p], s1 = esup_ptr[p + 1];
    for (int sb = s0; sb < s1; sb += kGeoBatch) {
        int slot[kGeoBatch];
        uchar4 pos[kGeoBatch];
        float4 ga[kGeoBatch], gb[kGeoBatch];
        double2 tm[kGeoBatch];
        float2 kr[kGeoBatch][3];
#pragma unroll
        for (int u = 0; u < kGeoBatch; ++u)
            if (sb + u < s1) {
                slot[u] = esup_slot[sb + u];
                pos[u] = lap_pos[sb + u];
                if (ROW64) {
                    const float2* k = k64 + 3 * (size_t)(sb + u);
                    kr[u][0] = k[0];
                    kr[u][1] = k[1];
                    kr[u][2] = k[2];
                }
            }
#pragma unroll
        for (int u = 0; u < kGeoBatch; ++u)
            if (sb + u < s1) {
                const int e = slot[u] / 3;
                if (need_geo) {
                    ga[u] = geo[2 * (size_t)e];
                    gb[u] = geo[2 * (size_t)e + 1];
                }
                if (gcl) tm[u] = terms[e];
            }
#pragma unroll
        for (int u = 0; u < kGeoBatch; ++u) {
            if (sb + u >= s1) break;
            if (gcl) {
                t1 = t1 + tm[u].x;
                t2 = t2 + tm[u].y;
            } else {
                m1.add(gb[u].z);
            }
            if (ROW64) {
                if (in_smem) {
                    df_acc(acc64[pos[u].x], kr[u][0]);
                    df_acc(acc64[pos[u].y], kr[u][1]);
                    df_acc(acc64[pos[u].z], kr[u][2]);
                }
                continue;
            }
            const int i = slot[u] - 3 * (slot[u] / 3);
            const float gx[3] = {ga[u].x, ga[u].y, ga[u].z}, gy[3] = {ga[u].w, gb[u].x, gb[u].y};
            const float q = gb[u].w;
            const float dxi = (i == 0) ? gx[0] : (i == 1 ? gx[1] : gx[2]);
            const float dyi = (i == 0) ? gy[0] : (i == 1 ? gy[1] : gy[2]);
            const unsigned char pj[3] = {pos[u].x, pos[u].y, pos[u].z};
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const float v = (dxi * gx[j] + dyi * gy[j]) * q;
                if (in_smem) acc[pj[j]] += v;
                else valf[r0 + pj[j]] += v;  // long rows (rare)
            }
        }
    }
    float idf;
    if (ROW64) {
        float diag;
        if (in_smem) {
            for (int k = 0; k < len; ++k) {
                valf[r0 + k] = acc64[k].x;
                val_lo[r0 + k] = acc64[k].y;
            }
            diag = acc64[0].x;
        } else {  // long rows (rare): one pass over the slots per entry
            diag = 0.f;
            for (int kk = 0; kk < len; ++kk) {
                float2 one = make_float2(0.f, 0.f);
                for (int sl = s0; sl < s1; ++sl) {
                    const float2* k = k64 + 3 * (size_t)sl;
                    const uchar4 ps = lap_pos[sl];
                    if (ps.x == kk) df_acc(one, k[0]);
                    if (ps.y == kk) df_acc(one, k[1]);
                    if (ps.z == kk) df_acc(one, k[2]);
                }
                valf[r0 + kk] = one.x;
                val_lo[r0 + kk] = one.y;
                if (kk == 0) diag = one.x;
            }
        }
        idf = 1.f / diag;  // the Jacobi scaling is FP32 in every pass
    } else {
        float diag;
        if (in_smem) {
            for (int k = 0; k < len; ++k) valf[r0 + k] = acc[k];
            diag = acc[0];
        } else {
            diag = valf[r0];
        }
        idf = 1.f / diag;
    }
    invdiagf[p] = idf;
    invdiag[p] = f2d_bits(idf);
    double m;
    if (gcl) {
        m = M[p] + (*dtp) * ((t1 + t2) * (1.0 / 3.0)) * 0.5;
        if (Wold) Wold[p] = W[p];  // putW (null: the caller swaps W buffers instead)
    } else {
        m = f2d_bits(m1.value()) * (1.0 / 3.0);
    }
    M[p] = m;
    invM[p] = 1.f / d2f_trunc(m);
    }
}
cudaError_t launch_node_geometry(bool row64, unsigned grid, cudaStream_t stream, int npoin,
                                 const int* esup_ptr, const int* esup_slot,
                                 const uchar4* lap_pos, const float4* geo, const double2* terms,
                                 const double* dtp, int gcl, const int* rowptr, float* valf,
                                 double* invdiag, float* invdiagf, double* M, float* invM,
                                 const float2* W, float2* Wold, const float2* k64,
                                 float* val_lo) {
    if (row64)
        k_node_geometry<true><<<grid, kGeoBlock, 0, stream>>>(
            npoin, esup_ptr, esup_slot, lap_pos, geo, terms, dtp, gcl, rowptr, valf, invdiag,
            invdiagf, M, invM, W, Wold, k64, val_lo);
    else
        k_node_geometry<false><<<grid, kGeoBlock, 0, stream>>>(
            npoin, esup_ptr, esup_slot, lap_pos, geo, terms, dtp, gcl, rowptr, valf, invdiag,
            invdiagf, M, invM, W, Wold, k64, val_lo);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

// The mesh-motion matrix assembled in FP64 (the mixed form under the relative stopping
// tests).  The FP32 assembly above rounds every entry afresh each step; the entries move by
// far more than an ulp per step, so that rounding is new noise in every step's operator,
// and the previous steps' solutions carry it into this step's residual (~1e-7 of it): a
// floor under every guess built from them.  Assembled in FP64 and held as valf + val_lo
// (split_bits, 2^-47), the operator moves as smoothly as the mesh, the first residual (the
// precise product) sees only that, and the FP32 iterations keep valf.  k_node_geometry<true>
// sums the rows.
//
// Per element: the 3x3 element matrix q (grad N_i . grad N_j) of mLaplace.f90:28-56,
// q = (a sum |grad N_i|^2)^2 / 3 with a the area.  With e_i = a2 grad N_i (the edge vectors
// from the first node, rotated; a2 = twice the signed area) the entries are
// (e_i . e_j) S^2 / (12 a2^4), S = sum |e_i|^2.  The edge vectors are FP64 differences of
// the FP64 coordinates (exact for the close nodes of an element); the rest runs in
// double-float (~2^-46, the accuracy of the valf + val_lo pair the rows end up in), so that
// 4 FP64 operations remain per element instead of ~40 and a division.  Row i goes, as
// (h, l) pairs, to the element's slot (e, i) in element-around-point order (slot_pos), so
// that the node pass reads each node's rows contiguously.
__global__ void k_elem_grad64(int nelem, const int4* __restrict__ elem,
                              const double* __restrict__ X, const double* __restrict__ Y,
                              const int* __restrict__ slot_pos, float2* __restrict__ k64) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nelem; e += gridDim.x * blockDim.x) {
        const int4 n = elem[e];
        const double X0 = X[n.x], Y0 = Y[n.x];
        const DF x1 = df_of(X[n.y] - X0), y1 = df_of(Y[n.y] - Y0);
        const DF x2 = df_of(X[n.z] - X0), y2 = df_of(Y[n.z] - Y0);
        const DF ex0 = df_sub(y1, y2), ey0 = df_sub(x2, x1);  // e_0; e_1 = (y2, -x2), e_2 = (-y1, x1)
        const DF d00 = df_add(df_mul(ex0, ex0), df_mul(ey0, ey0));
        const DF d11 = df_add(df_mul(y2, y2), df_mul(x2, x2));
        const DF d22 = df_add(df_mul(y1, y1), df_mul(x1, x1));
        const DF d01 = df_sub(df_mul(ex0, y2), df_mul(ey0, x2));
        const DF d02 = df_sub(df_mul(ey0, x1), df_mul(ex0, y1));
        const DF d12 = df_add(df_mul(y2, y1), df_mul(x2, x1));  // -d12
        const DF S = df_add(df_add(d00, d11), d22);
        const DF a2 = df_sub(df_mul(x1, y2), df_mul(x2, y1));
        const DF t = df_div(S, df_mul(a2, a2));
        const DF c = df_mul(df_mul(t, t), df_of(1.0 / 12.0));
        const DF k00 = df_mul(d00, c), k11 = df_mul(d11, c), k22 = df_mul(d22, c);
        const DF k01 = df_mul(d01, c), k02 = df_mul(d02, c), m12 = df_mul(d12, c);
        const float2 K[3][3] = {{make_float2(k00.h, k00.l), make_float2(k01.h, k01.l), make_float2(k02.h, k02.l)},
                                {make_float2(k01.h, k01.l), make_float2(k11.h, k11.l), make_float2(-m12.h, -m12.l)},
                                {make_float2(k02.h, k02.l), make_float2(-m12.h, -m12.l), make_float2(k22.h, k22.l)}};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            float2* r = k64 + 3 * (size_t)slot_pos[3 * (size_t)e + i];
            r[0] = K[i][0];
            r[1] = K[i][1];
            r[2] = K[i][2];
        }
    }
}

// geo -> the FP64 dNx/dNy (column-major [6][nelem]) and area the download entries read
__global__ void k_widen_geo(int nelem, const float4* __restrict__ geo, double* __restrict__ dN,
                            double* __restrict__ area) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    const size_t E = (size_t)nelem;
    const float4 ga = geo[2 * (size_t)e], gb = geo[2 * (size_t)e + 1];
    dN[e] = ga.x;
    dN[E + e] = ga.y;
    dN[2 * E + e] = ga.z;
    dN[3 * E + e] = ga.w;
    dN[4 * E + e] = gb.x;
    dN[5 * E + e] = gb.y;
    if (area) area[e] = gb.z;
}

// meshMove.f90:99-126: X += XPOS, W = XPOS/DTMIN (as XPOS*(1/DTMIN), the reciprocal formed
// once by k_dt_finalize), with the float shadows of (X, Y) and W
__global__ void k_motion_update_mixed(int npoin, const double* __restrict__ xpos,
                                      const double* __restrict__ ypos, const StepScal* __restrict__ sc,
                                      double* __restrict__ X, double* __restrict__ Y,
                                      double* __restrict__ WX, double* __restrict__ WY,
                                      float2* __restrict__ Xhi, float2* __restrict__ Xlo,
                                      float2* __restrict__ Wf) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npoin; p += gridDim.x * blockDim.x) {
    const double idt = sc->inv_dtmin;
    const double xp = xpos[p], yp = ypos[p];
    const double x = X[p] + xp, y = Y[p] + yp;
    X[p] = x;
    Y[p] = y;
    const double wx = xp * idt, wy = yp * idt;
    WX[p] = wx;
    WY[p] = wy;
    Wf[p] = make_float2(d2f_trunc(wx), d2f_trunc(wy));
    float hx, lx, hy, ly;
    split(x, hx, lx);
    split(y, hy, ly);
    Xhi[p] = make_float2(hx, hy);
    Xlo[p] = make_float2(lx, ly);
    }
}

// ------------------------------------------------------------------ end of the flow part
// TIME = TIME + DTMIN (ns2DComp.ALE.f90:163) and fluidStructure's motion increment
// (meshMove.f90:55-71 for the reference law: pitch pi/8 sin(10 t); the harmonic law: heave
// A_h sin(2 pi f t), pitch A_p sin(2 pi f t)), in the same operations as the FP64 form's
// host code
__device__ MotionScal motion_step(const MotionScal& m, double dt, int law, double heave_amp,
                                  double pitch_amp, double freq) {
    const double PI = 3.141592653589793;  // acos(-1)
    const double t = m.time + dt;
    const double alphav = m.disn1, yposrv = m.disn0;
    double d0 = m.disn0, d1 = m.disn1;
    if (law == CFD_MOTION_NEWMARK) {  // the increment needs this step's forces: later
        MotionScal o = m;
        o.time = t;
        o.dtmin = dt;
        return o;
    }
    if (law == CFD_MOTION_HARMONIC) {
        const double ph = 2.0 * PI * freq * t;
        d0 = heave_amp * sin(ph);
        d1 = pitch_amp * sin(ph);
    } else {
        d1 = (PI / 8.0) * sin(10.0 * t);
    }
    const double alpha = d1 - alphav;
    MotionScal o;
    o.time = t;
    o.disn0 = d0;
    o.disn1 = d1;
    o.ca = cos(alpha);
    o.sa = sin(alpha);
    o.yposr = d0 - yposrv;
    o.dtmin = dt;
    o.veln0 = m.veln0;
    o.veln1 = m.veln1;
    o.accn0 = m.accn0;
    o.accn1 = m.accn1;
    return o;
}

// TRANSF into x_fix and the Dirichlet values of the solves, entries k0, k0 + ks, ...
__device__ __forceinline__ void tail_transf(const MotionTailArgs& a, const MotionScal& mv,
                                            int k0, int ks);

// TRANSF (meshMove.f90:369-392) of moving-list entry k
__device__ __forceinline__ double2 transf_one(const MotionTailArgs& a, const MotionScal& mv,
                                              int k) {
    const int s = a.fix_set[k];
    if (s < 0) return make_double2(0.0, 0.0);
    const int n = a.fix_node[k];
    const double distx = a.X[n] - a.xref[s];
    const double disty = a.Y[n] - a.yref[s] + mv.yposr;
    return make_double2(mv.ca * distx + mv.sa * disty - distx,
                        -(mv.sa * distx) + mv.ca * disty - disty + mv.yposr);
}

// One launch of up to kTailBlocks blocks for FORCES (meshMove.f90:167-192; per-block trees of the
// edge terms, folded by a tree in block order by the last block) and/or the clock and the
// motion law,
// TRANSF into x_fix, and the Dirichlet values of the two BiCG solves (biconjGrad.f90:28:
// x(fix) = x_fix, in x and in its float shadow).  Every block forms the motion from the
// step-start MotionScal; the last block stores the new one.  The Newmark law runs both
// parts in one launch: its motion needs the forces.
__global__ void __launch_bounds__(256) k_motion_tail(MotionTailArgs a) {
    __shared__ MotionScal mv;
    __shared__ double red[9];
    __shared__ bool last;
    if (a.do_motion && threadIdx.x == 0)
        mv = motion_step(*a.m, a.sc->dtmin, a.law, a.heave_amp, a.pitch_amp, a.freq);
    __syncthreads();
    // items interleaved over the blocks (item k in block k % gridDim.x): the FP64 work of a
    // few thousand items spreads over as many SMs as there are blocks
    const int gt = threadIdx.x * gridDim.x + blockIdx.x, gs = gridDim.x * blockDim.x;
    const bool structural = a.law == CFD_MOTION_NEWMARK;
    if (a.do_motion && !structural) tail_transf(a, mv, gt, gs);
    if (a.do_forces)  // normales of the moved mesh, for the next step's wall condition
        for (int k = gt; k < a.nv.nwn; k += gs) normales_node(a.nv, k);
    if (a.do_motion && a.fgeo)  // the edge geometry FORCES will need, before the mesh moves
        for (int k = gt; k < a.set_ptr[a.nset]; k += gs) {
            const int2 ed = a.set_edges[k];
            a.fgeo[k] = make_double4_32a(a.Y[ed.y] - a.Y[ed.x], a.X[ed.x] - a.X[ed.y],
                                     (a.X[ed.x] + a.X[ed.y]) * 0.5, (a.Y[ed.y] + a.Y[ed.x]) * 0.5);
        }
    for (int s = 0; a.do_forces && s < a.nset; ++s) {
        double fx = 0.0, fy = 0.0, rm = 0.0;
        const double xr = a.xref[s], yr = a.yref[s];
        for (int k = a.set_ptr[s] + gt; k < a.set_ptr[s + 1]; k += gs) {
            const int2 ed = a.set_edges[k];
            const double d_press = ((double)a.P[ed.x] + (double)a.P[ed.y]) * 0.5;
            double4_32a g;  // Y(N2)-Y(N1), X(N1)-X(N2), the edge's midpoint
            if (a.fgeo) {
                g = a.fgeo[k];
            } else {
                g = make_double4_32a(a.Y[ed.y] - a.Y[ed.x], a.X[ed.x] - a.X[ed.y],
                                 (a.X[ed.x] + a.X[ed.y]) * 0.5, (a.Y[ed.y] + a.Y[ed.x]) * 0.5);
            }
            const double fa = d_press * g.x;
            const double fb = d_press * g.y;
            fx += fa;
            fy += fb;
            rm += fb * (g.z - xr) - fa * (g.w - yr);
        }
        fx = block_tree256(fx, red);
        fy = block_tree256(fy, red);
        rm = block_tree256(rm, red);
        if (threadIdx.x == 0) {
            a.part[(3 * s + 0) * gridDim.x + blockIdx.x] = fx;
            a.part[(3 * s + 1) * gridDim.x + blockIdx.x] = fy;
            a.part[(3 * s + 2) * gridDim.x + blockIdx.x] = rm;
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(a.count, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (a.do_forces)  // the blocks' partials of each sum, folded by a tree in block order
        for (int j = 0; j < 3 * a.nset; ++j) {
            double v = (threadIdx.x < gridDim.x) ? __ldcg(a.part + j * gridDim.x + threadIdx.x) : 0.0;
            v = block_tree256(v, red);
            if (threadIdx.x == 0) {
                const int s = j / 3, q = j % 3;
                (q == 0 ? a.sc->fx : q == 1 ? a.sc->fy : a.sc->rm)[s] = v;
            }
        }
    if (a.do_motion && structural) {  // the Newmark step under set 1's load, then TRANSF
        __syncthreads();
        if (threadIdx.x == 0) {
            NewmarkState ns;
            ns.dis[0] = mv.disn0;
            ns.dis[1] = mv.disn1;
            ns.vel[0] = mv.veln0;
            ns.vel[1] = mv.veln1;
            ns.acc[0] = mv.accn0;
            ns.acc[1] = mv.accn1;
            double F[2];
            newmark_load(ns, a.sc->fx[0], a.sc->fy[0], a.sc->rm[0], F);
            newmark_step(ns, F, mv.dtmin);
            const double alpha = ns.dis[1] - mv.disn1;
            mv.yposr = ns.dis[0] - mv.disn0;
            mv.ca = cos(alpha);
            mv.sa = sin(alpha);
            mv.disn0 = ns.dis[0];
            mv.disn1 = ns.dis[1];
            mv.veln0 = ns.vel[0];
            mv.veln1 = ns.vel[1];
            mv.accn0 = ns.acc[0];
            mv.accn1 = ns.acc[1];
        }
        __syncthreads();
        tail_transf(a, mv, threadIdx.x, blockDim.x);
    }
    if (threadIdx.x == 0) {
        if (a.do_motion) *a.m = mv;
        *a.count = 0u;
    }
}

__device__ __forceinline__ void tail_transf(const MotionTailArgs& a, const MotionScal& mv,
                                            int k0, int ks) {
    for (int k = k0; k < a.nnmove; k += ks) {
        const double2 d = transf_one(a, mv, k);
        a.xfix_x[k] = d.x;
        a.xfix_y[k] = d.y;
    }
    for (int k = k0; k < a.nufix; k += ks) {
        const int i = a.ufix_node[k];
        const double2 d = transf_one(a, mv, a.ufix_src[k]);
        a.x0[i] = d.x;
        a.xf0[i] = d2f_trunc(d.x);
        a.x1[i] = d.y;
        a.xf1[i] = d2f_trunc(d.y);
    }
}

// ------------------------------------------------------------------ host launchers
cudaError_t launch_elem_stage1_mixed(bool viscous, cudaStream_t st, int nelem, const int4* elem,
                                     const float4* Uhi, const float4* Ulo, const float4* geo,
                                     const float* VX, const float* VY, EstabConst ec,
                                     const StepScal* sc, GasConstF gc, const float2* W,
                                     const int* slot_pos, const float* T, float4* recInv,
                                     float4* recVisc, float2* mulam, const float* dte) {
    const unsigned grid = blocks_for(nelem, 128);
    if (viscous)
        k_elem_stage1_mixed<true><<<grid, 128, 0, st>>>(nelem, elem, Uhi, Ulo, geo, VX, VY, ec, sc,
                                                         gc, W, slot_pos, T, recInv, recVisc,
                                                         mulam, dte);
    else
        k_elem_stage1_mixed<false><<<grid, 128, 0, st>>>(nelem, elem, Uhi, Ulo, geo, VX, VY, ec,
                                                          sc, gc, W, slot_pos, T, recInv,
                                                          recVisc, mulam, dte);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ node pass, bulk-copy variant
// The viscous stages 2-4 with the block's slot records staged by the bulk-copy engine: a
// block's 128 nodes own one contiguous range of slots (element-around-point order), so one
// thread issues two cp.async.bulk copies (the recVisc records and the slot ids) into shared
// memory, completing on an mbarrier, while every thread loads its node's own data; the
// threads then gather the slots' mu, lambda (all of a node's gathers in flight at once) and
// sum from shared memory in slot order.  The wait is bounded (kSpinLimit polls, kWaitNs of
// the global timer): past either the block sets *err and leaves.
__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

template <bool LAST>
__global__ void __launch_bounds__(kNodeTB)
k_node_mixed_bulk(int npoin, const int* __restrict__ esup_ptr, const int* __restrict__ esup_slot,
                  const float2* __restrict__ mulam, const float4* __restrict__ recVisc,
                  float4* __restrict__ invSum, GasConst gc, GasConstF gf, const double* U,
                  float4* __restrict__ Uhi, float4* __restrict__ Ulo, const float* __restrict__ invM,
                  float rk_fact, const unsigned char* __restrict__ bcflag,
                  const double* __restrict__ bcval, const double2* __restrict__ nrm,
                  const double* __restrict__ WX, const double* __restrict__ WY, double* U1,
                  float* __restrict__ RHO, float* __restrict__ VX, float* __restrict__ VY,
                  float* __restrict__ Eo, float* __restrict__ Po, float* __restrict__ Tout,
                  float* __restrict__ RMACH, int* __restrict__ err) {
    extern __shared__ __align__(128) unsigned char stage_raw[];
    __shared__ __align__(8) unsigned long long bar;
    const int p0 = blockIdx.x * kNodeTB;
    const int p1 = min(p0 + kNodeTB, npoin);
    const int S0 = esup_ptr[p0], S1 = esup_ptr[p1];
    const int S0a = S0 & ~3, S1a = (S1 + 3) & ~3;  // 16-byte aligned range of slot ids
    const unsigned bytesV = 16u * (unsigned)(S1 - S0), bytesE = 4u * (unsigned)(S1a - S0a);
    const float4* sv = reinterpret_cast<const float4*>(stage_raw);
    const int* se = reinterpret_cast<const int*>(stage_raw + bytesV);
    const unsigned ubar = smem_u32(&bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ubar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ubar),
                     "r"(bytesV + bytesE)
                     : "memory");
        if (bytesV)
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                    "r"(smem_u32(stage_raw)), "l"(recVisc + S0), "r"(bytesV), "r"(ubar)
                : "memory");
        if (bytesE)
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                    "r"(smem_u32(stage_raw + bytesV)), "l"(esup_slot + S0a), "r"(bytesE), "r"(ubar)
                : "memory");
    }
    const int p = p0 + threadIdx.x;
    const bool live = p < npoin;
    const int s0 = live ? esup_ptr[p] : 0, s1 = live ? esup_ptr[p + 1] : 0;
    NodePre pre{};
    if (live) pre = node_pre<false>(p, invSum, invM, bcflag, Uhi);
    // bounded wait for the copies (phase 0)
    if (!mbar_wait_bounded(ubar, 0u)) {
        if (threadIdx.x == 0) atomicExch(err, (int)CFD_ERR_BARRIER);
        return;
    }
    if (!live) return;
    Acc v1, v2, v3;
    v1.init();
    v2.init();
    v3.init();
    for (int s = s0; s < s1; s += 8) {
        float2 ml[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (s + j < s1) ml[j] = mulam[se[s + j - S0a] / 3];
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (s + j < s1) {
                const float4 rv = sv[s + j - S0];
                v1.add(ml[j].x * rv.x);
                v2.add(ml[j].x * rv.y);
                v3.add(ml[j].x * rv.z + ml[j].y * rv.w);
            }
    }
    node_finish<false, LAST>(p, pre, make_float4(0.f, 0.f, 0.f, 0.f), v1.value(), v2.value(), v3.value(),
                             invSum, gc, gf, U, Uhi, Ulo, invM, rk_fact, bcflag, bcval, nrm, WX,
                             WY, U1, RHO, VX, VY, Eo, Po, Tout, RMACH);
}

cudaError_t launch_node_mixed(cudaStream_t st, int npoin, const int* esup_ptr, const int* esup_slot,
                              const float2* mulam, const float4* recInv, const float4* recVisc,
                              float4* invSum, int first_stage, GasConst gc, GasConstF gf,
                              int viscous, const double* U, float4* Uhi, float4* Ulo,
                              const float* invM, float rk_fact, int last_stage,
                              const unsigned char* bcflag, const double* bcval, const double2* nrm,
                              const double* WX, const double* WY, double* U1, float* RHO,
                              float* VX, float* VY, float* E, float* P, float* Tout, float* RMACH,
                              int bulk_smem, int* bulk_err) {
    const unsigned grid = blocks_for(npoin, kNodeTB);
    if (bulk_smem > 0 && viscous && !first_stage) {  // the bulk-copy variant
        if (last_stage)
            k_node_mixed_bulk<true><<<grid, kNodeTB, bulk_smem, st>>>(
                npoin, esup_ptr, esup_slot, mulam, recVisc, invSum, gc, gf, U, Uhi, Ulo, invM,
                rk_fact, bcflag, bcval, nrm, WX, WY, U1, RHO, VX, VY, E, P, Tout, RMACH, bulk_err);
        else
            k_node_mixed_bulk<false><<<grid, kNodeTB, bulk_smem, st>>>(
                npoin, esup_ptr, esup_slot, mulam, recVisc, invSum, gc, gf, U, Uhi, Ulo, invM,
                rk_fact, bcflag, bcval, nrm, WX, WY, U1, RHO, VX, VY, E, P, Tout, RMACH, bulk_err);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        return cudaGetLastError();
    }
#define CFD_NODE_ARGS                                                                          \
    npoin, esup_ptr, esup_slot, mulam, recInv, recVisc, invSum, gc, gf, viscous, U, Uhi, Ulo, invM, \
        rk_fact, bcflag, bcval, nrm, WX, WY, U1, RHO, VX, VY, E, P, Tout, RMACH
    if (first_stage)
        k_node_mixed<true, false><<<grid, kNodeTB, 0, st>>>(CFD_NODE_ARGS);
    else if (last_stage)
        k_node_mixed<false, true><<<grid, kNodeTB, 0, st>>>(CFD_NODE_ARGS);
    else
        k_node_mixed<false, false><<<grid, kNodeTB, 0, st>>>(CFD_NODE_ARGS);
#undef CFD_NODE_ARGS
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}


// Shared memory the bulk-copy node pass needs for the largest block of this mesh (0: more
// than the variant takes), with the kernel attributes set for it
int node_bulk_smem(const int* esup_ptr, int npoin) {
    long worst = 0;
    for (int p0 = 0; p0 < npoin; p0 += kNodeTB) {
        const int S0 = esup_ptr[p0], S1 = esup_ptr[std::min(p0 + kNodeTB, npoin)];
        const long b = 16L * (S1 - S0) + 4L * (((S1 + 3) & ~3) - (S0 & ~3));
        worst = std::max(worst, b);
    }
    if (worst > 200 * 1024) return 0;
    const int smem = (int)std::max(worst, 16L);
    if (cudaFuncSetAttribute(k_node_mixed_bulk<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess ||
        cudaFuncSetAttribute(k_node_mixed_bulk<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    return smem;
}

}  // namespace cfd

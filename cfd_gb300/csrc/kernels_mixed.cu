// kernels_mixed.cu — the mixed-precision form of the step (CFD_PREC_MIXED), sm_103a.
//
// FP32 for calcRHS, FUENTE, ESTAB, deltat and the Laplacian values; FP64 for the
// conserved-state update U1 = U - rk_fact/M*RHS, the areas and the gcl mass update, and
// (in the BiCG kernel) the vectors, dots and scalars.  Per-node sums of the FP32
// contributions are compensated (Neumaier), then widened to FP64.
//
// Stage invariance (the reference calls calcRHS/FUENTE with the step-start U in all four
// RK stages, subrutinas.f90:685, :1064; only the module T changes, through mu and lambda
// at calcRHS.f90:49-51): stage 1 evaluates every element once and stores, per (element,
// local node) slot, the stage-invariant part Inv(0:3) (Galerkin, SUPG, shock capturing,
// FUENTE) and the coefficients of the viscous part, which is linear in (mu, lambda):
// Vmu(1:3), Vlam(3).  Slots are stored in element-around-point order, so each RK stage
// is one node kernel that streams its node's slots, forms Inv + mu*Vmu + lambda*Vlam with
// the stage's mu and lambda, and applies the update and boundary conditions.
#include "cfd_kernels.cuh"

namespace cfd {

__device__ __forceinline__ float pow15f(float x) { return x * sqrtf(x); }

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
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// ------------------------------------------------------------------ deltat (FP32)
__global__ void k_deltat_mixed(int nelem, const int4* __restrict__ elem, const double* __restrict__ T,
                               const double* __restrict__ VX, const double* __restrict__ VY,
                               const double* __restrict__ WX, const double* __restrict__ WY,
                               const double* __restrict__ area, float fsafe, float t_inf,
                               unsigned long long* __restrict__ dtmin_bits) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long mybits = 0x7ff0000000000000ull;
    if (e < nelem) {
        int4 n = elem[e];
        const int nn[3] = {n.x, n.y, n.z};
        float vumax = 0.f, vvmax = 0.f;
        float T_iel = (float)((T[nn[0]] + T[nn[1]] + T[nn[2]]) * (1.0 / 3.0));
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            vumax = fmaxf(vumax, fabsf((float)(VX[nn[i]] - WX[nn[i]])));
            vvmax = fmaxf(vvmax, fabsf((float)(VY[nn[i]] - WY[nn[i]])));
        }
        float hh = sqrtf(2.f * (float)area[e]);
        float vel = sqrtf(vumax * vumax + vvmax * vvmax);
        float et = 0.017f * pow15f(T_iel / t_inf) * (t_inf + 110.f) / (T_iel + 110.f);
        float pe = (vel * hh) / (2.f * et);
        float alpha = fminf(pe / 3.f, 1.f);
        float a = 4.f * et / (hh * hh);
        // FSAFE/(1/DELTATC + 1/DELTATU) with 1/DELTATC = a, 1/DELTATU = a + alpha*vel/hh
        float dtelem = fsafe / (a + (a + alpha * vel / hh));
        double d = (double)dtelem;
        if (d < 1.0e20 && d > 0.0) mybits = (unsigned long long)__double_as_longlong(d);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        unsigned long long o = __shfl_down_sync(0xffffffffu, mybits, off);
        mybits = o < mybits ? o : mybits;
    }
    __shared__ unsigned long long wmin[32];
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = mybits;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = wmin[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = wmin[w] < m ? wmin[w] : m;
        atomicMin(dtmin_bits, m);
    }
}

// DTELEM in FP64 (subrutinas.f90:172-206), for the candidates of the FP32 minimum
__device__ double dtelem_fp64(int4 n, const double* __restrict__ T, const double* __restrict__ VX,
                              const double* __restrict__ VY, const double* __restrict__ WX,
                              const double* __restrict__ WY, double area, double fsafe,
                              double t_inf) {
    const int nn[3] = {n.x, n.y, n.z};
    double vumax = 0.0, vvmax = 0.0;
    const double T_iel = (T[nn[0]] + T[nn[1]] + T[nn[2]]) / 3.0;
    for (int i = 0; i < 3; ++i) {
        const double vu = fabs(VX[nn[i]] - WX[nn[i]]), vv = fabs(VY[nn[i]] - WY[nn[i]]);
        if (vu > vumax) vumax = vu;
        if (vv > vvmax) vvmax = vv;
    }
    const double hh = sqrt(2.0 * area);
    const double vel = sqrt(vumax * vumax + vvmax * vvmax);
    const double et = 0.017 * (T_iel / t_inf) * sqrt(T_iel / t_inf) * (t_inf + 110.0) / (T_iel + 110.0);
    const double pe = (vel * hh) / (2.0 * et);
    const double alpha = fmin(pe / 3.0, 1.0);
    const double deltatu = 1.0 / (4.0 * et / (hh * hh) + alpha * vel / hh);
    const double deltatc = 1.0 / (4.0 * et / (hh * hh));
    return fsafe / (1.0 / deltatc + 1.0 / deltatu);
}

// Second pass of the mixed deltat: elements whose FP32 DTELEM is within 1e-4 of the FP32
// minimum get their FP64 DTELEM; the FP64 minimum over them is DTMIN, so the 1%
// hysteresis of ns2DComp.ALE.f90:146-156 sees an FP64-accurate value.
__global__ void k_deltat_refine(int nelem, const int4* __restrict__ elem, const double* __restrict__ T,
                                const double* __restrict__ VX, const double* __restrict__ VY,
                                const double* __restrict__ WX, const double* __restrict__ WY,
                                const double* __restrict__ area, float fsafe, float t_inf,
                                StepScal* __restrict__ sc) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    const double m32 = __longlong_as_double((long long)sc->dtmin32_bits);
    const int4 n = elem[e];
    const int nn[3] = {n.x, n.y, n.z};
    float vumax = 0.f, vvmax = 0.f;
    const float T_iel = (float)((T[nn[0]] + T[nn[1]] + T[nn[2]]) * (1.0 / 3.0));
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        vumax = fmaxf(vumax, fabsf((float)(VX[nn[i]] - WX[nn[i]])));
        vvmax = fmaxf(vvmax, fabsf((float)(VY[nn[i]] - WY[nn[i]])));
    }
    const float hh = sqrtf(2.f * (float)area[e]);
    const float vel = sqrtf(vumax * vumax + vvmax * vvmax);
    const float et = 0.017f * pow15f(T_iel / t_inf) * (t_inf + 110.f) / (T_iel + 110.f);
    const float alpha = fminf((vel * hh) / (2.f * et) / 3.f, 1.f);
    const float a = 4.f * et / (hh * hh);
    const float d32 = fsafe / (a + (a + alpha * vel / hh));
    if ((double)d32 <= m32 * (1.0 + 1.0e-4)) {
        const double d = dtelem_fp64(n, T, VX, VY, WX, WY, area[e], (double)fsafe, (double)t_inf);
        if (d > 0.0 && d < 1.0e20) atomicMin(&sc->dtmin_bits, (unsigned long long)__double_as_longlong(d));
    }
}

// ------------------------------------------------------------------ ESTAB (FP32)
// subrutinas.f90:346-443 in FP32; estab_mode as CFD_ESTAB_*.
__global__ void k_estab_mixed(int nelem, const int4* __restrict__ elem, const double* __restrict__ U,
                              const double* __restrict__ T, float gm, const double* __restrict__ VX,
                              const double* __restrict__ VY, const double* __restrict__ WX,
                              const double* __restrict__ WY, const double* __restrict__ geo,
                              float FR, const StepScal* __restrict__ sc, float RHOINF, float TINF,
                              int estab_mode, float eps_dir, float dirx, float diry,
                              float* __restrict__ SHOC,
                              float* __restrict__ TS1, float* __restrict__ TS2,
                              float* __restrict__ TS3) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    const size_t E = (size_t)nelem;
    const float DTMIN = (float)sc->dtmin;
    int4 n = elem[e];
    const int n1 = n.x, n2 = n.y, n3 = n.z;
    const float DX[3] = {(float)geo[e], (float)geo[E + e], (float)geo[2 * E + e]};
    const float DY[3] = {(float)geo[3 * E + e], (float)geo[4 * E + e], (float)geo[5 * E + e]};
    const double r1 = U[4 * (size_t)n1], r2 = U[4 * (size_t)n2], r3 = U[4 * (size_t)n3];
    const float rho_elem = (float)((r1 + r2 + r3) * (1.0 / 3.0));
    float vx = (float)(((VX[n1] + VX[n2] + VX[n3]) - (WX[n1] + WX[n2] + WX[n3])) * (1.0 / 3.0));
    float vy = (float)(((VY[n1] + VY[n2] + VY[n3]) - (WY[n1] + WY[n2] + WY[n3])) * (1.0 / 3.0));
    float vel2 = sqrtf(vx * vx + vy * vy);
    // gradients from differences to node 1 (sum of the shape-function gradients is 0)
    const float d2 = (float)(r2 - r1), d3 = (float)(r3 - r1);
    float drx = d2 * DX[1] + d3 * DX[2], dry = d2 * DY[1] + d3 * DY[2];
    const double t1 = T[n1], t2 = T[n2], t3 = T[n3];
    const float e2 = (float)(t2 - t1), e3 = (float)(t3 - t1);
    float dtx = e2 * DX[1] + e3 * DX[2], dty = e2 * DY[1] + e3 * DY[2];
    const float temp = (float)((t1 + t2 + t3) * (1.0 / 3.0));
    float dr2 = sqrtf(drx * drx + dry * dry) + 1.0e-20f;
    float dt2 = sqrtf(dtx * dtx + dty * dty) + 1.0e-20f;
    float dux = 0.f, duy = 0.f;
    if (estab_mode == CFD_ESTAB_REFERENCE) {
        dux = vel2 * DX[0] + vel2 * DX[1] + vel2 * DX[2];
        duy = vel2 * DY[0] + vel2 * DY[1] + vel2 * DY[2];
    }
    float du2 = sqrtf(dux * dux + duy * duy) + 1.0e-20f;
    float rtx = dtx / dt2, rty = dty / dt2;
    float rjx = drx / dr2, rjy = dry / dr2;
    float rux = dux / du2, ruy = duy / du2;
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
    const float fmu = 0.017f * pow15f(temp / TINF) * (TINF + 110.f) / (temp + 110.f);
    float tau = 0.f, h_rgne = 0.f, h_rgn = 0.f, h_jgn = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float term1 = fabsf(vx * DX[i] + vy * DY[i]);
        float term2 = fabsf(rjx * DX[i] + rjy * DY[i]);
        tau += term1 + term2 * c;
        h_rgne += fabsf(rtx * DX[i] + rty * DY[i]);
        h_rgn += fabsf(rux * DX[i] + ruy * DY[i]);
        h_jgn += term2;
    }
    tau = 1.f / tau;
    h_rgne = 2.f / h_rgne;
    h_rgn = 2.f / h_rgn;
    if (!(h_rgn <= 10.f)) h_rgn = 0.f;  // > 10 (and inf from 2/0) -> 0
    h_jgn = 2.f / h_jgn;
    if (!(h_jgn <= 10.f)) h_jgn = 0.f;
    const float tr1 = dr2 * h_jgn / rho_elem;
    const float zzz = h_jgn / (2.f * c);
    SHOC[e] = (tr1 + tr1 * tr1) * 0.5f * (c * c) * zzz;
    const float resumen = 1.f / (tau * tau) + (2.f / DTMIN) * (2.f / DTMIN);
    const float rrr = rsqrtf(resumen);
    float s2 = rrr, s3 = rrr;
    const float k4 = 4.f * fmu / RHOINF;
    // (resumen + 1/tau_s^2)^(-1/2) with tau_s = h^2/k4  ==  (resumen + k4^2/h^4)^(-1/2); h = 0 -> 0
    const float hr2 = h_rgn * h_rgn, he2 = h_rgne * h_rgne;
    s2 = (hr2 > 0.f) ? rsqrtf(resumen + (k4 * k4) / (hr2 * hr2)) : 0.f;
    s3 = (he2 > 0.f) ? rsqrtf(resumen + (k4 * k4) / (he2 * he2)) : 0.f;
    TS1[e] = rrr;
    TS2[e] = s2;
    TS3[e] = s3;
}

// ------------------------------------------------------------------ stage-1 element kernel
// calcRHS.f90:36-141 + FUENTE (subrutinas.f90:1060-1078) in FP32, folded with the
// step's area*dtl/3, written as slot records in element-around-point order.
struct __align__(16) SlotRec {
    float4 inv;   // stage-invariant contributions to the 4 equations
    float4 visc;  // Vmu(1), Vmu(2), Vmu(3), Vlam(3)
};

template <bool VISCOUS>
__global__ void __launch_bounds__(128)
k_elem_stage1_mixed(int nelem, const int4* __restrict__ elem, const double* __restrict__ U,
                    const double* __restrict__ geo, const double* __restrict__ area,
                    const float* __restrict__ shoc, const double* __restrict__ dtl_arr,
                    const double* __restrict__ dtl_scalar, const float* __restrict__ ts1,
                    const float* __restrict__ ts2, const float* __restrict__ ts3, GasConst gc,
                    const double* __restrict__ WX, const double* __restrict__ WY,
                    const int* __restrict__ slot_pos, SlotRec* __restrict__ rec) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    const size_t E = (size_t)nelem;
    const float g = (float)gc.gamma, Cv = (float)gc.cv;
    int4 n = elem[e];
    const int p[3] = {n.x, n.y, n.z};
    const float Nx[3] = {(float)geo[e], (float)geo[E + e], (float)geo[2 * E + e]};
    const float Ny[3] = {(float)geo[3 * E + e], (float)geo[4 * E + e], (float)geo[5 * E + e]};
    double Ud[3][4];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double2* u2 = reinterpret_cast<const double2*>(U + 4 * (size_t)p[i]);
        double2 a = u2[0], b = u2[1];
        Ud[i][0] = a.x; Ud[i][1] = a.y; Ud[i][2] = b.x; Ud[i][3] = b.y;
    }
    float Ux[4], Uy[4], Un[3][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float d1 = (float)(Ud[1][q] - Ud[0][q]), d2 = (float)(Ud[2][q] - Ud[0][q]);
        Ux[q] = d1 * Nx[1] + d2 * Nx[2];
        Uy[q] = d1 * Ny[1] + d2 * Ny[2];
#pragma unroll
        for (int i = 0; i < 3; ++i) Un[i][q] = (float)Ud[i][q];
    }
    const float tau[3] = {ts1[e], ts2[e], ts3[e]};
    const float nu = shoc[e] * (float)gc.cte;
    const double dtl = dtl_arr ? dtl_arr[e] : *dtl_scalar;
    const float scale = (float)(area[e] * dtl / 3.0);
    float r[3][4], vm[3][3], vl[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        vl[i] = 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) r[i][q] = 0.f;
#pragma unroll
        for (int q = 0; q < 3; ++q) vm[i][q] = 0.f;
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
        const float irho = 1.f / rho;
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
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float t = tau[i] * (Nx[i] * B1[q] + Ny[i] * B2[q]) + nu * (Nx[i] * Ux[q] + Ny[i] * Uy[q]);
                if (i != k) t += 0.5f * A[q];
                r[i][q] += t;
            }
        if (VISCOUS) {
            // K1, K2 of calcRHS.f90:121-132 split as mu*(...) + lambda*(...)
            const float icv = 1.f / (Cv * rho);
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
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                vm[i][0] += Nx[i] * m11 + Ny[i] * m12;
                vm[i][1] += Nx[i] * m12 + Ny[i] * m22;
                vm[i][2] += Nx[i] * m13 + Ny[i] * m23;
                vl[i] += Nx[i] * l13 + Ny[i] * l23;
            }
        }
    }
    // FUENTE: -AR*sum_k sp(i,k)*(Ux*wx_k + Uy*wy_k), AR = area*dtl/3 = scale
    {
        const float w0 = (float)WX[p[0]], w1 = (float)WX[p[1]], w2 = (float)WX[p[2]];
        const float y0 = (float)WY[p[0]], y1 = (float)WY[p[1]], y2 = (float)WY[p[2]];
        const float wx[3] = {0.5f * (w0 + w1), 0.5f * (w1 + w2), 0.5f * (w0 + w2)};
        const float wy[3] = {0.5f * (y0 + y1), 0.5f * (y1 + y2), 0.5f * (y0 + y2)};
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
        SlotRec o;
        o.inv = make_float4(r[i][0] * scale, r[i][1] * scale, r[i][2] * scale, r[i][3] * scale);
        o.visc = make_float4(vm[i][0] * scale, vm[i][1] * scale, vm[i][2] * scale, vl[i] * scale);
        rec[slot_pos[3 * (size_t)e + i]] = o;
    }
}

// ------------------------------------------------------------------ RK stage, node side
// subrutinas.f90:680-825 for one stage with the slot records: the node's RHS is the
// compensated sum over its slots of Inv + mu_e*Vmu + lambda_e*Vlam (mu, lambda from the
// stage's element temperature, calcRHS.f90:49-51); U1 = U - rk_fact/M*RHS in FP64.
// Nodes without a boundary condition keep U1 as updated and get their primitives in
// FP32; boundary nodes follow the reference's FP64 primitive round trip and BC order.
__global__ void __launch_bounds__(256)
k_node_mixed(int npoin, const int* __restrict__ esup_ptr, const int* __restrict__ esup_slot,
             const int4* __restrict__ elem, const SlotRec* __restrict__ rec,
             const double* __restrict__ Tst, GasConst gc, int viscous,
             const double* __restrict__ U, const double* __restrict__ invM, double rk_fact,
             const unsigned char* __restrict__ bcflag, const double* __restrict__ bcval,
             const double2* __restrict__ nrm, const double* __restrict__ WX,
             const double* __restrict__ WY, double* __restrict__ U1, double* __restrict__ RHO,
             double* __restrict__ VX, double* __restrict__ VY, double* __restrict__ Eo,
             double* __restrict__ Po, double* __restrict__ To, double* __restrict__ RMACH) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoin) return;
    const float t_inf = (float)gc.t_inf, mu_ref = (float)gc.mu_ref, lam_ref = (float)gc.lambda_ref;
    Acc a0, a1, a2, a3;
    a0.init(); a1.init(); a2.init(); a3.init();
    const int s0 = esup_ptr[p], s1 = esup_ptr[p + 1];
    for (int s = s0; s < s1; ++s) {
        const SlotRec rc = rec[s];
        float c1 = rc.inv.y, c2 = rc.inv.z, c3 = rc.inv.w;
        if (viscous) {
            const int4 n = elem[esup_slot[s] / 3];
            const float Ta = (float)((Tst[n.x] + Tst[n.y] + Tst[n.z]) * (1.0 / 3.0));
            const float r15 = pow15f(Ta / t_inf);
            const float mu = mu_ref * r15 * (t_inf + 110.f) / (Ta + 110.f);
            const float lam = lam_ref * r15 * (t_inf + 194.f) / (Ta + 194.f);
            c1 += mu * rc.visc.x;
            c2 += mu * rc.visc.y;
            c3 += mu * rc.visc.z + lam * rc.visc.w;
        }
        a0.add(rc.inv.x);
        a1.add(c1);
        a2.add(c2);
        a3.add(c3);
    }
    const double r0 = a0.value(), r1 = a1.value(), r2 = a2.value(), r3 = a3.value();
    const double2* u2 = reinterpret_cast<const double2*>(U + 4 * (size_t)p);
    const double2 ua = u2[0], ub = u2[1];
    const double f = rk_fact * invM[p];
    double u1_0 = ua.x - f * r0, u1_1 = ua.y - f * r1, u1_2 = ub.x - f * r2, u1_3 = ub.y - f * r3;
    const float g = (float)gc.gamma;
    const double FR = gc.fr;
    const unsigned char fl = bcflag[p];
    if (!fl) {
        const float rho = (float)u1_0, ir = 1.f / rho;
        const float vx = (float)u1_1 * ir, vy = (float)u1_2 * ir, ee = (float)u1_3 * ir;
        const float vel2 = vx * vx + vy * vy;
        const float pp = rho * (g - 1.f) * (ee - 0.5f * vel2);
        const float tt = pp / (rho * (float)FR);
        RHO[p] = u1_0; VX[p] = vx; VY[p] = vy; Eo[p] = ee; Po[p] = pp; To[p] = tt;
        RMACH[p] = sqrtf(vel2 / (tt * g * (float)FR));
    } else {
        const double gd = gc.gamma;
        double rho = u1_0;
        double vx = u1_1 / rho, vy = u1_2 / rho, ee = u1_3 / rho;
        const double vel2 = vx * vx + vy * vy;
        const double pp = rho * (gd - 1.0) * (ee - 0.5 * vel2);
        double tt = pp / (rho * FR);
        RMACH[p] = sqrt(vel2 / (tt * gd * FR));
        Po[p] = pp;
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
        RHO[p] = rho; VX[p] = vx; VY[p] = vy; Eo[p] = ee; To[p] = tt;
        u1_0 = rho; u1_1 = vx * rho; u1_2 = vy * rho; u1_3 = ee * rho;
    }
    double2* o = reinterpret_cast<double2*>(U1 + 4 * (size_t)p);
    o[0] = make_double2(u1_0, u1_1);
    o[1] = make_double2(u1_2, u1_3);
}

// ------------------------------------------------------------------ geometry (mixed)
// deriv (subrutinas.f90:99-115): area in FP64, gradients through one reciprocal.
__global__ void k_deriv_mixed(int nelem, const int4* __restrict__ elem, const double* __restrict__ X,
                              const double* __restrict__ Y, double* __restrict__ area,
                              double* __restrict__ geo) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    int4 n = elem[e];
    const double x0 = X[n.x], x1 = X[n.y], x2 = X[n.z];
    const double y0 = Y[n.x], y1 = Y[n.y], y2 = Y[n.z];
    // 2a = (x1-x0)(y2-y0) - (x2-x0)(y1-y0): the same signed area from differences
    const double a2 = (x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0);
    area[e] = 0.5 * a2;
    const double ia = 1.0 / a2;
    const size_t E = (size_t)nelem;
    geo[e] = (y1 - y2) * ia;
    geo[E + e] = (y2 - y0) * ia;
    geo[2 * E + e] = (y0 - y1) * ia;
    geo[3 * E + e] = (x2 - x1) * ia;
    geo[4 * E + e] = (x0 - x2) * ia;
    geo[5 * E + e] = (x1 - x0) * ia;
}

// gcl main (gcl.f90:29-45) as two passes: per element divW*area/3 and divW_old*area_old/3
// (FP64), then the node gather and M += dt*(tot1+tot2)/2; also 1/M for the RK update.
__global__ void k_gcl_elem(int nelem, const int4* __restrict__ elem, const double* __restrict__ geo,
                           const double* __restrict__ area, const double* __restrict__ area_old,
                           const double* __restrict__ Wx, const double* __restrict__ Wy,
                           const double* __restrict__ Wxo, const double* __restrict__ Wyo,
                           int literal, double2* __restrict__ terms) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    const size_t E = (size_t)nelem;
    int4 n = elem[e];
    const int nn[3] = {n.x, n.y, n.z};
    double divW = 0.0, divWo = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double dx = geo[i * E + e], dy = geo[(3 + i) * E + e];
        const double wy = literal ? Wx[nn[i]] : Wy[nn[i]];
        const double wyo = literal ? Wxo[nn[i]] : Wyo[nn[i]];
        divW += dx * Wx[nn[i]] + dy * wy;
        divWo += dx * Wxo[nn[i]] + dy * wyo;
    }
    terms[e] = make_double2(divW * area[e] * (1.0 / 3.0), divWo * area_old[e] * (1.0 / 3.0));
}

__global__ void k_mass_mixed(int npoin, const int* __restrict__ esup_ptr,
                             const int* __restrict__ esup_slot, const double* __restrict__ area,
                             const double2* __restrict__ terms, const double* __restrict__ dtp,
                             int gcl, double* __restrict__ M, double* __restrict__ invM) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoin) return;
    double m;
    if (gcl) {
        double t1 = 0.0, t2 = 0.0;
        for (int s = esup_ptr[p]; s < esup_ptr[p + 1]; ++s) {
            const double2 t = terms[esup_slot[s] / 3];
            t1 += t.x;
            t2 += t.y;
        }
        m = M[p] + (*dtp) * (t1 + t2) * 0.5;
    } else {
        double acc = 0.0;
        for (int s = esup_ptr[p]; s < esup_ptr[p + 1]; ++s) acc += area[esup_slot[s] / 3];
        m = acc * (1.0 / 3.0);
    }
    M[p] = m;
    invM[p] = 1.0 / m;
}

// mLaplace.f90:28-56 in arithmetic R (float by default), row owner, element-around-point
// order; writes the values as float (valf) and double (vals)
template <typename R>
__global__ void k_laplace_mixed_t(int npoin, int nelem, const int4* __restrict__ elem,
                                  const int* __restrict__ esup_ptr, const int* __restrict__ esup_slot,
                                  const uchar4* __restrict__ lap_pos, const double* __restrict__ geo,
                                  const double* __restrict__ X, const double* __restrict__ Y,
                                  const int* __restrict__ rowptr, float* __restrict__ valf,
                                  double* __restrict__ vals, double* __restrict__ diag,
                                  double* __restrict__ invdiag) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoin) return;
    const size_t E = (size_t)nelem;
    const int r0 = rowptr[p], r1 = rowptr[p + 1];
    R acc[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[k] = R(0);
    const int len = r1 - r0;
    if (len > 16)
        for (int k = r0; k < r1; ++k) vals[k] = 0.0;
    for (int s = esup_ptr[p]; s < esup_ptr[p + 1]; ++s) {
        const int slot = esup_slot[s];
        const int e = slot / 3, i = slot - 3 * e;
        const int4 n = elem[e];
        const double xa = X[n.x], ya = Y[n.x];
        const R x1 = (R)(X[n.y] - xa), y1 = (R)(Y[n.y] - ya);
        const R x2 = (R)(X[n.z] - xa), y2 = (R)(Y[n.z] - ya);
        // mu = 2*sqrt(3)*(2*area)/(l1+l2+l3) (mLaplace.f90:96-108) from edge vectors
        const R a2 = x1 * y2 - x2 * y1;
        const R l = (x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1) + x2 * x2 + y2 * y2 + x1 * x1 + y1 * y1;
        const R m = R(3.46410161513775) * a2 / l;
        const R q = R(1) / (m * m);
        const R dxi = (R)geo[i * E + e], dyi = (R)geo[(3 + i) * E + e];
        const uchar4 pos = lap_pos[s];
        const unsigned char pj[3] = {pos.x, pos.y, pos.z};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const R v = (dxi * (R)geo[j * E + e] + dyi * (R)geo[(3 + j) * E + e]) * q;
            if (len <= 16) {
#pragma unroll
                for (int k = 0; k < 16; ++k)
                    if (k == pj[j]) acc[k] += v;
            } else {
                vals[r0 + pj[j]] += v;  // long rows: accumulate in place (rare)
            }
        }
    }
    if (len <= 16) {
#pragma unroll
        for (int k = 0; k < 16; ++k)
            if (k < len) {
                valf[r0 + k] = (float)acc[k];
                vals[r0 + k] = (double)acc[k];
            }
    } else {
        for (int k = r0; k < r1; ++k) valf[k] = (float)vals[k];
    }
    diag[p] = vals[r0];
    invdiag[p] = 1.0 / vals[r0];
}

cudaError_t launch_laplace_mixed(bool fp64, cudaStream_t st, int npoin, int nelem, const int4* elem,
                                 const int* esup_ptr, const int* esup_slot, const uchar4* lap_pos,
                                 const double* geo, const double* X, const double* Y,
                                 const int* rowptr, float* valf, double* vals, double* diag,
                                 double* invdiag) {
    const unsigned grid = blocks_for(npoin, 128);
    if (fp64)
        k_laplace_mixed_t<double><<<grid, 128, 0, st>>>(npoin, nelem, elem, esup_ptr, esup_slot,
                                                        lap_pos, geo, X, Y, rowptr, valf, vals,
                                                        diag, invdiag);
    else
        k_laplace_mixed_t<float><<<grid, 128, 0, st>>>(npoin, nelem, elem, esup_ptr, esup_slot,
                                                       lap_pos, geo, X, Y, rowptr, valf, vals, diag,
                                                       invdiag);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

// FORCES (meshMove.f90:167-192) with a block tree per set instead of the serial sum
__global__ void k_forces_tree(int nset_numb, const int* __restrict__ set_ptr,
                              const int2* __restrict__ set_edges, const double* __restrict__ P,
                              const double* __restrict__ X, const double* __restrict__ Y,
                              const double* __restrict__ xref, const double* __restrict__ yref,
                              StepScal* __restrict__ sc) {
    __shared__ double red[9];
    for (int s = 0; s < nset_numb; ++s) {
        double fx = 0.0, fy = 0.0, rm = 0.0;
        const double xr = xref[s], yr = yref[s];
        for (int k = set_ptr[s] + threadIdx.x; k < set_ptr[s + 1]; k += blockDim.x) {
            const int2 ed = set_edges[k];
            const double d_press = (P[ed.x] + P[ed.y]) * 0.5;
            const double a = d_press * (Y[ed.y] - Y[ed.x]);
            const double b = d_press * (X[ed.x] - X[ed.y]);
            fx += a;
            fy += b;
            rm += b * ((X[ed.x] + X[ed.y]) * 0.5 - xr) - a * ((Y[ed.y] + Y[ed.x]) * 0.5 - yr);
        }
        fx = block_tree256(fx, red);
        fy = block_tree256(fy, red);
        rm = block_tree256(rm, red);
        if (threadIdx.x == 0) { sc->fx[s] = fx; sc->fy[s] = fy; sc->rm[s] = rm; }
    }
}

// ------------------------------------------------------------------ host launchers
cudaError_t launch_elem_stage1_mixed(bool viscous, cudaStream_t st, int nelem, const int4* elem,
                                     const double* U, const double* geo, const double* area,
                                     const float* shoc, const double* dtl_arr,
                                     const double* dtl_scalar, const float* ts1, const float* ts2,
                                     const float* ts3, GasConst gc, const double* WX,
                                     const double* WY, const int* slot_pos, void* rec) {
    const unsigned grid = blocks_for(nelem, 128);
    if (viscous)
        k_elem_stage1_mixed<true><<<grid, 128, 0, st>>>(nelem, elem, U, geo, area, shoc, dtl_arr,
                                                         dtl_scalar, ts1, ts2, ts3, gc, WX, WY,
                                                         slot_pos, (SlotRec*)rec);
    else
        k_elem_stage1_mixed<false><<<grid, 128, 0, st>>>(nelem, elem, U, geo, area, shoc, dtl_arr,
                                                          dtl_scalar, ts1, ts2, ts3, gc, WX, WY,
                                                          slot_pos, (SlotRec*)rec);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

cudaError_t launch_node_mixed(cudaStream_t st, int npoin, const int* esup_ptr, const int* esup_slot,
                              const int4* elem, const void* rec, const double* T, GasConst gc,
                              int viscous, const double* U, const double* invM, double rk_fact,
                              const unsigned char* bcflag, const double* bcval, const double2* nrm,
                              const double* WX, const double* WY, double* U1, double* RHO,
                              double* VX, double* VY, double* E, double* P, double* To,
                              double* RMACH) {
    k_node_mixed<<<blocks_for(npoin, 256), 256, 0, st>>>(npoin, esup_ptr, esup_slot, elem,
                                                          (const SlotRec*)rec, T, gc, viscous, U,
                                                          invM, rk_fact, bcflag, bcval, nrm, WX,
                                                          WY, U1, RHO, VX, VY, E, P, To, RMACH);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

size_t slot_record_bytes() { return sizeof(SlotRec); }

}  // namespace cfd

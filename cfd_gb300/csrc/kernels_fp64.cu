// kernels_fp64.cu — the plain FP64 step on sm_103a.
//
// Compiled with --fmad=false: every double operation is the IEEE operation the reference
// expression spells, in Fortran's evaluation order, so each kernel reproduces the CPU
// restatement bit for bit.  Scatters the reference does with OpenMP atomics
// (calcRHS.f90:143-150, subrutinas.f90:145-150, :1080-1089, gcl.f90:42-43) are gathers
// here: node p walks its element-around-point list (getEsup order = element order) and
// folds the per-element contributions in that order, which is deterministic and equal to
// the serial element loop.
#include "cfd_kernels.cuh"

namespace cfd {

__device__ __forceinline__ double pow15(double x) { return x * sqrt(x); }   // x**1.5d0
__device__ __forceinline__ double powm05(double x) { return 1.0 / sqrt(x); }  // x**(-.5d0)

// ------------------------------------------------------------------ deriv
// subrutinas.f90:99-120.  geo = [dNx1 | dNx2 | dNx3 | dNy1 | dNy2 | dNy3] each [nelem].
__global__ void k_deriv(int nelem, const int4* __restrict__ elem, const double* __restrict__ X,
                        const double* __restrict__ Y, double* __restrict__ area,
                        double* __restrict__ geo, double* __restrict__ hh,
                        double* __restrict__ hhx, double* __restrict__ hhy) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    int4 n = elem[e];
    double xl[3] = {X[n.x], X[n.y], X[n.z]};
    double yl[3] = {Y[n.x], Y[n.y], Y[n.z]};
    double a = (xl[1] * yl[2] + xl[2] * yl[0] + xl[0] * yl[1] -
                (xl[1] * yl[0] + xl[2] * yl[1] + xl[0] * yl[2])) / 2.0;
    area[e] = a;
    const size_t E = (size_t)nelem;
    geo[e] = (yl[1] - yl[2]) / (2.0 * a);
    geo[E + e] = (yl[2] - yl[0]) / (2.0 * a);
    geo[2 * E + e] = (yl[0] - yl[1]) / (2.0 * a);
    geo[3 * E + e] = (xl[2] - xl[1]) / (2.0 * a);
    geo[4 * E + e] = (xl[0] - xl[2]) / (2.0 * a);
    geo[5 * E + e] = (xl[1] - xl[0]) / (2.0 * a);
    if (hh) {
        hh[e] = sqrt(a);
        hhx[e] = fabs(fmin(fmin(xl[2] - xl[1], xl[0] - xl[2]), xl[1] - xl[0]));
        hhy[e] = fabs(fmin(fmin(yl[2] - yl[1], yl[0] - yl[2]), yl[1] - yl[0]));
    }
}

// ------------------------------------------------------------------ MASAS (gather)
// subrutinas.f90:137-152: M(p) = sum over elements of p, in element order, of area/3.
__global__ void k_mass(int npoin, const int* __restrict__ esup_ptr, const int* __restrict__ esup_slot,
                       const double* __restrict__ area, double* __restrict__ M) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoin) return;
    double acc = 0.0;
    for (int s = esup_ptr[p]; s < esup_ptr[p + 1]; ++s) acc = acc + div3(area[esup_slot[s] / 3]);
    M[p] = acc;
}

// ------------------------------------------------------------------ gcl main (gather)
// gcl.f90:29-45 with putW/putArea's saved arrays; literal divW (:38-41) or dNy.W_y.
// The element terms divW*area/3 and divW_old*area_old/3 (gcl.f90:27-45; divW as written,
// dNy.W_x, when literal), formed once per element: every node around the element adds the
// same two values, in the same expressions as the reference's per-node loop.
__global__ void k_gcl_terms(int nelem, const int4* __restrict__ elem,
                            const double* __restrict__ geo, const double* __restrict__ area,
                            const double* __restrict__ area_old, const double* __restrict__ Wx,
                            const double* __restrict__ Wy, const double* __restrict__ Wxo,
                            const double* __restrict__ Wyo, int literal,
                            double2* __restrict__ terms) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    const size_t E = (size_t)nelem;
    const int4 n = elem[e];
    const int nn[3] = {n.x, n.y, n.z};
    double wx[3], wy[3], wxo[3], wyo[3];
    for (int i = 0; i < 3; ++i) {
        wx[i] = Wx[nn[i]];
        wy[i] = literal ? Wx[nn[i]] : Wy[nn[i]];
        wxo[i] = Wxo[nn[i]];
        wyo[i] = literal ? Wxo[nn[i]] : Wyo[nn[i]];
    }
    const double d0 = geo[e], d1 = geo[E + e], d2 = geo[2 * E + e];
    const double f0 = geo[3 * E + e], f1 = geo[4 * E + e], f2 = geo[5 * E + e];
    const double divW = d0 * wx[0] + d1 * wx[1] + d2 * wx[2] + f0 * wy[0] + f1 * wy[1] + f2 * wy[2];
    const double divWo =
        d0 * wxo[0] + d1 * wxo[1] + d2 * wxo[2] + f0 * wyo[0] + f1 * wyo[1] + f2 * wyo[2];
    terms[e] = make_double2(div3(divW * area[e]), div3(divWo * area_old[e]));
}

// Per node: tot1, tot2 as the ordered sums over the elements around it, M += dt(t1 + t2)/2
__global__ void k_gcl(int npoin, const int* __restrict__ esup_ptr,
                      const int* __restrict__ esup_slot, const double2* __restrict__ terms,
                      const double* __restrict__ dtp, double* __restrict__ M) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoin) return;
    double t1 = 0.0, t2 = 0.0;
    for (int s = esup_ptr[p]; s < esup_ptr[p + 1]; ++s) {
        const double2 tm = terms[esup_slot[s] / 3];
        t1 = t1 + tm.x;
        t2 = t2 + tm.y;
    }
    M[p] = M[p] + (*dtp) * (t1 + t2) / 2.0;
}

cudaError_t launch_gcl(cudaStream_t st, int npoin, int nelem, const int4* elem,
                       const int* esup_ptr, const int* esup_slot, const double* geo,
                       const double* area, const double* area_old, const double* Wx,
                       const double* Wy, const double* Wxo, const double* Wyo, const double* dtp,
                       int literal, double2* scratch, double* M) {
    k_gcl_terms<<<blocks_for(nelem, 256), 256, 0, st>>>(nelem, elem, geo, area, area_old, Wx, Wy,
                                                        Wxo, Wyo, literal, scratch);
    k_gcl<<<blocks_for(npoin, 256), 256, 0, st>>>(npoin, esup_ptr, esup_slot, scratch, dtp, M);
    g_launches.fetch_add(2, std::memory_order_relaxed);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ deltat
// subrutinas.f90:170-210.  DT per element and the bit pattern of the positive minimum
// (positive doubles order like their bits, so the unsigned atomicMin is exact).
__global__ void k_deltat(int nelem, const int4* __restrict__ elem, const double* __restrict__ T,
                         const double* __restrict__ VX, const double* __restrict__ VY,
                         const double* __restrict__ WX, const double* __restrict__ WY,
                         const double* __restrict__ area, double fsafe, double t_inf,
                         double* __restrict__ DT, unsigned long long* __restrict__ dtmin_bits) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long mybits = 0x7ff0000000000000ull;  // +inf
    if (e < nelem) {
        int4 n = elem[e];
        int nn[3] = {n.x, n.y, n.z};
        double vumax = 0.0, vvmax = 0.0;
        double T_iel = div3(T[nn[0]] + T[nn[1]] + T[nn[2]]);
        for (int i = 0; i < 3; ++i) {
            double vu = fabs(VX[nn[i]] - WX[nn[i]]);
            double vv = fabs(VY[nn[i]] - WY[nn[i]]);
            if (vu > vumax) vumax = vu;
            if (vv > vvmax) vvmax = vv;
        }
        double hh = sqrt(2.0 * area[e]);
        double vel = sqrt(vumax * vumax + vvmax * vvmax);
        const double smu = 110.0;
        double fmu = 0.017 * pow15(T_iel / t_inf) * (t_inf + smu) / (T_iel + smu);
        double et = fmu;
        double pe = (vel * hh) / (2.0 * et);
        double alpha = fmin(div3(pe), 1.0);
        double deltatu = 1.0 / (4.0 * et / (hh * hh) + alpha * vel / hh);
        double deltatc = 1.0 / (4.0 * et / (hh * hh));
        double dtelem = fsafe / (1.0 / deltatc + 1.0 / deltatu);
        DT[e] = dtelem;
        if (dtelem < 1.0e20 && dtelem > 0.0) mybits = (unsigned long long)__double_as_longlong(dtelem);
    }
    // warp + block min, then one atomic per block
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

// DTMIN (1.d20 when no element is finite), the 1% hysteresis of ns2DComp.ALE.f90:146-156
// and the DT clamp of subrutinas.f90:211-215.  One thread.
__global__ void k_dt_finalize(StepScal* sc) {
    const unsigned long long b = sc->dtmin_bits;
    sc->dtmin_bits = 0x7ff0000000000000ull;  // ready for the next step's k_deltat
    dt_finalize_from(sc, b);
}

// ITLOCAL != 0 only: DTL = DTMIN*DTFACT + min(DT, COTA)*(1-DTFACT) (ns2DComp.ALE.f90:160-161)
__global__ void k_dtl(int nelem, double* __restrict__ DT, double* __restrict__ DTL,
                      const StepScal* __restrict__ sc, double dtfact) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    double d = DT[e];
    if (d > sc->cota) d = sc->cota;
    DT[e] = d;
    DTL[e] = sc->dtmin * dtfact + d * (1.0 - dtfact);
}

// ------------------------------------------------------------------ ESTAB
// subrutinas.f90:346-443 (GAMM is the uniform GAMA for NGAS=0, :78).
__global__ void k_estab(int nelem, const int4* __restrict__ elem, const double* __restrict__ U,
                        const double* __restrict__ T, double gamm,
                        const double* __restrict__ GAMM, const double* __restrict__ VX,
                        const double* __restrict__ VY, const double* __restrict__ WX,
                        const double* __restrict__ WY, const double* __restrict__ geo,
                        double FR, const StepScal* __restrict__ sc, double RHOINF, double TINF,
                        int estab_mode, double eps_dir, double dirx, double diry,
                        double* __restrict__ SHOC, double* __restrict__ TS1,
                        double* __restrict__ TS2, double* __restrict__ TS3) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    const size_t E = (size_t)nelem;
    const double DTMIN = sc->dtmin;
    int4 n = elem[e];
    const int n1 = n.x, n2 = n.y, n3 = n.z;
    const double DX[3] = {geo[e], geo[E + e], geo[2 * E + e]};
    const double DY[3] = {geo[3 * E + e], geo[4 * E + e], geo[5 * E + e]};
    double gm = GAMM ? div3(GAMM[n1] + GAMM[n2] + GAMM[n3]) : div3(gamm + gamm + gamm);
    double tau = 0.0, h_rgne = 0.0, h_rgn = 0.0, h_jgn = 0.0;
    const double r1 = U[4 * (size_t)n1], r2 = U[4 * (size_t)n2], r3 = U[4 * (size_t)n3];
    double rho_elem = div3(r1 + r2 + r3);
    double vx = div3(VX[n1] + VX[n2] + VX[n3]);
    double vy = div3(VY[n1] + VY[n2] + VY[n3]);
    double wx = div3(WX[n1] + WX[n2] + WX[n3]);
    double wy = div3(WY[n1] + WY[n2] + WY[n3]);
    vx = vx - wx;
    vy = vy - wy;
    double vel2 = sqrt(vx * vx + vy * vy);
    double drx = r1 * DX[0] + r2 * DX[1] + r3 * DX[2];
    double dry = r1 * DY[0] + r2 * DY[1] + r3 * DY[2];
    double dr2 = sqrt(drx * drx + dry * dry) + 1.0e-20;
    const double t1 = T[n1], t2 = T[n2], t3 = T[n3];
    double dtx = t1 * DX[0] + t2 * DX[1] + t3 * DX[2];
    double dty = t1 * DY[0] + t2 * DY[1] + t3 * DY[2];
    double dt2 = sqrt(dtx * dtx + dty * dty) + 1.0e-20;
    double dux = vel2 * DX[0] + vel2 * DX[1] + vel2 * DX[2];
    double duy = vel2 * DY[0] + vel2 * DY[1] + vel2 * DY[2];
    if (estab_mode != CFD_ESTAB_REFERENCE) {
        dux = 0.0;
        duy = 0.0;
    }
    double du2 = sqrt(dux * dux + duy * duy) + 1.0e-20;
    double rtx = dtx / dt2, rty = dty / dt2;
    double rjx = drx / dr2, rjy = dry / dr2;
    double rux = dux / du2, ruy = duy / du2;
    if (estab_mode == CFD_ESTAB_REGULARIZED) {
        // unit vectors continuous in the state: gradient + eps*scale*G_e along the
        // freestream direction, normalised; the velocity-gradient direction is that d
        double ge = 0.0;
        for (int i = 0; i < 3; ++i) ge += sqrt(DX[i] * DX[i] + DY[i] * DY[i]);
        const double sr = eps_dir * rho_elem * ge;
        const double st = eps_dir * (div3(t1 + t2 + t3)) * ge;
        const double gx = drx + sr * dirx, gy = dry + sr * diry;
        const double hx = dtx + st * dirx, hy = dty + st * diry;
        const double gn = sqrt(gx * gx + gy * gy), hn = sqrt(hx * hx + hy * hy);
        rjx = gx / gn;
        rjy = gy / gn;
        rtx = hx / hn;
        rty = hy / hn;
        rux = dirx;
        ruy = diry;
    }
    double temp = div3(t1 + t2 + t3);
    double c = sqrt(gm * FR * temp);
    const double smu = 110.0;
    double fmu = 0.017 * pow15(temp / TINF) * (TINF + smu) / (temp + smu);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double term1 = fabs(vx * DX[i] + vy * DY[i]);
        double term2 = fabs(rjx * DX[i] + rjy * DY[i]);
        double h1 = fabs(rtx * DX[i] + rty * DY[i]);
        double h2 = fabs(rux * DX[i] + ruy * DY[i]);
        tau = tau + term1 + term2 * c;
        h_rgne = h_rgne + h1;
        h_rgn = h_rgn + h2;
        h_jgn = h_jgn + term2;
    }
    tau = 1.0 / tau;
    h_rgne = 2.0 / h_rgne;
    h_rgn = 2.0 / h_rgn;
    if (h_rgn > 10.0) h_rgn = 0.0;
    h_jgn = 2.0 / h_jgn;
    if (h_jgn > 10.0) h_jgn = 0.0;
    double tr1 = dr2 * h_jgn / rho_elem;
    double zzz = h_jgn / (2.0 * c);
    SHOC[e] = (tr1 + tr1 * tr1) * 0.5 * (c * c) * zzz;
    double resumen = 1.0 / (tau * tau) + (2.0 / DTMIN) * (2.0 / DTMIN);
    double rrr = powm05(resumen);
    double s2 = rrr, s3 = rrr;
    if (fmu != 0.0) {
        double tau_sung3 = (h_rgn * h_rgn) / (4.0 * fmu / RHOINF);
        double tau_sung3_e = (h_rgne * h_rgne) / (4.0 * fmu / RHOINF);
        s2 = powm05(resumen + 1.0 / (tau_sung3 * tau_sung3));
        s3 = powm05(resumen + 1.0 / (tau_sung3_e * tau_sung3_e));
    }
    TS1[e] = rrr;
    TS2[e] = s2;
    TS3[e] = s3;
}

// ------------------------------------------------------------------ calcRHS + FUENTE
// One thread per element: the 12 calcRHS contributions (calcRHS.f90:36-141) and, when
// `fuente` is set, the 12 FUENTE contributions (subrutinas.f90:1060-1078), written to
// per-(element, local node) slots [3*e + i][4] for the ordered node gather.  The terms
// N(i,k)*AiUi with N(i,k) = 0 and theta (identically 0 on this path) are left out: both
// add a signed zero, which leaves every sum's value unchanged.
template <bool VISCOUS, bool THETA>
__global__ void __launch_bounds__(128)
k_elem_rhs(int nelem, const int4* __restrict__ elem, const double* __restrict__ U,
           const double* __restrict__ theta, const double* __restrict__ T,
           const double* __restrict__ geo, const double* __restrict__ area,
           const double* __restrict__ shoc, const double* __restrict__ dtl_arr,
           const double* __restrict__ dtl_scalar, const double* __restrict__ ts1,
           const double* __restrict__ ts2, const double* __restrict__ ts3, GasConst gc,
           double* __restrict__ contrib, const double* __restrict__ WX,
           const double* __restrict__ WY, double* __restrict__ contribF) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    const size_t E = (size_t)nelem;
    const double Cv = gc.cv, lambda_ref = gc.lambda_ref, mu_ref = gc.mu_ref, g = gc.gamma;
    const double T_inf = gc.t_inf, cte = gc.cte;
    int4 n = elem[e];
    const int p[3] = {n.x, n.y, n.z};
    const double Nx[3] = {geo[e], geo[E + e], geo[2 * E + e]};
    const double Ny[3] = {geo[3 * E + e], geo[4 * E + e], geo[5 * E + e]};
    double Un[3][4];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double2* u2 = reinterpret_cast<const double2*>(U + 4 * (size_t)p[i]);
        double2 a = u2[0], b = u2[1];
        Un[i][0] = a.x; Un[i][1] = a.y; Un[i][2] = b.x; Un[i][3] = b.y;
    }
    double Ux[4], Uy[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        Ux[q] = Un[0][q] * Nx[0] + Un[1][q] * Nx[1] + Un[2][q] * Nx[2];
        Uy[q] = Un[0][q] * Ny[0] + Un[1][q] * Ny[1] + Un[2][q] * Ny[2];
    }
    const double dtl = dtl_arr ? dtl_arr[e] : *dtl_scalar;
    const double ar = area[e];
    if (contrib) {
    const double tau[3] = {ts1[e], ts2[e], ts3[e]};
    const double nu = shoc[e] * cte;
    double mu = 0.0, lambda = 0.0;
    if (VISCOUS) {
        const double T_avg = div3(T[p[0]] + T[p[1]] + T[p[2]]);
        mu = mu_ref * pow15(T_avg / T_inf) * (T_inf + 110.0) / (T_avg + 110.0);
        lambda = lambda_ref * pow15(T_avg / T_inf) * (T_inf + 194.0) / (T_avg + 194.0);
    }
    double r[3][4];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) r[i][q] = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        // U_k = N(1,k) U1 + N(2,k) U2 + N(3,k) U3 with N(k,k) = 0: the two 0.5 terms in order
        const int ia = (k == 0) ? 1 : 0;
        const int ib = (k == 2) ? 1 : 2;
        double Uk[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) Uk[q] = 0.5 * Un[ia][q] + 0.5 * Un[ib][q];
        const double rho = Uk[0];
        const double v1 = Uk[1] / rho, v2 = Uk[2] / rho, ev = Uk[3] / rho;
        const double V_sq = v1 * v1 + v2 * v2;
        double A[4];
        A[0] = Ux[1] + Uy[2];
        A[1] = 0.5 * Ux[0] * (V_sq * (g - 1.0) - 2.0 * (v1 * v1)) - Ux[1] * v1 * (g - 3.0) -
               Ux[2] * v2 * (g - 1.0) + Ux[3] * (g - 1.0) - Uy[0] * v1 * v2 + Uy[1] * v2 +
               Uy[2] * v1;
        A[2] = -(Ux[0] * v1 * v2) + Ux[1] * v2 + Ux[2] * v1 +
               0.5 * Uy[0] * (V_sq * (g - 1.0) - 2.0 * (v2 * v2)) - Uy[1] * v1 * (g - 1.0) -
               Uy[2] * v2 * (g - 3.0) + Uy[3] * (g - 1.0);
        A[3] = Ux[0] * v1 * (V_sq * (g - 1.0) - ev * g) -
               0.5 * Ux[1] * (V_sq * (g - 1.0) - 2.0 * ev * g + 2.0 * (v1 * v1) * (g - 1.0)) -
               Ux[2] * v1 * v2 * (g - 1.0) + Ux[3] * g * v1 +
               Uy[0] * v2 * (V_sq * (g - 1.0) - ev * g) - Uy[1] * v1 * v2 * (g - 1.0) -
               0.5 * Uy[2] * (V_sq * (g - 1.0) - 2.0 * ev * g + 2.0 * (v2 * v2) * (g - 1.0)) +
               Uy[3] * g * v2;
        double At[4];
        if (THETA) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const double tk = 0.5 * theta[4 * (size_t)p[ia] + q] + 0.5 * theta[4 * (size_t)p[ib] + q];
                At[q] = tk + A[q];
            }
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) At[q] = A[q];
        }
        double B1[4], B2[4];
        B1[0] = At[1];
        B1[1] = v1 * (-g + 3.0) * At[1] - v2 * (g - 1.0) * At[2] + (g - 1.0) * At[3] +
                (0.5 * V_sq * (g - 1.0) - v1 * v1) * At[0];
        B1[2] = -(v1 * v2 * At[0]) + v1 * At[2] + v2 * At[1];
        B1[3] = g * v1 * At[3] - v1 * v2 * (g - 1.0) * At[2] +
                v1 * (V_sq * (g - 1.0) - ev * g) * At[0] +
                (-(0.5 * V_sq * (g - 1.0)) + ev * g - v1 * v1 * (g - 1.0)) * At[1];
        B2[0] = At[2];
        B2[1] = B1[2];
        B2[2] = -(v1 * (g - 1.0) * At[1]) + v2 * (-g + 3.0) * At[2] + (g - 1.0) * At[3] +
                (0.5 * V_sq * (g - 1.0) - v2 * v2) * At[0];
        B2[3] = g * v2 * At[3] - v1 * v2 * (g - 1.0) * At[1] +
                v2 * (V_sq * (g - 1.0) - ev * g) * At[0] +
                (-(0.5 * V_sq * (g - 1.0)) + ev * g - v2 * v2 * (g - 1.0)) * At[2];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                double t = r[i][q];
                if (i != k) t = t + 0.5 * A[q];
                r[i][q] = t + tau[i] * (Nx[i] * B1[q] + Ny[i] * B2[q]) +
                          nu * (Nx[i] * Ux[q] + Ny[i] * Uy[q]);
            }
        if (VISCOUS) {
            double K1[4], K2[4];
            K1[1] = 2.0 / 3.0 * mu * (-(2.0 * Ux[0] * v1) + 2.0 * Ux[1] + Uy[0] * v2 - Uy[2]) / rho;
            K1[2] = mu * (-(Ux[0] * v2) + Ux[2] - Uy[0] * v1 + Uy[1]) / rho;
            K1[3] = 1.0 / 3.0 *
                    (Cv * mu * (-(Uy[0] * v1 * v2) + 3.0 * Uy[1] * v2 - 2.0 * Uy[2] * v1) -
                     Ux[0] * (Cv * mu * (3.0 * V_sq + v1 * v1) - 3.0 * lambda * (V_sq - ev)) +
                     Ux[1] * v1 * (4.0 * Cv * mu - 3.0 * lambda) +
                     3.0 * Ux[2] * v2 * (Cv * mu - lambda) + 3.0 * Ux[3] * lambda) /
                    (Cv * rho);
            K2[1] = K1[2];
            K2[2] = 2.0 / 3.0 * mu * (Ux[0] * v1 - Ux[1] - 2.0 * Uy[0] * v2 + 2.0 * Uy[2]) / rho;
            K2[3] = 1.0 / 3.0 *
                    (Cv * mu * (-(Ux[0] * v1 * v2) - 2.0 * Ux[1] * v2 + 3.0 * Ux[2] * v1) -
                     Uy[0] * (Cv * mu * (3.0 * V_sq + v2 * v2) - 3.0 * lambda * (V_sq - ev)) +
                     3.0 * Uy[1] * v1 * (Cv * mu - lambda) +
                     Uy[2] * v2 * (4.0 * Cv * mu - 3.0 * lambda) + 3.0 * Uy[3] * lambda) /
                    (Cv * rho);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int q = 1; q < 4; ++q) r[i][q] = r[i][q] + (Nx[i] * K1[q] + Ny[i] * K2[q]);
        }
    }
    double* out = contrib + 12 * (size_t)e;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double2 a, b;
        a.x = div3(r[i][0] * ar * dtl);
        a.y = div3(r[i][1] * ar * dtl);
        b.x = div3(r[i][2] * ar * dtl);
        b.y = div3(r[i][3] * ar * dtl);
        reinterpret_cast<double2*>(out + 4 * i)[0] = a;
        reinterpret_cast<double2*>(out + 4 * i)[1] = b;
    }
    }  // contrib
    if (contribF) {
        // FUENTE (subrutinas.f90:1064-1078); its Ux/Uy expression equals calcRHS's.
        const double AR = div3(ar * dtl);
        const double w0 = WX[p[0]], w1 = WX[p[1]], w2 = WX[p[2]];
        const double y0 = WY[p[0]], y1 = WY[p[1]], y2 = WY[p[2]];
        // sp(:,1)=(.5,.5,0), sp(:,2)=(0,.5,.5), sp(:,3)=(.5,0,.5); zero terms dropped
        const double wx[3] = {0.5 * w0 + 0.5 * w1, 0.5 * w1 + 0.5 * w2, 0.5 * w0 + 0.5 * w2};
        const double wy[3] = {0.5 * y0 + 0.5 * y1, 0.5 * y1 + 0.5 * y2, 0.5 * y0 + 0.5 * y2};
        double* of = contribF + 12 * (size_t)e;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double q0 = Ux[q] * wx[0] + Uy[q] * wy[0];
            const double q1 = Ux[q] * wx[1] + Uy[q] * wy[1];
            const double q2 = Ux[q] * wx[2] + Uy[q] * wy[2];
            of[q] = -(AR * (0.5 * q0 + 0.5 * q2));      // node 1: sp(1,:) = (.5, 0, .5)
            of[4 + q] = -(AR * (0.5 * q0 + 0.5 * q1));  // node 2: sp(2,:) = (.5, .5, 0)
            of[8 + q] = -(AR * (0.5 * q1 + 0.5 * q2));  // node 3: sp(3,:) = (0, .5, .5)
        }
    }
}

cudaError_t launch_elem_rhs(bool viscous, bool with_theta, cudaStream_t stream, int nelem,
                            const int4* elem, const double* U, const double* theta,
                            const double* T, const double* geo, const double* area,
                            const double* shoc, const double* dtl_arr, const double* dtl_scalar,
                            const double* ts1, const double* ts2, const double* ts3, GasConst gc,
                            double* contrib, const double* WX, const double* WY,
                            double* contribF) {
    const unsigned grid = blocks_for(nelem, 128);
#define CFD_ELEM_ARGS nelem, elem, U, theta, T, geo, area, shoc, dtl_arr, dtl_scalar, ts1, ts2, \
                      ts3, gc, contrib, WX, WY, contribF
    if (viscous && with_theta) k_elem_rhs<true, true><<<grid, 128, 0, stream>>>(CFD_ELEM_ARGS);
    else if (viscous) k_elem_rhs<true, false><<<grid, 128, 0, stream>>>(CFD_ELEM_ARGS);
    else if (with_theta) k_elem_rhs<false, true><<<grid, 128, 0, stream>>>(CFD_ELEM_ARGS);
    else k_elem_rhs<false, false><<<grid, 128, 0, stream>>>(CFD_ELEM_ARGS);
#undef CFD_ELEM_ARGS
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

// VEL_X = rho u / rho, VEL_Y = rho v / rho from U(4,npoin) (either output may be null)
__global__ void k_vel_from_U(int npoin, const double* __restrict__ U, double* __restrict__ VX,
                             double* __restrict__ VY) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npoin) return;
    const double2 a = reinterpret_cast<const double2*>(U + 4 * (size_t)i)[0];
    const double b = U[4 * (size_t)i + 2];
    if (VX) VX[i] = a.y / a.x;
    if (VY) VY[i] = b / a.x;
}

// ------------------------------------------------------------------ calcRHS, stage-invariant split
// All four RK stages evaluate calcRHS at the step-start U (subrutinas.f90:685); between the
// stages only T changes, and T enters only mu and lambda (calcRHS.f90:49-51), i.e. only
// the viscous K-flux terms (:119-137).  The per-node sums of calcRHS.f90:109-117 and
// :133-135 are left-associative and interleave the quadrature points: for local node i,
// variable q and quadrature point k the running sum takes
//     (+ 0.5*AiUi_k(q) if i != k)  + tau_i*(Nx_i*B1_k(q) + Ny_i*B2_k(q))
//     + nu*(Nx_i*Ux(q) + Ny_i*Uy(q))  [+ Nx_i*K1_k(q) + Ny_i*K2_k(q) for q = 2..4],
// so caching the individual addends (not their sum) and replaying the adds in the same
// order reproduces every bit.  k_elem_inv forms, once per step, the stage-invariant addends
// and the mu-independent factors of K1, K2; k_elem_replay forms, per stage, mu and lambda,
// K1, K2 and the sums.  Variable 1 (continuity) has no viscous term: its contribution is
// final after k_elem_inv.
//
// Cache planes (kInvPlanes, each nelem doubles, plane-major so a warp's loads coalesce):
constexpr int kC0 = 0;    // [i]        final continuity contribution of local node i
constexpr int kA1 = 3;    // [k][q-1]   0.5*AiUi_k(q)
constexpr int kA2 = 12;   // [i][k][q-1] tau_i*(Nx_i*B1_k(q) + Ny_i*B2_k(q))
constexpr int kA3 = 39;   // [i][q-1]   nu*(Nx_i*Ux(q) + Ny_i*Uy(q))
constexpr int kV = 48;    // [k][14]    mu-independent factors of K1_k, K2_k (below)
constexpr int kVG = 90;   // [4]        Ux(1), Uy(1), 3*Ux(4), 3*Uy(4)
constexpr int kRc = 94;   // [k][2]     RN(1/rho_k), RN(1/(Cv*rho_k)): the replay's quotients
                          //            by them take div_rcp (bit-identical, fewer FP64 ops)
constexpr int kInvPlanes = 100;
static_assert(kInvPlanes == kElemInvPlanes, "cache planes");
// kV + 14*k + m: 0 rho, 1 P11, 2 P12, 3 P13a, 4 P13b, 5 P13c, 6 Ux(2)*v1, 7 3*Ux(3)*v2,
// 8 Cv*rho, 9 P22, 10 P23a, 11 P23b, 12 3*Uy(2)*v1, 13 Uy(3)*v2

template <bool VISCOUS>
__global__ void __launch_bounds__(128)
k_elem_inv(int nelem, const int4* __restrict__ elem, const double* __restrict__ U,
           const double* __restrict__ geo, const double* __restrict__ area,
           const double* __restrict__ shoc, const double* __restrict__ dtl_arr,
           const double* __restrict__ dtl_scalar, const double* __restrict__ ts1,
           const double* __restrict__ ts2, const double* __restrict__ ts3, GasConst gc,
           double* __restrict__ cache, double* __restrict__ contrib,
           const double* __restrict__ WX, const double* __restrict__ WY,
           double* __restrict__ contribF) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    const size_t E = (size_t)nelem;
    const double Cv = gc.cv, g = gc.gamma, cte = gc.cte;
    int4 n = elem[e];
    const int p[3] = {n.x, n.y, n.z};
    const double Nx[3] = {geo[e], geo[E + e], geo[2 * E + e]};
    const double Ny[3] = {geo[3 * E + e], geo[4 * E + e], geo[5 * E + e]};
    double Un[3][4];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double2* u2 = reinterpret_cast<const double2*>(U + 4 * (size_t)p[i]);
        double2 a = u2[0], b = u2[1];
        Un[i][0] = a.x; Un[i][1] = a.y; Un[i][2] = b.x; Un[i][3] = b.y;
    }
    double Ux[4], Uy[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        Ux[q] = Un[0][q] * Nx[0] + Un[1][q] * Nx[1] + Un[2][q] * Nx[2];
        Uy[q] = Un[0][q] * Ny[0] + Un[1][q] * Ny[1] + Un[2][q] * Ny[2];
    }
    const double dtl = dtl_arr ? dtl_arr[e] : *dtl_scalar;
    const double ar = area[e];
    const double tau[3] = {ts1[e], ts2[e], ts3[e]};
    const double nu = shoc[e] * cte;
    auto C = [&](int plane) -> double& { return cache[(size_t)plane * E + e]; };
    double a3[3][4];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) a3[i][q] = nu * (Nx[i] * Ux[q] + Ny[i] * Uy[q]);
    double r[3][4];  // non-viscous sums (all four variables when !VISCOUS, else continuity)
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) r[i][q] = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int ia = (k == 0) ? 1 : 0;
        const int ib = (k == 2) ? 1 : 2;
        double Uk[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) Uk[q] = 0.5 * Un[ia][q] + 0.5 * Un[ib][q];
        const double rho = Uk[0];
        const double v1 = Uk[1] / rho, v2 = Uk[2] / rho, ev = Uk[3] / rho;
        const double V_sq = v1 * v1 + v2 * v2;
        double A[4];
        A[0] = Ux[1] + Uy[2];
        A[1] = 0.5 * Ux[0] * (V_sq * (g - 1.0) - 2.0 * (v1 * v1)) - Ux[1] * v1 * (g - 3.0) -
               Ux[2] * v2 * (g - 1.0) + Ux[3] * (g - 1.0) - Uy[0] * v1 * v2 + Uy[1] * v2 +
               Uy[2] * v1;
        A[2] = -(Ux[0] * v1 * v2) + Ux[1] * v2 + Ux[2] * v1 +
               0.5 * Uy[0] * (V_sq * (g - 1.0) - 2.0 * (v2 * v2)) - Uy[1] * v1 * (g - 1.0) -
               Uy[2] * v2 * (g - 3.0) + Uy[3] * (g - 1.0);
        A[3] = Ux[0] * v1 * (V_sq * (g - 1.0) - ev * g) -
               0.5 * Ux[1] * (V_sq * (g - 1.0) - 2.0 * ev * g + 2.0 * (v1 * v1) * (g - 1.0)) -
               Ux[2] * v1 * v2 * (g - 1.0) + Ux[3] * g * v1 +
               Uy[0] * v2 * (V_sq * (g - 1.0) - ev * g) - Uy[1] * v1 * v2 * (g - 1.0) -
               0.5 * Uy[2] * (V_sq * (g - 1.0) - 2.0 * ev * g + 2.0 * (v2 * v2) * (g - 1.0)) +
               Uy[3] * g * v2;
        const double* At = A;
        double B1[4], B2[4];
        B1[0] = At[1];
        B1[1] = v1 * (-g + 3.0) * At[1] - v2 * (g - 1.0) * At[2] + (g - 1.0) * At[3] +
                (0.5 * V_sq * (g - 1.0) - v1 * v1) * At[0];
        B1[2] = -(v1 * v2 * At[0]) + v1 * At[2] + v2 * At[1];
        B1[3] = g * v1 * At[3] - v1 * v2 * (g - 1.0) * At[2] +
                v1 * (V_sq * (g - 1.0) - ev * g) * At[0] +
                (-(0.5 * V_sq * (g - 1.0)) + ev * g - v1 * v1 * (g - 1.0)) * At[1];
        B2[0] = At[2];
        B2[1] = B1[2];
        B2[2] = -(v1 * (g - 1.0) * At[1]) + v2 * (-g + 3.0) * At[2] + (g - 1.0) * At[3] +
                (0.5 * V_sq * (g - 1.0) - v2 * v2) * At[0];
        B2[3] = g * v2 * At[3] - v1 * v2 * (g - 1.0) * At[1] +
                v2 * (V_sq * (g - 1.0) - ev * g) * At[0] +
                (-(0.5 * V_sq * (g - 1.0)) + ev * g - v2 * v2 * (g - 1.0)) * At[2];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const double a2 = tau[i] * (Nx[i] * B1[q] + Ny[i] * B2[q]);
                if (!VISCOUS || q == 0) {
                    double t = r[i][q];
                    if (i != k) t = t + 0.5 * A[q];
                    r[i][q] = t + a2 + a3[i][q];
                } else {
                    C(kA2 + 9 * i + 3 * k + (q - 1)) = a2;
                }
            }
        if (VISCOUS) {
#pragma unroll
            for (int q = 1; q < 4; ++q) C(kA1 + 3 * k + (q - 1)) = 0.5 * A[q];
            // the mu-independent factors of K1_k, K2_k (calcRHS.f90:119-137), each formed
            // exactly as the full expression forms it
            C(kV + 14 * k + 0) = rho;
            C(kV + 14 * k + 1) = -(2.0 * Ux[0] * v1) + 2.0 * Ux[1] + Uy[0] * v2 - Uy[2];
            C(kV + 14 * k + 2) = -(Ux[0] * v2) + Ux[2] - Uy[0] * v1 + Uy[1];
            C(kV + 14 * k + 3) = -(Uy[0] * v1 * v2) + 3.0 * Uy[1] * v2 - 2.0 * Uy[2] * v1;
            C(kV + 14 * k + 4) = 3.0 * V_sq + v1 * v1;
            C(kV + 14 * k + 5) = V_sq - ev;
            C(kV + 14 * k + 6) = Ux[1] * v1;
            C(kV + 14 * k + 7) = 3.0 * Ux[2] * v2;
            C(kV + 14 * k + 8) = Cv * rho;
            C(kRc + 2 * k) = 1.0 / rho;
            C(kRc + 2 * k + 1) = 1.0 / (Cv * rho);
            C(kV + 14 * k + 9) = Ux[0] * v1 - Ux[1] - 2.0 * Uy[0] * v2 + 2.0 * Uy[2];
            C(kV + 14 * k + 10) = -(Ux[0] * v1 * v2) - 2.0 * Ux[1] * v2 + 3.0 * Ux[2] * v1;
            C(kV + 14 * k + 11) = 3.0 * V_sq + v2 * v2;
            C(kV + 14 * k + 12) = 3.0 * Uy[1] * v1;
            C(kV + 14 * k + 13) = Uy[2] * v2;
        }
    }
    if (VISCOUS) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            C(kC0 + i) = div3(r[i][0] * ar * dtl);
#pragma unroll
            for (int q = 1; q < 4; ++q) C(kA3 + 3 * i + (q - 1)) = a3[i][q];
        }
        C(kVG + 0) = Ux[0];
        C(kVG + 1) = Uy[0];
        C(kVG + 2) = 3.0 * Ux[3];
        C(kVG + 3) = 3.0 * Uy[3];
    } else {
        double* out = contrib + 12 * (size_t)e;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            double2 a, b;
            a.x = div3(r[i][0] * ar * dtl);
            a.y = div3(r[i][1] * ar * dtl);
            b.x = div3(r[i][2] * ar * dtl);
            b.y = div3(r[i][3] * ar * dtl);
            reinterpret_cast<double2*>(out + 4 * i)[0] = a;
            reinterpret_cast<double2*>(out + 4 * i)[1] = b;
        }
    }
    if (contribF) {
        // FUENTE (subrutinas.f90:1064-1078), as in k_elem_rhs
        const double AR = div3(ar * dtl);
        const double w0 = WX[p[0]], w1 = WX[p[1]], w2 = WX[p[2]];
        const double y0 = WY[p[0]], y1 = WY[p[1]], y2 = WY[p[2]];
        const double wx[3] = {0.5 * w0 + 0.5 * w1, 0.5 * w1 + 0.5 * w2, 0.5 * w0 + 0.5 * w2};
        const double wy[3] = {0.5 * y0 + 0.5 * y1, 0.5 * y1 + 0.5 * y2, 0.5 * y0 + 0.5 * y2};
        double* of = contribF + 12 * (size_t)e;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double q0 = Ux[q] * wx[0] + Uy[q] * wy[0];
            const double q1 = Ux[q] * wx[1] + Uy[q] * wy[1];
            const double q2 = Ux[q] * wx[2] + Uy[q] * wy[2];
            of[q] = -(AR * (0.5 * q0 + 0.5 * q2));
            of[4 + q] = -(AR * (0.5 * q0 + 0.5 * q1));
            of[8 + q] = -(AR * (0.5 * q1 + 0.5 * q2));
        }
    }
}

// One RK stage of the viscous calcRHS from the cache: mu, lambda from this stage's T, the
// K fluxes (calcRHS.f90:119-137 with the cached factors) and the sums replayed in the order
// of k_elem_rhs; writes all 12 contributions (continuity copied from the cache).
__global__ void __launch_bounds__(128)
k_elem_replay(int nelem, const int4* __restrict__ elem, const double* __restrict__ T,
              const double* __restrict__ geo, const double* __restrict__ area,
              const double* __restrict__ dtl_arr, const double* __restrict__ dtl_scalar,
              GasConst gc, const double* __restrict__ cache, double* __restrict__ contrib) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    const size_t E = (size_t)nelem;
    auto C = [&](int plane) -> double { return __ldcs(cache + (size_t)plane * E + e); };
    const double Cv = gc.cv, lambda_ref = gc.lambda_ref, mu_ref = gc.mu_ref, T_inf = gc.t_inf;
    const int4 n = elem[e];
    const double T_avg = div3(T[n.x] + T[n.y] + T[n.z]);
    const double mu = mu_ref * pow15(T_avg / T_inf) * (T_inf + 110.0) / (T_avg + 110.0);
    const double lambda = lambda_ref * pow15(T_avg / T_inf) * (T_inf + 194.0) / (T_avg + 194.0);
    const double Nx[3] = {geo[e], geo[E + e], geo[2 * E + e]};
    const double Ny[3] = {geo[3 * E + e], geo[4 * E + e], geo[5 * E + e]};
    const double dtl = dtl_arr ? dtl_arr[e] : *dtl_scalar;
    const double ar = area[e];
    // the mu, lambda subexpressions as calcRHS.f90:119-137 group them
    const double c23m = 2.0 / 3.0 * mu;
    const double cm = Cv * mu;
    const double l3 = 3.0 * lambda;
    const double c4m_l3 = 4.0 * Cv * mu - 3.0 * lambda;
    const double cm_l = Cv * mu - lambda;
    const double Ux0 = C(kVG + 0), Uy0 = C(kVG + 1);
    const double t5x = C(kVG + 2) * lambda, t5y = C(kVG + 3) * lambda;
    double r[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int q = 0; q < 3; ++q) r[i][q] = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int b = kV + 14 * k;
        const double rho = C(b + 0);
        const double P13c = C(b + 5);
        const double crho = C(b + 8);
        const double rr = C(kRc + 2 * k), rc = C(kRc + 2 * k + 1);
        double K1[3], K2[3];
        K1[0] = div_rcp(c23m * C(b + 1), rho, rr);
        K1[1] = div_rcp(mu * C(b + 2), rho, rr);
        K1[2] = div_rcp(1.0 / 3.0 *
                            (cm * C(b + 3) - Ux0 * (cm * C(b + 4) - l3 * P13c) +
                             C(b + 6) * c4m_l3 + C(b + 7) * cm_l + t5x),
                        crho, rc);
        K2[0] = K1[1];
        K2[1] = div_rcp(c23m * C(b + 9), rho, rr);
        K2[2] = div_rcp(1.0 / 3.0 *
                            (cm * C(b + 10) - Uy0 * (cm * C(b + 11) - l3 * P13c) +
                             C(b + 12) * cm_l + C(b + 13) * c4m_l3 + t5y),
                        crho, rc);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                double t = r[i][q];
                if (i != k) t = t + C(kA1 + 3 * k + q);
                t = t + C(kA2 + 9 * i + 3 * k + q) + C(kA3 + 3 * i + q);
                r[i][q] = t + (Nx[i] * K1[q] + Ny[i] * K2[q]);
            }
    }
    double* out = contrib + 12 * (size_t)e;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double2 a, b;
        a.x = C(kC0 + i);
        a.y = div3(r[i][0] * ar * dtl);
        b.x = div3(r[i][1] * ar * dtl);
        b.y = div3(r[i][2] * ar * dtl);
        reinterpret_cast<double2*>(out + 4 * i)[0] = a;
        reinterpret_cast<double2*>(out + 4 * i)[1] = b;
    }
}

cudaError_t launch_elem_inv(bool viscous, cudaStream_t stream, int nelem, const int4* elem,
                            const double* U, const double* geo, const double* area,
                            const double* shoc, const double* dtl_arr, const double* dtl_scalar,
                            const double* ts1, const double* ts2, const double* ts3, GasConst gc,
                            double* cache, double* contrib, const double* WX, const double* WY,
                            double* contribF) {
    const unsigned grid = blocks_for(nelem, 128);
    if (viscous)
        k_elem_inv<true><<<grid, 128, 0, stream>>>(nelem, elem, U, geo, area, shoc, dtl_arr,
                                                   dtl_scalar, ts1, ts2, ts3, gc, cache, contrib,
                                                   WX, WY, contribF);
    else
        k_elem_inv<false><<<grid, 128, 0, stream>>>(nelem, elem, U, geo, area, shoc, dtl_arr,
                                                    dtl_scalar, ts1, ts2, ts3, gc, cache, contrib,
                                                    WX, WY, contribF);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

cudaError_t launch_elem_replay(cudaStream_t stream, int nelem, const int4* elem, const double* T,
                               const double* geo, const double* area, const double* dtl_arr,
                               const double* dtl_scalar, GasConst gc, const double* cache,
                               double* contrib) {
    k_elem_replay<<<blocks_for(nelem, 128), 128, 0, stream>>>(nelem, elem, T, geo, area, dtl_arr,
                                                               dtl_scalar, gc, cache, contrib);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ RK stage, node side
// subrutinas.f90:680-825 for one stage: RHS = ordered sum of the calcRHS then the FUENTE
// contributions of the node's elements; U1 = U - rk_fact/M*RHS; primitives; FIXVEL,
// NORMALVEL, FIX (applied per node: every node's list entries are resolved on the host
// with the reference's last-write-wins order); U1 rebuilt from the primitives.
__global__ void k_node_update(int npoin, const int* __restrict__ esup_ptr,
                              const int* __restrict__ esup_slot, const double* __restrict__ contrib,
                              const double* __restrict__ contribF, const double* __restrict__ U,
                              const double* __restrict__ M, double rk_fact, double gamm, double FR,
                              const unsigned char* __restrict__ bcflag,
                              const double* __restrict__ bcval, const double2* __restrict__ nrm,
                              const double* __restrict__ WX, const double* __restrict__ WY,
                              double* __restrict__ U1, double* __restrict__ RHO,
                              double* __restrict__ VX, double* __restrict__ VY,
                              double* __restrict__ Eo, double* __restrict__ Po,
                              double* __restrict__ To, double* __restrict__ RMACH,
                              const double* __restrict__ rhs_init, double* __restrict__ rhs_out) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoin) return;
    double r0 = 0.0, r1 = 0.0, r2 = 0.0, r3 = 0.0;
    if (rhs_init) {  // drop-in calls accumulate into the caller's rhs
        const double2* c = reinterpret_cast<const double2*>(rhs_init + 4 * (size_t)p);
        double2 a = c[0], b = c[1];
        r0 = a.x; r1 = a.y; r2 = b.x; r3 = b.y;
    }
    const int s0 = esup_ptr[p], s1 = esup_ptr[p + 1];
    for (int s = s0; s < s1; ++s) {
        const double2* c = reinterpret_cast<const double2*>(contrib + 4 * (size_t)esup_slot[s]);
        double2 a = c[0], b = c[1];
        r0 = r0 + a.x; r1 = r1 + a.y; r2 = r2 + b.x; r3 = r3 + b.y;
    }
    if (contribF) {
        for (int s = s0; s < s1; ++s) {
            const double2* c = reinterpret_cast<const double2*>(contribF + 4 * (size_t)esup_slot[s]);
            double2 a = c[0], b = c[1];
            r0 = r0 + a.x; r1 = r1 + a.y; r2 = r2 + b.x; r3 = r3 + b.y;
        }
    }
    if (rhs_out) {
        double2* o = reinterpret_cast<double2*>(rhs_out + 4 * (size_t)p);
        o[0] = make_double2(r0, r1);
        o[1] = make_double2(r2, r3);
    }
    if (!U1) return;
    const double2* u2 = reinterpret_cast<const double2*>(U + 4 * (size_t)p);
    double2 ua = u2[0], ub = u2[1];
    const double f = rk_fact / M[p];
    const double u1_0 = ua.x - f * r0, u1_1 = ua.y - f * r1, u1_2 = ub.x - f * r2, u1_3 = ub.y - f * r3;
    double rho = u1_0;
    double vx = u1_1 / rho, vy = u1_2 / rho, ee = u1_3 / rho;
    double vel2 = vx * vx + vy * vy;
    double pp = rho * (gamm - 1.0) * (ee - 0.5 * vel2);
    double tt = pp / (rho * FR);
    RMACH[p] = sqrt(vel2 / (tt * gamm * FR));
    Po[p] = pp;
    const unsigned char fl = bcflag[p];
    if (fl) {
        const double2* b2 = reinterpret_cast<const double2*>(bcval + 4 * (size_t)p);
        const double2 bva = b2[0], bvb = b2[1];
        const double4_32a bv = {bva.x, bva.y, bvb.x, bvb.y};
        if (fl & BC_FIXV) { vx = bv.x; vy = bv.y; }
        if (fl & BC_NORMAL) {
            double2 nn = nrm[p];
            double wx = WX[p], wy = WY[p];
            double q = -(nn.y * (vx - wx)) + nn.x * (vy - wy);
            vx = -(nn.y * q) + wx;
            vy = nn.x * q + wy;
        }
        if (fl & BC_FIXRHO) rho = bv.z;
        if (fl & BC_FIXT) {
            double gm = gamm - 1.0;
            tt = bv.w;
            ee = tt * FR / gm + 0.5 * (vx * vx + vy * vy);
        }
    }
    RHO[p] = rho; VX[p] = vx; VY[p] = vy; Eo[p] = ee; To[p] = tt;
    double2* o = reinterpret_cast<double2*>(U1 + 4 * (size_t)p);
    o[0] = make_double2(rho, vx * rho);
    o[1] = make_double2(vy * rho, ee * rho);
}

// ------------------------------------------------------------------ normales (gather)
// subrutinas.f90:21-63: per wall node, the wall edges touching it in edge order; the
// nodes kept by the reference's compaction (den > 1d-6 and |l| > 0.2) get BC_NORMAL.
__global__ void k_normales(int nwn, const int* __restrict__ wnode, const int* __restrict__ wptr,
                           const int2* __restrict__ wedge_of, const int2* __restrict__ walls,
                           const double* __restrict__ X, const double* __restrict__ Y,
                           unsigned char* __restrict__ bcflag, double2* __restrict__ nrm) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nwn) return;
    normales_node(NormalsArgs{nwn, wnode, wptr, wedge_of, walls, X, Y, bcflag, nrm}, k);
}

// ------------------------------------------------------------------ laplace values
// mLaplace.f90:28-56, row owner: row p walks its elements in esup order; lap_pos gives,
// per esup slot and local column j, the offset of node inpoel(j,e) within row p (the
// reference's linear search, done once on the host).
__device__ __forceinline__ double mesh_mu(const double* X3, const double* Y3) {
    const double TWOSQRT3 = 3.46410161513775;
    double a = X3[1] * Y3[2] + X3[2] * Y3[0] + X3[0] * Y3[1] -
               (X3[1] * Y3[0] + X3[2] * Y3[1] + X3[0] * Y3[2]);
    double l1 = (X3[2] - X3[1]) * (X3[2] - X3[1]) + (Y3[2] - Y3[1]) * (Y3[2] - Y3[1]);
    double l2 = (X3[0] - X3[2]) * (X3[0] - X3[2]) + (Y3[0] - Y3[2]) * (Y3[0] - Y3[2]);
    double l3 = (X3[1] - X3[0]) * (X3[1] - X3[0]) + (Y3[1] - Y3[0]) * (Y3[1] - Y3[0]);
    double l = l1 + l2 + l3;
    return TWOSQRT3 * a / l;
}

// Each element's weight q = 1/mu^2 (mLaplace.f90:40), formed once: the reference forms it
// for every (node, element) pair of its loop, with the same value each time
__global__ void k_lap_q(int nelem, const int4* __restrict__ elem, const double* __restrict__ X,
                        const double* __restrict__ Y, double* __restrict__ q) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    const int4 n = elem[e];
    const double X3[3] = {X[n.x], X[n.y], X[n.z]};
    const double Y3[3] = {Y[n.x], Y[n.y], Y[n.z]};
    const double m = mesh_mu(X3, Y3);
    q[e] = 1.0 / (m * m);
}

__global__ void k_laplace(int npoin, int nelem, const int* __restrict__ esup_ptr,
                          const int* __restrict__ esup_slot, const uchar4* __restrict__ lap_pos,
                          const double* __restrict__ geo, const double* __restrict__ qe,
                          const int* __restrict__ rowptr, double* __restrict__ vals,
                          double* __restrict__ diag) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoin) return;
    const size_t E = (size_t)nelem;
    const int r0 = rowptr[p], r1 = rowptr[p + 1];
    for (int k = r0; k < r1; ++k) vals[k] = 0.0;
    for (int s = esup_ptr[p]; s < esup_ptr[p + 1]; ++s) {
        const int slot = esup_slot[s];
        const int e = slot / 3, i = slot - 3 * e;
        const double q = qe[e];
        const double dxi = geo[i * E + e], dyi = geo[(3 + i) * E + e];
        uchar4 pos = lap_pos[s];
        const unsigned char pj[3] = {pos.x, pos.y, pos.z};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int k = r0 + pj[j];
            vals[k] = vals[k] + (dxi * geo[j * E + e] + dyi * geo[(3 + j) * E + e]) * q;
        }
    }
    diag[p] = vals[r0];
}

cudaError_t launch_laplace(cudaStream_t st, int npoin, int nelem, const int4* elem,
                           const int* esup_ptr, const int* esup_slot, const uchar4* lap_pos,
                           const double* geo, const double* X, const double* Y, const int* rowptr,
                           double* scratch, double* vals, double* diag) {
    k_lap_q<<<blocks_for(nelem, 256), 256, 0, st>>>(nelem, elem, X, Y, scratch);
    k_laplace<<<blocks_for(npoin, 128), 128, 0, st>>>(npoin, nelem, esup_ptr, esup_slot, lap_pos,
                                                      geo, scratch, rowptr, vals, diag);
    g_launches.fetch_add(2, std::memory_order_relaxed);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ FORCES
// meshMove.f90:167-192: pressure force and moment per set.  One block: edge terms in
// parallel, then the reference's serial order of accumulation by thread 0.
__global__ void k_forces(int nset_numb, const int* __restrict__ set_ptr,
                         const int2* __restrict__ set_edges, const double* __restrict__ P,
                         const double* __restrict__ X, const double* __restrict__ Y,
                         const double* __restrict__ xref, const double* __restrict__ yref,
                         StepScal* __restrict__ sc) {
    __shared__ double dfx[256], dfy[256], dm1[256], dm2[256];
    for (int s = 0; s < nset_numb; ++s) {
        double fx = 0.0, fy = 0.0, rm = 0.0;
        const double xr = xref[s], yr = yref[s];
        for (int base = set_ptr[s]; base < set_ptr[s + 1]; base += 256) {
            int k = base + threadIdx.x;
            if (k < set_ptr[s + 1]) {
                int2 ed = set_edges[k];
                double d_press = (P[ed.x] + P[ed.y]) / 2.0;
                double rlx = X[ed.x] - X[ed.y];
                double rly = Y[ed.y] - Y[ed.x];
                double a = d_press * rly, b = d_press * rlx;
                double xc = (X[ed.x] + X[ed.y]) / 2.0;
                double yc = (Y[ed.y] + Y[ed.x]) / 2.0;
                dfx[threadIdx.x] = a;
                dfy[threadIdx.x] = b;
                dm1[threadIdx.x] = b * (xc - xr);
                dm2[threadIdx.x] = a * (yc - yr);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                int cnt = min(256, set_ptr[s + 1] - base);
                for (int t = 0; t < cnt; ++t) {
                    fx = fx + dfx[t];
                    fy = fy + dfy[t];
                    rm = rm + dm1[t] - dm2[t];
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) { sc->fx[s] = fx; sc->fy[s] = fy; sc->rm[s] = rm; }
    }
}

// ------------------------------------------------------------------ TRANSF -> x_fix
// meshMove.f90:378-389 evaluated for each moving node of ilaux (its last set in the
// reference's loop order); fixed-movement nodes get 0 (meshMove.f90:80-82).
__global__ void k_transf(int nnmove, const int* __restrict__ fix_node, const int* __restrict__ fix_set,
                         const double* __restrict__ X, const double* __restrict__ Y,
                         const double* __restrict__ xref, const double* __restrict__ yref,
                         double ca, double sa, double yposr, double* __restrict__ xfix_x,
                         double* __restrict__ xfix_y) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nnmove) return;
    int s = fix_set[k];
    double dx = 0.0, dy = 0.0;
    if (s >= 0) {
        int n = fix_node[k];
        double distx = X[n] - xref[s];
        double disty = Y[n] - yref[s] + yposr;
        dx = ca * distx + sa * disty - distx;
        dy = -(sa * distx) + ca * disty - disty + yposr;
    }
    xfix_x[k] = dx;
    xfix_y[k] = dy;
}

// meshMove.f90:99-126: X += XPOS, W_X = XPOS/DTMIN (and y)
__global__ void k_motion_update(int npoin, const double* __restrict__ xpos, const double* __restrict__ ypos,
                                const StepScal* __restrict__ sc, double* __restrict__ X,
                                double* __restrict__ Y, double* __restrict__ WX,
                                double* __restrict__ WY) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoin) return;
    const double dt = sc->dtmin;
    double xp = xpos[p], yp = ypos[p];
    X[p] = X[p] + xp;
    WX[p] = xp / dt;
    Y[p] = Y[p] + yp;
    WY[p] = yp / dt;
}

}  // namespace cfd

namespace cfd {

// DT = min(DT, 10*DTMIN) (subrutinas.f90:211-215)
__global__ void k_dt_clamp(int nelem, double* __restrict__ DT, const StepScal* __restrict__ sc) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    if (DT[e] > sc->cota) DT[e] = sc->cota;
}

// bit pattern of the smallest positive finite value of x (minval of deriv's HH)
__global__ void k_min_positive(long n, const double* __restrict__ x, unsigned long long* bits) {
    unsigned long long m = 0x7ff0000000000000ull;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double v = x[i];
        if (v > 0.0 && v < 1.0e308) {
            unsigned long long b = (unsigned long long)__double_as_longlong(v);
            m = b < m ? b : m;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        unsigned long long o = __shfl_down_sync(0xffffffffu, m, off);
        m = o < m ? o : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMin(bits, m);
}

// ------------------------------------------------------------------ FORCE_VISC
// ns2DComp.ALE.f90:819-893: per wall edge of the force sets, the stress of its element on
// the edge's outward normal (Sutherland mu at the edge's mean T with the hard-coded 0.017,
// :838-840; element-mean pressure and velocity gradients), in the reference's operation
// order.  One thread per edge writes its two force terms and its SKIN.DAT row (:887); the
// per-set sums run in edge order in a second kernel, as the reference's loop does.
struct DnStrided {  // dNx(j, e) = dnx[e*se + j*sj], dNy likewise
    const double *dnx, *dny;
    size_t se, sj;
    __device__ void get(int e, double nx[3], double ny[3]) const {
        for (int j = 0; j < 3; ++j) {
            nx[j] = dnx[e * se + j * sj];
            ny[j] = dny[e * se + j * sj];
        }
    }
};
struct DnGeo8 {  // the mixed form's per-element float4 pair
    const float4* g;
    __device__ void get(int e, double nx[3], double ny[3]) const {
        const float4 a = g[2 * (size_t)e], b = g[2 * (size_t)e + 1];
        nx[0] = a.x; nx[1] = a.y; nx[2] = a.z;
        ny[0] = a.w; ny[1] = b.x; ny[2] = b.y;
    }
};

template <class Dn, class Fld>
__global__ void k_force_visc_terms(int nedges, const int2* __restrict__ edges,
                                   const int* __restrict__ eelem, const int4* __restrict__ elem,
                                   Dn dn, const Fld* __restrict__ P, const Fld* __restrict__ T,
                                   const Fld* __restrict__ VX, const Fld* __restrict__ VY,
                                   const double* __restrict__ X, const double* __restrict__ Y,
                                   double u_inf, double v_inf, double rho_inf, double t_inf,
                                   double* __restrict__ terms, double* __restrict__ skin) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nedges) return;
    const int2 ed = edges[k];
    const int nn1 = ed.x, nn2 = ed.y, ielem = eelem[k];
    const double temp = ((double)T[nn1] + (double)T[nn2]) / 2.0;
    const double smu = 110.0;
    const double r = temp / t_inf;
    const double fmu = 0.017 * (r * sqrt(r)) * (t_inf + smu) / (temp + smu);
    double rly = -(X[nn2] - X[nn1]);
    double rlx = Y[nn2] - Y[nn1];
    const double rmod = sqrt(rlx * rlx + rly * rly);
    rlx = rlx / rmod;
    rly = rly / rmod;
    double nx[3], ny[3];
    dn.get(ielem, nx, ny);
    const int4 el = elem[ielem];
    const int nn[3] = {el.x, el.y, el.z};
    double dux = 0.0, duy = 0.0, dvx = 0.0, dvy = 0.0, press = 0.0;
    for (int jj = 0; jj < 3; ++jj) {
        const double vx = VX[nn[jj]], vy = VY[nn[jj]];
        dux = dux + nx[jj] * vx;
        duy = duy + ny[jj] * vx;
        dvx = dvx + nx[jj] * vy;
        dvy = dvy + ny[jj] * vy;
        press = press + (double)P[nn[jj]];
    }
    press = div3(press);
    const double txx = -press - fmu * (2.0 / 3.0 * (dux + dvy) - 2.0 * dux);
    const double txy = fmu * (duy + dvx);
    const double tyx = txy;
    const double tyy = -press - fmu * (2.0 / 3.0 * (dux + dvy) - 2.0 * dvy);
    const double ttx = txx * rlx + txy * rly;
    const double tty = tyx * rlx + tyy * rly;
    const double tmod = -ttx * rly + tty * rlx;
    const double uu = u_inf * u_inf + v_inf * v_inf;
    terms[2 * k] = ttx * rmod;
    terms[2 * k + 1] = tty * rmod;
    if (skin) {
        skin[3 * k] = tmod / (.5 * rho_inf * uu);
        skin[3 * k + 1] = (X[nn2] + X[nn1]) / 2.0;
        skin[3 * k + 2] = press / 82713.27;
    }
}

__global__ void k_force_visc_sum(int nset, const int* __restrict__ set_ptr,
                                 const double* __restrict__ terms, double* __restrict__ fv) {
    const int s = threadIdx.x;
    if (s >= 10) return;
    double fx = 0.0, fy = 0.0;
    if (s < nset)
        for (int k = set_ptr[s]; k < set_ptr[s + 1]; ++k) {
            fx = fx + terms[2 * k];
            fy = fy + terms[2 * k + 1];
        }
    fv[s] = fx;
    fv[10 + s] = fy;
}

cudaError_t launch_force_visc(cudaStream_t st, int form, int nset, const int* set_ptr,
                              int nedges, const int2* edges, const int* eelem, const int4* elem,
                              const double* dnx, const double* dny, size_t se, size_t sj,
                              const float4* geo8, const void* P, const void* T, const void* VX,
                              const void* VY, const double* X, const double* Y, double u_inf,
                              double v_inf, double rho_inf, double t_inf, double* terms,
                              double* skin, double* fv) {
    const unsigned grid = blocks_for(nedges > 0 ? nedges : 1, 128);
    if (nedges > 0) {
        if (form == 0)
            k_force_visc_terms<<<grid, 128, 0, st>>>(
                nedges, edges, eelem, elem, DnStrided{dnx, dny, se, sj}, (const double*)P,
                (const double*)T, (const double*)VX, (const double*)VY, X, Y, u_inf, v_inf,
                rho_inf, t_inf, terms, skin);
        else
            k_force_visc_terms<<<grid, 128, 0, st>>>(
                nedges, edges, eelem, elem, DnGeo8{geo8}, (const float*)P, (const float*)T,
                (const float*)VX, (const float*)VY, X, Y, u_inf, v_inf, rho_inf, t_inf, terms,
                skin);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    k_force_visc_sum<<<1, 32, 0, st>>>(nset, set_ptr, terms, fv);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ step report
__global__ void k_pack_report(const StepScal* __restrict__ sc, const MotionScal* __restrict__ ms,
                              const int* __restrict__ it, const int* __restrict__ cv,
                              const double* __restrict__ rz, const GridBar* __restrict__ bar,
                              const int* __restrict__ wait_err, StepOut* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    out->sc = *sc;
    out->has_motion = ms != nullptr;
    if (ms) out->ms = *ms;
    for (int s = 0; s < 2; ++s) {
        out->it[s] = it[s];
        out->cv[s] = cv[s];
        out->rz[s] = rz[s];
        out->relres[s] = rz[2 + s];
    }
    out->bar_err = bar->err | (wait_err ? *wait_err : 0);
}

// ------------------------------------------------------------------ div3 self-test
// div3 against the division x / 3.0 over n inputs: a third raw 64-bit patterns (splitmix64
// of seed + i: every exponent and sign, zeros, subnormals, infinities, NaNs), a third
// values of magnitude 2^-40 .. 2^40, a third multiples of 3 times a power of two moved by
// up to +-2^12 ulps (quotients next to binade edges and halfway cases).  Counts the inputs
// whose results differ in any bit (two NaNs count as equal).
__global__ void k_selftest_div3(long long n, unsigned long long seed,
                                unsigned long long* __restrict__ bad) {
    unsigned long long local = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
        unsigned long long z = seed + (unsigned long long)i * 0x9e3779b97f4a7c15ull;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        unsigned long long bits = z;
        const int kind = (int)(i % 3);
        if (kind == 1) {  // sign | exponent 1023-40 .. 1023+40 | random significand
            const unsigned long long ex = 983ull + (z >> 52) % 81ull;
            bits = (z & 0x800fffffffffffffull) | (ex << 52);
        } else if (kind == 2) {  // 3 * 2^k, then +-(up to 4096) ulps
            const int k = (int)((z >> 40) % 121ull) - 60;
            const long long d = (long long)(z & 0x1fffull) - 4096;
            const long long b3 = __double_as_longlong(ldexp(3.0, k)) + d;
            bits = (unsigned long long)b3 | (z & 0x8000000000000000ull);
        }
        const double x = __longlong_as_double((long long)bits);
        const double a = div3(x), b = x / 3.0;
        if (__double_as_longlong(a) != __double_as_longlong(b) && !(a != a && b != b)) ++local;
    }
    if (local) atomicAdd(bad, local);
}

cudaError_t launch_selftest_div3(long long n, unsigned long long seed, unsigned long long* bad) {
    k_selftest_div3<<<152 * 8, 256>>>(n, seed, bad);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}

}  // namespace cfd

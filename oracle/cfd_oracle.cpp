// cfd_oracle.cpp — CPU restatement of the reference's FP64 step.
//
// TEST INFRASTRUCTURE ONLY (see cfd_oracle.h): the checker of the cfd_gb300 GPU path and
// the timed CPU baseline.  Build: oracle/build_oracle.py (g++ -O2 -ffp-contract=off
// -fopenmp).  Each routine cites the reference file:line it restates.  Parity with the
// reference is unpinned (no tests, fixtures or Fortran compiler for the reference).
#include "cfd_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// x**1.5d0, x**.5d0 and x**(-.5d0): see the header for why these compositions.  With
// or_set_pow_mode(1) they are std::pow (the C library's pow), which is how a Fortran
// compiler without unsafe-math options evaluates a real exponent: the mode measures how far
// a build of the reference that calls pow sits from the compositions.
int g_pow_mode = 0;
inline double pow15(double x) { return g_pow_mode ? std::pow(x, 1.5) : x * std::sqrt(x); }
inline double powm05(double x) { return g_pow_mode ? std::pow(x, -0.5) : 1.0 / std::sqrt(x); }
inline double pow05(double x) { return g_pow_mode ? std::pow(x, 0.5) : std::sqrt(x); }

// calcRHS and FUENTE scatter their element contributions with OpenMP atomics, as the
// reference does: with more than one thread the adds into a node arrive in thread order.
// With or_set_ordered_scatter(1) the elements are still formed in parallel but the adds
// run in element order afterwards, so any thread count gives the one-thread result.
int g_ordered_scatter = 0;

// The thread count of every parallel loop, given on each loop (num_threads) rather than
// through the OpenMP runtime's per-thread default, which another library in the same
// process (one that shares the runtime) may change.
int g_threads = 1;

// ESTAB's DUX/DUY evaluation (CFD_ESTAB_*), set by or_set_estab_mode / the case params
int g_estab_mode = CFD_ESTAB_REFERENCE;
double g_estab_eps = 1.0e-3;  // CFD_ESTAB_REGULARIZED: relative gradient scale
double g_dir[2] = {1.0, 0.0};  // CFD_ESTAB_REGULARIZED: freestream direction

struct Clock {
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    double sec() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

}  // namespace

extern "C" {

void or_set_threads(int n) { g_threads = n > 0 ? n : 1; }

void or_set_ordered_scatter(int on) { g_ordered_scatter = on; }
void or_set_estab_mode(int mode) { g_estab_mode = mode; }
void or_set_pow_mode(int mode) { g_pow_mode = mode; }
int or_get_pow_mode(void) { return g_pow_mode; }

// How many of x[0..n) give pow(x, 1.5) != x*sqrt(x), pow(x, -0.5) != 1/sqrt(x) and
// pow(x, 0.5) != sqrt(x) (the three non-integer powers of the reference's step)
void or_pow_census(int n, const double* x, long long* out3) {
    long long c15 = 0, cm05 = 0, c05 = 0;
    for (int i = 0; i < n; ++i) {
        const double v = x[i];
        if (std::pow(v, 1.5) != v * std::sqrt(v)) ++c15;
        if (std::pow(v, -0.5) != 1.0 / std::sqrt(v)) ++cm05;
        if (std::pow(v, 0.5) != std::sqrt(v)) ++c05;
    }
    out3[0] = c15;
    out3[1] = cm05;
    out3[2] = c05;
}
void or_set_estab_eps(double eps) { g_estab_eps = eps; }
void or_set_estab_dir(double ux, double uy) {
    const double n = std::sqrt(ux * ux + uy * uy);
    g_dir[0] = n > 0.0 ? ux / n : 1.0;
    g_dir[1] = n > 0.0 ? uy / n : 0.0;
}

int or_get_threads(void) {
#ifdef _OPENMP
    return g_threads;
#else
    return 1;
#endif
}

// deriv: subrutinas.f90:88-126
void or_deriv(int npoin, int nelem, const double* X, const double* Y, const int* inpoel,
              double* area, double* dNx, double* dNy, double* HH, double* HHX,
              double* HHY, double* hmin) {
    (void)npoin;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int e = 0; e < nelem; ++e) {
        double xl[3], yl[3];
        for (int i = 0; i < 3; ++i) {
            int p = inpoel[3 * e + i] - 1;
            xl[i] = X[p];
            yl[i] = Y[p];
        }
        // :106-107
        double a = (xl[1] * yl[2] + xl[2] * yl[0] + xl[0] * yl[1] -
                    (xl[1] * yl[0] + xl[2] * yl[1] + xl[0] * yl[2])) / 2.0;
        area[e] = a;
        // :110-115
        dNx[3 * e + 0] = (yl[1] - yl[2]) / (2.0 * a);
        dNx[3 * e + 1] = (yl[2] - yl[0]) / (2.0 * a);
        dNx[3 * e + 2] = (yl[0] - yl[1]) / (2.0 * a);
        dNy[3 * e + 0] = (xl[2] - xl[1]) / (2.0 * a);
        dNy[3 * e + 1] = (xl[0] - xl[2]) / (2.0 * a);
        dNy[3 * e + 2] = (xl[1] - xl[0]) / (2.0 * a);
        // :117-119
        if (HH) HH[e] = std::sqrt(a);
        if (HHX) HHX[e] = std::fabs(std::min(std::min(xl[2] - xl[1], xl[0] - xl[2]), xl[1] - xl[0]));
        if (HHY) HHY[e] = std::fabs(std::min(std::min(yl[2] - yl[1], yl[0] - yl[2]), yl[1] - yl[0]));
    }
    if (hmin) {  // :124-125
        double h = 0.0;
        for (int e = 0; e < nelem; ++e) {
            double v = std::sqrt(area[e]);
            if (e == 0 || v < h) h = v;
        }
        if (h > 1.0e10) h = 1.0e10;
        *hmin = h;
    }
}

// MASAS: subrutinas.f90:128-153 (element order)
void or_masas(int npoin, int nelem, const double* area, const int* inpoel, double* M) {
    for (int p = 0; p < npoin; ++p) M[p] = 0.0;
    for (int e = 0; e < nelem; ++e)
        for (int i = 0; i < 3; ++i) {
            int p = inpoel[3 * e + i] - 1;
            M[p] = M[p] + area[e] / 3.0;
        }
}

// deltat: subrutinas.f90:155-218 (serial, as the reference)
void or_deltat(int npoin, int nelem, const double* T, const double* VEL_X,
               const double* VEL_Y, const double* W_X, const double* W_Y,
               const double* area, const int* inpoel, double FSAFE, double FR,
               double GAMA, double T_inf, double* DT, double* DTMIN) {
    (void)npoin; (void)FR; (void)GAMA;  // VC = sqrt(GAMA*FR*T_iel) is computed but unused (:179)
    double dtmin = 1.0e20;
    for (int e = 0; e < nelem; ++e) {
        double vumax = 0.0, vvmax = 0.0;
        const int* n = inpoel + 3 * e;
        double T_iel = (T[n[0] - 1] + T[n[1] - 1] + T[n[2] - 1]) / 3.0;
        for (int i = 0; i < 3; ++i) {
            int p = n[i] - 1;
            double vu = std::fabs(VEL_X[p] - W_X[p]);
            double vv = std::fabs(VEL_Y[p] - W_Y[p]);
            if (vu > vumax) vumax = vu;
            if (vv > vvmax) vvmax = vv;
        }
        double hh = std::sqrt(2.0 * area[e]);
        double vel = pow05(vumax * vumax + vvmax * vvmax);  // :194 (**.5D0)
        const double smu = 110.0;
        double fmu = 0.017 * pow15(T_iel / T_inf) * (T_inf + smu) / (T_iel + smu);
        double et = fmu;
        double pe = (vel * hh) / (2.0 * et);
        double alpha = std::min(pe / 3.0, 1.0);
        double deltatu = 1.0 / (4.0 * et / (hh * hh) + alpha * vel / hh);
        double deltatc = 1.0 / (4.0 * et / (hh * hh));
        double dtelem = FSAFE / (1.0 / deltatc + 1.0 / deltatu);
        DT[e] = dtelem;
        if (dtelem < dtmin) dtmin = dtelem;
    }
    double cota = 10.0 * dtmin;  // :211-215
    for (int e = 0; e < nelem; ++e)
        if (DT[e] > cota) DT[e] = cota;
    *DTMIN = dtmin;
}

// ESTAB: subrutinas.f90:332-446 (serial, as the reference)
void or_estab(int npoin, int nelem, const double* U, const double* T, const double* GAMM,
              const double* VEL_X, const double* VEL_Y, const double* W_X,
              const double* W_Y, const double* dNx, const double* dNy, const int* inpoel,
              double GAMA, double FR, double DTMIN, double RHOINF, double TINF,
              double* SHOC, double* TS1, double* TS2, double* TS3) {
    (void)npoin; (void)GAMA;
    for (int e = 0; e < nelem; ++e) {
        int n1 = inpoel[3 * e] - 1, n2 = inpoel[3 * e + 1] - 1, n3 = inpoel[3 * e + 2] - 1;
        const double* DX = dNx + 3 * e;
        const double* DY = dNy + 3 * e;
        double gm = (GAMM[n1] + GAMM[n2] + GAMM[n3]) / 3.0;
        double tau = 0.0, h_rgne = 0.0, h_rgn = 0.0, h_jgn = 0.0;
        double rho_elem = (U[4 * n1] + U[4 * n2] + U[4 * n3]) / 3.0;
        double vx = (VEL_X[n1] + VEL_X[n2] + VEL_X[n3]) / 3.0;
        double vy = (VEL_Y[n1] + VEL_Y[n2] + VEL_Y[n3]) / 3.0;
        double wx = (W_X[n1] + W_X[n2] + W_X[n3]) / 3.0;
        double wy = (W_Y[n1] + W_Y[n2] + W_Y[n3]) / 3.0;
        vx = vx - wx;
        vy = vy - wy;
        double vel2 = std::sqrt(vx * vx + vy * vy);
        double drx = U[4 * n1] * DX[0] + U[4 * n2] * DX[1] + U[4 * n3] * DX[2];
        double dry = U[4 * n1] * DY[0] + U[4 * n2] * DY[1] + U[4 * n3] * DY[2];
        double dr2 = std::sqrt(drx * drx + dry * dry) + 1.0e-20;
        double dtx = T[n1] * DX[0] + T[n2] * DX[1] + T[n3] * DX[2];
        double dty = T[n1] * DY[0] + T[n2] * DY[1] + T[n3] * DY[2];
        double dt2 = std::sqrt(dtx * dtx + dty * dty) + 1.0e-20;
        double dux = vel2 * DX[0] + vel2 * DX[1] + vel2 * DX[2];  // :380-383 (A-4)
        double duy = vel2 * DY[0] + vel2 * DY[1] + vel2 * DY[2];
        if (g_estab_mode != CFD_ESTAB_REFERENCE) {
            dux = 0.0;
            duy = 0.0;
        }
        double du2 = std::sqrt(dux * dux + duy * duy) + 1.0e-20;
        double rtx = dtx / dt2, rty = dty / dt2;
        double rjx = drx / dr2, rjy = dry / dr2;
        double rux = dux / du2, ruy = duy / du2;
        if (g_estab_mode == CFD_ESTAB_REGULARIZED) {
            // unit vectors that stay unit vectors but are continuous in the state: the
            // gradient plus eps*scale*G_e along the freestream direction d, normalised;
            // the "velocity gradient" direction (zero in exact arithmetic) is d itself
            double ge = 0.0;
            for (int i = 0; i < 3; ++i) ge += std::sqrt(DX[i] * DX[i] + DY[i] * DY[i]);
            const double sr = g_estab_eps * rho_elem * ge;
            const double st = g_estab_eps * ((T[n1] + T[n2] + T[n3]) / 3.0) * ge;
            const double gx = drx + sr * g_dir[0], gy = dry + sr * g_dir[1];
            const double hx = dtx + st * g_dir[0], hy = dty + st * g_dir[1];
            const double gn = std::sqrt(gx * gx + gy * gy), hn = std::sqrt(hx * hx + hy * hy);
            rjx = gx / gn;
            rjy = gy / gn;
            rtx = hx / hn;
            rty = hy / hn;
            rux = g_dir[0];
            ruy = g_dir[1];
        }
        double temp = (T[n1] + T[n2] + T[n3]) / 3.0;
        double c = std::sqrt(gm * FR * temp);
        const double smu = 110.0;
        double fmu = 0.017 * pow15(temp / TINF) * (TINF + smu) / (temp + smu);
        for (int i = 0; i < 3; ++i) {
            double term1 = std::fabs(vx * DX[i] + vy * DY[i]);
            double term2 = std::fabs(rjx * DX[i] + rjy * DY[i]);
            double h1 = std::fabs(rtx * DX[i] + rty * DY[i]);
            double h2 = std::fabs(rux * DX[i] + ruy * DY[i]);
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
        TS1[e] = rrr;
        TS2[e] = rrr;
        TS3[e] = rrr;
        if (fmu != 0.0) {  // :433-440
            double tau_sung3 = (h_rgn * h_rgn) / (4.0 * fmu / RHOINF);
            double tau_sung3_e = (h_rgne * h_rgne) / (4.0 * fmu / RHOINF);
            TS2[e] = powm05(resumen + 1.0 / (tau_sung3 * tau_sung3));
            TS3[e] = powm05(resumen + 1.0 / (tau_sung3_e * tau_sung3_e));
        }
    }
}

// The adds of the held element rows r[e][i][q] into rhs, element by element: the order in
// which the one-thread loop makes them (the twelve adds of one element go to distinct
// entries, so only the element order matters).
static void scatter_in_order(double* rhs, const double* held, const int* inpoel, int nelem) {
    for (int e = 0; e < nelem; ++e)
        for (int i = 0; i < 3; ++i) {
            const int p = inpoel[3 * e + i] - 1;
            for (int q = 0; q < 4; ++q) rhs[4 * p + q] += held[12 * (size_t)e + 4 * i + q];
        }
}

// calcRHS: calcRHS.f90:4-154.  OpenMP atomics like the reference; 1 thread = element order.
void or_calcrhs(double* rhs, const double* U, const double* theta, const double* dNx,
                const double* dNy, const double* area, const double* shoc,
                const double* dtl, const double* ts1, const double* ts2,
                const double* ts3, const int* inpoel, int nelem, int npoin,
                const double* T, const double* gas6) {
    (void)npoin;
    const double Cv = gas6[0], lambda_ref = gas6[1], mu_ref = gas6[2], g = gas6[3];
    const double T_inf = gas6[4], cte = gas6[5];
    // N(3,3) of calcRHS.f90:18-23, N[i][k] = N(i+1,k+1)
    static const double N[3][3] = {{0.0, 0.5, 0.5}, {0.5, 0.0, 0.5}, {0.5, 0.5, 0.0}};
    const bool viscous = mu_ref > 2.2250738585072014e-308;  // tiny(0d0), :119
    const bool ordered = g_ordered_scatter && or_get_threads() > 1;
    std::vector<double> held(ordered ? 12 * (size_t)nelem : 0);
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int e = 0; e < nelem; ++e) {
        double r[3][4] = {{0}};
        const int p[3] = {inpoel[3 * e] - 1, inpoel[3 * e + 1] - 1, inpoel[3 * e + 2] - 1};
        const double Nx[3] = {dNx[3 * e], dNx[3 * e + 1], dNx[3 * e + 2]};
        const double Ny[3] = {dNy[3 * e], dNy[3 * e + 1], dNy[3 * e + 2]};
        double Ux[4], Uy[4];
        for (int q = 0; q < 4; ++q) {  // :43-44
            Ux[q] = U[4 * p[0] + q] * Nx[0] + U[4 * p[1] + q] * Nx[1] + U[4 * p[2] + q] * Nx[2];
            Uy[q] = U[4 * p[0] + q] * Ny[0] + U[4 * p[1] + q] * Ny[1] + U[4 * p[2] + q] * Ny[2];
        }
        const double tau[3] = {ts1[e], ts2[e], ts3[e]};  // :45-47 (per local node, A-3)
        const double nu = shoc[e] * cte;
        const double T_avg = (T[p[0]] + T[p[1]] + T[p[2]]) / 3.0;  // :49-51
        const double mu = mu_ref * pow15(T_avg / T_inf) * (T_inf + 110.0) / (T_avg + 110.0);
        const double lambda = lambda_ref * pow15(T_avg / T_inf) * (T_inf + 194.0) / (T_avg + 194.0);
        for (int k = 0; k < 3; ++k) {
            double Uk[4], th[4];
            for (int q = 0; q < 4; ++q) {  // :53-60
                Uk[q] = N[0][k] * U[4 * p[0] + q] + N[1][k] * U[4 * p[1] + q] + N[2][k] * U[4 * p[2] + q];
                th[q] = N[0][k] * theta[4 * p[0] + q] + N[1][k] * theta[4 * p[1] + q] + N[2][k] * theta[4 * p[2] + q];
            }
            const double rho = Uk[0];
            const double v1 = Uk[1] / rho, v2 = Uk[2] / rho, ev = Uk[3] / rho;
            const double V_sq = v1 * v1 + v2 * v2;
            double A[4];  // AiUi, :73-84
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
            double At[4];  // :86
            for (int q = 0; q < 4; ++q) At[q] = th[q] + A[q];
            double B1[4], B2[4];  // A1AiUi_theta, A2AiUi_theta, :88-107
            B1[0] = At[1];
            B1[1] = v1 * (-g + 3.0) * At[1] - v2 * (g - 1.0) * At[2] + (g - 1.0) * At[3] +
                    (0.5 * V_sq * (g - 1.0) - v1 * v1) * At[0];
            B1[2] = -(v1 * v2 * At[0]) + v1 * At[2] + v2 * At[1];
            B1[3] = g * v1 * At[3] - v1 * v2 * (g - 1.0) * At[2] +
                    v1 * (V_sq * (g - 1.0) - ev * g) * At[0] +
                    (-(0.5 * V_sq * (g - 1.0)) + ev * g - v1 * v1 * (g - 1.0)) * At[1];
            B2[0] = At[2];
            B2[1] = -(v1 * v2 * At[0]) + v1 * At[2] + v2 * At[1];
            B2[2] = -(v1 * (g - 1.0) * At[1]) + v2 * (-g + 3.0) * At[2] + (g - 1.0) * At[3] +
                    (0.5 * V_sq * (g - 1.0) - v2 * v2) * At[0];
            B2[3] = g * v2 * At[3] - v1 * v2 * (g - 1.0) * At[1] +
                    v2 * (V_sq * (g - 1.0) - ev * g) * At[0] +
                    (-(0.5 * V_sq * (g - 1.0)) + ev * g - v2 * v2 * (g - 1.0)) * At[2];
            for (int i = 0; i < 3; ++i)  // :109-117
                for (int q = 0; q < 4; ++q)
                    r[i][q] = r[i][q] + N[i][k] * A[q] + tau[i] * (Nx[i] * B1[q] + Ny[i] * B2[q]) +
                              nu * (Nx[i] * Ux[q] + Ny[i] * Uy[q]);
            if (viscous) {  // :119-137
                double K1[4], K2[4];
                K1[1] = 2.0 / 3.0 * mu * (-(2.0 * Ux[0] * v1) + 2.0 * Ux[1] + Uy[0] * v2 - Uy[2]) / rho;
                K1[2] = mu * (-(Ux[0] * v2) + Ux[2] - Uy[0] * v1 + Uy[1]) / rho;
                K1[3] = 1.0 / 3.0 *
                        (Cv * mu * (-(Uy[0] * v1 * v2) + 3.0 * Uy[1] * v2 - 2.0 * Uy[2] * v1) -
                         Ux[0] * (Cv * mu * (3.0 * V_sq + v1 * v1) - 3.0 * lambda * (V_sq - ev)) +
                         Ux[1] * v1 * (4.0 * Cv * mu - 3.0 * lambda) +
                         3.0 * Ux[2] * v2 * (Cv * mu - lambda) + 3.0 * Ux[3] * lambda) /
                        (Cv * rho);
                K2[1] = mu * (-(Ux[0] * v2) + Ux[2] - Uy[0] * v1 + Uy[1]) / rho;
                K2[2] = 2.0 / 3.0 * mu * (Ux[0] * v1 - Ux[1] - 2.0 * Uy[0] * v2 + 2.0 * Uy[2]) / rho;
                K2[3] = 1.0 / 3.0 *
                        (Cv * mu * (-(Ux[0] * v1 * v2) - 2.0 * Ux[1] * v2 + 3.0 * Ux[2] * v1) -
                         Uy[0] * (Cv * mu * (3.0 * V_sq + v2 * v2) - 3.0 * lambda * (V_sq - ev)) +
                         3.0 * Uy[1] * v1 * (Cv * mu - lambda) +
                         Uy[2] * v2 * (4.0 * Cv * mu - 3.0 * lambda) + 3.0 * Uy[3] * lambda) /
                        (Cv * rho);
                for (int i = 0; i < 3; ++i)
                    for (int q = 1; q < 4; ++q) r[i][q] = r[i][q] + (Nx[i] * K1[q] + Ny[i] * K2[q]);
            }
        }
        for (int i = 0; i < 3; ++i)  // :141
            for (int q = 0; q < 4; ++q) r[i][q] = r[i][q] * area[e] * dtl[e] / 3.0;
        if (ordered) {
            std::memcpy(&held[12 * (size_t)e], r, sizeof(r));
            continue;
        }
        for (int q = 0; q < 4; ++q)  // :143-150
            for (int i = 0; i < 3; ++i) {
#pragma omp atomic
                rhs[4 * p[i] + q] += r[i][q];
            }
    }
    if (ordered) scatter_in_order(rhs, held.data(), inpoel, nelem);
}

// FUENTE: subrutinas.f90:1036-1094
void or_fuente(double* rhs, const double* U, const double* W_X, const double* W_Y,
               const double* dNx, const double* dNy, const double* area,
               const double* dtl, const int* inpoel, int nelem, int npoin) {
    (void)npoin;
    // sp(:,k) of :1052-1054, sp[i][k] = sp(i+1,k+1)
    static const double sp[3][3] = {{0.5, 0.0, 0.5}, {0.5, 0.5, 0.0}, {0.0, 0.5, 0.5}};
    const bool ordered = g_ordered_scatter && or_get_threads() > 1;
    std::vector<double> held(ordered ? 12 * (size_t)nelem : 0);
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int e = 0; e < nelem; ++e) {
        const int p[3] = {inpoel[3 * e] - 1, inpoel[3 * e + 1] - 1, inpoel[3 * e + 2] - 1};
        double Ux[4], Uy[4];
        for (int q = 0; q < 4; ++q) {
            Ux[q] = U[4 * p[0] + q] * dNx[3 * e] + U[4 * p[1] + q] * dNx[3 * e + 1] + U[4 * p[2] + q] * dNx[3 * e + 2];
            Uy[q] = U[4 * p[0] + q] * dNy[3 * e] + U[4 * p[1] + q] * dNy[3 * e + 1] + U[4 * p[2] + q] * dNy[3 * e + 2];
        }
        const double AR = area[e] * dtl[e] / 3.0;
        double wx[3], wy[3];
        for (int k = 0; k < 3; ++k) {  // sum(sp(:,k)*w(ipoin(:))), left to right
            wx[k] = sp[0][k] * W_X[p[0]] + sp[1][k] * W_X[p[1]] + sp[2][k] * W_X[p[2]];
            wy[k] = sp[0][k] * W_Y[p[0]] + sp[1][k] * W_Y[p[1]] + sp[2][k] * W_Y[p[2]];
        }
        double r[3][4];
        for (int i = 0; i < 3; ++i)  // :1076-1078
            for (int q = 0; q < 4; ++q)
                r[i][q] = -(AR * (sp[i][0] * (Ux[q] * wx[0] + Uy[q] * wy[0]) +
                                  sp[i][1] * (Ux[q] * wx[1] + Uy[q] * wy[1]) +
                                  sp[i][2] * (Ux[q] * wx[2] + Uy[q] * wy[2])));
        if (ordered) {
            std::memcpy(&held[12 * (size_t)e], r, sizeof(r));
            continue;
        }
        for (int i = 0; i < 3; ++i)
            for (int q = 0; q < 4; ++q) {
#pragma omp atomic
                rhs[4 * p[i] + q] += r[i][q];
            }
    }
    if (ordered) scatter_in_order(rhs, held.data(), inpoel, nelem);
}

// gcl_mod::main: gcl.f90:8-46 (mode 1 literal divW, mode 2 dNy.W_y)
void or_gcl(double* M, const double* W_x, const double* W_y, const double* W_x_old,
            const double* W_y_old, const double* dNx, const double* dNy,
            const double* area, const double* area_old, const int* inpoel, int nelem,
            int npoin, double dt, int mode) {
    std::vector<double> tot1(npoin, 0.0), tot2(npoin, 0.0);
    const bool literal = (mode != CFD_MASS_GCL_CORRECTED);
    for (int e = 0; e < nelem; ++e) {
        const int* n = inpoel + 3 * e;
        double wx[3], wy[3], wxo[3], wyo[3];
        for (int i = 0; i < 3; ++i) {
            wx[i] = W_x[n[i] - 1];
            wy[i] = literal ? W_x[n[i] - 1] : W_y[n[i] - 1];
            wxo[i] = W_x_old[n[i] - 1];
            wyo[i] = literal ? W_x_old[n[i] - 1] : W_y_old[n[i] - 1];
        }
        const double* DX = dNx + 3 * e;
        const double* DY = dNy + 3 * e;
        double divW = DX[0] * wx[0] + DX[1] * wx[1] + DX[2] * wx[2] + DY[0] * wy[0] + DY[1] * wy[1] + DY[2] * wy[2];
        double divWo = DX[0] * wxo[0] + DX[1] * wxo[1] + DX[2] * wxo[2] + DY[0] * wyo[0] + DY[1] * wyo[1] + DY[2] * wyo[2];
        for (int i = 0; i < 3; ++i) {
            int p = n[i] - 1;
            tot1[p] = tot1[p] + divW * area[e] / 3.0;
            tot2[p] = tot2[p] + divWo * area_old[e] / 3.0;
        }
    }
    for (int p = 0; p < npoin; ++p) M[p] = M[p] + dt * (tot1[p] + tot2[p]) / 2.0;
}

// getEsup: pointNeighbor.f90:5-43 (1-based output)
int or_get_esup(const int* inpoel, int nelem, int npoin, int* esup1, int* esup2) {
    for (int i = 0; i <= npoin; ++i) esup2[i] = 0;
    for (int e = 0; e < nelem; ++e)
        for (int i = 0; i < 3; ++i) {
            int p = inpoel[3 * e + i];
            if (p < 1 || p > npoin) return CFD_ERR_MESH;
            esup2[p] += 1;  // esup2(ipoin+1) with 1-based ipoin
        }
    for (int p = 1; p <= npoin; ++p) esup2[p] += esup2[p - 1];
    for (int e = 0; e < nelem; ++e)
        for (int i = 0; i < 3; ++i) {
            int p = inpoel[3 * e + i];
            int istor = esup2[p - 1] + 1;
            esup2[p - 1] = istor;
            esup1[istor - 1] = e + 1;
        }
    for (int p = npoin; p >= 1; --p) esup2[p] = esup2[p - 1];
    esup2[0] = 0;
    return CFD_OK;
}

// getPsup: pointNeighbor.f90:45-91 (1-based output).  psup1 == NULL: count only.
int or_get_psup(const int* inpoel, int nelem, int npoin, int* psup1, int* psup2,
                int* npsup) {
    std::vector<int> esup1(3 * (size_t)nelem), esup2(npoin + 1);
    int st = or_get_esup(inpoel, nelem, npoin, esup1.data(), esup2.data());
    if (st) return st;
    std::vector<int> lpoin(npoin + 1, 0);
    std::vector<int> p2(npoin + 1, 0);
    int istor = 0;
    for (int ip = 1; ip <= npoin; ++ip) {
        for (int s = esup2[ip - 1]; s < esup2[ip]; ++s) {
            int e = esup1[s] - 1;
            for (int i = 0; i < 3; ++i) {
                int jp = inpoel[3 * e + i];
                if (jp != ip && lpoin[jp] != ip) {
                    if (psup1) psup1[istor] = jp;
                    ++istor;
                    lpoin[jp] = ip;
                }
            }
        }
        p2[ip] = istor;
    }
    if (psup2) std::memcpy(psup2, p2.data(), sizeof(int) * (npoin + 1));
    if (npsup) *npsup = istor;
    return CFD_OK;
}

// Mlaplace::initialize: mLaplace.f90:60-94
int or_laplace_pattern(const int* inpoel, int nelem, int npoin, int* lap_rowptr,
                       int* lap_idx, int* nnz) {
    int npsup = 0;
    int st = or_get_psup(inpoel, nelem, npoin, nullptr, nullptr, &npsup);
    if (st) return st;
    if (nnz) *nnz = npsup + npoin;
    if (!lap_idx) return CFD_OK;
    std::vector<int> psup1(npsup > 0 ? npsup : 1), psup2(npoin + 1);
    or_get_psup(inpoel, nelem, npoin, psup1.data(), psup2.data(), nullptr);
    lap_rowptr[0] = 0;
    for (int i = 2; i <= npoin + 1; ++i) lap_rowptr[i - 1] = psup2[i - 1] + i - 1;
    for (int ip = 1; ip <= npoin; ++ip) {
        lap_idx[lap_rowptr[ip - 1]] = ip;
        int ips = psup2[ip - 1];
        for (int k = lap_rowptr[ip - 1] + 1; k < lap_rowptr[ip]; ++k) lap_idx[k] = psup1[ips++];
    }
    return CFD_OK;
}

// mu of mLaplace.f90:96-108 (and smoothing.f90:305-317)
static inline double mesh_mu(const double* X3, const double* Y3) {
    const double TWOSQRT3 = 3.46410161513775;
    double a = X3[1] * Y3[2] + X3[2] * Y3[0] + X3[0] * Y3[1] -
               (X3[1] * Y3[0] + X3[2] * Y3[1] + X3[0] * Y3[2]);
    double l1 = (X3[2] - X3[1]) * (X3[2] - X3[1]) + (Y3[2] - Y3[1]) * (Y3[2] - Y3[1]);
    double l2 = (X3[0] - X3[2]) * (X3[0] - X3[2]) + (Y3[0] - Y3[2]) * (Y3[0] - Y3[2]);
    double l3 = (X3[1] - X3[0]) * (X3[1] - X3[0]) + (Y3[1] - Y3[0]) * (Y3[1] - Y3[0]);
    double l = l1 + l2 + l3;
    return TWOSQRT3 * a / l;
}

// Mlaplace::laplace: mLaplace.f90:7-58 (row-owner, esup order)
void or_laplace(const int* inpoel, const double* dNx, const double* dNy, int nelem,
                int npoin, const double* X, const double* Y, const int* esup1,
                const int* esup2, double* lap_sparse, const int* lap_idx,
                const int* lap_rowptr, double* lap_diag) {
    (void)nelem;
    for (int k = 0; k < lap_rowptr[npoin]; ++k) lap_sparse[k] = 0.0;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int ip = 1; ip <= npoin; ++ip) {
        for (int s = esup2[ip - 1]; s < esup2[ip]; ++s) {
            int e = esup1[s] - 1;
            double X3[3], Y3[3];
            for (int i = 0; i < 3; ++i) {
                X3[i] = X[inpoel[3 * e + i] - 1];
                Y3[i] = Y[inpoel[3 * e + i] - 1];
            }
            double m = mesh_mu(X3, Y3);
            double q = 1.0 / (m * m);
            for (int i = 0; i < 3; ++i) {
                if (inpoel[3 * e + i] != ip) continue;
                for (int j = 0; j < 3; ++j) {
                    int kp = inpoel[3 * e + j];
                    for (int k = lap_rowptr[ip - 1]; k < lap_rowptr[ip]; ++k)
                        if (lap_idx[k] == kp)
                            lap_sparse[k] = lap_sparse[k] +
                                (dNx[3 * e + i] * dNx[3 * e + j] + dNy[3 * e + i] * dNy[3 * e + j]) * q;
                }
            }
        }
        lap_diag[ip - 1] = lap_sparse[lap_rowptr[ip - 1]];
    }
}

// vecdot (biconjGrad.f90:153-169) with its OpenMP REDUCTION(+) order pinned to a fixed
// tree: chunks of 1024 products (256 lanes x 4 strided terms, then a 32-lane shuffle-down
// tree per warp and an 8-way tree over warps); chunk partials folded by 256 lanes with a
// stride of 256, then the same 256-lane tree.  The GPU kernels take exactly this order.
static double tree256(double* s) {
    double w[8];
    for (int wi = 0; wi < 8; ++wi) {
        double* v = s + 32 * wi;
        for (int off = 16; off > 0; off >>= 1)
            for (int l = 0; l < off; ++l) v[l] = v[l] + v[l + off];
        w[wi] = v[0];
    }
    for (int off = 4; off > 0; off >>= 1)
        for (int l = 0; l < off; ++l) w[l] = w[l] + w[l + off];
    return w[0];
}

double or_vecdot(int n, const double* x, const double* y) {
    const long nc = (n + 1023) / 1024;
    std::vector<double> part(nc > 0 ? nc : 1);
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (long c = 0; c < nc; ++c) {
        double s[256];
        long base = c * 1024;
        for (int t = 0; t < 256; ++t) {
            long i = base + t;
            double acc = (i < n) ? x[i] * y[i] : 0.0;
            for (int k = 1; k < 4; ++k) {
                long j = i + 256L * k;
                if (j < n) acc = acc + x[j] * y[j];
            }
            s[t] = acc;
        }
        part[c] = tree256(s);
    }
    double s[256];
    for (int t = 0; t < 256; ++t) {
        double acc = (t < nc) ? part[t] : 0.0;
        for (long c = t + 256; c < nc; c += 256) acc = acc + part[c];
        s[t] = acc;
    }
    return tree256(s);
}

// biCG: biconjGrad.f90:8-62 (+ vecdiv/vecsum/assign2/copy1/copy2/SpMV :64-190).
// tol_mode CFD_BICG_TOL_ABS is the reference's test (|r.z| > tol continues, :47; early exit
// on r.r < tol, :35).  The relative modes (not in the reference) test the same iterates on
// r.r <= tol^2 * ref.ref, with ref = b - A.x_D (x_D: the Dirichlet values, 0 elsewhere;
// ref(fix) = 0) or ref = r_0; r.r is the vecdot of the residual after its update.
void or_bicg_mode(const double* spMtx, const int* spIdx, const int* spRowptr,
                  const double* diagMtx, double* x, const double* b, const double* x_fix,
                  const int* x_fixIdx, int npoin, int nfix, double tol, int maxit, int tol_mode,
                  cfd_solve_info* info) {
    std::vector<double> y(npoin), p(npoin), r(npoin), z(npoin);
    auto spmv = [&](const double* v, double* out) {
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < npoin; ++i) {
            double dot = 0.0;
            for (int j = spRowptr[i]; j < spRowptr[i + 1]; ++j) dot = dot + spMtx[j] * v[spIdx[j] - 1];
            out[i] = dot;
        }
    };
    auto copy2 = [&](const double* v, double* out) {
        for (int i = 0; i < nfix; ++i) out[x_fixIdx[i] - 1] = 1.0e30 * v[x_fixIdx[i] - 1];
    };
    const bool rel = tol_mode != CFD_BICG_TOL_ABS;
    int k = 0;
    for (int i = 0; i < nfix; ++i) x[x_fixIdx[i] - 1] = 1.0 * x_fix[i];  // copy1
    double ref2 = 0.0;
    if (tol_mode == CFD_BICG_TOL_REL) {  // e = b - A.x_D, e(fix) = 0
        std::vector<double> xd(npoin, 0.0), e(npoin);
        for (int i = 0; i < nfix; ++i) xd[x_fixIdx[i] - 1] = x[x_fixIdx[i] - 1];
        spmv(xd.data(), e.data());
        for (int i = 0; i < npoin; ++i) e[i] = -1.0 * e[i] + b[i];
        for (int i = 0; i < nfix; ++i) e[x_fixIdx[i] - 1] = 0.0;
        ref2 = or_vecdot(npoin, e.data(), e.data());
    }
    spmv(x, y.data());
    copy2(x, y.data());
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int i = 0; i < npoin; ++i) r[i] = -1.0 * y[i] + b[i];  // vecsum(-1, y, b, r)
    for (int i = 0; i < nfix; ++i) r[x_fixIdx[i] - 1] = 0.0;  // assign2
    double rr = or_vecdot(npoin, r.data(), r.data());
    if (tol_mode == CFD_BICG_TOL_REL_R0) ref2 = rr;
    const double thr = (tol * tol) * ref2;
    auto relres = [&](double q) { return (rel && ref2 > 0.0) ? std::sqrt(q / ref2) : 0.0; };
    if (rel ? rr <= thr : rr < tol) {
        if (info) { info->iters = 0; info->converged = 1; info->rz = rr; info->relres = relres(rr); }
        return;
    }
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int i = 0; i < npoin; ++i) p[i] = r[i] / diagMtx[i];
    double err_new = or_vecdot(npoin, r.data(), p.data());
    spmv(p.data(), y.data());
    copy2(p.data(), y.data());
    double py = or_vecdot(npoin, p.data(), y.data());
    double alfa = err_new / py;
#pragma omp parallel for schedule(static) num_threads(g_threads)
    for (int i = 0; i < npoin; ++i) x[i] = alfa * p[i] + x[i];
    double err_old = err_new;
    while ((rel ? rr > thr : std::fabs(err_old) > tol) && k < maxit) {
        k = k + 1;
        const double malfa = -alfa;
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < npoin; ++i) {
            r[i] = malfa * y[i] + r[i];
            z[i] = r[i] / diagMtx[i];
        }
        err_new = or_vecdot(npoin, r.data(), z.data());
        if (rel) rr = or_vecdot(npoin, r.data(), r.data());
        double beta = err_new / err_old;
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < npoin; ++i) p[i] = beta * p[i] + z[i];
        spmv(p.data(), y.data());
        copy2(p.data(), y.data());
        py = or_vecdot(npoin, p.data(), y.data());
        alfa = err_new / py;
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < npoin; ++i) x[i] = alfa * p[i] + x[i];
        err_old = err_new;
    }
    if (info) {
        info->iters = k;
        info->converged = (rel ? rr > thr : std::fabs(err_old) > tol) ? 0 : 1;
        info->rz = std::fabs(err_old);
        info->relres = relres(rr);
    }
}

void or_bicg(const double* spMtx, const int* spIdx, const int* spRowptr,
             const double* diagMtx, double* x, const double* b, const double* x_fix,
             const int* x_fixIdx, int npoin, int nfix, double tol, int maxit,
             cfd_solve_info* info) {
    or_bicg_mode(spMtx, spIdx, spRowptr, diagMtx, x, b, x_fix, x_fixIdx, npoin, nfix, tol, maxit,
                 CFD_BICG_TOL_ABS, info);
}

// normales: subrutinas.f90:7-64 (wall-edge order).  Returns m.
// FORCE_VISC (ns2DComp.ALE.f90:819-893): per set and wall edge, the stress of the owning
// element (Sutherland mu at the edge's mean T, hard-coded 0.017, :838-840; velocity
// gradients through dNx, dNy; element-mean pressure) on the edge's outward normal.  F_VX,
// F_VY summed in edge order; skin (nullable) gets per edge, in set and edge order, the
// SKIN.DAT row (:887): SKIN, the edge's mean x, press/82713.27.  RMU and RHO of the
// reference's argument list are unused by its body and left out.
void or_force_visc(int nelem, int npoin, int nsets, const int* ielem_sets, const int* iset,
                   const int* inpoel, int nset_numb, double u_inf, double v_inf, double rho_inf,
                   double t_inf, const double* X, const double* Y, const double* P,
                   const double* T, const double* VEL_X, const double* VEL_Y, const double* dNx,
                   const double* dNy, double* F_VX, double* F_VY, double* skin) {
    (void)nelem;
    (void)npoin;
    (void)nsets;
    for (int s = 0; s < 10; ++s) {
        F_VX[s] = 0.0;
        F_VY[s] = 0.0;
    }
    long row = 0;
    for (int sn = 0; sn < nset_numb; ++sn)
        for (int ii = 0; ii < ielem_sets[sn]; ++ii) {
            const int* e = iset + 3 * (sn + 10 * (size_t)ii);
            const int nn1 = e[0] - 1, nn2 = e[1] - 1, ielem = e[2] - 1;
            const double temp = (T[nn1] + T[nn2]) / 2.0;
            const double smu = 110.0;
            const double r = temp / t_inf;
            const double fmu = 0.017 * pow15(r) * (t_inf + smu) / (temp + smu);
            double rly = -(X[nn2] - X[nn1]);
            double rlx = Y[nn2] - Y[nn1];
            const double rmod = std::sqrt(rlx * rlx + rly * rly);
            rlx = rlx / rmod;
            rly = rly / rmod;
            double dux = 0.0, duy = 0.0, dvx = 0.0, dvy = 0.0, press = 0.0;
            for (int jj = 0; jj < 3; ++jj) {
                const int nn = inpoel[3 * (size_t)ielem + jj] - 1;
                const double nx = dNx[3 * (size_t)ielem + jj], ny = dNy[3 * (size_t)ielem + jj];
                dux = dux + nx * VEL_X[nn];
                duy = duy + ny * VEL_X[nn];
                dvx = dvx + nx * VEL_Y[nn];
                dvy = dvy + ny * VEL_Y[nn];
                press = press + P[nn];
            }
            press = press / 3.0;
            const double txx = -press - fmu * (2.0 / 3.0 * (dux + dvy) - 2.0 * dux);
            const double txy = fmu * (duy + dvx);
            const double tyx = txy;
            const double tyy = -press - fmu * (2.0 / 3.0 * (dux + dvy) - 2.0 * dvy);
            const double ttx = txx * rlx + txy * rly;
            const double tty = tyx * rlx + tyy * rly;
            const double tmod = -ttx * rly + tty * rlx;
            const double uu = u_inf * u_inf + v_inf * v_inf;
            const double sk = tmod / (.5 * rho_inf * uu);
            F_VX[sn] = F_VX[sn] + ttx * rmod;
            F_VY[sn] = F_VY[sn] + tty * rmod;
            if (skin) {
                skin[3 * row] = sk;
                skin[3 * row + 1] = (X[nn2] + X[nn1]) / 2.0;
                skin[3 * row + 2] = press / 82713.27;
            }
            ++row;
        }
}

int or_normales(int npoin, int nwall, const int* wall, const double* X, const double* Y,
                int* n_ipoin, double* n_x, double* n_y) {
    std::vector<double> nlx(npoin, 0.0), nly(npoin, 0.0), den(npoin, 0.0);
    for (int w = 0; w < nwall; ++w) {
        int a = wall[2 * w] - 1, b = wall[2 * w + 1] - 1;
        double lex = Y[b] - Y[a];
        double ley = -(X[b] - X[a]);
        double le = std::sqrt(lex * lex + ley * ley);
        nlx[a] = nlx[a] + lex; nly[a] = nly[a] + ley; den[a] = den[a] + le;
        nlx[b] = nlx[b] + lex; nly[b] = nly[b] + ley; den[b] = den[b] + le;
    }
    int m = 0;
    for (int p = 0; p < npoin; ++p) {
        if (den[p] > 1.0e-6) {
            double lx = nlx[p] / den[p];
            double ly = nly[p] / den[p];
            double nrm = std::sqrt(lx * lx + ly * ly);
            if (nrm > 0.2) {
                n_ipoin[m] = p + 1;
                n_x[m] = lx / nrm;
                n_y[m] = ly / nrm;
                ++m;
            }
        }
    }
    return m;
}

}  // extern "C"

// ------------------------------------------------------------------ smoothing
// smoothing_mod: smoothing.f90:1-387, the setup-time path (no dX/dY: SWITCH_TOL_MOVE off)
namespace {

struct Smoother {
    int npoin, nelem;
    const int* inpoel;
    double* X;
    double* Y;
    std::vector<int> esup1, esup2, psup1, psup2;
    std::vector<char> smoothable;
    double H_MIN_GLOBAL = 1.0;
    static constexpr int MAX_ELEM_PER_NODE = 20, NITER = 100, MITER = 2, NTRY = 8;
    static constexpr double TOL_METRIC = 0.85, FACTOR_TOL_DIST = 1e-2, FACTOR_DELTA = 1e-2;
    static constexpr double FACTOR_PLUS = 1.0, FACTOR_STEP = 3.0;

    void loc(int e, double* xl, double* yl) const {
        for (int i = 0; i < 3; ++i) {
            xl[i] = X[inpoel[3 * e + i] - 1];
            yl[i] = Y[inpoel[3 * e + i] - 1];
        }
    }
    static double hfun(const double* xl, const double* yl) {  // :319-332
        double a = xl[1] * yl[2] + xl[2] * yl[0] + xl[0] * yl[1] -
                   (xl[1] * yl[0] + xl[2] * yl[1] + xl[0] * yl[2]);
        double d1 = std::fabs(xl[2] - xl[1]) + std::fabs(yl[2] - yl[1]);
        double d2 = std::fabs(xl[0] - xl[2]) + std::fabs(yl[0] - yl[2]);
        double d3 = std::fabs(xl[1] - xl[0]) + std::fabs(yl[1] - yl[0]);
        double d = d1 + d2 + d3;
        return std::fabs(a) / d;
    }
    // getMu_vec :173-199 (mu_vec 1-based positions stored 0-based); returns min_idx (1-based)
    int getMu_vec(double* mu_vec, int ip) const {
        int min_idx = 1;
        double mu_min = 1.0;
        for (int s = esup2[ip - 1]; s < esup2[ip]; ++s) {
            double xl[3], yl[3];
            loc(esup1[s] - 1, xl, yl);
            double m1 = mesh_mu(xl, yl);
            int pos = s - esup2[ip - 1] + 1;
            mu_vec[pos - 1] = m1;
            if (m1 < mu_min) { mu_min = m1; min_idx = pos; }
        }
        return min_idx;
    }
    double getMu_min(int ip) const {  // :201-219
        double r = 1.0;
        for (int s = esup2[ip - 1]; s < esup2[ip]; ++s) {
            double xl[3], yl[3];
            loc(esup1[s] - 1, xl, yl);
            double m1 = mesh_mu(xl, yl);
            if (m1 <= r) r = m1;
        }
        return r;
    }
    double getH_min(int ip) const {  // :274-291
        double r = 1.0;
        for (int s = esup2[ip - 1]; s < esup2[ip]; ++s) {
            double xl[3], yl[3];
            loc(esup1[s] - 1, xl, yl);
            double h1 = hfun(xl, yl);
            if (h1 < r) r = h1;
        }
        return r;
    }
    void getG(double* gx, double* gy, int ip, const double* mu_vec) {  // :221-243
        double delta = H_MIN_GLOBAL * FACTOR_DELTA;
        int n = esup2[ip] - esup2[ip - 1];
        double x_old = X[ip - 1];
        X[ip - 1] = X[ip - 1] + delta;
        getMu_vec(gx, ip);
        for (int i = 0; i < n; ++i) gx[i] = (gx[i] - mu_vec[i]) / delta;
        X[ip - 1] = x_old;
        double y_old = Y[ip - 1];
        Y[ip - 1] = Y[ip - 1] + delta;
        getMu_vec(gy, ip);
        for (int i = 0; i < n; ++i) gy[i] = (gy[i] - mu_vec[i]) / delta;
        Y[ip - 1] = y_old;
    }
    double getStep(const double* gx, const double* gy, const double* mu_vec, int min_idx,
                   int ip) const {  // :245-272
        double gxm = gx[min_idx - 1], gym = gy[min_idx - 1], mum = mu_vec[min_idx - 1];
        double g2 = gxm * gxm + gym * gym;
        double st = tol_move ? tol_move[ip - 1] / ((std::fabs(gxm) + std::fabs(gym)) * NITER)
                             : getH_min(ip) * FACTOR_STEP / (std::fabs(gxm) + std::fabs(gym));
        int n = esup2[ip] - esup2[ip - 1];
        for (int i = 0; i < n; ++i) {
            double gg = gxm * gx[i] + gym * gy[i];
            if (gg < 0) {
                double s1 = (mu_vec[i] - mum) / (g2 - gg);
                if (s1 < st) st = s1;
            }
        }
        return st;
    }
    void update_list(int ip) {  // :293-303
        for (int s = psup2[ip - 1]; s < psup2[ip]; ++s) smoothable[psup1[s] - 1] = 1;
    }
    void moveIpoin(int ip, double* mu_vec, int& min_idx, double& d_max) {  // :116-171
        double gx[MAX_ELEM_PER_NODE], gy[MAX_ELEM_PER_NODE];
        double x0 = X[ip - 1], y0 = Y[ip - 1];
        for (int it = 0; it < MITER; ++it) {
            double mu_min = mu_vec[min_idx - 1];
            double x_old = X[ip - 1], y_old = Y[ip - 1];
            getG(gx, gy, ip, mu_vec);
            double step = getStep(gx, gy, mu_vec, min_idx, ip);
            bool accepted = false;
            for (int j = 0; j < NTRY; ++j) {
                double dx = step * gx[min_idx - 1];
                double dy = step * gy[min_idx - 1];
                X[ip - 1] = X[ip - 1] + dx;
                Y[ip - 1] = Y[ip - 1] + dy;
                int mnew = getMu_vec(mu_vec, ip);
                if (mu_vec[mnew - 1] > mu_min * FACTOR_PLUS) {
                    min_idx = mnew;
                    accepted = true;
                    break;
                } else {
                    step = 0.5 * step;
                }
            }
            if (!accepted) {
                X[ip - 1] = x_old;
                Y[ip - 1] = y_old;
                break;
            }
        }
        double d_move = (X[ip - 1] - x0) * (X[ip - 1] - x0) + (Y[ip - 1] - y0) * (Y[ip - 1] - y0);
        if (d_move > d_max) d_max = d_move;
        if (d_move > 2.2250738585072014e-308) update_list(ip);
    }
    const int* order = nullptr;  // 0-based visiting order of the nodes (null: 1..npoin)
    const double* tol_move = nullptr;  // setTol_move (:372-386): |dX| + |dY| per node, or null
    int node_at(int k) const { return (order ? order[k] : k) + 1; }
    void laplacianSmoothing(const int* fixed) {  // :74-114
        for (int k = 0; k < npoin; ++k) {
            const int ip = node_at(k);
            if (!(smoothable[ip - 1] && !fixed[ip - 1])) continue;
            double xn = 0.0, yn = 0.0;
            double mu_old = getMu_min(ip);
            double xo = X[ip - 1], yo = Y[ip - 1];
            int n = psup2[ip] - psup2[ip - 1];
            for (int s = psup2[ip - 1]; s < psup2[ip]; ++s) {
                xn = xn + X[psup1[s] - 1];
                yn = yn + Y[psup1[s] - 1];
            }
            xn = xn / n;
            yn = yn / n;
            if (tol_move) {  // SWITCH_TOL_MOVE (:98-102)
                const double dX = xn - xo, dY = yn - yo;
                xn = xo + dX / (std::fabs(dX) + std::fabs(dY)) * tol_move[ip - 1] / 2 * FACTOR_STEP;
                yn = yo + dY / (std::fabs(dX) + std::fabs(dY)) * tol_move[ip - 1] / 2 * FACTOR_STEP;
            }
            X[ip - 1] = xn;
            Y[ip - 1] = yn;
            if (getMu_min(ip) < mu_old) {
                X[ip - 1] = xo;
                Y[ip - 1] = yo;
            }
        }
    }
    void checkMesh() {  // :351-370
        H_MIN_GLOBAL = 1.0;
        std::fill(smoothable.begin(), smoothable.end(), 0);
        for (int e = 0; e < nelem; ++e) {
            double xl[3], yl[3];
            loc(e, xl, yl);
            if (mesh_mu(xl, yl) < TOL_METRIC)
                for (int i = 0; i < 3; ++i) smoothable[inpoel[3 * e + i] - 1] = 1;
            double h1 = hfun(xl, yl);
            if (h1 < H_MIN_GLOBAL) H_MIN_GLOBAL = h1;
        }
    }
    double quality() const {  // getMeshQuality :334-349
        double q = 1.0;
        for (int e = 0; e < nelem; ++e) {
            double xl[3], yl[3];
            loc(e, xl, yl);
            double m1 = mesh_mu(xl, yl);
            if (m1 < q) q = m1;
        }
        return q;
    }
    int run(const int* fixed) {  // smoothing :21-72
        checkMesh();
        bool any = false;
        for (int i = 0; i < npoin; ++i) any = any || smoothable[i];
        if (!any) return 0;
        for (int it = 0; it < 2; ++it) laplacianSmoothing(fixed);
        double tol_dist = FACTOR_TOL_DIST * H_MIN_GLOBAL;
        double mu_vec[MAX_ELEM_PER_NODE];
        int iter;
        for (iter = 1; iter <= NITER; ++iter) {
            double d_max = 0.0;
            for (int k = 0; k < npoin; ++k) {
                const int ip = node_at(k);
                if (smoothable[ip - 1] && !fixed[ip - 1]) {
                    smoothable[ip - 1] = 0;
                    int min_idx = getMu_vec(mu_vec, ip);
                    if (mu_vec[min_idx - 1] < TOL_METRIC) moveIpoin(ip, mu_vec, min_idx, d_max);
                }
            }
            if (d_max < tol_dist) break;
        }
        return iter > NITER ? NITER : iter;
    }
};

}  // namespace

// The same algorithm visiting the nodes in `order` (0-based, a permutation) instead of node
// order in its Laplacian passes and sweeps: the reference's sequential semantics (each node
// sees every move made before it) in another order.  Test infrastructure for the GPU
// smoothing, which moves one colour of mutually non-adjacent nodes at a time: with its
// colour order here the two must agree exactly.
// tol_move: setTol_move's |dX| + |dY| per node (:372-386), or null (SWITCH_TOL_MOVE off).
extern "C" void or_smoothing_ordered(double* X, double* Y, const int* inpoel, const int* fixed,
                                     int npoin, int nelem, const int* order,
                                     const double* tol_move, int* iters_out,
                                     double* min_quality_out);

extern "C" void or_smoothing(double* X, double* Y, const int* inpoel, const int* fixed,
                             int npoin, int nelem, int* iters_out, double* min_quality_out) {
    or_smoothing_ordered(X, Y, inpoel, fixed, npoin, nelem, nullptr, nullptr, iters_out,
                         min_quality_out);
}

extern "C" void or_smoothing_ordered(double* X, double* Y, const int* inpoel, const int* fixed,
                                     int npoin, int nelem, const int* order,
                                     const double* tol_move, int* iters_out,
                                     double* min_quality_out) {
    Smoother s;
    s.order = order;
    s.tol_move = tol_move;
    s.npoin = npoin;
    s.nelem = nelem;
    s.inpoel = inpoel;
    s.X = X;
    s.Y = Y;
    s.esup1.resize(3 * (size_t)nelem);
    s.esup2.resize(npoin + 1);
    or_get_esup(inpoel, nelem, npoin, s.esup1.data(), s.esup2.data());
    int npsup = 0;
    or_get_psup(inpoel, nelem, npoin, nullptr, nullptr, &npsup);
    s.psup1.resize(npsup > 0 ? npsup : 1);
    s.psup2.resize(npoin + 1);
    or_get_psup(inpoel, nelem, npoin, s.psup1.data(), s.psup2.data(), nullptr);
    s.smoothable.assign(npoin, 0);
    int it = s.run(fixed);
    if (iters_out) *iters_out = it;
    if (min_quality_out) *min_quality_out = s.quality();
}

// ------------------------------------------------------------------ driver
// PROGRAM NSComp2D (ns2DComp.ALE.f90:8-282) with the module state made explicit.
enum { TM_DELTAT, TM_ESTAB, TM_CALCRHS, TM_FUENTE, TM_UPDATE, TM_FORCES, TM_TRANSF,
       TM_GRAD, TM_NORMALES, TM_DERIV, TM_MASAS, TM_LAPLACE, TM_N };

struct or_case {
    int npoin, nelem;
    cfd_params p;
    std::vector<int> inpoel;
    std::vector<double> X, Y;
    // BC lists (dataLoader.f90:130-199)
    std::vector<int> ifixrho; std::vector<double> rfixrho;
    std::vector<int> ifixv; std::vector<double> rfixvx, rfixvy;
    std::vector<int> ifixt; std::vector<double> rfixt;
    std::vector<int> wall;
    int nsets, nset_numb; int ielem_sets[10]; std::vector<int> iset;
    int nmove, nfix_move; std::vector<int> ilaux;
    // state
    std::vector<double> U, U1, RHS, UN, T, RHO, E, P, RMACH, VEL_X, VEL_Y, W_X, W_Y, GAMM;
    std::vector<double> area, dNx, dNy, M, DT, DTL, SHOC, TS1, TS2, TS3;
    std::vector<double> W_x_old, W_y_old, area_old;
    std::vector<int> esup1, esup2, lap_rowptr, lap_idx;
    std::vector<double> lap_sparse, lap_diag, xpos, ypos;
    std::vector<double> xprev[2];          // CFD_GUESS_EXTRAPOLATED: x_{n-2} of both solves
    double xhist_dt[2] = {0.0, 0.0};       // DTMIN of the last two steps
    int xhist_n = 0;                       // solutions kept
    int m = 0; std::vector<int> n_ipoin; std::vector<double> n_x, n_y;
    int iter = 0, bandera = 1;
    double time = 0.0, dtmin = 0.0, dtmin1 = 0.0, disn[2] = {0.0, 0.0};
    double veln[2] = {0.0, 0.0}, accn[2] = {0.0, 0.0};  // setNewmarkCondition (meshMove.f90:14-25)
    bool fv_each = false;  // FORCE_VISC every step at the print block's point
    int smooth_every = 0;    // smooth the moved mesh every this many steps (0: never)
    std::vector<int> sm_order;  // the visiting order of that smoothing (0-based)
    double fvx[10] = {0}, fvy[10] = {0};
    std::vector<double> skin;
    double fx[10], fy[10], rm[10];
    cfd_solve_info sx{}, sy{};
    double timers[TM_N] = {0};
};

namespace {

void geometry(or_case* c) {  // ns2DComp.ALE.f90:88-100 / :259-275
    Clock t;
    c->m = or_normales(c->npoin, (int)c->wall.size() / 2, c->wall.data(), c->X.data(),
                       c->Y.data(), c->n_ipoin.data(), c->n_x.data(), c->n_y.data());
    c->timers[TM_NORMALES] += t.sec();
    Clock t2;
    or_deriv(c->npoin, c->nelem, c->X.data(), c->Y.data(), c->inpoel.data(), c->area.data(),
             c->dNx.data(), c->dNy.data(), nullptr, nullptr, nullptr, nullptr);
    c->timers[TM_DERIV] += t2.sec();
}

void laplace_values(or_case* c) {
    Clock t;
    or_laplace(c->inpoel.data(), c->dNx.data(), c->dNy.data(), c->nelem, c->npoin, c->X.data(),
               c->Y.data(), c->esup1.data(), c->esup2.data(), c->lap_sparse.data(),
               c->lap_idx.data(), c->lap_rowptr.data(), c->lap_diag.data());
    c->timers[TM_LAPLACE] += t.sec();
}

// RK: subrutinas.f90:645-849 (NGAS=0)
void rk(or_case* c, double dtmin) {
    const int N = c->npoin;
    const cfd_params& p = c->p;
    const double gas6[6] = {p.fcv, p.fk, p.fmu, p.gama, p.t_inf, p.cte};
    const int NRK = 4;
    for (int irk = 1; irk <= NRK; ++irk) {
        const double rk_fact = 1.0 / (NRK + 1 - irk);
        if (irk == 1) {
            // CUARTO_ORDEN's output is zeroed before use (:673-674): theta = 0
            std::fill(c->UN.begin(), c->UN.end(), 0.0);
            Clock t;
            or_estab(N, c->nelem, c->U.data(), c->T.data(), c->GAMM.data(), c->VEL_X.data(),
                     c->VEL_Y.data(), c->W_X.data(), c->W_Y.data(), c->dNx.data(), c->dNy.data(),
                     c->inpoel.data(), p.gama, p.fr, dtmin, p.rho_inf, p.t_inf, c->SHOC.data(),
                     c->TS1.data(), c->TS2.data(), c->TS3.data());
            c->timers[TM_ESTAB] += t.sec();
        }
        std::fill(c->RHS.begin(), c->RHS.end(), 0.0);
        Clock t1;
        or_calcrhs(c->RHS.data(), c->U.data(), c->UN.data(), c->dNx.data(), c->dNy.data(),
                   c->area.data(), c->SHOC.data(), c->DTL.data(), c->TS1.data(), c->TS2.data(),
                   c->TS3.data(), c->inpoel.data(), c->nelem, N, c->T.data(), gas6);
        c->timers[TM_CALCRHS] += t1.sec();
        Clock t2;
        or_fuente(c->RHS.data(), c->U.data(), c->W_X.data(), c->W_Y.data(), c->dNx.data(),
                  c->dNy.data(), c->area.data(), c->DTL.data(), c->inpoel.data(), c->nelem, N);
        c->timers[TM_FUENTE] += t2.sec();
        Clock t3;
        double* U = c->U.data();
        double* U1 = c->U1.data();
        const double* R = c->RHS.data();
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < N; ++i) {  // :696-698 and :708-717
            for (int q = 0; q < 4; ++q) U1[4 * i + q] = U[4 * i + q] - rk_fact / c->M[i] * R[4 * i + q];
            double rho = U1[4 * i];
            c->RHO[i] = rho;
            c->VEL_X[i] = U1[4 * i + 1] / rho;
            c->VEL_Y[i] = U1[4 * i + 2] / rho;
            c->E[i] = U1[4 * i + 3] / rho;
            double vel2 = c->VEL_X[i] * c->VEL_X[i] + c->VEL_Y[i] * c->VEL_Y[i];
            c->P[i] = rho * (c->GAMM[i] - 1.0) * (c->E[i] - 0.5 * vel2);
            c->T[i] = c->P[i] / (rho * p.fr);
            c->RMACH[i] = std::sqrt(vel2 / (c->T[i] * c->GAMM[i] * p.fr));
        }
        for (size_t i = 0; i < c->ifixv.size(); ++i) {  // FIXVEL :601-616
            int j = c->ifixv[i] - 1;
            c->VEL_X[j] = c->rfixvx[i];
            c->VEL_Y[j] = c->rfixvy[i];
        }
        for (int i = 0; i < c->m; ++i) {  // NORMALVEL :66-85
            int ip = c->n_ipoin[i] - 1;
            double vx = c->VEL_X[ip], vy = c->VEL_Y[ip], wx = c->W_X[ip], wy = c->W_Y[ip];
            double pp = -(c->n_y[i] * (vx - wx)) + c->n_x[i] * (vy - wy);
            c->VEL_X[ip] = -(c->n_y[i] * pp) + wx;
            c->VEL_Y[ip] = c->n_x[i] * pp + wy;
        }
        for (size_t i = 0; i < c->ifixrho.size(); ++i) c->RHO[c->ifixrho[i] - 1] = c->rfixrho[i];  // FIX
        for (size_t i = 0; i < c->ifixt.size(); ++i) {
            int j = c->ifixt[i] - 1;
            double gm = c->GAMM[j] - 1.0;
            c->T[j] = c->rfixt[i];
            c->E[j] = c->T[j] * p.fr / gm + 0.5 * (c->VEL_X[j] * c->VEL_X[j] + c->VEL_Y[j] * c->VEL_Y[j]);
        }
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < N; ++i) {  // :820-825
            U1[4 * i] = c->RHO[i];
            U1[4 * i + 1] = c->VEL_X[i] * c->RHO[i];
            U1[4 * i + 2] = c->VEL_Y[i] * c->RHO[i];
            U1[4 * i + 3] = c->E[i] * c->RHO[i];
        }
        c->timers[TM_UPDATE] += t3.sec();
    }
}

// FORCES: meshMove.f90:153-194
void forces(or_case* c) {
    for (int s = 0; s < c->nset_numb; ++s) { c->fx[s] = 0.0; c->fy[s] = 0.0; c->rm[s] = 0.0; }
    for (int s = 0; s < c->nset_numb; ++s) {
        for (int ii = 0; ii < c->ielem_sets[s]; ++ii) {
            const int* e = c->iset.data() + 3 * (s + 10 * ii);
            int n1 = e[0] - 1, n2 = e[1] - 1;
            double d_press = (c->P[n1] + c->P[n2]) / 2.0;
            double rlx = c->X[n1] - c->X[n2];
            double rly = c->Y[n2] - c->Y[n1];
            double dfx = d_press * rly, dfy = d_press * rlx;
            c->fx[s] = c->fx[s] + dfx;
            c->fy[s] = c->fy[s] + dfy;
            double xc = (c->X[n1] + c->X[n2]) / 2.0;
            double yc = (c->Y[n2] + c->Y[n1]) / 2.0;
            c->rm[s] = c->rm[s] + dfy * (xc - c->p.xref[s]) - dfx * (yc - c->p.yref[s]);
        }
    }
}

// fluidStructure: meshMove.f90:28-142 with the motion law as an option
// NEWMARK_METHOD(H) (meshMove.f90:196-310) with MATVEC (:312-324) and GAUSS (:326-346) for
// NDIM = 2, statement by statement; DISN, VELN, ACCN and the load F are the module arrays.
void newmark_method(double H, const double F[2], double DISN[2], double VELN[2], double ACCN[2]) {
    const double GR = 1.0;                                       // :239
    const double GAMA = .5, BETA = .25;                          // :246
    const double A1 = 1.0 / (BETA * H * H), A2 = 1.0 / (BETA * H), A3 = 1.0 / (2.0 * BETA) - 1.0,
                 A4 = (1.0 - GAMA) * H, A5 = GAMA * H;            // :248
    const double A1D = GAMA / (BETA * H), A2D = GAMA / BETA - 1.0,
                 A3D = 0.5 * H * (GAMA / BETA - 2.0);            // :249
    double MASA[2][2], C[2][2], K[2][2], CTEN[2] = {0.0, 0.0};
    MASA[0][0] = 51.5; MASA[0][1] = -51.5 * .0429;               // :258-259
    MASA[1][0] = -51.5 * .0429; MASA[1][1] = 2.275;
    C[0][0] = 32.358 / GR; C[0][1] = 0.0;                        // :262-263
    C[1][0] = 0.0; C[1][1] = 5.718 / GR;
    K[0][0] = 50828.463 / GR; K[0][1] = 0.0;                     // :266-267
    K[1][0] = 0.0; K[1][1] = 35923.241 / GR;
    for (int i = 0; i < 2; ++i)                                  // :280 K=K+A1*MASA+A1D*C
        for (int j = 0; j < 2; ++j) K[i][j] = K[i][j] + A1 * MASA[i][j] + A1D * C[i][j];
    for (int I = 0; I < 1; ++I)                                  // :283-290
        for (int J = I + 1; J < 2; ++J) {
            CTEN[J] = K[J][I] / K[I][I];
            for (int l = I + 1; l < 2; ++l) K[J][l] = K[J][l] - CTEN[J] * K[I][l];
        }
    double DISS[2], VELS[2], ACCS[2], R[2], G[2], G1[2];
    for (int i = 0; i < 2; ++i) { DISS[i] = DISN[i]; VELS[i] = VELN[i]; ACCS[i] = ACCN[i]; }
    auto matvec = [](const double A[2][2], const double* X, double* AUX) {
        for (int i = 0; i < 2; ++i) {
            AUX[i] = 0.0;
            for (int j = 0; j < 2; ++j) AUX[i] = AUX[i] + A[i][j] * X[j];
        }
    };
    for (int i = 0; i < 2; ++i) G[i] = A1 * DISN[i] + A2 * VELN[i] + A3 * ACCN[i];  // :303
    matvec(MASA, G, G1);
    for (int i = 0; i < 2; ++i) R[i] = F[i] + G1[i];
    for (int i = 0; i < 2; ++i) G[i] = A1D * DISN[i] + A2D * VELN[i] + A3D * ACCN[i];  // :308
    matvec(C, G, G1);
    for (int i = 0; i < 2; ++i) R[i] = R[i] + G1[i];
    for (int I = 0; I < 1; ++I)                                  // GAUSS :333-337
        for (int J = I + 1; J < 2; ++J) R[J] = R[J] - CTEN[J] * R[I];
    for (int I = 1; I >= 0; --I) {                               // :340-346
        double S = 0.0;
        for (int J = I + 1; J < 2; ++J) S = S + K[I][J] * DISN[J];
        DISN[I] = (R[I] - S) / K[I][I];
    }
    for (int i = 0; i < 2; ++i) ACCN[i] = A1 * (DISN[i] - DISS[i]) - A2 * VELS[i] - A3 * ACCS[i];
    for (int i = 0; i < 2; ++i) VELN[i] = VELS[i] + A4 * ACCS[i] + A5 * ACCN[i];
}

// The moved mesh smoothed on the setTol_move path (smoothing.f90:372-386) with this step's
// displacement, the mesh-motion nodes fixed, in c->sm_order; W becomes the whole move over
// DTMIN at the nodes the smoothing moved.  The reference's loop has no such call (its calls
// of the older SMOOTH_MESH are commented out, meshMove.f90:133): this restates the GPU
// context's per-step smoothing option for its tests.
void smooth_moved_mesh(or_case* c, double dtmin) {
    const int N = c->npoin;
    std::vector<double> tol(N), xb(c->X), yb(c->Y);
    for (int i = 0; i < N; ++i) tol[i] = std::fabs(c->xpos[i]) + std::fabs(c->ypos[i]);
    std::vector<int> fixed(N, 0);
    for (int v : c->ilaux) fixed[v - 1] = 1;
    or_smoothing_ordered(c->X.data(), c->Y.data(), c->inpoel.data(), fixed.data(), N, c->nelem,
                         c->sm_order.empty() ? nullptr : c->sm_order.data(), tol.data(),
                         nullptr, nullptr);
    for (int i = 0; i < N; ++i) {
        const double dx = c->X[i] - xb[i], dy = c->Y[i] - yb[i];
        if (dx == 0.0 && dy == 0.0) continue;
        c->W_X[i] = (c->xpos[i] + dx) / dtmin;
        c->W_Y[i] = (c->ypos[i] + dy) / dtmin;
    }
}

// CFD_GUESS_EXTRAPOLATED (no counterpart in the reference, whose guess is the previous
// increment, meshMove.f90:97): the two solves start from the last two increments
// extrapolated with the mesh velocity linear in time through the last two steps' midpoints,
// x = c1 x_{n-1} + c2 x_{n-2}, h = (dt_n + dt1)/(dt1 + dt2), c1 = dt_n/dt1 (1 + h),
// c2 = -(dt_n/dt2) h; the previous increment until two are kept.  The rows biCG fixes are
// overwritten by their Dirichlet values in the solve.
void extrapolate_guess(or_case* c, double dtn) {
    const int N = c->npoin;
    const bool two = c->xhist_n >= 2;
    double c1 = 1.0, c2 = 0.0;
    if (two) {
        const double h = (dtn + c->xhist_dt[0]) / (c->xhist_dt[0] + c->xhist_dt[1]);
        c1 = dtn / c->xhist_dt[0] * (1.0 + h);
        c2 = -(dtn / c->xhist_dt[1]) * h;
    }
    double* x[2] = {c->xpos.data(), c->ypos.data()};
    for (int s = 0; s < 2; ++s) {
        double* xp = c->xprev[s].data();
        for (int i = 0; i < N; ++i) {
            const double x1 = x[s][i];
            if (two) x[s][i] = c1 * x1 + c2 * xp[i];
            xp[i] = x1;
        }
    }
    c->xhist_dt[1] = c->xhist_dt[0];
    c->xhist_dt[0] = dtn;
    c->xhist_n += 1;
}

void fluid_structure(or_case* c, double dtmin, double time) {
    const int N = c->npoin;
    std::vector<double> dxpos(N, 0.0), dypos(N, 0.0);
    const double PI = std::acos(-1.0);
    c->p.xref[1] = 1.4;  // :58
    c->p.yref[1] = 0.0;
    Clock tf;
    forces(c);
    c->timers[TM_FORCES] += tf.sec();
    double alphav = c->disn[1], yposrv = c->disn[0];
    if (c->p.motion_law == CFD_MOTION_HARMONIC) {
        double ph = 2.0 * PI * c->p.motion_freq * time;
        c->disn[0] = c->p.heave_amp * std::sin(ph);
        c->disn[1] = c->p.pitch_amp * std::sin(ph);
    } else if (c->p.motion_law == CFD_MOTION_NEWMARK) {
        // the load lines :61-62 and the NEWMARK_METHOD call :67, enabled
        double F[2];
        F[0] = std::cos(c->disn[1]) * c->fy[0] - std::sin(c->disn[1]) * c->fx[0];
        F[1] = c->rm[0] + 0.1 * std::sin(c->disn[1]) * c->fx[0] - std::cos(c->disn[1]) * 0.1 * c->fy[0];
        newmark_method(dtmin, F, c->disn, c->veln, c->accn);
    } else {
        const double ampli = PI / 8.0;
        c->disn[1] = ampli * std::sin(10.0 * time);  // :70
    }
    double alpha = c->disn[1] - alphav, yposr = c->disn[0] - yposrv;
    Clock tt;
    const double ca = std::cos(alpha), sa = std::sin(alpha);
    for (int s = 0; s < c->nset_numb; ++s)  // TRANSF :369-392
        for (int ii = 0; ii < c->ielem_sets[s]; ++ii)
            for (int jj = 0; jj < 2; ++jj) {
                int n = c->iset[3 * (s + 10 * ii) + jj] - 1;
                double distx = c->X[n] - c->p.xref[s];
                double disty = c->Y[n] - c->p.yref[s] + yposr;
                dxpos[n] = ca * distx + sa * disty - distx;
                dypos[n] = -(sa * distx) + ca * disty - disty + yposr;
            }
    c->timers[TM_TRANSF] += tt.sec();
    const int nn = c->nmove + c->nfix_move;
    std::vector<double> pos_aux(nn, 0.0), b(N, 0.0);
    if (c->p.guess_mode == CFD_GUESS_EXTRAPOLATED ||
        c->p.guess_mode == CFD_GUESS_LEARNED_EXTRAPOLATED)  // no network here: its fallback
        extrapolate_guess(c, dtmin);
    for (int i = 0; i < c->nmove; ++i) pos_aux[i] = dxpos[c->ilaux[i] - 1];
    Clock tg;
    or_bicg_mode(c->lap_sparse.data(), c->lap_idx.data(), c->lap_rowptr.data(), c->lap_diag.data(),
            c->xpos.data(), b.data(), pos_aux.data(), c->ilaux.data(), N, nn, c->p.bicg_tol,
            c->p.bicg_maxit, c->p.bicg_tol_mode, &c->sx);
    c->timers[TM_GRAD] += tg.sec();
    for (int i = 0; i < N; ++i) {
        c->X[i] = c->X[i] + c->xpos[i];
        c->W_X[i] = c->xpos[i] / dtmin;
    }
    for (int i = 0; i < c->nmove; ++i) pos_aux[i] = dypos[c->ilaux[i] - 1];
    Clock tg2;
    or_bicg_mode(c->lap_sparse.data(), c->lap_idx.data(), c->lap_rowptr.data(), c->lap_diag.data(),
            c->ypos.data(), b.data(), pos_aux.data(), c->ilaux.data(), N, nn, c->p.bicg_tol,
            c->p.bicg_maxit, c->p.bicg_tol_mode, &c->sy);
    c->timers[TM_GRAD] += tg2.sec();
    for (int i = 0; i < N; ++i) {
        c->Y[i] = c->Y[i] + c->ypos[i];
        c->W_Y[i] = c->ypos[i] / dtmin;
    }
}

void mass_update(or_case* c, double dt) {
    Clock t;
    if (c->p.mass_mode == CFD_MASS_MASAS) {
        or_masas(c->npoin, c->nelem, c->area.data(), c->inpoel.data(), c->M.data());
    } else {
        or_gcl(c->M.data(), c->W_X.data(), c->W_Y.data(), c->W_x_old.data(), c->W_y_old.data(),
               c->dNx.data(), c->dNy.data(), c->area.data(), c->area_old.data(),
               c->inpoel.data(), c->nelem, c->npoin, dt, c->p.mass_mode);
        c->W_x_old = c->W_X;  // putW
        c->W_y_old = c->W_Y;
        c->area_old = c->area;  // putArea
    }
    c->timers[TM_MASAS] += t.sec();
}

}  // namespace

extern "C" {

static void or_case_force_visc_now(or_case* c) {
    or_force_visc(c->nelem, c->npoin, c->nsets, c->ielem_sets, c->iset.data(), c->inpoel.data(),
                  c->nset_numb, c->p.u_inf, c->p.v_inf, c->p.rho_inf, c->p.t_inf, c->X.data(),
                  c->Y.data(), c->P.data(), c->T.data(), c->VEL_X.data(), c->VEL_Y.data(),
                  c->dNx.data(), c->dNy.data(), c->fvx, c->fvy, c->skin.data());
}

or_case* or_case_create(const cfd_mesh* mesh, const cfd_params* prm, int do_smoothing) {
    or_case* c = new or_case();
    const int N = mesh->npoin, NE = mesh->nelem;
    c->npoin = N;
    c->nelem = NE;
    c->p = *prm;
    if (c->p.bicg_maxit <= 0) c->p.bicg_maxit = 1000;
    if (!(c->p.bicg_tol > 0.0)) c->p.bicg_tol = 1.0e-10;
    c->inpoel.assign(mesh->inpoel, mesh->inpoel + 3 * (size_t)NE);
    c->X.assign(mesh->x, mesh->x + N);
    c->Y.assign(mesh->y, mesh->y + N);
    c->ifixrho.assign(mesh->ifixrho_node, mesh->ifixrho_node + mesh->nfixrho);
    c->rfixrho.assign(mesh->rfixrho_value, mesh->rfixrho_value + mesh->nfixrho);
    c->ifixv.assign(mesh->ifixv_node, mesh->ifixv_node + mesh->nfixv);
    c->rfixvx.assign(mesh->rfixv_valuex, mesh->rfixv_valuex + mesh->nfixv);
    c->rfixvy.assign(mesh->rfixv_valuey, mesh->rfixv_valuey + mesh->nfixv);
    c->ifixt.assign(mesh->ifixt_node, mesh->ifixt_node + mesh->nfixt);
    c->rfixt.assign(mesh->rfixt_value, mesh->rfixt_value + mesh->nfixt);
    c->wall.assign(mesh->wall, mesh->wall + 2 * (size_t)mesh->nwall);
    c->nsets = mesh->nsets;
    c->nset_numb = mesh->nset_numb;
    for (int i = 0; i < 10; ++i) c->ielem_sets[i] = mesh->ielem_sets[i];
    c->iset.assign(mesh->iset, mesh->iset + 30 * (size_t)mesh->nsets);
    c->nmove = mesh->nmove;
    c->nfix_move = mesh->nfix_move;
    c->ilaux.assign(mesh->ilaux, mesh->ilaux + mesh->nmove + mesh->nfix_move);
    auto z4 = [&](std::vector<double>& v) { v.assign(4 * (size_t)N, 0.0); };
    z4(c->U); z4(c->U1); z4(c->RHS); z4(c->UN);
    for (auto* v : {&c->T, &c->RHO, &c->E, &c->P, &c->RMACH, &c->VEL_X, &c->VEL_Y, &c->W_X,
                    &c->W_Y, &c->GAMM, &c->M, &c->lap_diag, &c->xpos, &c->ypos, &c->n_x, &c->n_y,
                    &c->W_x_old, &c->W_y_old, &c->xprev[0], &c->xprev[1]})
        v->assign(N, 0.0);
    c->n_ipoin.assign(N, 0);
    for (auto* v : {&c->area, &c->DT, &c->DTL, &c->SHOC, &c->TS1, &c->TS2, &c->TS3, &c->area_old})
        v->assign(NE, 0.0);
    c->dNx.assign(3 * (size_t)NE, 0.0);
    c->dNy.assign(3 * (size_t)NE, 0.0);
    // GAMM = GAMA; RESTART (ns2DComp.ALE.f90:59-60, :404-420), freestream
    const cfd_params& p = c->p;
    for (int i = 0; i < N; ++i) {
        c->GAMM[i] = p.gama;
        double rhoamb = p.rho_inf, tamb = p.t_inf, uamb = p.u_inf, vamb = p.v_inf;
        double pamb = p.rho_inf * p.fr * p.t_inf;
        c->U[4 * i] = rhoamb;
        c->U[4 * i + 1] = rhoamb * uamb;
        c->U[4 * i + 2] = rhoamb * vamb;
        double energia = pamb / ((c->GAMM[i] - 1.0) * rhoamb) + 0.5 * (uamb * uamb + vamb * vamb);
        c->U[4 * i + 3] = energia * rhoamb;
        c->VEL_X[i] = uamb;
        c->VEL_Y[i] = vamb;
        c->T[i] = tamb;
        c->RMACH[i] = (p.u_inf * p.u_inf + p.v_inf * p.v_inf) / std::sqrt(p.gama * p.fr * p.t_inf);
    }
    if (do_smoothing) {  // :63-76
        std::vector<int> fixed(N, 0);
        for (int i = 0; i < c->nmove + c->nfix_move; ++i) fixed[c->ilaux[i] - 1] = 1;
        or_smoothing(c->X.data(), c->Y.data(), c->inpoel.data(), fixed.data(), N, NE, nullptr, nullptr);
    }
    c->esup1.resize(3 * (size_t)NE);
    c->esup2.resize(N + 1);
    or_get_esup(c->inpoel.data(), NE, N, c->esup1.data(), c->esup2.data());
    int nnz = 0;
    or_laplace_pattern(c->inpoel.data(), NE, N, nullptr, nullptr, &nnz);
    c->lap_rowptr.resize(N + 1);
    c->lap_idx.resize(nnz);
    c->lap_sparse.assign(nnz, 0.0);
    or_laplace_pattern(c->inpoel.data(), NE, N, c->lap_rowptr.data(), c->lap_idx.data(), &nnz);
    geometry(c);
    or_masas(N, NE, c->area.data(), c->inpoel.data(), c->M.data());
    c->area_old = c->area;  // putArea at setup for the gcl wiring; W_old = 0
    laplace_values(c);
    return c;
}

void or_case_destroy(or_case* c) { delete c; }

// loop body ns2DComp.ALE.f90:140-280
int or_case_step(or_case* c, int nsteps, cfd_step_report* rep) {
    const int N = c->npoin;
    const int saved_mode = g_estab_mode;  // the case's mode for its steps only
    const double saved_dir[2] = {g_dir[0], g_dir[1]};
    g_estab_mode = c->p.estab_mode;
    or_set_estab_dir(c->p.u_inf, c->p.v_inf);
    for (int s = 0; s < nsteps; ++s) {
        c->iter += 1;
        Clock t;
        double dtmin = 0.0;
        or_deltat(N, c->nelem, c->T.data(), c->VEL_X.data(), c->VEL_Y.data(), c->W_X.data(),
                  c->W_Y.data(), c->area.data(), c->inpoel.data(), c->p.fsafe, c->p.fr,
                  c->p.gama, c->p.t_inf, c->DT.data(), &dtmin);
        c->timers[TM_DELTAT] += t.sec();
        if (c->bandera == 1) {  // :146-156
            c->dtmin1 = dtmin;
            c->bandera = 2;
        }
        double porc = std::fabs((dtmin - c->dtmin1) / dtmin);
        if (100.0 * porc <= 1.0) {
            dtmin = c->dtmin1;
        } else {
            c->dtmin1 = dtmin;
            c->bandera = 2;
        }
        if (c->p.itlocal != 0) {  // :159-164
            double dtfact = 1.0 - std::exp(-(c->iter * 4.6 / c->p.itlocal));
            for (int e = 0; e < c->nelem; ++e) c->DTL[e] = dtmin * dtfact + c->DT[e] * (1.0 - dtfact);
        } else {
            for (int e = 0; e < c->nelem; ++e) c->DTL[e] = dtmin;
        }
        c->time = c->time + dtmin;
        c->dtmin = dtmin;
        c->U1 = c->U;
        rk(c, dtmin);
        fluid_structure(c, dtmin, c->time);
        if (c->smooth_every > 0 && c->iter % c->smooth_every == 0) smooth_moved_mesh(c, dtmin);
        if (c->fv_each) {  // the print block (:224-230): after the move, before deriv
            c->skin.assign(3 * (size_t)std::max(1, (int)(c->iset.size() / 3)), 0.0);
            or_case_force_visc_now(c);
        }
        c->bandera += 1;
        if (c->p.moving == 1) {  // :259-275
            geometry(c);
            mass_update(c, dtmin);
            laplace_values(c);
        }
        c->U.swap(c->U1);  // :277-281 (U = U1)
    }
    g_estab_mode = saved_mode;
    g_dir[0] = saved_dir[0];
    g_dir[1] = saved_dir[1];
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->iter = c->iter;
        rep->time = c->time;
        rep->dtmin = c->dtmin;
        rep->bicg_iters[0] = c->sx.iters;
        rep->bicg_iters[1] = c->sy.iters;
        rep->bicg_rz[0] = c->sx.rz;
        rep->bicg_rz[1] = c->sy.rz;
        rep->bicg_relres[0] = c->sx.relres;
        rep->bicg_relres[1] = c->sy.relres;
        rep->bicg_converged[0] = c->sx.converged;
        rep->bicg_converged[1] = c->sy.converged;
        rep->nset_numb = c->nset_numb;
        for (int i = 0; i < 10; ++i) { rep->fx[i] = c->fx[i]; rep->fy[i] = c->fy[i]; rep->rm[i] = c->rm[i]; }
    }
    return CFD_OK;
}

void or_case_get(or_case* c, double* U, double* T, double* X, double* Y) {
    if (U) std::memcpy(U, c->U.data(), sizeof(double) * 4 * c->npoin);
    if (T) std::memcpy(T, c->T.data(), sizeof(double) * c->npoin);
    if (X) std::memcpy(X, c->X.data(), sizeof(double) * c->npoin);
    if (Y) std::memcpy(Y, c->Y.data(), sizeof(double) * c->npoin);
}

void or_case_get_fields(or_case* c, double* RHO, double* VEL_X, double* VEL_Y, double* E,
                        double* P, double* RMACH, double* W_X, double* W_Y) {
    const size_t n = sizeof(double) * c->npoin;
    if (RHO) std::memcpy(RHO, c->RHO.data(), n);
    if (VEL_X) std::memcpy(VEL_X, c->VEL_X.data(), n);
    if (VEL_Y) std::memcpy(VEL_Y, c->VEL_Y.data(), n);
    if (E) std::memcpy(E, c->E.data(), n);
    if (P) std::memcpy(P, c->P.data(), n);
    if (RMACH) std::memcpy(RMACH, c->RMACH.data(), n);
    if (W_X) std::memcpy(W_X, c->W_X.data(), n);
    if (W_Y) std::memcpy(W_Y, c->W_Y.data(), n);
}

void or_case_set_force_visc(or_case* c, int each_step) { c->fv_each = each_step != 0; }

void or_case_set_smoothing(or_case* c, int every, const int* order) {
    c->smooth_every = every;
    if (order) c->sm_order.assign(order, order + c->npoin);
    else c->sm_order.clear();
}

void or_case_force_visc(or_case* c, double* F_VX, double* F_VY, double* skin) {
    if (!c->fv_each) {
        c->skin.assign(3 * (size_t)std::max(1, (int)(c->iset.size() / 3)), 0.0);
        or_case_force_visc_now(c);
    }
    for (int s = 0; s < 10; ++s) {
        F_VX[s] = c->fvx[s];
        F_VY[s] = c->fvy[s];
    }
    if (skin) {
        int ne = 0;
        for (int s = 0; s < c->nset_numb; ++s) ne += c->ielem_sets[s];
        std::memcpy(skin, c->skin.data(), sizeof(double) * 3 * (size_t)ne);
    }
}

void or_case_get_motion(or_case* c, double* xpos, double* ypos) {
    if (xpos) std::memcpy(xpos, c->xpos.data(), sizeof(double) * c->npoin);
    if (ypos) std::memcpy(ypos, c->ypos.data(), sizeof(double) * c->npoin);
}

void or_case_get_geometry(or_case* c, double* area, double* dNx, double* dNy, double* M) {
    if (area) std::memcpy(area, c->area.data(), sizeof(double) * c->nelem);
    if (dNx) std::memcpy(dNx, c->dNx.data(), sizeof(double) * 3 * c->nelem);
    if (dNy) std::memcpy(dNy, c->dNy.data(), sizeof(double) * 3 * c->nelem);
    if (M) std::memcpy(M, c->M.data(), sizeof(double) * c->npoin);
}

void or_case_set_state(or_case* c, const double* U, const double* T, const double* VEL_X,
                       const double* VEL_Y) {
    const int N = c->npoin;
    if (U) std::memcpy(c->U.data(), U, sizeof(double) * 4 * N);
    if (T) std::memcpy(c->T.data(), T, sizeof(double) * N);
    if (VEL_X) std::memcpy(c->VEL_X.data(), VEL_X, sizeof(double) * N);
    else if (U) for (int i = 0; i < N; ++i) c->VEL_X[i] = c->U[4 * i + 1] / c->U[4 * i];
    if (VEL_Y) std::memcpy(c->VEL_Y.data(), VEL_Y, sizeof(double) * N);
    else if (U) for (int i = 0; i < N; ++i) c->VEL_Y[i] = c->U[4 * i + 2] / c->U[4 * i];
}

void or_case_set_mesh(or_case* c, const double* X, const double* Y, const double* W_X,
                      const double* W_Y, const double* xpos, const double* ypos) {
    const size_t n = sizeof(double) * c->npoin;
    if (X) std::memcpy(c->X.data(), X, n);
    if (Y) std::memcpy(c->Y.data(), Y, n);
    if (W_X) std::memcpy(c->W_X.data(), W_X, n);
    if (W_Y) std::memcpy(c->W_Y.data(), W_Y, n);
    if (xpos) std::memcpy(c->xpos.data(), xpos, n);
    if (ypos) std::memcpy(c->ypos.data(), ypos, n);
    if (X || Y) {
        geometry(c);
        or_masas(c->npoin, c->nelem, c->area.data(), c->inpoel.data(), c->M.data());
        laplace_values(c);
    }
}

void or_case_set_clock(or_case* c, int iter, double time, double dtmin1, int bandera,
                       double disn1, double disn2) {
    c->iter = iter;
    c->time = time;
    c->dtmin1 = dtmin1;
    c->bandera = bandera;
    c->disn[0] = disn1;
    c->disn[1] = disn2;
}

void or_case_timers(or_case* c, double* seconds, int max, int* n) {
    int k = max < TM_N ? max : TM_N;
    for (int i = 0; i < k; ++i) seconds[i] = c->timers[i];
    if (n) *n = k;
}

// one NEWMARK_METHOD step on a state (dis, vel, acc: 2 each), for unit tests
void or_newmark_step(double H, const double* F, double* dis, double* vel, double* acc) {
    newmark_method(H, F, dis, vel, acc);
}

}  // extern "C"

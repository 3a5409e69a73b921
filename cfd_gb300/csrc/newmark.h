// newmark.h — the 2-DOF structural model of meshMove.f90:196-367 (NEWMARK_METHOD, MATVEC,
// GAUSS): heave and pitch of the body under the fluid load, integrated with Newmark's
// average-acceleration scheme (gamma = 1/2, beta = 1/4).  The reference has the routine
// but disables its call (meshMove.f90:67) and the load lines (:61-62); CFD_MOTION_NEWMARK
// enables both.  The arithmetic follows the Fortran expressions in order (no FMA on the
// host side), so the FP64 form reproduces the oracle's restatement bit for bit.
//
// Host and device: the FP64 form runs it on the host after reading the step's forces, the
// mixed form in the last block of its motion-tail kernel.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define CFD_HD __host__ __device__
#else
#define CFD_HD
#endif

namespace cfd {

struct NewmarkState {
    double dis[2];  // DISN: heave, pitch
    double vel[2];  // VELN
    double acc[2];  // ACCN
};

// The load of the commented lines meshMove.f90:61-62 from set 1's pressure force and
// moment, in the body axes of the current pitch DISN(2)
CFD_HD inline void newmark_load(const NewmarkState& s, double fx, double fy, double rm,
                                double F[2]) {
    const double c = cos(s.dis[1]), sn = sin(s.dis[1]);
    F[0] = c * fy - sn * fx;
    F[1] = rm + 0.1 * sn * fx - c * 0.1 * fy;
}

// One NEWMARK_METHOD(H) step: the reference's mass, damping and stiffness matrices
// (meshMove.f90:251-261, GR = 1), the effective stiffness K + a1 M + a1d C triangularised
// (:275-283) and the back substitution of GAUSS (:329-346).
CFD_HD inline void newmark_step(NewmarkState& s, const double F[2], double H) {
    const double GAMA = 0.5, BETA = 0.25, GR = 1.0;
    const double A1 = 1.0 / (BETA * H * H), A2 = 1.0 / (BETA * H), A3 = 1.0 / (2.0 * BETA) - 1.0;
    const double A4 = (1.0 - GAMA) * H, A5 = GAMA * H;
    const double A1D = GAMA / (BETA * H), A2D = GAMA / BETA - 1.0;
    const double A3D = 0.5 * H * (GAMA / BETA - 2.0);
    const double M[2][2] = {{51.5, -51.5 * 0.0429}, {-51.5 * 0.0429, 2.275}};
    const double C[2][2] = {{32.358 / GR, 0.0}, {0.0, 5.718 / GR}};
    double K[2][2] = {{50828.463 / GR, 0.0}, {0.0, 35923.241 / GR}};
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) K[i][j] = K[i][j] + A1 * M[i][j] + A1D * C[i][j];
    const double cten = K[1][0] / K[0][0];
    K[1][1] = K[1][1] - cten * K[0][1];
    const double diss[2] = {s.dis[0], s.dis[1]}, vels[2] = {s.vel[0], s.vel[1]},
                 accs[2] = {s.acc[0], s.acc[1]};
    double G[2], R[2];
    for (int i = 0; i < 2; ++i) G[i] = A1 * s.dis[i] + A2 * s.vel[i] + A3 * s.acc[i];
    for (int i = 0; i < 2; ++i) R[i] = F[i] + (0.0 + M[i][0] * G[0] + M[i][1] * G[1]);
    for (int i = 0; i < 2; ++i) G[i] = A1D * s.dis[i] + A2D * s.vel[i] + A3D * s.acc[i];
    for (int i = 0; i < 2; ++i) R[i] = R[i] + (0.0 + C[i][0] * G[0] + C[i][1] * G[1]);
    R[1] = R[1] - cten * R[0];
    s.dis[1] = (R[1] - 0.0) / K[1][1];
    s.dis[0] = (R[0] - (0.0 + K[0][1] * s.dis[1])) / K[0][0];
    for (int i = 0; i < 2; ++i) s.acc[i] = A1 * (s.dis[i] - diss[i]) - A2 * vels[i] - A3 * accs[i];
    for (int i = 0; i < 2; ++i) s.vel[i] = vels[i] + A4 * accs[i] + A5 * s.acc[i];
}

}  // namespace cfd

// mpnn.cuh — the learned initial guess of the mesh-motion solve: an edge message-passing
// network over the mesh graph (point neighbours), 4 layers of width 64.
//
// The mesh-motion solve is linear, with one scalar operator for both components, so the
// displacement of any affine motion of the body, g = t + M (p - c) on the body and 0 on
// the outer boundary, is u = t Phi + M (Psi_x, Psi_y) with the three fields
// Phi = L^-1[1], Psi_x = L^-1[x - c_x], Psi_y = L^-1[y - c_y] (boundary data on the body).
// The network predicts those fields (Phi, Psi_x / L, Psi_y / L) from the mesh geometry
// alone; the guess combines them with the affine fit (t, M) of the prescribed body
// displacement.  Rigid motions of any angle are affine motions.
//
// The network, its features and its loss are restated in numpy by the test oracle
// (oracle/mpnn_ref.py); the packing of the parameters below is the one both use.
//   f (10 node features) -> h0 = relu(W_in f + b_in)
//   layer l: z_ij = A h_i + B h_j + C e_ij + c;  agg_i = mean_j relu(z_ij);
//            h_i += relu(U [h_i; agg_i] + u)
//   y = W_out h + b_out  (3 outputs)
#pragma once
#include <cuda_bf16.h>

#include "cfd_common.cuh"

namespace cfd {
namespace mpnn {

constexpr int F_IN = 10, HID = 64, E_F = 3, LAYERS = 4, OUT = 3;
constexpr int OFF_W_IN = 0, OFF_B_IN = HID * F_IN;
constexpr int LAYER0 = OFF_B_IN + HID;
// per layer: A (64x64) B (64x64) C (64x3) c (64) U (64x128) u (64)
constexpr int L_A = 0, L_B = HID * HID, L_C = 2 * HID * HID, L_c = L_C + HID * E_F,
              L_U = L_c + HID, L_u = L_U + HID * 2 * HID, L_SIZE = L_u + HID;
constexpr int OFF_W_OUT = LAYER0 + LAYERS * L_SIZE, OFF_B_OUT = OFF_W_OUT + OUT * HID;
constexpr int N_PARAMS = OFF_B_OUT + OUT;
__host__ __device__ constexpr int layer_off(int l) { return LAYER0 + l * L_SIZE; }

// node kinds
enum : int { KIND_FREE = 0, KIND_BODY = 1, KIND_OUTER = 2 };

// Globals of one graph: body geometry, and the least-squares affine fit g = t + M (p - c)
// of the prescribed body displacement
struct Globals {
    double cx, cy;  // mean body position
    double L;       // 2 max |p - c| over the body
    double R;       // mean |p - c| over the outer boundary
    double tx, ty;  // translation
    double m11, m12, m21, m22;
    double ea, eb;  // semi-axes of the body's second-moment ellipse (uniform sampling in
    double ec, es;  //   the parametric angle), cos and sin of its major-axis angle
};

}  // namespace mpnn
}  // namespace cfd

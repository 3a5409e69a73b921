// mpnn_kernels.cuh — declarations of the kernels in kernels_mpnn.cu.
#pragma once
#include "mpnn.cuh"

namespace cfd {
namespace mpnn {

constexpr int DT = 32;  // nodes per block of the FP32 dense kernels
constexpr int WG = 64;  // rows per weight-gradient partial

// kernels with a `gate` argument return at once when gate != null and *gate == 0
__global__ void k_globals(int nb, const int* bnode, const int* bkind, const double* gx,
                          const double* gy, const double* X, const double* Y, Globals* G,
                          const int* gate);
__global__ void k_scatter_bc(int nb, const int* bnode, const double* gx, const double* gy,
                             double* gnx, double* gny, const int* gate);
__global__ void k_fields_seed(int n, const float* y, const int* kind, const Globals* G, double* F);
__global__ void k_fields_guess(int n, const int* kind, const Globals* G, const double* F,
                               const double* x0, const double* x1, double* c0, double* c1);
__global__ void k_fields_update(int n, const int* kind, const Globals* G, const double* x0,
                                const double* x1, double* F);
__global__ void k_features(int n, const double* X, const double* Y, const int* kind,
                           const Globals* G, float* f, const int* gate);
__global__ void k_edge_features(int m, const int* src, const int* nbr, const double* X,
                                const double* Y, const Globals* G, float* e, const int* gate);
__global__ void k_dense(int n, const float* X1, int I1, const float* X2, int I2, const float* W,
                        const float* b, int O, float* Y);
__global__ void k_dense_t(int n, const float* dY, int O, const float* W, int I, float* dX);
__global__ void k_wgrad(int n, const float* dY, int O, const float* X1, int I1, const float* X2,
                        int I2, int with_bias, float* part);
__global__ void k_fold(int nchunk, int stride, const float* part, int accumulate, float* out);
__global__ void k_relu(long n, const float* a, float* h);
__global__ void k_residual(long n, const float* h0, const float* v, float* h1);
__global__ void k_relu_bwd(long n, const float* g, const float* a, float* d);
__global__ void k_add_dh(int n, const float* dhc, const float* dpqh, float* dh);
__global__ void k_edge_fwd(int m, const int* src, const int* nbr, const float* PQ, const float* e,
                           const float* C, const float* c, float* z);
__global__ void k_node_agg(int n, const int* ptr, const float* z, float* agg);
__global__ void k_edge_bwd(int m, const int* src, const int* ptr, const float* dhc, const float* z,
                           float* dz);
__global__ void k_node_dpq(int n, const int* ptr, const int* rev, const float* dz, float* dPQ);
__global__ void k_loss(int n, const float* y, const float* t, const int* kind, float inv_nfree,
                       float* dy, float* part);
__global__ void k_adam(int np, float* w, const float* g, float* m, float* v, float lr, float b1,
                       float b2, float eps, float bc1, float bc2);
__global__ void k_targets(int n, const double* phi, const double* psx, const double* psy,
                          const Globals* G, float* t);
__global__ void k_guess(int n, const float* y, const int* kind, const double* gnx,
                        const double* gny, const Globals* G, double* ux, double* uy,
                        const int* gate);

// BF16 tensor-core inference: y[n][OUT] from the features; wb (BF16 copy of w) is refreshed
// when *wb_valid is false
int infer_bf16(cudaStream_t st, const float* w, __nv_bfloat16* wb, bool* wb_valid, int n,
               const int* ptr, const int* nbr, const float* f, const float* e,
               __nv_bfloat16* hb, __nv_bfloat16* pqb, float* y, const int* gate, int* err);

}  // namespace mpnn
}  // namespace cfd

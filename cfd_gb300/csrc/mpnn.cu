// mpnn.cu — host side of the learned mesh-motion guess: the network object (parameters,
// Adam state, BF16 copy for inference), the graph object (mesh adjacency, features, the
// buffers of one forward/backward pass) and their extern "C" entries (include/cfd_gpu.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "cfd_context.cuh"
#include "host_prep.h"
#include "mpnn.cuh"
#include "mpnn_kernels.cuh"

using namespace cfd;
using namespace cfd::mpnn;

namespace cfd {
namespace mpnn {

template <class T>
static int dev_alloc(std::vector<void*>& owned, T** p, size_t n) {
    void* v = nullptr;
    CFD_CUDA(cudaMalloc(&v, (n ? n : 1) * sizeof(T)));
    owned.push_back(v);
    *p = (T*)v;
    return CFD_OK;
}

}  // namespace mpnn
}  // namespace cfd

struct cfd_mpnn {
    std::vector<void*> owned;
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16* wb = nullptr;  // BF16 weights (inference)
    bool wb_valid = false;
    int t = 0;  // Adam step count
    ~cfd_mpnn() {
        for (void* p : owned) cudaFree(p);
    }
};

struct cfd_mpnn_graph {
    std::vector<void*> owned;
    cudaStream_t stream = nullptr;
    int n = 0, m = 0, nb = 0, nfree = 0;
    int *ptr = nullptr, *nbr = nullptr, *src = nullptr, *rev = nullptr, *kind = nullptr;
    int *bnode = nullptr, *bkind = nullptr;
    double *X = nullptr, *Y = nullptr, *bgx = nullptr, *bgy = nullptr, *gnx = nullptr,
           *gny = nullptr;
    Globals* G = nullptr;
    // refined learned guess: per-node basis fields (3 planes of n doubles), allocated on
    // first use
    double* F = nullptr;
    float *f = nullptr, *e = nullptr, *target = nullptr;
    // forward cache
    float* a0 = nullptr;                 // n x HID (pre-activation of h0)
    float* h[LAYERS + 1] = {};           // n x HID
    float* agg[LAYERS] = {};             // n x HID
    float* v[LAYERS] = {};               // n x HID
    float* z[LAYERS] = {};               // m x HID
    float *pq = nullptr, *y = nullptr;   // n x 2HID, n x OUT
    // backward
    float *dy = nullptr, *dh = nullptr, *dhc = nullptr, *dz = nullptr, *dpq = nullptr,
          *dpqh = nullptr, *part = nullptr, *lpart = nullptr;
    size_t part_floats = 0;
    // inference (BF16)
    __nv_bfloat16 *hb = nullptr, *pqb = nullptr;
    float* yb = nullptr;
    int* tc_err = nullptr;  // set when a tensor-core pass's bounded wait gave up
    double *ux = nullptr, *uy = nullptr, *uz = nullptr;
    bool training = false;
    ~cfd_mpnn_graph() {
        if (stream) {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
        for (void* p : owned) cudaFree(p);
    }
};

namespace {

int arg_err(const char* what) {
    set_last_message(std::string("invalid argument: ") + what);
    return CFD_ERR_ARG;
}

inline unsigned nb_of(long n, int t) { return blocks_for(n, t); }

// Y = [X1|X2] W^T + b
int dense(cudaStream_t st, int n, const float* X1, int I1, const float* X2, int I2,
          const float* W, const float* b, int O, float* Y) {
    CFD_LAUNCH(k_dense, nb_of(n, DT), 128, 0, st, n, X1, I1, X2, I2, W, b, O, Y);
    return CFD_OK;
}

int dense_t(cudaStream_t st, int n, const float* dY, int O, const float* W, int I, float* dX) {
    CFD_LAUNCH(k_dense_t, nb_of(n, DT), 128, 0, st, n, dY, O, W, I, dX);
    return CFD_OK;
}

// gradient of the weights W (O x (I1+I2)) [and bias] into out (+= when accumulate)
int wgrad(cudaStream_t st, cfd_mpnn_graph& g, int rows, const float* dY, int O, const float* X1,
          int I1, const float* X2, int I2, bool bias, float* out) {
    const int I = I1 + I2;
    const int nchunk = (int)nb_of(rows, WG);
    const int stride = O * I + (bias ? O : 0);
    if ((size_t)nchunk * stride > g.part_floats) {
        set_last_message("mpnn: gradient partial buffer too small");
        return CFD_ERR_LIMIT;
    }
    const size_t smem = sizeof(float) * WG * (O + I);
    CFD_LAUNCH(k_wgrad, nchunk, 256, smem, st, rows, dY, O, X1, I1, X2, I2, bias ? 1 : 0, g.part);
    CFD_LAUNCH(k_fold, nb_of(stride, 256), 256, 0, st, nchunk, stride, (const float*)g.part, 0, out);
    return CFD_OK;
}

int forward_fp32(cfd_mpnn& net, cfd_mpnn_graph& g) {
    cudaStream_t st = g.stream;
    const int n = g.n, m = g.m;
    const long nh = (long)n * HID, mh = (long)m * HID;
    int rc;
    if ((rc = dense(st, n, g.f, F_IN, nullptr, 0, net.w + OFF_W_IN, net.w + OFF_B_IN, HID, g.a0)))
        return rc;
    CFD_LAUNCH(k_relu, nb_of(nh, 256), 256, 0, st, nh, (const float*)g.a0, g.h[0]);
    for (int l = 0; l < LAYERS; ++l) {
        const float* W = net.w + layer_off(l);
        if ((rc = dense(st, n, g.h[l], HID, nullptr, 0, W + L_A, nullptr, 2 * HID, g.pq))) return rc;
        CFD_LAUNCH(k_edge_fwd, nb_of(mh, 256), 256, 0, st, m, g.src, g.nbr, (const float*)g.pq,
                   (const float*)g.e, W + L_C, W + L_c, g.z[l]);
        CFD_LAUNCH(k_node_agg, nb_of(nh, 256), 256, 0, st, n, g.ptr, (const float*)g.z[l], g.agg[l]);
        if ((rc = dense(st, n, g.h[l], HID, g.agg[l], HID, W + L_U, W + L_u, HID, g.v[l]))) return rc;
        CFD_LAUNCH(k_residual, nb_of(nh, 256), 256, 0, st, nh, (const float*)g.h[l],
                   (const float*)g.v[l], g.h[l + 1]);
    }
    return dense(st, n, g.h[LAYERS], HID, nullptr, 0, net.w + OFF_W_OUT, net.w + OFF_B_OUT, OUT, g.y);
}

int backward_fp32(cfd_mpnn& net, cfd_mpnn_graph& g, float* loss_out) {
    cudaStream_t st = g.stream;
    const int n = g.n, m = g.m;
    const long nh = (long)n * HID, mh = (long)m * HID;
    int rc;
    const int nlb = (int)nb_of(n, 256);
    CFD_LAUNCH(k_loss, nlb, 256, 0, st, n, (const float*)g.y, (const float*)g.target, g.kind,
               1.f / (float)std::max(g.nfree, 1), g.dy, g.lpart);
    float* lsum = g.lpart + nlb;
    CFD_LAUNCH(k_fold, 1, 256, 0, st, nlb, 1, (const float*)g.lpart, 0, lsum);
    // decoder
    if ((rc = wgrad(st, g, n, g.dy, OUT, g.h[LAYERS], HID, nullptr, 0, true, net.g + OFF_W_OUT)))
        return rc;
    if ((rc = dense_t(st, n, g.dy, OUT, net.w + OFF_W_OUT, HID, g.dh))) return rc;
    for (int l = LAYERS - 1; l >= 0; --l) {
        const float* W = net.w + layer_off(l);
        float* GW = net.g + layer_off(l);
        // h_{l+1} = h_l + relu(v): dv = dh * (v > 0)
        float* dv = g.dpqh;  // scratch n x HID
        CFD_LAUNCH(k_relu_bwd, nb_of(nh, 256), 256, 0, st, nh, (const float*)g.dh,
                   (const float*)g.v[l], dv);
        if ((rc = wgrad(st, g, n, dv, HID, g.h[l], HID, g.agg[l], HID, true, GW + L_U))) return rc;
        if ((rc = dense_t(st, n, dv, HID, W + L_U, 2 * HID, g.dhc))) return rc;
        // agg_i = mean_j relu(z_ij)
        CFD_LAUNCH(k_edge_bwd, nb_of(mh, 256), 256, 0, st, m, g.src, g.ptr, (const float*)g.dhc,
                   (const float*)g.z[l], g.dz);
        if ((rc = wgrad(st, g, m, g.dz, HID, g.e, E_F, nullptr, 0, true, GW + L_C))) return rc;
        CFD_LAUNCH(k_node_dpq, nb_of(nh, 256), 256, 0, st, n, g.ptr, g.rev, (const float*)g.dz, g.dpq);
        if ((rc = wgrad(st, g, n, g.dpq, 2 * HID, g.h[l], HID, nullptr, 0, false, GW + L_A))) return rc;
        if ((rc = dense_t(st, n, g.dpq, 2 * HID, W + L_A, HID, g.dpqh))) return rc;
        CFD_LAUNCH(k_add_dh, nb_of(nh, 256), 256, 0, st, n, (const float*)g.dhc,
                   (const float*)g.dpqh, g.dh);
    }
    float* da0 = g.dpqh;
    CFD_LAUNCH(k_relu_bwd, nb_of(nh, 256), 256, 0, st, nh, (const float*)g.dh, (const float*)g.a0, da0);
    if ((rc = wgrad(st, g, n, da0, HID, g.f, F_IN, nullptr, 0, true, net.g + OFF_W_IN))) return rc;
    if (loss_out) {
        CFD_CUDA(cudaMemcpyAsync(loss_out, lsum, sizeof(float), cudaMemcpyDeviceToHost, st));
        CFD_CUDA(cudaStreamSynchronize(st));
        *loss_out /= (float)std::max(g.nfree, 1);
    }
    return CFD_OK;
}

}  // namespace

namespace cfd {
namespace mpnn {

// Graph from the Laplacian pattern (rowptr, col: 0-based, diagonal first), host coordinates,
// boundary nodes (0-based) and kinds.  training = false leaves out the buffers of the FP32
// forward/backward passes.  Features are formed on `st` (the graph's own stream if null).
int graph_build(cfd_mpnn_graph** out, int npoin, const std::vector<int>& rowptr,
                const std::vector<int>& col, const double* x, const double* y, int nb,
                const int* bnode0, const int* bkind, bool training, cudaStream_t st) {
    *out = nullptr;
    for (int k = 0; k < nb; ++k) {
        if (bkind[k] != KIND_BODY && bkind[k] != KIND_OUTER) return arg_err("bkind (1 body, 2 outer)");
        if (bnode0[k] < 0 || bnode0[k] >= npoin) return arg_err("boundary node index");
    }
    // neighbours = the Laplacian pattern without its diagonal (first entry of each row)
    std::vector<int> ptr(npoin + 1, 0), nbr, src, rev;
    for (int i = 0; i < npoin; ++i) {
        for (int k = rowptr[i] + 1; k < rowptr[i + 1]; ++k) {
            nbr.push_back(col[k]);
            src.push_back(i);
        }
        ptr[i + 1] = (int)nbr.size();
    }
    const int m = (int)nbr.size();
    rev.assign(m, -1);
    for (int k = 0; k < m; ++k) {
        const int i = src[k], j = nbr[k];
        for (int q = ptr[j]; q < ptr[j + 1]; ++q)
            if (nbr[q] == i) {
                rev[k] = q;
                break;
            }
        if (rev[k] < 0) {
            set_last_message("mpnn: point neighbours are not symmetric");
            return CFD_ERR_MESH;
        }
    }
    std::vector<int> kind(npoin, KIND_FREE);
    for (int k = 0; k < nb; ++k) kind[bnode0[k]] = bkind[k];
    int nfree = 0;
    for (int i = 0; i < npoin; ++i) nfree += kind[i] == KIND_FREE;
    std::unique_ptr<cfd_mpnn_graph> g(new cfd_mpnn_graph());
    g->n = npoin;
    g->m = m;
    g->nb = nb;
    g->nfree = nfree;
    CFD_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    if (!st) st = g->stream;
    auto& o = g->owned;
    auto up = [&](auto** p, const auto* h, size_t cnt) -> int {
        int r = dev_alloc(o, p, cnt);
        if (r) return r;
        CFD_CUDA(cudaMemcpy(*p, h, cnt * sizeof(**p), cudaMemcpyHostToDevice));
        return CFD_OK;
    };
    int rc;
    if ((rc = up(&g->ptr, ptr.data(), npoin + 1))) return rc;
    if ((rc = up(&g->nbr, nbr.data(), m))) return rc;
    if ((rc = up(&g->src, src.data(), m))) return rc;
    if ((rc = up(&g->rev, rev.data(), m))) return rc;
    if ((rc = up(&g->kind, kind.data(), npoin))) return rc;
    if ((rc = up(&g->bnode, bnode0, nb))) return rc;
    if ((rc = up(&g->bkind, bkind, nb))) return rc;
    if ((rc = up(&g->X, x, npoin))) return rc;
    if ((rc = up(&g->Y, y, npoin))) return rc;
    for (double** q : {&g->bgx, &g->bgy})
        if ((rc = dev_alloc(o, q, nb))) return rc;
    for (double** q : {&g->gnx, &g->gny, &g->ux, &g->uy, &g->uz})
        if ((rc = dev_alloc(o, q, npoin))) return rc;
    CFD_CUDA(cudaMemset(g->gnx, 0, sizeof(double) * npoin));
    CFD_CUDA(cudaMemset(g->gny, 0, sizeof(double) * npoin));
    CFD_CUDA(cudaMemset(g->bgx, 0, sizeof(double) * nb));
    CFD_CUDA(cudaMemset(g->bgy, 0, sizeof(double) * nb));
    if ((rc = dev_alloc(o, &g->G, 1))) return rc;
    const size_t n = npoin;
    if ((rc = dev_alloc(o, &g->f, n * F_IN))) return rc;
    if ((rc = dev_alloc(o, &g->e, (size_t)m * E_F))) return rc;
    if (training) {
        if ((rc = dev_alloc(o, &g->target, n * OUT))) return rc;
        if ((rc = dev_alloc(o, &g->a0, n * HID))) return rc;
        for (int l = 0; l <= LAYERS; ++l)
            if ((rc = dev_alloc(o, &g->h[l], n * HID))) return rc;
        for (int l = 0; l < LAYERS; ++l) {
            if ((rc = dev_alloc(o, &g->agg[l], n * HID))) return rc;
            if ((rc = dev_alloc(o, &g->v[l], n * HID))) return rc;
            if ((rc = dev_alloc(o, &g->z[l], (size_t)m * HID))) return rc;
        }
        if ((rc = dev_alloc(o, &g->pq, n * 2 * HID))) return rc;
        if ((rc = dev_alloc(o, &g->y, n * OUT))) return rc;
        if ((rc = dev_alloc(o, &g->dy, n * OUT))) return rc;
        if ((rc = dev_alloc(o, &g->dh, n * HID))) return rc;
        if ((rc = dev_alloc(o, &g->dhc, n * 2 * HID))) return rc;
        if ((rc = dev_alloc(o, &g->dz, (size_t)m * HID))) return rc;
        if ((rc = dev_alloc(o, &g->dpq, n * 2 * HID))) return rc;
        if ((rc = dev_alloc(o, &g->dpqh, n * HID))) return rc;
        // partials of the largest weight gradient: rows/WG chunks x (128*64 + 128) floats
        const long rows = std::max<long>(npoin, m);
        g->part_floats = (size_t)blocks_for(rows, WG) * (2 * HID * HID + 2 * HID);
        if ((rc = dev_alloc(o, &g->part, g->part_floats))) return rc;
        if ((rc = dev_alloc(o, &g->lpart, blocks_for(npoin, 256) + 1))) return rc;
    }
    g->training = training;
    if ((rc = dev_alloc(o, &g->hb, n * HID))) return rc;
    if ((rc = dev_alloc(o, &g->pqb, 2 * n * 2 * HID))) return rc;  // two P|Q buffers
    if ((rc = dev_alloc(o, &g->yb, n * OUT))) return rc;
    if ((rc = dev_alloc(o, &g->tc_err, 1))) return rc;
    CFD_CUDA(cudaMemsetAsync(g->tc_err, 0, sizeof(int), st));
    // geometry globals (zero displacement), node and edge features
    const int* ng = nullptr;
    CFD_LAUNCH(k_globals, 1, 256, 0, st, g->nb, g->bnode, g->bkind, (const double*)g->bgx,
               (const double*)g->bgy, (const double*)g->X, (const double*)g->Y, g->G, ng);
    CFD_LAUNCH(k_features, blocks_for(g->n, 256), 256, 0, st, g->n, (const double*)g->X,
               (const double*)g->Y, g->kind, (const Globals*)g->G, g->f, ng);
    CFD_LAUNCH(k_edge_features, blocks_for(g->m, 256), 256, 0, st, g->m, g->src, g->nbr,
               (const double*)g->X, (const double*)g->Y, (const Globals*)g->G, g->e, ng);
    CFD_CUDA(cudaStreamSynchronize(st));
    *out = g.release();
    return CFD_OK;
}

// The guess (ux, uy) on stream st for the mesh (X, Y) and the boundary displacement
// (bgx, bgy) in bnode order (device arrays); every kernel returns at once when gate is
// non-null and *gate == 0.
int guess_on_stream(cfd_mpnn* net, cfd_mpnn_graph* g, cudaStream_t st, const double* X,
                    const double* Y, const double* bgx, const double* bgy, double* ux,
                    double* uy, const int* gate) {
    // grid-stride launches of a few waves: a closed gate costs little
    const unsigned gs = 1216;
    const int nbk = (int)blocks_for(g->nb, 256);
    CFD_LAUNCH(k_scatter_bc, nbk, 256, 0, st, g->nb, g->bnode, bgx, bgy, g->gnx, g->gny, gate);
    CFD_LAUNCH(k_globals, 1, 256, 0, st, g->nb, g->bnode, g->bkind, bgx, bgy, X, Y, g->G, gate);
    CFD_LAUNCH(k_features, std::min(blocks_for(g->n, 256), gs), 256, 0, st, g->n, X, Y, g->kind,
               (const Globals*)g->G, g->f, gate);
    CFD_LAUNCH(k_edge_features, std::min(blocks_for(g->m, 256), gs), 256, 0, st, g->m, g->src,
               g->nbr, X, Y, (const Globals*)g->G, g->e, gate);
    int rc = infer_bf16(st, net->w, net->wb, &net->wb_valid, g->n, g->ptr, g->nbr, g->f, g->e,
                        g->hb, g->pqb, g->yb, gate, g->tc_err);
    if (rc) return rc;
    CFD_LAUNCH(k_guess, std::min(blocks_for(g->n, 256), gs), 256, 0, st, g->n,
               (const float*)g->yb, g->kind, (const double*)g->gnx, (const double*)g->gny,
               (const Globals*)g->G, ux, uy, gate);
    return CFD_OK;
}

// Refined learned guess (mesh motion in a resident context), three steps on stream st:
//  fields_seed: the basis fields from the network's last run (its output and the globals of
//    that run's fit, as guess_on_stream leaves them);
//  fields_guess: the affine fit of the boundary data (bgx, bgy; bnode order) and the guess
//    c = t Phi + M Psi from the fields;
//  fields_update: after the solves, the per-node correction by their solutions (x0, x1),
//    with the fit the last guess_on_stream or fields_guess formed.
int fields_seed(cfd_mpnn_graph* g, cudaStream_t st) {
    if (!g->F) {
        int rc = dev_alloc(g->owned, &g->F, 3 * (size_t)g->n);
        if (rc) return rc;
    }
    CFD_LAUNCH(k_fields_seed, std::min(blocks_for(g->n, 256), 1216u), 256, 0, st, g->n,
               (const float*)g->yb, g->kind, (const Globals*)g->G, g->F);
    return CFD_OK;
}

int fields_guess(cfd_mpnn_graph* g, cudaStream_t st, const double* X, const double* Y,
                 const double* bgx, const double* bgy, const double* x0, const double* x1,
                 double* c0, double* c1) {
    const int* ng = nullptr;
    CFD_LAUNCH(k_globals, 1, 256, 0, st, g->nb, g->bnode, g->bkind, bgx, bgy, X, Y, g->G, ng);
    CFD_LAUNCH(k_fields_guess, std::min(blocks_for(g->n, 256), 1216u), 256, 0, st, g->n, g->kind,
               (const Globals*)g->G, (const double*)g->F, x0, x1, c0, c1);
    return CFD_OK;
}

int fields_update(cfd_mpnn_graph* g, cudaStream_t st, const double* x0, const double* x1) {
    CFD_LAUNCH(k_fields_update, std::min(blocks_for(g->n, 256), 1216u), 256, 0, st, g->n, g->kind,
               (const Globals*)g->G, x0, x1, g->F);
    return CFD_OK;
}

void graph_free(cfd_mpnn_graph* g) { delete g; }

}  // namespace mpnn
}  // namespace cfd

// ------------------------------------------------------------------ extern "C"
extern "C" {

int cfd_mpnn_nparams(void) { return N_PARAMS; }

int cfd_mpnn_create(cfd_mpnn** out, const float* w) {
    if (!out || !w) return arg_err("null pointer");
    *out = nullptr;
    std::unique_ptr<cfd_mpnn> net(new cfd_mpnn());
    int rc;
    for (float** q : {&net->w, &net->g, &net->m, &net->v})
        if ((rc = dev_alloc(net->owned, q, N_PARAMS))) return rc;
    if ((rc = dev_alloc(net->owned, &net->wb, N_PARAMS))) return rc;
    CFD_CUDA(cudaMemcpy(net->w, w, sizeof(float) * N_PARAMS, cudaMemcpyHostToDevice));
    CFD_CUDA(cudaMemset(net->m, 0, sizeof(float) * N_PARAMS));
    CFD_CUDA(cudaMemset(net->v, 0, sizeof(float) * N_PARAMS));
    CFD_CUDA(cudaMemset(net->g, 0, sizeof(float) * N_PARAMS));
    *out = net.release();
    return CFD_OK;
}

void cfd_mpnn_destroy(cfd_mpnn* net) { delete net; }

int cfd_mpnn_get_weights(cfd_mpnn* net, float* w) {
    if (!net || !w) return arg_err("null pointer");
    CFD_CUDA(cudaMemcpy(w, net->w, sizeof(float) * N_PARAMS, cudaMemcpyDeviceToHost));
    return CFD_OK;
}

int cfd_mpnn_set_weights(cfd_mpnn* net, const float* w) {
    if (!net || !w) return arg_err("null pointer");
    CFD_CUDA(cudaMemcpy(net->w, w, sizeof(float) * N_PARAMS, cudaMemcpyHostToDevice));
    net->wb_valid = false;
    return CFD_OK;
}

int cfd_mpnn_graph_create(cfd_mpnn_graph** out, int npoin, int nelem, const int* inpoel,
                          const double* x, const double* y, int nb, const int* bnode,
                          const int* bkind) {
    if (!out || !inpoel || !x || !y || !bnode || !bkind) return arg_err("null pointer");
    *out = nullptr;
    if (npoin <= 0 || nelem <= 0 || nb <= 0) return arg_err("sizes");
    if (!check_index_range(inpoel, 3L * nelem, 1, npoin) || !check_index_range(bnode, nb, 1, npoin))
        return CFD_ERR_MESH;
    Adjacency adj;
    std::string why;
    int rc = build_adjacency(npoin, nelem, inpoel, adj, &why);
    if (rc) {
        set_last_message(why);
        return rc;
    }
    std::vector<int> bn(nb);
    for (int k = 0; k < nb; ++k) bn[k] = bnode[k] - 1;
    return graph_build(out, npoin, adj.rowptr, adj.col, x, y, nb, bn.data(), bkind, true, nullptr);
}

void cfd_mpnn_graph_destroy(cfd_mpnn_graph* g) { delete g; }

int cfd_mpnn_graph_set_bc(cfd_mpnn_graph* g, const double* gx, const double* gy) {
    if (!g || !gx || !gy) return arg_err("null pointer");
    cudaStream_t st = g->stream;
    CFD_CUDA(cudaMemcpyAsync(g->bgx, gx, sizeof(double) * g->nb, cudaMemcpyHostToDevice, st));
    CFD_CUDA(cudaMemcpyAsync(g->bgy, gy, sizeof(double) * g->nb, cudaMemcpyHostToDevice, st));
    const int* ng = nullptr;
    CFD_LAUNCH(k_scatter_bc, blocks_for(g->nb, 256), 256, 0, st, g->nb, g->bnode,
               (const double*)g->bgx, (const double*)g->bgy, g->gnx, g->gny, ng);
    CFD_LAUNCH(k_globals, 1, 256, 0, st, g->nb, g->bnode, g->bkind, (const double*)g->bgx,
               (const double*)g->bgy, (const double*)g->X, (const double*)g->Y, g->G, ng);
    CFD_CUDA(cudaStreamSynchronize(st));
    return CFD_OK;
}

int cfd_mpnn_graph_globals(cfd_mpnn_graph* g, double* out10) {
    if (!g || !out10) return arg_err("null pointer");
    Globals h;
    CFD_CUDA(cudaMemcpyAsync(&h, g->G, sizeof(h), cudaMemcpyDeviceToHost, g->stream));
    CFD_CUDA(cudaStreamSynchronize(g->stream));
    const double v[10] = {h.cx, h.cy, h.L, h.R, h.tx, h.ty, h.m11, h.m12, h.m21, h.m22};
    std::memcpy(out10, v, sizeof(v));
    return CFD_OK;
}

int cfd_mpnn_graph_set_target(cfd_mpnn_graph* g, const double* phi, const double* psi_x,
                              const double* psi_y) {
    if (!g || !phi || !psi_x || !psi_y) return arg_err("null pointer");
    if (!g->training) return arg_err("graph without training buffers");
    cudaStream_t st = g->stream;
    CFD_CUDA(cudaMemcpyAsync(g->ux, phi, sizeof(double) * g->n, cudaMemcpyHostToDevice, st));
    CFD_CUDA(cudaMemcpyAsync(g->uy, psi_x, sizeof(double) * g->n, cudaMemcpyHostToDevice, st));
    CFD_CUDA(cudaMemcpyAsync(g->uz, psi_y, sizeof(double) * g->n, cudaMemcpyHostToDevice, st));
    CFD_LAUNCH(k_targets, blocks_for(g->n, 256), 256, 0, st, g->n, (const double*)g->ux,
               (const double*)g->uy, (const double*)g->uz, (const Globals*)g->G, g->target);
    CFD_CUDA(cudaStreamSynchronize(st));
    return CFD_OK;
}

int cfd_mpnn_loss_grad(cfd_mpnn* net, cfd_mpnn_graph* g, float* loss, float* grad) {
    if (!net || !g) return arg_err("null pointer");
    if (!g->training) return arg_err("graph without training buffers");
    int rc = forward_fp32(*net, *g);
    if (rc) return rc;
    float l = 0.f;
    if ((rc = backward_fp32(*net, *g, &l))) return rc;
    if (loss) *loss = l;
    if (grad) {
        CFD_CUDA(cudaMemcpyAsync(grad, net->g, sizeof(float) * N_PARAMS, cudaMemcpyDeviceToHost,
                                 g->stream));
        CFD_CUDA(cudaStreamSynchronize(g->stream));
    }
    return CFD_OK;
}

int cfd_mpnn_train_step(cfd_mpnn* net, cfd_mpnn_graph* g, float lr, float* loss) {
    if (!net || !g) return arg_err("null pointer");
    if (!(lr > 0.f)) return arg_err("lr");
    if (!g->training) return arg_err("graph without training buffers");
    int rc = forward_fp32(*net, *g);
    if (rc) return rc;
    float l = 0.f;
    if ((rc = backward_fp32(*net, *g, loss ? &l : nullptr))) return rc;
    net->t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.f - std::pow(b1, (float)net->t), bc2 = 1.f - std::pow(b2, (float)net->t);
    CFD_LAUNCH(k_adam, blocks_for(N_PARAMS, 256), 256, 0, g->stream, N_PARAMS, net->w,
               (const float*)net->g, net->m, net->v, lr, b1, b2, 1e-8f, bc1, bc2);
    net->wb_valid = false;
    CFD_CUDA(cudaStreamSynchronize(g->stream));
    if (loss) *loss = l;
    return CFD_OK;
}

int cfd_mpnn_adam_state(cfd_mpnn* net, float* m, float* v, int* t) {
    if (!net) return arg_err("null pointer");
    if (m) CFD_CUDA(cudaMemcpy(m, net->m, sizeof(float) * N_PARAMS, cudaMemcpyDeviceToHost));
    if (v) CFD_CUDA(cudaMemcpy(v, net->v, sizeof(float) * N_PARAMS, cudaMemcpyDeviceToHost));
    if (t) *t = net->t;
    return CFD_OK;
}

int cfd_mpnn_forward(cfd_mpnn* net, cfd_mpnn_graph* g, int bf16, double* ux, double* uy) {
    if (!net || !g) return arg_err("null pointer");
    if (!bf16 && !g->training) return arg_err("graph without training buffers (FP32 pass)");
    int rc;
    const float* y = nullptr;
    if (bf16) {
        if ((rc = infer_bf16(g->stream, net->w, net->wb, &net->wb_valid, g->n, g->ptr, g->nbr, g->f,
                             g->e, g->hb, g->pqb, g->yb, nullptr, g->tc_err)))
            return rc;
        y = g->yb;
    } else {
        if ((rc = forward_fp32(*net, *g))) return rc;
        y = g->y;
    }
    CFD_LAUNCH(k_guess, blocks_for(g->n, 256), 256, 0, g->stream, g->n, y, g->kind,
               (const double*)g->gnx, (const double*)g->gny, (const Globals*)g->G, g->ux, g->uy,
               (const int*)nullptr);
    if (ux) CFD_CUDA(cudaMemcpyAsync(ux, g->ux, sizeof(double) * g->n, cudaMemcpyDeviceToHost, g->stream));
    if (uy) CFD_CUDA(cudaMemcpyAsync(uy, g->uy, sizeof(double) * g->n, cudaMemcpyDeviceToHost, g->stream));
    int tc_err = 0;
    CFD_CUDA(cudaMemcpyAsync(&tc_err, g->tc_err, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    CFD_CUDA(cudaStreamSynchronize(g->stream));
    if (tc_err) {
        CFD_CUDA(cudaMemsetAsync(g->tc_err, 0, sizeof(int), g->stream));
        set_last_message("a tensor-core inference pass timed out on its mbarrier");
        return tc_err;
    }
    return CFD_OK;
}

}  // extern "C"

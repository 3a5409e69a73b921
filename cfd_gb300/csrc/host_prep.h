// host_prep.h — setup-time mesh preprocessing on the host (once per context).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/cfd_gpu.h"

namespace cfd {

struct Adjacency {
    // element-around-point (pointNeighbor.f90:5-43), 0-based; slot = 3*e + local index
    std::vector<int> esup_ptr;   // npoin+1
    std::vector<int> esup_slot;  // 3*nelem, element order within each node
    // point-around-point (pointNeighbor.f90:45-91), 0-based, discovery order
    std::vector<int> psup_ptr, psup;
    // Laplacian pattern (mLaplace.f90:60-94): rowptr 0-based offsets, col 0-based,
    // diagonal first then psup order
    std::vector<int> rowptr, col;
    // per esup slot: offsets in row p of the element's three nodes (x,y,z), w unused
    std::vector<uint8_t> lap_pos;  // 4 * 3*nelem
};

// Builds esup/psup/pattern/positions; returns CFD_OK or CFD_ERR_MESH (bad index,
// repeated node in an element, row longer than 255).
int build_adjacency(int npoin, int nelem, const int* inpoel_1based, Adjacency& adj,
                    std::string* why);

struct BcTables {
    std::vector<uint8_t> flag;     // npoin: BC_FIXV | BC_FIXRHO | BC_FIXT (BC_NORMAL on device)
    std::vector<double> val;       // 4*npoin: vx, vy, rho, T (last entry of each list wins)
    // wall nodes for normales: node list, CSR of incident wall edges (edge order)
    std::vector<int> wnode, wptr, wedge;  // wedge: edge index (0-based)
    std::vector<int> walls;        // 2*nwall, 0-based
    // FORCES sets: per set the (n1, n2) edges in ISET order
    std::vector<int> set_ptr, set_edges;  // set_edges 2 per edge, 0-based
    std::vector<int> set_elem;            // owning element of each set edge, 0-based
    int nset_numb = 0;
    // mesh-motion Dirichlet list: ilaux order; per entry the node and the set whose
    // TRANSF write wins for it (-1: none / fixed-movement entry)
    std::vector<int> fix_node, fix_set;
    // unique fixed nodes with the ilaux entry that wins (copy1's last write)
    std::vector<int> ufix_node, ufix_src;
    std::vector<uint8_t> isfix;    // npoin
};

int build_bc_tables(const cfd_mesh* m, BcTables& bc, std::string* why);

// 1-based index checks of a routine's arrays
bool check_index_range(const int* idx, long n, int lo, int hi);

}  // namespace cfd

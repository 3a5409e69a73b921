// host_prep.cpp — setup-time mesh preprocessing (adjacency, Laplacian pattern, BC tables).
#include "host_prep.h"

#include <algorithm>
#include <cstring>

namespace cfd {

enum : uint8_t { HB_FIXV = 1, HB_NORMAL = 2, HB_FIXRHO = 4, HB_FIXT = 8 };

bool check_index_range(const int* idx, long n, int lo, int hi) {
    for (long i = 0; i < n; ++i)
        if (idx[i] < lo || idx[i] > hi) return false;
    return true;
}

int build_adjacency(int npoin, int nelem, const int* inpoel, Adjacency& a, std::string* why) {
    if (npoin <= 0 || nelem <= 0) {
        if (why) *why = "npoin and nelem must be positive";
        return CFD_ERR_ARG;
    }
    for (long e = 0; e < nelem; ++e) {
        const int* n = inpoel + 3 * e;
        for (int i = 0; i < 3; ++i)
            if (n[i] < 1 || n[i] > npoin) {
                if (why) *why = "inpoel(" + std::to_string(i + 1) + "," + std::to_string(e + 1) +
                                ") = " + std::to_string(n[i]) + " is outside 1..npoin";
                return CFD_ERR_MESH;
            }
        if (n[0] == n[1] || n[1] == n[2] || n[0] == n[2]) {
            if (why) *why = "element " + std::to_string(e + 1) + " repeats a node";
            return CFD_ERR_MESH;
        }
    }
    // getEsup: histogram, scan, fill in element order
    a.esup_ptr.assign(npoin + 1, 0);
    for (long e = 0; e < nelem; ++e)
        for (int i = 0; i < 3; ++i) a.esup_ptr[inpoel[3 * e + i]] += 1;
    for (int p = 1; p <= npoin; ++p) a.esup_ptr[p] += a.esup_ptr[p - 1];
    a.esup_slot.assign(3 * (size_t)nelem, 0);
    std::vector<int> fill(a.esup_ptr.begin(), a.esup_ptr.end() - 1);
    for (long e = 0; e < nelem; ++e)
        for (int i = 0; i < 3; ++i) {
            int p = inpoel[3 * e + i] - 1;
            a.esup_slot[fill[p]++] = (int)(3 * e + i);
        }
    // getPsup: per node, the other nodes of its elements in discovery order
    a.psup_ptr.assign(npoin + 1, 0);
    a.psup.clear();
    a.psup.reserve(6 * (size_t)npoin);
    std::vector<int> lpoin(npoin, -1);
    for (int p = 0; p < npoin; ++p) {
        for (int s = a.esup_ptr[p]; s < a.esup_ptr[p + 1]; ++s) {
            int e = a.esup_slot[s] / 3;
            for (int i = 0; i < 3; ++i) {
                int q = inpoel[3 * e + i] - 1;
                if (q != p && lpoin[q] != p) {
                    a.psup.push_back(q);
                    lpoin[q] = p;
                }
            }
        }
        a.psup_ptr[p + 1] = (int)a.psup.size();
    }
    // pattern: diagonal first, then psup
    a.rowptr.assign(npoin + 1, 0);
    for (int p = 0; p < npoin; ++p) a.rowptr[p + 1] = a.rowptr[p] + 1 + (a.psup_ptr[p + 1] - a.psup_ptr[p]);
    a.col.assign(a.rowptr[npoin], 0);
    for (int p = 0; p < npoin; ++p) {
        int k = a.rowptr[p];
        a.col[k++] = p;
        for (int s = a.psup_ptr[p]; s < a.psup_ptr[p + 1]; ++s) a.col[k++] = a.psup[s];
        if (a.rowptr[p + 1] - a.rowptr[p] > 255) {
            if (why) *why = "node " + std::to_string(p + 1) + " has more than 254 neighbours";
            return CFD_ERR_MESH;
        }
    }
    // the linear search of mLaplace.f90:46-50, once
    a.lap_pos.assign(4 * (size_t)3 * nelem, 0);
    for (int p = 0; p < npoin; ++p) {
        const int r0 = a.rowptr[p], r1 = a.rowptr[p + 1];
        for (int s = a.esup_ptr[p]; s < a.esup_ptr[p + 1]; ++s) {
            int e = a.esup_slot[s] / 3;
            for (int j = 0; j < 3; ++j) {
                int q = inpoel[3 * e + j] - 1;
                int off = -1;
                for (int k = r0; k < r1; ++k)
                    if (a.col[k] == q) { off = k - r0; break; }
                a.lap_pos[4 * (size_t)s + j] = (uint8_t)off;
            }
        }
    }
    return CFD_OK;
}

int build_bc_tables(const cfd_mesh* m, BcTables& bc, std::string* why) {
    const int N = m->npoin;
    auto bad = [&](const char* what) {
        if (why) *why = std::string(what) + " holds a node index outside 1..npoin";
        return CFD_ERR_MESH;
    };
    if (m->nfixrho < 0 || m->nfixv < 0 || m->nfixt < 0 || m->nwall < 0 || m->nsets < 0 ||
        m->nmove < 0 || m->nfix_move < 0 || m->nset_numb < 0 || m->nset_numb > 10) {
        if (why) *why = "negative list length or nset_numb > 10";
        return CFD_ERR_ARG;
    }
    if (m->nfixrho && !check_index_range(m->ifixrho_node, m->nfixrho, 1, N)) return bad("ifixrho_node");
    if (m->nfixv && !check_index_range(m->ifixv_node, m->nfixv, 1, N)) return bad("ifixv_node");
    if (m->nfixt && !check_index_range(m->ifixt_node, m->nfixt, 1, N)) return bad("ifixt_node");
    if (m->nwall && !check_index_range(m->wall, 2L * m->nwall, 1, N)) return bad("wall");
    const int nn = m->nmove + m->nfix_move;
    if (nn && !check_index_range(m->ilaux, nn, 1, N)) return bad("ilaux");
    bc.flag.assign(N, 0);
    bc.val.assign(4 * (size_t)N, 0.0);
    for (int i = 0; i < m->nfixv; ++i) {  // FIXVEL order: last wins
        int p = m->ifixv_node[i] - 1;
        bc.flag[p] |= HB_FIXV;
        bc.val[4 * p] = m->rfixv_valuex[i];
        bc.val[4 * p + 1] = m->rfixv_valuey[i];
    }
    for (int i = 0; i < m->nfixrho; ++i) {
        int p = m->ifixrho_node[i] - 1;
        bc.flag[p] |= HB_FIXRHO;
        bc.val[4 * p + 2] = m->rfixrho_value[i];
    }
    for (int i = 0; i < m->nfixt; ++i) {
        int p = m->ifixt_node[i] - 1;
        bc.flag[p] |= HB_FIXT;
        bc.val[4 * p + 3] = m->rfixt_value[i];
    }
    // wall incidence in edge order
    bc.walls.assign(2 * (size_t)m->nwall, 0);
    std::vector<int> cnt(N, 0);
    for (int w = 0; w < m->nwall; ++w)
        for (int j = 0; j < 2; ++j) {
            int p = m->wall[2 * w + j] - 1;
            bc.walls[2 * w + j] = p;
            cnt[p] += 1;
        }
    bc.wnode.clear();
    std::vector<int> slot(N, -1);
    for (int p = 0; p < N; ++p)
        if (cnt[p]) { slot[p] = (int)bc.wnode.size(); bc.wnode.push_back(p); }
    bc.wptr.assign(bc.wnode.size() + 1, 0);
    for (size_t k = 0; k < bc.wnode.size(); ++k) bc.wptr[k + 1] = bc.wptr[k] + cnt[bc.wnode[k]];
    bc.wedge.assign(bc.wptr.back(), 0);
    std::vector<int> fill(bc.wptr.begin(), bc.wptr.end() - 1);
    for (int w = 0; w < m->nwall; ++w)
        for (int j = 0; j < 2; ++j) {
            int p = bc.walls[2 * w + j];
            bc.wedge[fill[slot[p]]++] = w;
        }
    // force sets: ISET(3,10,nsets), entry (j, s, ii) at j + 3*s + 30*ii
    bc.nset_numb = m->nset_numb;
    bc.set_ptr.assign(11, 0);
    bc.set_edges.clear();
    bc.set_elem.clear();
    std::vector<int> last_set(N, -1);
    for (int s = 0; s < m->nset_numb; ++s) {
        if (m->ielem_sets[s] < 0 || m->ielem_sets[s] > m->nsets) {
            if (why) *why = "ielem_sets exceeds nsets";
            return CFD_ERR_ARG;
        }
        for (int ii = 0; ii < m->ielem_sets[s]; ++ii) {
            const int* e = m->iset + 3 * (s + 10 * (size_t)ii);
            if (e[0] < 1 || e[0] > N || e[1] < 1 || e[1] > N || e[2] < 1 || e[2] > m->nelem)
                return bad("iset");
            bc.set_edges.push_back(e[0] - 1);
            bc.set_edges.push_back(e[1] - 1);
            bc.set_elem.push_back(e[2] - 1);
            last_set[e[0] - 1] = s;  // TRANSF loop order: set, edge, JJ=1,2
            last_set[e[1] - 1] = s;
        }
        bc.set_ptr[s + 1] = (int)bc.set_edges.size() / 2;
    }
    for (int s = m->nset_numb; s < 10; ++s) bc.set_ptr[s + 1] = bc.set_ptr[s];
    // mesh-motion Dirichlet list (meshMove.f90:80-89 with ilaux of dataLoader.f90:258-268)
    bc.fix_node.assign(nn, 0);
    bc.fix_set.assign(nn, -1);
    std::vector<int> last_src(N, -1);
    for (int k = 0; k < nn; ++k) {
        int p = m->ilaux[k] - 1;
        bc.fix_node[k] = p;
        bc.fix_set[k] = (k < m->nmove) ? last_set[p] : -1;
        last_src[p] = k;
    }
    bc.isfix.assign(N, 0);
    bc.ufix_node.clear();
    bc.ufix_src.clear();
    for (int p = 0; p < N; ++p)
        if (last_src[p] >= 0) {
            bc.isfix[p] = 1;
            bc.ufix_node.push_back(p);
            bc.ufix_src.push_back(last_src[p]);
        }
    return CFD_OK;
}

}  // namespace cfd

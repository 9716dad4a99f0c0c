// .su2 reading, O(N) mesh assembly with the reference's numbering,
// synthetic .su2 writers and the initial field -- host side of fvgb.
//
// The assembly reproduces, in O(N) with a hash map instead of the reference's
// linear edge search (FVMR/src/legacy/FVM_2D.cpp:105-114), the numbering and
// geometry of SU2MeshReader::read_mesh_and_process
// (FVMR/src/input/SU2MeshReader.cpp:10-251) followed by OldDataConverter
// (FVMR/src/solvers/OldDataConverter.cpp:35-195):
//   * quads are split into (n0,n1,n3) and (n3,n1,n2) (SU2MeshReader.cpp:104-119);
//   * a triangle with negative signed area swaps nodes 1 and 2 (FVM_2D.cpp:50-70);
//   * edges are numbered in first-seen order over the elements' (n0n1, n1n2,
//     n2n0) sides, the first owner being L (FVM_2D.cpp:72-81, 116-134);
//   * edge lengths are rounded through float (FVM_2D.cpp:189-198);
//   * periodic edges take the partner at reversed index in the paired set
//     (BoundaryManager_2D.cpp:304-323) and its L cell as R
//     (OldDataConverter.cpp:154-172).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

namespace fvgb {

namespace {

struct EdgeMap {  // open addressing: unordered node pair -> edge index
    std::vector<uint64_t> key;
    std::vector<int> val;
    size_t mask = 0;
    explicit EdgeMap(size_t n) {
        size_t cap = 16;
        while (cap < 2 * n) cap <<= 1;
        key.assign(cap, 0);
        val.assign(cap, -1);
        mask = cap - 1;
    }
    static uint64_t k(int a, int b) {
        uint32_t lo = (uint32_t)(a < b ? a : b), hi = (uint32_t)(a < b ? b : a);
        return ((uint64_t)lo << 32) | hi;
    }
    static size_t h(uint64_t x) {
        x ^= x >> 31;
        x *= 0x9e3779b97f4a7c15ULL;
        x ^= x >> 29;
        return (size_t)x;
    }
    int get(int a, int b) const {
        uint64_t kk = k(a, b);
        for (size_t i = h(kk) & mask;; i = (i + 1) & mask) {
            if (val[i] < 0) return -1;
            if (key[i] == kk) return val[i];
        }
    }
    void put(int a, int b, int v) {
        uint64_t kk = k(a, b);
        for (size_t i = h(kk) & mask;; i = (i + 1) & mask) {
            if (val[i] < 0) {
                key[i] = kk;
                val[i] = v;
                return;
            }
        }
    }
};

// BoundaryManager::boundaryNameToType, FVMR/src/boundary_condition/BoundaryManager.cpp:15-45
int name_to_type(const std::string& n, int equation) {
    if (n == "wall" || n == "obstacle" || n == "airfoil" || n == "foil")
        return equation == 1 ? BC_WALL_NONVISCOUS : BC_WALL_ADIABAT;
    if (n == "wall_nonViscous" || n == "wall_slippery" || n == "slippery" || n == "slippery_wall")
        return BC_WALL_NONVISCOUS;
    if (n == "inlet") return BC_INLET;
    if (n == "outlet") return BC_OUTLET;
    if (n == "inf" || n == "infinity" || n == "far" || n == "farfield") return BC_INF;
    if (n == "dsr") return BC_DSR;
    if (n == "symmetry") return BC_SYMMETRY;
    if (n.compare(0, 8, "periodic") == 0 && !n.empty()) {
        char c = n.back();
        if (c >= '0' && c <= '9') return BC_PERIODIC_0 + (c - '0');
    }
    return -2;
}

bool is_periodic(int t) { return t >= BC_PERIODIC_0 && t <= BC_PERIODIC_9; }

// Splits a line the way StringProcessor::splitString does after '=' has been
// widened to " = " (SU2MeshReader.cpp:46-48): words end at ' ', '\t', ',' and
// '=' is a word of its own.
int split(char* s, char** w, int maxw) {
    int n = 0;
    while (*s && n < maxw) {
        while (*s == ' ' || *s == '\t' || *s == ',') s++;
        if (!*s) break;
        if (*s == '=') {
            *s++ = 0;
            w[n++] = (char*)"=";
            continue;
        }
        w[n++] = s;
        while (*s && *s != ' ' && *s != '\t' && *s != ',' && *s != '=') s++;
        if (*s == '=') {
            *s++ = 0;
            if (n < maxw) w[n++] = (char*)"=";
            continue;
        }
        if (*s) *s++ = 0;
    }
    return n;
}

}  // namespace

int read_su2(const char* path, int equation, double scale, HostMesh& m) {
    RawMesh r;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(FVGB_ERR_IO, std::string("cannot open mesh file ") + path);
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::vector<char> buf((size_t)sz + 1);
    size_t got = std::fread(buf.data(), 1, (size_t)sz, f);
    std::fclose(f);
    buf[got] = 0;

    std::vector<double>& nx = r.nx;
    std::vector<double>& ny = r.ny;
    std::vector<int>& nid = r.nid;
    std::vector<int>& tri = r.tri;
    std::vector<RawMesh::Marker>& mk = r.mk;
    int& maxnodeID = r.maxnodeID;
    enum { S_START, S_NDIME, S_NPOIN, S_NELEM, S_NMARK } state = S_START;

    char* p = buf.data();
    char* end = p + got;
    while (p < end) {
        char* line = p;
        while (p < end && *p != '\n') p++;
        if (p < end) *p++ = 0;
        char* w[16];
        int nw = split(line, w, 16);
        if (nw == 0 || std::strcmp(w[0], "%") == 0) continue;
        if (!std::strcmp(w[0], "NDIME")) state = S_NDIME;
        else if (!std::strcmp(w[0], "NPOIN")) state = S_NPOIN;
        else if (!std::strcmp(w[0], "NELEM")) state = S_NELEM;
        else if (!std::strcmp(w[0], "NMARK")) state = S_NMARK;
        if (state == S_NDIME) {
            if (!(nw == 3 && !std::strcmp(w[2], "2"))) return fail(FVGB_ERR_FORMAT, "SU2 mesh dimension is not 2D");
        } else if (state == S_NPOIN && w[0][0] != 'N') {
            if (nw < 3) return fail(FVGB_ERR_FORMAT, "malformed node line in .su2");
            nx.push_back(std::strtod(w[0], nullptr));
            ny.push_back(std::strtod(w[1], nullptr));
            int id = (nw == 3) ? (int)std::strtod(w[2], nullptr) + 1 : (int)std::strtod(w[3], nullptr) + 1;
            nid.push_back(id);
            if (id > maxnodeID) maxnodeID = id;
        } else if (state == S_NELEM && w[0][0] != 'N') {
            if (!std::strcmp(w[0], "5")) {
                if (nw < 4) return fail(FVGB_ERR_FORMAT, "malformed triangle line in .su2");
                tri.push_back((int)std::strtod(w[1], nullptr) + 1);
                tri.push_back((int)std::strtod(w[2], nullptr) + 1);
                tri.push_back((int)std::strtod(w[3], nullptr) + 1);
            } else if (!std::strcmp(w[0], "9")) {
                if (nw < 5) return fail(FVGB_ERR_FORMAT, "malformed quad line in .su2");
                int q1 = (int)std::strtod(w[1], nullptr) + 1, q2 = (int)std::strtod(w[2], nullptr) + 1;
                int q3 = (int)std::strtod(w[3], nullptr) + 1, q4 = (int)std::strtod(w[4], nullptr) + 1;
                tri.insert(tri.end(), {q1, q2, q4, q4, q2, q3});
            }
        } else if (state == S_NMARK) {
            if (!std::strcmp(w[0], "NMARK") || !std::strcmp(w[0], "MARKER_ELEMS")) {
            } else if (!std::strcmp(w[0], "MARKER_TAG")) {
                if (nw < 3) return fail(FVGB_ERR_FORMAT, "malformed MARKER_TAG line");
                mk.push_back(RawMesh::Marker{w[2], {}});
            } else {
                if (mk.empty() || nw < 3) return fail(FVGB_ERR_FORMAT, "boundary element before MARKER_TAG");
                mk.back().e.push_back(std::atoi(w[1]) + 1);
                mk.back().e.push_back(std::atoi(w[2]) + 1);
            }
        }
    }
    if (nx.empty() || tri.empty()) return fail(FVGB_ERR_FORMAT, "mesh has no nodes or no elements");
    {  // scaleMesh, SU2MeshReader.cpp:157-173
        double res = scale - 1.0;
        if (!(res > -0.01 && res < 0.01)) {
            if (scale < 0.0) return fail(FVGB_ERR_ARG, "mesh scale factor should be positive");
            for (size_t i = 0; i < nx.size(); i++) {
                nx[i] *= scale;
                ny[i] *= scale;
            }
        }
    }
    return assemble(r, equation, m);
}

// FVM_2D::iniEdges .. iniEdges_lengths (FVMR/src/legacy/FVM_2D.cpp:36-198), the boundary
// sets of SU2MeshReader.cpp:201-243 / ContinueFileReader::process (ContinueFileReader.cpp:457-494)
// and OldDataConverter, in O(N): the reference's numbering and arrays.
int assemble(RawMesh& r, int equation, HostMesh& m) {
    std::vector<double>& nx = r.nx;
    std::vector<double>& ny = r.ny;
    std::vector<int>& nid = r.nid;
    std::vector<int>& tri = r.tri;
    std::vector<RawMesh::Marker>& mk = r.mk;
    const int maxnodeID = r.maxnodeID;
    std::vector<int> idx((size_t)maxnodeID + 1, -1);
    for (size_t i = 0; i < nid.size(); i++)
        if (nid[i] >= 0) idx[nid[i]] = (int)i;

    const int N = (int)(tri.size() / 3);
    const int V = (int)nx.size();
    m = HostMesh();
    m.N = N;
    m.V = V;
    m.elem_vol.resize(N);
    m.elem_xy.resize(2 * (size_t)N);
    for (int e = 0; e < N; e++) {
        int* t = &tri[3 * (size_t)e];
        double xn[3], yn[3];
        for (int i = 0; i < 3; i++) {
            if (t[i] < 0 || t[i] > maxnodeID || idx[t[i]] < 0)
                return fail(FVGB_ERR_MESH, "element names an unknown node");
            xn[i] = nx[idx[t[i]]];
            yn[i] = ny[idx[t[i]]];
        }
        double area = 0.5 * (xn[0] * (yn[1] - yn[2]) + xn[1] * (yn[2] - yn[0]) + xn[2] * (yn[0] - yn[1]));
        if (area < 0) {
            m.elem_vol[e] = -area;
            std::swap(t[1], t[2]);
        } else {
            m.elem_vol[e] = area;
        }
    }
    EdgeMap hm((size_t)N * 2 + 16);
    std::vector<int> en0, en1, eL, eR;
    en0.reserve((size_t)N * 3 / 2 + 16);
    en1.reserve(en0.capacity());
    eL.reserve(en0.capacity());
    eR.reserve(en0.capacity());
    for (int e = 0; e < N; e++) {
        const int* t = &tri[3 * (size_t)e];
        for (int k = 0; k < 3; k++) {
            int a = t[k], b = t[(k + 1) % 3];
            int ei = hm.get(a, b);
            if (ei < 0) {
                hm.put(a, b, (int)en0.size());
                en0.push_back(a);
                en1.push_back(b);
                eL.push_back(e);
                eR.push_back(-1);
            } else {
                eR[ei] = e;
            }
        }
    }
    const int E = (int)en0.size();
    m.E = E;
    std::vector<int> pedges(3 * (size_t)N);
    for (int e = 0; e < N; e++) {
        const int* t = &tri[3 * (size_t)e];
        double sx = 0, sy = 0;
        for (int i = 0; i < 3; i++) {
            sx += nx[idx[t[i]]];
            sy += ny[idx[t[i]]];
        }
        m.elem_xy[e] = sx / 3.0;
        m.elem_xy[(size_t)N + e] = sy / 3.0;
        for (int k = 0; k < 3; k++) pedges[3 * (size_t)e + k] = hm.get(t[k], t[(k + 1) % 3]);
    }
    // boundary sets, SU2MeshReader.cpp:201-243
    const int NB = (int)mk.size();
    m.NB = NB;
    m.bc_type.resize(NB);
    m.bc_name.resize(NB);
    m.edge_set.assign(E, -1);
    std::vector<std::vector<int>> setedges(NB);
    struct Pair { int type, s0, s1; };
    std::vector<Pair> pairs;
    for (int s = 0; s < NB; s++) {
        int bt = name_to_type(mk[s].name, equation);
        if (bt == -2) return fail(FVGB_ERR_MESH, "unknown boundary type " + mk[s].name);
        m.bc_type[s] = bt;
        m.bc_name[s] = mk[s].name;
        size_t ne = r.marker_edge_ids ? mk[s].e.size() : mk[s].e.size() / 2;
        setedges[s].resize(ne);
        for (size_t k = 0; k < ne; k++) {
            // edge IDs are 1-based positions in the assembled order (FVM_2D.cpp:121)
            int ei = r.marker_edge_ids ? ((mk[s].e[k] >= 1 && mk[s].e[k] <= E) ? mk[s].e[k] - 1 : -1)
                                       : hm.get(mk[s].e[2 * k], mk[s].e[2 * k + 1]);
            if (ei < 0) return fail(FVGB_ERR_MESH, "boundary edge is not an edge of the mesh");
            m.edge_set[ei] = s + 1;
            setedges[s][k] = ei;
        }
        if (is_periodic(bt)) {
            int ip = -1;
            for (size_t q = 0; q < pairs.size(); q++)
                if (pairs[q].type == bt) ip = (int)q;
            if (ip != -1) pairs[ip].s1 = s + 1;
            else pairs.push_back(Pair{bt, s + 1, -1});
        }
    }
    auto ex = [&](int ei) { return (nx[idx[en0[ei]]] + nx[idx[en1[ei]]]) / 2.0; };
    auto ey = [&](int ei) { return (ny[idx[en0[ei]]] + ny[idx[en1[ei]]]) / 2.0; };
    // BoundaryManager_2D::checkPeriodPairs, BoundaryManager_2D.cpp:183-255
    for (const Pair& pr : pairs) {
        if (pr.s0 == -1 || pr.s1 == -1) return fail(FVGB_ERR_MESH, "periodic boundaries do not appear in pairs");
        const auto& a = setedges[pr.s0 - 1];
        const auto& b = setedges[pr.s1 - 1];
        if (a.size() != b.size()) return fail(FVGB_ERR_MESH, "periodic boundary edge counts do not match");
        const int n = (int)a.size();
        if (n == 0) continue;
        double tx = ex(b[n - 1]) - ex(a[0]), ty = ey(b[n - 1]) - ey(a[0]);
        for (int k = 0; k < n; k++) {
            double rx = ex(b[n - 1 - k]) - (ex(a[k]) + tx), ry = ey(b[n - 1 - k]) - (ey(a[k]) + ty);
            if ((rx * rx + ry * ry) / (tx * tx + ty * ty) >= 0.0001)
                return fail(FVGB_ERR_MESH, "periodic boundary is not a translation of its pair");
        }
    }
    m.node_id = nid;
    m.set_edges = setedges;
    // OldDataConverter
    m.node_xy.resize(2 * (size_t)V);
    for (int i = 0; i < V; i++) {
        m.node_xy[i] = nx[i];
        m.node_xy[(size_t)V + i] = ny[i];
    }
    m.elem_nodes.resize(4 * (size_t)N);
    m.elem_edges.resize(4 * (size_t)N);
    m.elem_nbrs.resize(4 * (size_t)N);
    for (int e = 0; e < N; e++) {
        for (int j = 0; j < 3; j++) {
            m.elem_nodes[(size_t)j * N + e] = idx[tri[3 * (size_t)e + j]];
            m.elem_edges[(size_t)j * N + e] = pedges[3 * (size_t)e + j];
            int ei = pedges[3 * (size_t)e + j];
            int nb = -1;  // Element_2D::findNeighbor, FVMR/src/legacy/Element_2D.cpp:19-48
            if (eL[ei] == e) nb = eR[ei];
            else if (eR[ei] == e) nb = eL[ei];
            m.elem_nbrs[(size_t)j * N + e] = nb;
        }
        m.elem_nodes[3 * (size_t)N + e] = -1;
        m.elem_edges[3 * (size_t)N + e] = -1;
        m.elem_nbrs[3 * (size_t)N + e] = -1;
    }
    m.edge_nodes.resize(2 * (size_t)E);
    m.edge_L = eL;
    m.edge_R = eR;
    m.edge_pair.assign(E, -1);
    m.edge_len.resize(E);
    m.edge_dist.resize(E);
    m.edge_xy.resize(2 * (size_t)E);
    m.edge_normal.resize(2 * (size_t)E);
    for (int i = 0; i < E; i++) {
        const int a = idx[en0[i]], b = idx[en1[i]];
        const double x0 = nx[a], y0 = ny[a], x1 = nx[b], y1 = ny[b];
        m.edge_nodes[i] = a;
        m.edge_nodes[(size_t)E + i] = b;
        // Edge_2D::getLength then (float), FVMR/src/legacy/Edge_2D.cpp:19-28
        m.edge_len[i] = (double)(float)std::sqrt((x0 - x1) * (x0 - x1) + (y0 - y1) * (y0 - y1));
        // Edge_2D::getRefLength in float arithmetic, Edge_2D.cpp:30-52
        float xl = (float)m.elem_xy[eL[i]], yl = (float)m.elem_xy[(size_t)N + eL[i]];
        if (eR[i] < 0) {
            float dx = (float)((x0 + x1) / 2.0) - xl, dy = (float)((y0 + y1) / 2.0) - yl;
            m.edge_dist[i] = (double)(2.0f * std::sqrt(dx * dx + dy * dy));
        } else {
            float dx = (float)m.elem_xy[eR[i]] - xl, dy = (float)m.elem_xy[(size_t)N + eR[i]] - yl;
            m.edge_dist[i] = (double)std::sqrt(dx * dx + dy * dy);
        }
        m.edge_xy[i] = (x0 + x1) / 2.0;
        m.edge_xy[(size_t)E + i] = (y0 + y1) / 2.0;
        double dx = x1 - x0, dy = y1 - y0;
        m.edge_normal[i] = dy / m.edge_len[i];
        m.edge_normal[(size_t)E + i] = -dx / m.edge_len[i];
    }
    for (int s = 0; s < NB; s++) {
        if (!is_periodic(m.bc_type[s])) continue;
        int other = -1;
        for (const Pair& pr : pairs)
            if (pr.type == m.bc_type[s]) {
                other = (pr.s0 == s + 1) ? pr.s1 : pr.s0;
                break;
            }
        const auto& a = setedges[s];
        const auto& b = setedges[other - 1];
        const int n = (int)a.size();
        for (int k = 0; k < n; k++) {
            int index0 = k;  // VirtualBoundarySet_2D::getEdgeIndex returns the first position
            for (int q = 0; q < k; q++)
                if (a[q] == a[k]) {
                    index0 = q;
                    break;
                }
            int pe = b[n - 1 - index0];
            m.edge_R[a[k]] = m.edge_L[pe];
            m.edge_pair[a[k]] = pe;
        }
    }
    return 0;
}

void mesh_view(const HostMesh& m, fvgb_mesh_soa& s) {
    s.num_node = m.V;
    s.num_element = m.N;
    s.num_edge = m.E;
    s.num_boundary = m.NB;
    s.node_xy = m.node_xy.data();
    s.elem_nodes = m.elem_nodes.data();
    s.elem_edges = m.elem_edges.data();
    s.elem_neighbors = m.elem_nbrs.data();
    s.elem_xy = m.elem_xy.data();
    s.elem_volume = m.elem_vol.data();
    s.edge_nodes = m.edge_nodes.data();
    s.edge_L = m.edge_L.data();
    s.edge_R = m.edge_R.data();
    s.edge_setID = m.edge_set.data();
    s.edge_periodicPair = m.edge_pair.data();
    s.edge_length = m.edge_len.data();
    s.edge_distance = m.edge_dist.data();
    s.edge_xy = m.edge_xy.data();
    s.edge_normal = m.edge_normal.data();
    s.boundary_type = m.bc_type.data();
    m.set_off.assign(1, 0);
    m.set_list.clear();
    m.name_ptrs.clear();
    for (int b = 0; b < m.NB; b++) {
        if (b < (int)m.set_edges.size()) m.set_list.insert(m.set_list.end(), m.set_edges[b].begin(), m.set_edges[b].end());
        m.set_off.push_back((int)m.set_list.size());
        m.name_ptrs.push_back(b < (int)m.bc_name.size() ? m.bc_name[b].c_str() : "");
    }
    const bool have_sets = (int)m.set_edges.size() == m.NB;
    s.set_edge_offsets = have_sets ? m.set_off.data() : nullptr;
    s.set_edge_list = have_sets ? m.set_list.data() : nullptr;
    s.set_names = m.name_ptrs.data();
}

// ruvp2U_host, FVMR/src/math/PhysicalKernel.h:20-27
static void ruvp_to_U(const double* r, double* U, double gamma) {
    U[0] = r[0];
    U[1] = r[0] * r[1];
    U[2] = r[0] * r[2];
    U[3] = r[3] / (gamma - 1) + 0.5 * r[0] * (r[1] * r[1] + r[2] * r[2]);
}

int initial_field(const fvgb_mesh_soa& s, const fvgb_params& p, double* U) {
    const int N = s.num_element;
    const double gamma = p.gamma;
    double u4[4];
    switch (p.ic_type) {
    case 1:  // setInitialUniform, FVMR/src/input/FieldInitializer.cpp:129-137
        ruvp_to_U(p.inf, u4, gamma);
        for (int e = 0; e < N; e++)
            for (int j = 0; j < 4; j++) U[(size_t)j * N + e] = u4[j];
        return 0;
    case 2: {  // setInitialIsentropicVortex, FieldInitializer.cpp:139-177
        const double xc = p.vortex[0], yc = p.vortex[1], chi = p.vortex[2];
        const double ga1 = gamma - 1.0;
        const double c_du = chi / (2.0 * kPi);
        const double c_dT = ga1 * (chi * chi) / (8. * gamma * (kPi * kPi));
        for (int e = 0; e < N; e++) {
            double dx = s.elem_xy[e] - xc, dy = s.elem_xy[(size_t)N + e] - yc;
            double one_minus_r2 = 1.0 - (dx * dx + dy * dy);
            double c_distance = std::exp(0.5 * one_minus_r2);
            double u = p.inf[1] + c_du * c_distance * (-dy);
            double v = p.inf[2] + c_du * c_distance * dx;
            double dT = -c_dT * std::exp(one_minus_r2);
            double rho = std::pow(p.inf[3] + dT, 1. / ga1);
            double r[4] = {rho, u, v, rho * (p.inf[3] + dT)};
            ruvp_to_U(r, u4, gamma);
            for (int j = 0; j < 4; j++) U[(size_t)j * N + e] = u4[j];
        }
        return 0;
    }
    case 3: {  // setInitialShockTube, FieldInitializer.cpp:179-222
        double sx = p.shock[0], sy = p.shock[1], nxs = p.shock[2], nys = p.shock[3];
        if (nxs == 0.0 && nys == 0.0) nxs = 1.0;
        double li = 1.0 / std::sqrt(nxs * nxs + nys * nys);
        nxs *= li;
        nys *= li;
        double ui[4], uo[4];
        ruvp_to_U(p.inlet, ui, gamma);
        ruvp_to_U(p.outlet, uo, gamma);
        for (int e = 0; e < N; e++) {
            double x = s.elem_xy[e], y = s.elem_xy[(size_t)N + e];
            bool inlet;
            if (nxs == 1.0) inlet = x < sx;
            else inlet = !((x - sx) * nxs + (y - sy) * nys > 0);
            for (int j = 0; j < 4; j++) U[(size_t)j * N + e] = inlet ? ui[j] : uo[j];
        }
        return 0;
    }
    case 4: {  // setInitialDoubleShockReflection, FieldInitializer.cpp:224-260: upstream of the
               // shock line (CBoundaryDoubleShockReflect::isUpStreamOfShock_forElement,
               // CBoundaryDoubleShockReflect.cpp:17-33) takes the inlet state
        const double angle = p.dsr[2] * kPi / 180.0;
        const double nxs = -std::sin(angle), nys = std::cos(angle);
        double ui[4], uo[4];
        ruvp_to_U(p.inlet, ui, gamma);
        ruvp_to_U(p.outlet, uo, gamma);
        for (int e = 0; e < N; e++) {
            const double rx = s.elem_xy[e] - p.dsr[0], ry = s.elem_xy[(size_t)N + e] - p.dsr[1];
            const bool upstream = rx * nxs + ry * nys > 0;
            for (int j = 0; j < 4; j++) U[(size_t)j * N + e] = upstream ? ui[j] : uo[j];
        }
        return 0;
    }
    default:
        return fail(FVGB_ERR_UNSUPPORTED, "initialCondition.type not supported on this path");
    }
}

}  // namespace fvgb

using namespace fvgb;

extern "C" int fvgb_mesh_read_su2(const char* path, int equation, double scale, fvgb_mesh** out) {
    if (!path || !out) return fail(FVGB_ERR_ARG, "null argument");
    fvgb_mesh* m = new fvgb_mesh();
    int rc = read_su2(path, equation, scale, m->m);
    if (rc) {
        delete m;
        *out = nullptr;
        return rc;
    }
    *out = m;
    return 0;
}

extern "C" int fvgb_mesh_view(const fvgb_mesh* m, fvgb_mesh_soa* soa) {
    if (!m || !soa) return fail(FVGB_ERR_ARG, "null argument");
    mesh_view(m->m, *soa);
    return 0;
}

extern "C" void fvgb_mesh_free(fvgb_mesh* m) { delete m; }

extern "C" int fvgb_initial_field(const fvgb_mesh_soa* mesh, const fvgb_params* p, double* U) {
    if (!mesh || !p || !U) return fail(FVGB_ERR_ARG, "null argument");
    return initial_field(*mesh, *p, U);
}

// ---- synthetic meshes -------------------------------------------------------

namespace {
struct Writer {
    FILE* f;
    std::vector<char> buf;
    size_t n = 0;
    explicit Writer(FILE* ff) : f(ff), buf(1 << 22) {}
    void flush() {
        std::fwrite(buf.data(), 1, n, f);
        n = 0;
    }
    void printf_(const char* fmt, ...) __attribute__((format(printf, 2, 3))) {
        if (buf.size() - n < 512) flush();
        va_list ap;
        va_start(ap, fmt);
        int k = std::vsnprintf(buf.data() + n, buf.size() - n, fmt, ap);
        va_end(ap);
        n += (size_t)k;
    }
    ~Writer() { flush(); }
};

// splitmix64: deterministic on every platform
uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
double uniform(uint64_t& s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }
}  // namespace

extern "C" int fvgb_write_su2_periodic_square(const char* path, int n, double L, double jitter, unsigned long long seed) {
    if (!path || n < 2 || !(L > 0)) return fail(FVGB_ERR_ARG, "bad square mesh arguments");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(FVGB_ERR_IO, std::string("cannot write ") + path);
    {
        Writer w(f);
        const double h = L / n;
        const int nn = n + 1;
        w.printf_("%% periodic square [0,%.17g]^2, %d x %d quads, jitter %.17g h, seed %llu\nNDIME= 2\n", L, n, n,
                  jitter, seed);
        w.printf_("NELEM= %lld\n", (long long)n * n);
        long long q = 0;
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++)  // CCW: (i,j) (i+1,j) (i+1,j+1) (i,j+1)
                w.printf_("9 %d %d %d %d %lld\n", j * nn + i, j * nn + i + 1, (j + 1) * nn + i + 1, (j + 1) * nn + i, q++);
        w.printf_("NPOIN= %d\n", nn * nn);
        uint64_t st = seed;
        for (int j = 0; j < nn; j++)
            for (int i = 0; i < nn; i++) {
                double x = i * h, y = j * h;
                if (i == n) x = L;
                if (j == n) y = L;
                if (i > 0 && i < n && j > 0 && j < n && jitter > 0) {
                    x += (2.0 * uniform(st) - 1.0) * jitter * h;
                    y += (2.0 * uniform(st) - 1.0) * jitter * h;
                }
                w.printf_("%.17g %.17g %d\n", x, y, j * nn + i);
            }
        // periodic_1: x=0 ascending y and x=L descending y; periodic_2: y=L ascending x
        // and y=0 descending x (the marker orientation of the reference's vortex case)
        w.printf_("NMARK= 4\n");
        w.printf_("MARKER_TAG= periodic_1\nMARKER_ELEMS= %d\n", n);
        for (int j = 0; j < n; j++) w.printf_("3 %d %d\n", j * nn, (j + 1) * nn);
        w.printf_("MARKER_TAG= periodic_1\nMARKER_ELEMS= %d\n", n);
        for (int j = n; j > 0; j--) w.printf_("3 %d %d\n", j * nn + n, (j - 1) * nn + n);
        w.printf_("MARKER_TAG= periodic_2\nMARKER_ELEMS= %d\n", n);
        for (int i = 0; i < n; i++) w.printf_("3 %d %d\n", n * nn + i, n * nn + i + 1);
        w.printf_("MARKER_TAG= periodic_2\nMARKER_ELEMS= %d\n", n);
        for (int i = n; i > 0; i--) w.printf_("3 %d %d\n", i, i - 1);
    }
    std::fclose(f);
    return 0;
}

extern "C" int fvgb_write_su2_cylinder(const char* path, int nt, int nr, double r0, double r1, double first_dr) {
    if (!path || nt < 3 || nr < 1 || !(r1 > r0) || !(r0 > 0) || !(first_dr > 0))
        return fail(FVGB_ERR_ARG, "bad cylinder mesh arguments");
    // geometric radial spacing: r_k = r0 + d1 (q^k - 1)/(q - 1) with r_nr = r1
    std::vector<double> r(nr + 1);
    const double span = r1 - r0;
    if (first_dr * nr >= span) {
        for (int k = 0; k <= nr; k++) r[k] = r0 + span * k / nr;
    } else {
        double lo = 1.0 + 1e-12, hi = 2.0;
        auto total = [&](double q) { return first_dr * (std::pow(q, nr) - 1.0) / (q - 1.0); };
        while (total(hi) < span) hi *= 2.0;
        for (int it = 0; it < 200; it++) {
            double mid = 0.5 * (lo + hi);
            if (total(mid) < span) lo = mid;
            else hi = mid;
        }
        double q = 0.5 * (lo + hi);
        for (int k = 0; k <= nr; k++) r[k] = r0 + first_dr * (std::pow(q, k) - 1.0) / (q - 1.0);
        r[nr] = r1;
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(FVGB_ERR_IO, std::string("cannot write ") + path);
    {
        Writer w(f);
        w.printf_("%% cylinder O-grid r0=%.17g r1=%.17g, %d x %d quads, first spacing %.17g\nNDIME= 2\n", r0, r1, nt, nr,
                  first_dr);
        auto node = [&](int i, int k) { return k * nt + (i % nt); };
        w.printf_("NELEM= %lld\n", (long long)nt * nr);
        long long q = 0;
        for (int k = 0; k < nr; k++)
            for (int i = 0; i < nt; i++)  // CCW: inner (i), outer (i), outer (i+1), inner (i+1)
                w.printf_("9 %d %d %d %d %lld\n", node(i, k), node(i, k + 1), node(i + 1, k + 1), node(i + 1, k), q++);
        w.printf_("NPOIN= %d\n", nt * (nr + 1));
        for (int k = 0; k <= nr; k++)
            for (int i = 0; i < nt; i++) {
                double th = 2.0 * kPi * i / nt;
                w.printf_("%.17g %.17g %d\n", r[k] * std::cos(th), r[k] * std::sin(th), node(i, k));
            }
        w.printf_("NMARK= 2\nMARKER_TAG= wall\nMARKER_ELEMS= %d\n", nt);
        for (int i = 0; i < nt; i++) w.printf_("3 %d %d\n", node(i, 0), node(i + 1, 0));
        w.printf_("MARKER_TAG= farfield\nMARKER_ELEMS= %d\n", nt);
        for (int i = 0; i < nt; i++) w.printf_("3 %d %d\n", node(i, nr), node(i + 1, nr));
    }
    std::fclose(f);
    return 0;
}

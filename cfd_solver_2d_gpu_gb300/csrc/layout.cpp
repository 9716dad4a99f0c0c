// Device layout of one mesh: cell renumbering, edge ordering and the per-cell /
// per-edge geometric coefficients the kernels read, all derived on the host
// from the reference-order mesh.
//
// Every coefficient is computed with the reference's own operation sequence,
// so the values the kernels start from are the reference's bit for bit:
//   * least-squares weights B = (A^T A)^-1 A^T per cell with the 2x2 inverse of
//     FVMR/src/math/MatrixKernel.h:45-59 (GradientLeastSquare_2,
//     FVMR/src/space/gradient/Gradient.cpp:160-246 forms the same products);
//   * Green-Gauss face weights g_C, 1-g_C, S_f*sign and 1/vol
//     (Gradient.cpp:248-458);
//   * vertex offsets x_node - x_cell of the Barth limiter (Gradient.cpp:88-95);
//   * reconstruction offsets x_face - x_cell for both sides of every edge, the
//     periodic R side using its partner's midpoint (FVMR/src/space/Flux.cpp:165-184);
//   * -1/vol of calculateFunctionF (FVMR/src/time/Evolve.cpp:107).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <vector>

#include "layout.h"

namespace fvgb {

namespace {
uint64_t spread(uint32_t x) {
    uint64_t v = x;
    v = (v | (v << 16)) & 0x0000FFFF0000FFFFULL;
    v = (v | (v << 8)) & 0x00FF00FF00FF00FFULL;
    v = (v | (v << 4)) & 0x0F0F0F0F0F0F0F0FULL;
    v = (v | (v << 2)) & 0x3333333333333333ULL;
    v = (v | (v << 1)) & 0x5555555555555555ULL;
    return v;
}
bool is_periodic(int t) { return t >= BC_PERIODIC_0 && t <= BC_PERIODIC_9; }

}  // namespace

// The caller's arrays are checked before anything indexes them, so that a bad
// index is an error code rather than a host crash or an out-of-bounds gather on
// the device (every device index is derived from these).
int validate_mesh(const fvgb_mesh_soa& m) {
    const int N = m.num_element, E = m.num_edge, V = m.num_node, NB = m.num_boundary;
    if (N < 0 || E < 0 || V < 0 || NB < 0) return fail(FVGB_ERR_MESH, "negative mesh sizes");
    if (N == 0) return fail(FVGB_ERR_MESH, "mesh has no cells");  // as the su2 reader refuses one
    if ((N > 0 && (!m.elem_edges || !m.elem_nodes || !m.elem_neighbors || !m.elem_xy || !m.elem_volume)) ||
        (E > 0 && (!m.edge_L || !m.edge_R || !m.edge_setID || !m.edge_periodicPair || !m.edge_length ||
                   !m.edge_xy || !m.edge_normal || !m.edge_nodes)) ||
        (V > 0 && !m.node_xy) || (NB > 0 && !m.boundary_type))
        return fail(FVGB_ERR_MESH, "a mesh array is NULL");
    auto in = [](int x, int lo, int hi) { return x >= lo && x < hi; };
    for (int e = 0; e < E; e++) {
        const int s = m.edge_setID[e];
        if (!in(m.edge_L[e], 0, N) || !in(m.edge_R[e], -1, N) || !(s == -1 || in(s, 1, NB + 1)) ||
            !in(m.edge_periodicPair[e], -1, E) || !in(m.edge_nodes[e], 0, V) ||
            !in(m.edge_nodes[(size_t)E + e], 0, V))
            return fail(FVGB_ERR_MESH, "edge " + std::to_string(e) + " refers outside the mesh");
    }
    for (int c = 0; c < N; c++)
        for (int j = 0; j < 3; j++)
            if (!in(m.elem_edges[(size_t)j * N + c], 0, E) || !in(m.elem_nodes[(size_t)j * N + c], 0, V) ||
                !in(m.elem_neighbors[(size_t)j * N + c], -1, N))
                return fail(FVGB_ERR_MESH, "cell " + std::to_string(c) + " refers outside the mesh");
    if (m.set_edge_offsets && m.set_edge_list) {
        if (m.set_edge_offsets[0] != 0) return fail(FVGB_ERR_MESH, "boundary set offsets do not start at 0");
        for (int b = 0; b < NB; b++)
            if (m.set_edge_offsets[b + 1] < m.set_edge_offsets[b]) return fail(FVGB_ERR_MESH, "boundary set offsets decrease");
        for (int i = 0; i < (NB > 0 ? m.set_edge_offsets[NB] : 0); i++)
            if (!in(m.set_edge_list[i], 0, E)) return fail(FVGB_ERR_MESH, "boundary set edge outside the mesh");
    }
    return 0;
}

int build_layout(const fvgb_mesh_soa& m, const fvgb_params& p, Layout& L) {
    if (int rc = validate_mesh(m)) return rc;
    const int N = m.num_element, E = m.num_edge, V = m.num_node;
    L = Layout();
    L.N = N;
    L.E = E;
    // ---- cell order -------------------------------------------------------
    L.cell_new.resize(N);
    L.cell_ref.resize(N);
    std::iota(L.cell_ref.begin(), L.cell_ref.end(), 0);
    if (p.renumber == 1 && N > 1) {
        double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
        for (int c = 0; c < N; c++) {
            xmin = std::min(xmin, m.elem_xy[c]);
            xmax = std::max(xmax, m.elem_xy[c]);
            ymin = std::min(ymin, m.elem_xy[(size_t)N + c]);
            ymax = std::max(ymax, m.elem_xy[(size_t)N + c]);
        }
        double sx = (xmax > xmin) ? 1048575.0 / (xmax - xmin) : 0.0;
        double sy = (ymax > ymin) ? 1048575.0 / (ymax - ymin) : 0.0;
        std::vector<uint64_t> code(N);
        for (int c = 0; c < N; c++) {
            uint32_t ix = (uint32_t)((m.elem_xy[c] - xmin) * sx);
            uint32_t iy = (uint32_t)((m.elem_xy[(size_t)N + c] - ymin) * sy);
            code[c] = spread(ix) | (spread(iy) << 1);
        }
        std::stable_sort(L.cell_ref.begin(), L.cell_ref.end(), [&](int a, int b) { return code[a] < code[b]; });
    }
    for (int i = 0; i < N; i++) L.cell_new[L.cell_ref[i]] = i;

    // ---- edge order: interior and periodic edges first, then the other boundary
    // edges grouped by type; inside a group by the new index of their L cell -----
    auto bc_of = [&](int e) {
        int s = m.edge_setID[e];
        if (s == -1) return (int)BC_INTERIOR;
        int t = m.boundary_type[s - 1];
        return is_periodic(t) ? (int)BC_INTERIOR : t;
    };
    L.edge_ref.resize(E);
    std::iota(L.edge_ref.begin(), L.edge_ref.end(), 0);
    std::stable_sort(L.edge_ref.begin(), L.edge_ref.end(), [&](int a, int b) {
        int ta = bc_of(a), tb = bc_of(b);
        if (ta != tb) return ta < tb;  // -1 (interior) sorts first
        if (p.renumber == 1) return L.cell_new[m.edge_L[a]] < L.cell_new[m.edge_L[b]];
        return false;
    });
    L.edge_new.resize(E);
    for (int i = 0; i < E; i++) L.edge_new[L.edge_ref[i]] = i;
    L.E_int = 0;
    while (L.E_int < E && bc_of(L.edge_ref[L.E_int]) == BC_INTERIOR) L.E_int++;

    // ---- per-edge arrays ----------------------------------------------------
    L.e_L.resize(E);
    L.e_R.resize(E);
    L.e_bc.resize(E);
    L.e_geom.resize((size_t)E * 8);
    for (int i = 0; i < E; i++) {
        const int e = L.edge_ref[i];
        const int l = m.edge_L[e], r = m.edge_R[e];
        L.e_L[i] = L.cell_new[l];
        L.e_R[i] = r < 0 ? -1 : L.cell_new[r];
        L.e_bc[i] = bc_of(e);
        double* g = &L.e_geom[(size_t)i * 8];
        const double fx = m.edge_xy[e], fy = m.edge_xy[(size_t)E + e];
        g[0] = m.edge_normal[e];
        g[1] = m.edge_normal[(size_t)E + e];
        g[2] = m.edge_length[e];
        g[3] = 0.0;
        g[4] = fx - m.elem_xy[l];
        g[5] = fy - m.elem_xy[(size_t)N + l];
        if (r >= 0) {
            double rx = fx, ry = fy;
            if (m.edge_setID[e] != -1) {  // periodic: R is reconstructed at the partner's midpoint
                const int pe = m.edge_periodicPair[e];
                if (pe < 0 || pe >= E) return fail(FVGB_ERR_MESH, "periodic edge without a partner");
                rx = m.edge_xy[pe];
                ry = m.edge_xy[(size_t)E + pe];
            }
            g[6] = rx - m.elem_xy[r];
            g[7] = ry - m.elem_xy[(size_t)N + r];
        } else {  // boundary edge: its midpoint (the double-Mach-reflection boundary tests it)
            g[6] = fx;
            g[7] = fy;
        }
    }

    // ---- per-cell arrays ----------------------------------------------------
    L.c_edge.resize((size_t)N * 3);
    L.c_nbr.resize((size_t)N * 3);
    L.c_nnb.resize(N);
    L.c_mvol.resize(N);
    L.c_vol.resize(N);
    L.c_lsq.assign((size_t)N * 6, 0.0);
    L.c_vtx.resize((size_t)N * 6);
    const bool gg = (p.gradient == 2);
    if (gg) {
        L.c_gg.assign((size_t)N * 12, 0.0);
        L.c_ggout.assign((size_t)N * 3, -1);
        L.c_ginv.resize(N);
    }
    for (int i = 0; i < N; i++) {
        const int c = L.cell_ref[i];
        const double xc = m.elem_xy[c], yc = m.elem_xy[(size_t)N + c];
        L.c_vol[i] = m.elem_volume[c];
        L.c_mvol[i] = -1.0 / m.elem_volume[c];
        for (int j = 0; j < 3; j++) {
            int e = m.elem_edges[(size_t)j * N + c];
            if (e < 0 || e >= E) return fail(FVGB_ERR_MESH, "triangle without three edges");
            int ne = L.edge_new[e];
            L.c_edge[(size_t)i * 3 + j] = (c != m.edge_R[e]) ? ne : ~ne;  // sign of add_edge_flux_to_element_flux
            int nd = m.elem_nodes[(size_t)j * N + c];
            L.c_vtx[(size_t)i * 6 + 2 * j] = m.node_xy[nd] - xc;
            L.c_vtx[(size_t)i * 6 + 2 * j + 1] = m.node_xy[(size_t)V + nd] - yc;
        }
        // valid face neighbours in slot order (getElementT3ValidNeighbor, Gradient.cpp:35-47)
        int nb[3], nvn = 0;
        for (int j = 0; j < 3; j++) {
            int q = m.elem_neighbors[(size_t)j * N + c];
            if (q != -1) nb[nvn++] = q;
        }
        L.c_nnb[i] = nvn;
        for (int k = 0; k < 3; k++) L.c_nbr[(size_t)i * 3 + k] = k < nvn ? L.cell_new[nb[k]] : -1;
        if (p.gradient == 1 && nvn > 0) {
            double dX[6], dXt[6], A[4], B[6];
            for (int k = 0; k < nvn; k++) {
                dX[k * 2 + 0] = m.elem_xy[nb[k]] - xc;
                dX[k * 2 + 1] = m.elem_xy[(size_t)N + nb[k]] - yc;
            }
            for (int x = 0; x < nvn; x++)
                for (int y = 0; y < 2; y++) dXt[y * nvn + x] = dX[x * 2 + y];
            for (int x = 0; x < 2; x++)
                for (int y = 0; y < 2; y++) {
                    A[x * 2 + y] = 0.0;
                    for (int z = 0; z < nvn; z++) A[x * 2 + y] += dXt[x * nvn + z] * dX[z * 2 + y];
                }
            double det = A[0] * A[3] - A[1] * A[2];
            if (p.lsq_det_ref) {  // MatrixKernel.h:48-49: every det >= EPS becomes -EPS
                if (det >= 0 && det < kEps) det = kEps;
                else if (det > -kEps) det = -kEps;
            } else {
                if (det >= 0 && det < kEps) det = kEps;
                else if (det < 0 && det > -kEps) det = -kEps;
            }
            const double inv_det = 1.0 / det;
            const double Ai[4] = {A[3] * inv_det, -A[1] * inv_det, -A[2] * inv_det, A[0] * inv_det};
            for (int x = 0; x < 2; x++)
                for (int y = 0; y < nvn; y++) {
                    B[x * nvn + y] = 0.0;
                    for (int z = 0; z < 2; z++) B[x * nvn + y] += Ai[x * 2 + z] * dXt[z * nvn + y];
                }
            for (int x = 0; x < 2; x++)
                for (int k = 0; k < nvn; k++) L.c_lsq[(size_t)i * 6 + x * 3 + k] = B[x * nvn + k];
        } else if (p.gradient == 1 && nvn == 0) {
            return fail(FVGB_ERR_MESH, "least-squares gradient of a cell without neighbours");
        }
        if (gg) {
            for (int j = 0; j < 3; j++) {
                const int e = m.elem_edges[(size_t)j * N + c];
                int sign, out;
                if (c != m.edge_R[e]) { sign = 1; out = m.edge_R[e]; }
                else { sign = -1; out = m.edge_L[e]; }
                const double Sx = m.edge_normal[e] * m.edge_length[e];
                const double Sy = m.edge_normal[(size_t)E + e] * m.edge_length[e];
                double gC = 0.5;
                if (out != -1) {
                    const double fx = m.edge_xy[e], fy = m.edge_xy[(size_t)E + e];
                    double Fx = m.elem_xy[out], Fy = m.elem_xy[(size_t)N + out];
                    if (m.edge_setID[e] != -1) {
                        const int pe = m.edge_periodicPair[e];
                        Fx += fx - m.edge_xy[pe];
                        Fy += fy - m.edge_xy[(size_t)E + pe];
                    }
                    double dfx = fx - Fx, dfy = fy - Fy, dcx = xc - Fx, dcy = yc - Fy;
                    double dFf = std::sqrt(dfx * dfx + dfy * dfy);
                    double dFC = std::sqrt(dcx * dcx + dcy * dcy);
                    if (dFC < kEps) dFC = kEps;
                    gC = dFf / dFC;
                }
                double* w = &L.c_gg[(size_t)i * 12 + 4 * j];
                w[0] = gC;
                w[1] = 1.0 - gC;
                w[2] = Sx * (double)sign;  // (phif*Sx)*sign == phif*(Sx*sign): a sign flip is exact
                w[3] = Sy * (double)sign;
                L.c_ggout[(size_t)i * 3 + j] = out < 0 ? -1 : L.cell_new[out];
            }
            L.c_ginv[i] = 1 / m.elem_volume[c];
        }
    }
    // ---- time-step contributions: per cell, the edges touching it in reference
    // edge order (update_alphaC_host, FVMR/src/time/CalculateDt.cpp:207-247) ----
    L.dt_ptr.assign((size_t)N + 1, 0);
    for (int e = 0; e < E; e++) {
        L.dt_ptr[L.cell_new[m.edge_L[e]] + 1]++;
        if (m.edge_R[e] != -1) L.dt_ptr[L.cell_new[m.edge_R[e]] + 1]++;
    }
    for (int i = 0; i < N; i++) L.dt_ptr[i + 1] += L.dt_ptr[i];
    L.dt_edge.resize(L.dt_ptr[N]);
    std::vector<int> fill(L.dt_ptr.begin(), L.dt_ptr.end() - 1);
    for (int e = 0; e < E; e++) {
        L.dt_edge[fill[L.cell_new[m.edge_L[e]]]++] = L.edge_new[e];
        if (m.edge_R[e] != -1) L.dt_edge[fill[L.cell_new[m.edge_R[e]]]++] = L.edge_new[e];
    }
    if (p.edge_colour) return build_edge_colours(L);
    return 0;
}

// Greedy edge colouring for the coloured scatter: edges visited in device order take the
// smallest colour that no edge already coloured uses at a cell this edge writes (its L cell,
// and its R cell where the edge is in R's edge list).  The colours' edge lists keep the device
// order.  A cell writes at most three edge slots, so at most five colours are needed.
int build_edge_colours(Layout& L) {
    const int N = L.N, E = L.E;
    L.e_in_r.assign(E, 0);
    for (int c = 0; c < N; c++)
        for (int j = 0; j < 3; j++) {
            const int r = L.c_edge[(size_t)c * 3 + j];
            if (r < 0) L.e_in_r[~r] = 1;
        }
    std::vector<uint32_t> used(N, 0u);
    std::vector<int> colour(E);
    int nc = 0;
    for (int e = 0; e < E; e++) {
        const int l = L.e_L[e], r = L.e_in_r[e] ? L.e_R[e] : -1;
        const uint32_t busy = used[l] | (r >= 0 ? used[r] : 0u);
        if (busy == 0xffffffffu) return fail(FVGB_ERR_MESH, "edge colouring needs more than 32 colours");
        int k = 0;
        while (busy & (1u << k)) k++;
        colour[e] = k;
        used[l] |= 1u << k;
        if (r >= 0) used[r] |= 1u << k;
        nc = std::max(nc, k + 1);
    }
    L.col_ptr.assign((size_t)nc + 1, 0);
    for (int e = 0; e < E; e++) L.col_ptr[colour[e] + 1]++;
    for (int k = 0; k < nc; k++) L.col_ptr[k + 1] += L.col_ptr[k];
    L.col_edge.resize(E);
    std::vector<int> fill(L.col_ptr.begin(), L.col_ptr.end() - 1);
    for (int e = 0; e < E; e++) L.col_edge[fill[colour[e]]++] = e;
    L.e_colour = colour;
    return 0;
}

}  // namespace fvgb

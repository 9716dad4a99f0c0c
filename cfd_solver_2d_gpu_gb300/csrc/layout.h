// Device layout of one mesh (host-side description; see layout.cpp).
#pragma once
#include <vector>

#include "internal.h"

namespace fvgb {

struct Layout {
    int N = 0, E = 0, E_int = 0;     // cells, edges, interior+periodic edges (first E_int)
    std::vector<int> cell_new, cell_ref;  // reference <-> device cell index
    std::vector<int> edge_new, edge_ref;  // reference <-> device edge index
    // edges (device order)
    std::vector<int> e_L, e_R, e_bc;
    std::vector<double> e_geom;      // [E][8]: nx, ny, length, 0, dLx, dLy, dRx, dRy
                                     // (boundary edges: the midpoint x, y in place of dRx, dRy)
    // cells (device order)
    std::vector<int> c_edge;         // [N][3]: edge index, or ~index where the cell is R
    std::vector<int> c_nbr;          // [N][3]: valid face neighbours first, -1 after
    std::vector<int> c_nnb;          // [N]
    std::vector<double> c_mvol;      // [N] -1/vol
    std::vector<double> c_vol;       // [N]
    std::vector<double> c_lsq;       // [N][2][3] least-squares weights
    std::vector<double> c_vtx;       // [N][3][2] vertex - centroid
    std::vector<double> c_gg;        // [N][3][4] g_C, 1-g_C, Sx*sign, Sy*sign
    std::vector<int> c_ggout;        // [N][3] Green-Gauss outer cell, -1 on boundaries
    std::vector<double> c_ginv;      // [N] 1/vol as the Green-Gauss gradient forms it
    std::vector<int> dt_ptr, dt_edge;  // CSR: edges whose spectral radius a cell sums
    // edge colouring ([gpu] edge_colour = 1): per edge whether R's edge list holds it, its
    // colour, and per colour the edges (device order) in col_edge[col_ptr[k] .. col_ptr[k+1])
    std::vector<int> e_in_r, e_colour, col_ptr, col_edge;
};

// Checks the caller's mesh arrays (sizes, NULL arrays, every index in range) on the
// host; FVGB_ERR_MESH with the reason, 0 if the mesh may be indexed.
int validate_mesh(const fvgb_mesh_soa& m);
int build_layout(const fvgb_mesh_soa& m, const fvgb_params& p, Layout& L);
int build_edge_colours(Layout& L);

}  // namespace fvgb

// Shared declarations of the fvgb library (host side).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "bc_types.h"
#include "fvgb.h"

namespace fvgb {

// constants of FVMR/src/math/CommonValue.h:16-29
constexpr double kEps = 1e-10;
constexpr double kRhoMax = 300.0;
constexpr double kPMax = 400.0 * 101325.0;
constexpr double kPi = 3.1415926535897;

// Host mesh in the reference's numbering and [row][index] layout.
struct HostMesh {
    int N = 0, E = 0, V = 0, NB = 0;
    std::vector<double> node_xy;    // 2V
    std::vector<int> elem_nodes;    // 4N
    std::vector<int> elem_edges;    // 4N
    std::vector<int> elem_nbrs;     // 4N
    std::vector<double> elem_xy;    // 2N
    std::vector<double> elem_vol;   // N
    std::vector<int> edge_nodes;    // 2E
    std::vector<int> edge_L, edge_R, edge_set, edge_pair;  // E
    std::vector<double> edge_len, edge_dist;                // E
    std::vector<double> edge_xy, edge_normal;               // 2E
    std::vector<int> bc_type;       // NB
    std::vector<std::string> bc_name;
    std::vector<int> node_id;                  // V: the reference's node IDs (file index + 1)
    std::vector<std::vector<int>> set_edges;   // NB: each boundary set's edges in set order
    std::vector<double> U;                     // 4N: the state read with a continue file, else empty
    // flattened set_edges and the names' C strings, filled by mesh_view for fvgb_mesh_soa
    mutable std::vector<int> set_off, set_list;
    mutable std::vector<const char*> name_ptrs;
};

// A mesh as read from a file, before assembly: node coordinates and IDs, triangles
// as node IDs (quads already split), and the boundary markers, each a list of
// node-ID pairs (.su2) or of 1-based edge IDs (continue file).
struct RawMesh {
    std::vector<double> nx, ny;
    std::vector<int> nid;
    std::vector<int> tri;
    struct Marker {
        std::string name;
        std::vector<int> e;
    };
    std::vector<Marker> mk;
    bool marker_edge_ids = false;
    int maxnodeID = 1;
};

void set_error(const std::string& msg);
int fail(int code, const std::string& msg);

int read_su2(const char* path, int equation, double scale, HostMesh& m);
int assemble(RawMesh& r, int equation, HostMesh& m);
void mesh_view(const HostMesh& m, fvgb_mesh_soa& s);
int initial_field(const fvgb_mesh_soa& s, const fvgb_params& p, double* U);

}  // namespace fvgb

struct fvgb_mesh {
    fvgb::HostMesh m;
};

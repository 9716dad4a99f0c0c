// Continue ("pause") files: the reference's restart format.
//
//   t, istep, CFL
//   <t> <istep> <CFL>
//   nodes: ID, x, y
//   <node ID> <x> <y>                                   one line per node
//   elements: ID, nodes, U
//   <element ID> <n0> <n1> <n2> <U0> <U1> <U2> <U3>      node IDs, one line per triangle
//   boundaries: ID, name; edgeIDs
//   <set ID> <name>                                     then the set's edge IDs, ten a line
//
// written by FieldWriter::writeContinueFile_1 (FVMR/src/output/FieldWriter.cpp:264-326)
// and read by ContinueFileReader::readContinueFile_1 + process
// (FVMR/src/input/ContinueFileReader.cpp:19-158, 457-494), which rebuilds the
// mesh from the element list with the same assembly as the .su2 path.  Edge IDs
// are 1-based positions in that assembly's order (FVM_2D.cpp:121).  The file
// carries the whole mesh, so a restart needs no .su2 file.
//
// The reference writes with the stream's default 6 significant digits; this
// writer uses 17, so the state and the node coordinates round-trip exactly and
// a restarted run continues bit for bit.  Either reader accepts either file.
#include <dirent.h>

#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

namespace fvgb {
namespace {

// StringProcessor::splitString (FVMR/src/global/StringProcessor.cpp:21-45): space, tab
// and comma separate words ('\r' too, for files written on Windows)
int words(char* s, char** w, int maxw) {
    int n = 0;
    while (*s) {
        while (*s == ' ' || *s == '\t' || *s == ',' || *s == '\r') s++;
        if (!*s) break;
        if (n < maxw) w[n] = s;
        n++;
        while (*s && *s != ' ' && *s != '\t' && *s != ',' && *s != '\r') s++;
        if (*s) *s++ = 0;
    }
    return n < maxw ? n : maxw;
}

}  // namespace

int read_continue(const char* path, int equation, HostMesh& m, double* t, int* istep, double* cfl, bool* has_cfl) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(FVGB_ERR_IO, std::string("cannot open continue file ") + path);
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::vector<char> buf((size_t)sz + 1);
    size_t got = std::fread(buf.data(), 1, (size_t)sz, f);
    std::fclose(f);
    buf[got] = 0;

    RawMesh r;
    r.marker_edge_ids = true;
    std::vector<double> U;  // element-major while reading
    double tt = 0.0, cf = 0.0;
    int is = 0;
    bool seen_t = false, seen_cfl = false;
    int state = -1;
    char* p = buf.data();
    char* end = p + got;
    while (p < end) {
        char* line = p;
        while (p < end && *p != '\n') p++;
        if (p < end) *p++ = 0;
        char* w[24];
        int nw = words(line, w, 24);
        if (nw == 0) continue;
        if (!std::strcmp(w[0], "t")) state = 0;
        else if (!std::strcmp(w[0], "nodes:")) state = 1;
        else if (!std::strcmp(w[0], "edges:")) state = 2;
        else if (!std::strcmp(w[0], "elements:")) state = 3;
        else if (!std::strcmp(w[0], "boundaries:")) state = 4;
        if (state == 0 && w[0][0] != 't') {
            if (nw < 2) return fail(FVGB_ERR_FORMAT, "malformed t, istep line in continue file");
            tt = std::strtod(w[0], nullptr);
            is = (int)std::strtod(w[1], nullptr);
            seen_t = true;
            if (nw == 3) {
                cf = std::strtod(w[2], nullptr);
                seen_cfl = true;
            }
        } else if (state == 1 && w[0][0] != 'n') {
            if (nw < 3) return fail(FVGB_ERR_FORMAT, "malformed node line in continue file");
            const int id = (int)std::strtod(w[0], nullptr);
            r.nid.push_back(id);
            r.nx.push_back(std::strtod(w[1], nullptr));
            r.ny.push_back(std::strtod(w[2], nullptr));
            if (id > r.maxnodeID) r.maxnodeID = id;
        } else if (state == 3 && w[0][0] != 'e') {
            if (nw < 8) return fail(FVGB_ERR_FORMAT, "malformed element line in continue file");
            for (int k = 1; k <= 3; k++) r.tri.push_back((int)std::strtod(w[k], nullptr));
            for (int k = 4; k <= 7; k++) U.push_back(std::strtod(w[k], nullptr));
        } else if (state == 4 && w[0][0] != 'b') {
            if (nw >= 2 && !std::isdigit((unsigned char)w[1][0])) {
                r.mk.push_back(RawMesh::Marker{w[1], {}});
            } else {
                if (r.mk.empty()) return fail(FVGB_ERR_FORMAT, "edge IDs before a boundary name in continue file");
                for (int k = 0; k < nw; k++) r.mk.back().e.push_back(std::atoi(w[k]));
            }
        }
    }
    if (!seen_t) return fail(FVGB_ERR_FORMAT, "continue file has no t, istep line");
    if (r.nx.empty() || r.tri.empty()) return fail(FVGB_ERR_FORMAT, "continue file has no nodes or no elements");
    for (int id : r.nid)
        if (id < 0) return fail(FVGB_ERR_FORMAT, "negative node ID in continue file");
    int rc = assemble(r, equation, m);
    if (rc) return rc;
    const int N = m.N;
    m.U.resize(4 * (size_t)N);
    for (int e = 0; e < N; e++)
        for (int v = 0; v < 4; v++) m.U[(size_t)v * N + e] = U[4 * (size_t)e + v];
    if (t) *t = tt;
    if (istep) *istep = is;
    if (cfl) *cfl = cf;
    if (has_cfl) *has_cfl = seen_cfl;
    return 0;
}

int write_continue(const HostMesh& m, const char* path, double t, int istep, double cfl, const double* U) {
    if ((int)m.node_id.size() != m.V || (int)m.set_edges.size() != m.NB)
        return fail(FVGB_ERR_ARG, "mesh lacks node IDs or boundary edge lists (read it with fvgb_mesh_read_su2 "
                                  "or fvgb_read_continue)");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(FVGB_ERR_IO, std::string("cannot write continue file ") + path);
    const int N = m.N, V = m.V;
    std::fprintf(f, "t, istep, CFL\n%.17g %d %.17g\n", t, istep, cfl);
    std::fprintf(f, "nodes: ID, x, y\n");
    for (int i = 0; i < V; i++)
        std::fprintf(f, "%d %.17g %.17g\n", m.node_id[i], m.node_xy[i], m.node_xy[(size_t)V + i]);
    std::fprintf(f, "elements: ID, nodes, U\n");
    for (int e = 0; e < N; e++) {
        std::fprintf(f, "%d %d %d %d", e + 1, m.node_id[m.elem_nodes[e]], m.node_id[m.elem_nodes[(size_t)N + e]],
                     m.node_id[m.elem_nodes[2 * (size_t)N + e]]);
        for (int v = 0; v < 4; v++) std::fprintf(f, " %.17g", U[(size_t)v * N + e]);
        std::fputc('\n', f);
    }
    std::fprintf(f, "boundaries: ID, name; edgeIDs\n");
    for (int s = 0; s < m.NB; s++) {
        std::fprintf(f, "%d %s\n", s + 1, m.bc_name[s].c_str());
        const std::vector<int>& es = m.set_edges[s];
        bool at_line_start = false;
        for (size_t k = 0; k < es.size(); k++) {
            std::fprintf(f, "%d", es[k] + 1);
            at_line_start = (k % 10 == 9);
            std::fputc(at_line_start ? '\n' : ' ', f);
        }
        if (!at_line_start) std::fputc('\n', f);
    }
    const bool ok = std::ferror(f) == 0;
    if (std::fclose(f) != 0 || !ok) return fail(FVGB_ERR_IO, std::string("write failed: ") + path);
    return 0;
}

}  // namespace fvgb

using namespace fvgb;

extern "C" int fvgb_read_continue(const char* path, int equation, fvgb_mesh** out, double* t, int* istep,
                                  double* cfl) {
    if (!path || !out) return fail(FVGB_ERR_ARG, "path or out is NULL");
    *out = nullptr;
    fvgb_mesh* m = new fvgb_mesh();
    bool has_cfl = false;
    double c = 0.0;
    int rc = read_continue(path, equation, m->m, t, istep, &c, &has_cfl);
    if (rc) {
        delete m;
        return rc;
    }
    if (cfl) *cfl = has_cfl ? c : -1.0;
    *out = m;
    return 0;
}

extern "C" int fvgb_continue_state(const fvgb_mesh* m, double* U) {
    if (!m || !U) return fail(FVGB_ERR_ARG, "mesh or U is NULL");
    if (m->m.U.empty()) return fail(FVGB_ERR_ARG, "mesh was not read from a continue file");
    std::memcpy(U, m->m.U.data(), sizeof(double) * m->m.U.size());
    return 0;
}

extern "C" int fvgb_write_continue(const fvgb_mesh* m, const char* path, double t, int istep, double cfl,
                                   const double* U) {
    if (!m || !path || !U) return fail(FVGB_ERR_ARG, "mesh, path or U is NULL");
    return write_continue(m->m, path, t, istep, cfl, U);
}

// ContinueFileReader.cpp:24-53: among the files named pause_<name>[<n>].dat in the
// folder, the one with the largest n (n > 0: a step-0 file is never chosen, as there)
extern "C" int fvgb_find_continue_file(const char* directory, const char* name, char* path_out, int path_len) {
    if (!directory || !name || !path_out || path_len <= 0) return fail(FVGB_ERR_ARG, "bad arguments");
    DIR* d = opendir(directory);
    if (!d) return fail(FVGB_ERR_IO, std::string("cannot list folder ") + directory);
    const std::string prefix = std::string("pause_") + name + "[";
    std::string best;
    long best_n = 0;
    while (dirent* e = readdir(d)) {
        const std::string f = e->d_name;
        if (f.size() <= prefix.size() + 5 || f.compare(0, prefix.size(), prefix) != 0) continue;
        if (f.compare(f.size() - 5, 5, "].dat") != 0) continue;
        const std::string num = f.substr(prefix.size(), f.size() - prefix.size() - 5);
        char* endp = nullptr;
        const long n = std::strtol(num.c_str(), &endp, 10);
        if (num.empty() || *endp != 0) continue;
        if (n > best_n) {
            best_n = n;
            best = f;
        }
    }
    closedir(d);
    if (best.empty()) return fail(FVGB_ERR_IO, std::string("no pause_") + name + "[n].dat in " + directory);
    std::string full = std::string(directory);
    if (!full.empty() && full.back() != '/') full += '/';
    full += best;
    if ((int)full.size() >= path_len) return fail(FVGB_ERR_ARG, "path buffer too small");
    std::memcpy(path_out, full.c_str(), full.size() + 1);
    return 0;
}

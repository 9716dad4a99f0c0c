// Field output: node values, boundary forces, Tecplot files and the headless
// field colouring.
//
//   node values     FieldWriter::update_nodeField (FVMR/src/output/FieldWriter.cpp:364-453):
//                   per node the mean of its cells' rho, u, v, p (U2ruvp_host,
//                   FVMR/src/math/PhysicalKernel.h:11-16), summed in cell order;
//                   Cp = (p - p_inf) / (1/2 rho_inf V_inf^2); Ma = sqrt(V^2 / (gamma p / rho))
//   forces          ReferenceData::calculate_edgeSet_force (FieldWriter.cpp:175-210) per
//                   boundary set, HistData::set_CDCL_wall (FieldWriter.cpp:611-632) over walls
//   Tecplot files   write_tecplot_volume_file / write_tecplot_boundary_file
//                   (FieldWriter.cpp:44-172), with the output schemes of FieldWriter.cpp:464-553
//   colouring       the GUI's cell -> node -> colour kernels (FVMR/src/gui/cuda/
//                   CudaGrid_kernels.cu:18-164, 225-245), into a device buffer instead of
//                   an OpenGL vertex buffer
//
// Both kernels gather over a node -> cell list in increasing reference cell order,
// so they reproduce the reference's sums (host loop over cells) exactly and are
// deterministic where the reference's colouring kernel races.  Their arithmetic
// uses explicit round-to-nearest operations (no contraction), the order written
// in the reference.  The node values are taken from the current state; the
// reference's writers read the primitive variables of the previous step's start.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"
#include "solver.h"

namespace fvgb {

struct OutputState {
    int* d_node_ptr = nullptr;    // V+1
    int* d_node_cells = nullptr;  // 3N device cell indices, increasing reference cell order per node
    double* d_field = nullptr;    // [6][V]: rho u v p Cp Ma
    float* d_rgb = nullptr;       // [V][3]
    float* d_node_value = nullptr;
    d4* d_cell_ruvp = nullptr;    // [N]: each cell's rho u v p, computed once per call
    std::vector<double> h_field;  // host copy of d_field
};

namespace dev {

// U2ruvp_host once per cell: rho, U1/U0, U2/U0, rho (gamma-1) (U3/U0 - (u u + v v) 0.5)
__global__ void __launch_bounds__(256) k_cell_ruvp(const d4* __restrict__ U, int N, double gm1,
                                                   d4* __restrict__ ruvp) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const d4 u = ld4(&U[c]);
    const double uu = __ddiv_rn(u.y, u.x), vv = __ddiv_rn(u.z, u.x);
    const double q = __dmul_rn(__dadd_rn(__dmul_rn(uu, uu), __dmul_rn(vv, vv)), 0.5);
    ruvp[c] = mk4(u.x, uu, vv, __dmul_rn(__dmul_rn(u.x, gm1), __dsub_rn(__ddiv_rn(u.w, u.x), q)));
}

__global__ void __launch_bounds__(256) k_node_field(const d4* __restrict__ ruvp, const int* __restrict__ ptr,
                                                    const int* __restrict__ cells, int V, double gamma,
                                                    double p_inf, double pdyn_inf, double* __restrict__ f) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= V) return;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    const int b = ptr[n], e = ptr[n + 1];
    for (int k = b; k < e; k++) {
        const d4 w = ld4(&ruvp[cells[k]]);
        s0 = __dadd_rn(s0, w.x);
        s1 = __dadd_rn(s1, w.y);
        s2 = __dadd_rn(s2, w.z);
        s3 = __dadd_rn(s3, w.w);
    }
    if (e > b) {
        const double c = (double)(e - b);
        s0 = __ddiv_rn(s0, c);
        s1 = __ddiv_rn(s1, c);
        s2 = __ddiv_rn(s2, c);
        s3 = __ddiv_rn(s3, c);
    }
    const double v2 = __dadd_rn(__dmul_rn(s1, s1), __dmul_rn(s2, s2));
    const double a2 = __ddiv_rn(__dmul_rn(gamma, s3), s0);
    f[n] = s0;
    f[(size_t)V + n] = s1;
    f[2 * (size_t)V + n] = s2;
    f[3 * (size_t)V + n] = s3;
    f[4 * (size_t)V + n] = __ddiv_rn(__dsub_rn(s3, p_inf), pdyn_inf);
    f[5 * (size_t)V + n] = __dsqrt_rn(__ddiv_rn(v2, a2));
}

// the default colour map of CudaGrid.cpp:31-37: red, yellow, green, blue, magenta at 0, 1/4, 1/2, 3/4, 1
__constant__ float4 c_colormap[5] = {{1.0f, 0.0f, 0.0f, 0.00f},
                                     {1.0f, 1.0f, 0.0f, 0.25f},
                                     {0.0f, 1.0f, 0.0f, 0.50f},
                                     {0.0f, 0.0f, 1.0f, 0.75f},
                                     {1.0f, 0.0f, 1.0f, 1.00f}};

// getColor_device (CudaGrid_kernels.cu:24-66): clamp to [0, 1], find the interval, blend
// c0, (c0 + c1)/2 twice and c1 with the cubic weights (1-n)^3, 3(1-n)^2 n, 3(1-n) n^2, n^3
__device__ __forceinline__ void colour_of(float x, float* rgb) {
    if (x < 0.0f) x = 0.0f;
    if (x > 1.0f) x = 1.0f;
    for (int i = 0; i < 4; i++) {
        const float4 a = c_colormap[i], z = c_colormap[i + 1];
        if (x >= a.w && x <= z.w) {
            const float c0[3] = {a.x, a.y, a.z}, c1[3] = {z.x, z.y, z.z};
            const float n = __fdiv_rn(__fsub_rn(x, a.w), __fsub_rn(z.w, a.w));
            const float omn = __fsub_rn(1.0f, n);
            const float omn2 = __fmul_rn(omn, omn), omn3 = __fmul_rn(omn2, omn);
            const float n2 = __fmul_rn(n, n), n3 = __fmul_rn(n2, n);
            const float w1 = __fmul_rn(__fmul_rn(3.0f, omn2), n);
            const float w2 = __fmul_rn(__fmul_rn(3.0f, omn), n2);
            for (int k = 0; k < 3; k++) {
                const float cm = __fmul_rn(0.5f, __fadd_rn(c0[k], c1[k]));
                float s = __fmul_rn(omn3, c0[k]);
                s = __fadd_rn(s, __fmul_rn(w1, cm));
                s = __fadd_rn(s, __fmul_rn(w2, cm));
                rgb[k] = __fadd_rn(s, __fmul_rn(n3, c1[k]));
            }
            return;
        }
    }
    rgb[0] = 252.0f / 255.0f;  // outside every interval (NaN): the reference's magenta
    rgb[1] = 3.0f / 255.0f;
    rgb[2] = 253.0f / 255.0f;
}

// accumulateElementDataToNodeData_k + divideNodeData_k + nodeDataToVertexColor_k
// (CudaGrid_kernels.cu:79-130): the node value is the largest rho x count over the
// node's cells (0 when all are negative), times 1/count; then normalised by the range
__global__ void __launch_bounds__(256) k_colour(const d4* __restrict__ U, const int* __restrict__ ptr,
                                                const int* __restrict__ cells, int V, float lo, float hi,
                                                float* __restrict__ rgb, float* __restrict__ node_value) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= V) return;
    const int b = ptr[n], e = ptr[n + 1];
    const float cnt = (float)(e - b);
    float v = 0.0f;
    for (int k = b; k < e; k++) {
        const float x = __fmul_rn(__double2float_rn(U[cells[k]].x), cnt);
        v = (v > x) ? v : x;
    }
    float div = __double2float_rn(__ddiv_rn(1.0, (double)(e - b)));
    if (div > 1e5f) div = 1.0f;
    v = __fmul_rn(v, div);
    node_value[n] = v;
    const float len = fabsf(__fsub_rn(hi, lo));
    const float x = (len == 0.0f) ? 0.0f : __fdiv_rn(__fsub_rn(v, lo), len);
    float c[3];
    colour_of(x, c);
    rgb[3 * (size_t)n] = c[0];
    rgb[3 * (size_t)n + 1] = c[1];
    rgb[3 * (size_t)n + 2] = c[2];
}

}  // namespace dev

#define OK_(call)                                                                                              \
    do {                                                                                                       \
        cudaError_t e_ = (call);                                                                               \
        if (e_ != cudaSuccess) return fail(FVGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int Solver::keep_output_mesh(const fvgb_mesh_soa& m) {
    om = OutputMesh();
    const int V = m.num_node, NB = m.num_boundary, Nn = m.num_element, Ee = m.num_edge;
    om.V = V;
    om.NB = NB;
    om.node_xy.assign(m.node_xy, m.node_xy + 2 * (size_t)V);
    om.elem_nodes.resize(3 * (size_t)Nn);
    for (int j = 0; j < 3; j++)
        for (int c = 0; c < Nn; c++) {
            const int q = m.elem_nodes[(size_t)j * Nn + c];
            if (q < 0 || q >= V) return fail(FVGB_ERR_MESH, "element names a node out of range");
            om.elem_nodes[(size_t)j * Nn + c] = q;
        }
    om.set_off.assign(1, 0);
    for (int s = 0; s < NB; s++) {
        std::vector<int> es;
        if (m.set_edge_offsets && m.set_edge_list) {
            es.assign(m.set_edge_list + m.set_edge_offsets[s], m.set_edge_list + m.set_edge_offsets[s + 1]);
        } else {
            for (int e = 0; e < Ee; e++)
                if (m.edge_setID[e] == s + 1) es.push_back(e);
        }
        for (int e : es) {
            if (e < 0 || e >= Ee) return fail(FVGB_ERR_MESH, "boundary set names an edge out of range");
            om.set_n0.push_back(m.edge_nodes[e]);
            om.set_n1.push_back(m.edge_nodes[(size_t)Ee + e]);
            om.set_nx.push_back(m.edge_normal[e]);
            om.set_ny.push_back(m.edge_normal[(size_t)Ee + e]);
            om.set_len.push_back(m.edge_length[e]);
        }
        om.set_off.push_back((int)om.set_n0.size());
        om.set_type.push_back(m.boundary_type[s]);
        om.set_name.push_back(m.set_names && m.set_names[s] ? m.set_names[s] : ("set" + std::to_string(s + 1)));
    }
    return 0;
}

void Solver::release_output() {
    if (!out) return;
    cudaFree(out->d_node_ptr);
    cudaFree(out->d_node_cells);
    cudaFree(out->d_field);
    cudaFree(out->d_rgb);
    cudaFree(out->d_node_value);
    cudaFree(out->d_cell_ruvp);
    delete out;
    out = nullptr;
}

// the node -> cell lists and output buffers, on first use
static int output_ready(Solver& s) {
    if (s.out) return 0;
    const int V = s.om.V, N = s.N;
    std::vector<int> ptr((size_t)V + 1, 0), cells(3 * (size_t)N);
    for (int c = 0; c < N; c++)
        for (int j = 0; j < 3; j++) ptr[s.om.elem_nodes[(size_t)j * N + c] + 1]++;
    for (int i = 0; i < V; i++) ptr[i + 1] += ptr[i];
    std::vector<int> pos(ptr.begin(), ptr.end() - 1);
    for (int c = 0; c < N; c++)
        for (int j = 0; j < 3; j++) cells[pos[s.om.elem_nodes[(size_t)j * N + c]]++] = s.L.cell_new[c];
    OutputState* o = new OutputState();
    s.out = o;
    OK_(cudaMalloc(&o->d_node_ptr, sizeof(int) * ptr.size()));
    OK_(cudaMalloc(&o->d_node_cells, sizeof(int) * cells.size()));
    OK_(cudaMalloc(&o->d_field, sizeof(double) * 6 * (size_t)V));
    OK_(cudaMalloc(&o->d_rgb, sizeof(float) * 3 * (size_t)V));
    OK_(cudaMalloc(&o->d_node_value, sizeof(float) * (size_t)V));
    OK_(cudaMalloc(&o->d_cell_ruvp, sizeof(d4) * (size_t)(N > 0 ? N : 1)));
    OK_(cudaMemcpyAsync(o->d_node_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice, s.stream));
    OK_(cudaMemcpyAsync(o->d_node_cells, cells.data(), sizeof(int) * cells.size(), cudaMemcpyHostToDevice, s.stream));
    OK_(cudaStreamSynchronize(s.stream));
    return 0;
}

// FieldWriter::ReferenceData::update_farfield (FieldWriter.cpp:540-549)
static void farfield_reference(const fvgb_params& p, double* p_inf, double* pdyn) {
    const double V2 = p.inf[1] * p.inf[1] + p.inf[2] * p.inf[2];
    *p_inf = p.inf[3];
    *pdyn = 0.5 * p.inf[0] * V2;
}

static void launch_node_field(Solver& s, double p_inf, double pdyn) {
    const int V = s.om.V, N = s.N;
    if (N > 0) dev::k_cell_ruvp<<<(N + 255) / 256, 256, 0, s.stream>>>(s.d_U, N, s.p.gamma - 1, s.out->d_cell_ruvp);
    if (V > 0)
        dev::k_node_field<<<(V + 255) / 256, 256, 0, s.stream>>>(s.out->d_cell_ruvp, s.out->d_node_ptr,
                                                                 s.out->d_node_cells, V, s.p.gamma, p_inf, pdyn,
                                                                 s.out->d_field);
    s.launches += 2;
}

static int node_field(Solver& s) {
    int rc = output_ready(s);
    if (rc) return rc;
    const int V = s.om.V;
    double p_inf, pdyn;
    farfield_reference(s.p, &p_inf, &pdyn);
    launch_node_field(s, p_inf, pdyn);
    OK_(cudaGetLastError());
    s.out->h_field.resize(6 * (size_t)V);
    OK_(cudaMemcpyAsync(s.out->h_field.data(), s.out->d_field, sizeof(double) * 6 * (size_t)V, cudaMemcpyDeviceToHost,
                        s.stream));
    OK_(cudaStreamSynchronize(s.stream));
    return 0;
}

// calculate_edgeSet_force over the node Cp of the last node_field()
static void forces(const Solver& s, double* cd, double* cl, double* cd_wall, double* cl_wall) {
    const int V = s.om.V;
    const double* Cp = s.out->h_field.data() + 4 * (size_t)V;
    const double one_on_Sref = 1 / s.p.ref_area;
    double dw = 0.0, lw = 0.0;
    for (int b = 0; b < s.om.NB; b++) {
        double CD = 0.0, CL = 0.0;
        for (int k = s.om.set_off[b]; k < s.om.set_off[b + 1]; k++) {
            const double c = 0.5 * (Cp[s.om.set_n0[k]] + Cp[s.om.set_n1[k]]);
            const double dC = c * one_on_Sref * s.om.set_len[k];
            CD += dC * s.om.set_nx[k];
            CL += dC * s.om.set_ny[k];
        }
        if (cd) cd[b] = CD;
        if (cl) cl[b] = CL;
        const int t = s.om.set_type[b];
        if (t == BC_WALL_NONVISCOUS || t == BC_WALL_ADIABAT || t == BC_WALL_ISOTHERMAL) {  // set_CDCL_wall: the wall types
            dw += CD;
            lw += CL;
        }
    }
    if (cd_wall) *cd_wall = dw;
    if (cl_wall) *cl_wall = lw;
}

// ---- Tecplot text ---------------------------------------------------------
namespace {

struct Text {
    FILE* f = nullptr;
    std::string buf;
    void flush() {
        if (!buf.empty()) std::fwrite(buf.data(), 1, buf.size(), f);
        buf.clear();
    }
    void put(const char* s) {
        buf += s;
        if (f && buf.size() > (1u << 22)) flush();
    }
    void e(double x) {  // std::scientific, default precision: %e
        char t[40];
        std::snprintf(t, sizeof t, "%e", x);
        put(t);
    }
};

// FieldOutputScheme::updateBoolDataByPreset / get_variable_names (FieldWriter.cpp:464-517)
const char* variable_names(int preset) {
    switch (preset) {
    case 0: return "\"x\", \"y\", \"rho\", \"u\", \"v\", \"p\"";
    case 1: return "\"x\", \"y\", \"rho\", \"u\", \"v\", \"p\", \"Cp\"";
    default: return "\"x\", \"y\", \"rho\", \"u\", \"v\", \"p\", \"Ma\"";
    }
}

// FieldOutputScheme::get_variable_value_string (FieldWriter.cpp:520-541)
void node_line(Text& o, const Solver& s, int n, int preset) {
    const int V = s.om.V;
    const double* f = s.out->h_field.data();
    double vals[7] = {s.om.node_xy[n], s.om.node_xy[(size_t)V + n], f[n], f[(size_t)V + n], f[2 * (size_t)V + n],
                      f[3 * (size_t)V + n], 0.0};
    int k = 6;
    if (preset == 1) vals[k++] = f[4 * (size_t)V + n];
    else if (preset == 2) vals[k++] = f[5 * (size_t)V + n];
    for (int i = 0; i < k; i++) {
        o.e(vals[i]);
        o.put(i + 1 < k ? " " : "\n");
    }
}

}  // namespace

static int write_volume(Solver& s, const char* path, const char* title, double t, int preset) {
    Text o;
    o.f = std::fopen(path, "wb");
    if (!o.f) return fail(FVGB_ERR_IO, std::string("cannot write ") + path);
    char line[512];
    std::snprintf(line, sizeof line,
                  "title= \"%s\"\nvariables= %s\nzone t= \"volume field\", nodes= %d, elements= %d, datapacking= point, "
                  "zonetype= fequadrilateral, solutiontime= %e\n",
                  title, variable_names(preset), s.om.V, s.N, t);
    o.put(line);
    o.flush();
    // the node lines, then the cells' node lists: formatted in chunks on host threads, written in order
    const int V = s.om.V, N = s.N;
    const long long total = (long long)V + N;
    const int nthreads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const long long chunk = 1 << 16;
    for (long long base = 0; base < total; base += chunk * nthreads) {
        std::vector<std::string> parts(nthreads);
        std::vector<std::thread> pool;
        for (int w = 0; w < nthreads; w++) {
            const long long lo = base + (long long)w * chunk, hi = std::min(total, lo + chunk);
            if (lo >= hi) break;
            pool.emplace_back([&, w, lo, hi] {
                Text part;
                char l[64];
                for (long long i = lo; i < hi; i++) {
                    if (i < V) {
                        node_line(part, s, (int)i, preset);
                    } else {
                        const int c = (int)(i - V);
                        const int a = s.om.elem_nodes[c] + 1, b = s.om.elem_nodes[(size_t)N + c] + 1,
                                  d = s.om.elem_nodes[2 * (size_t)N + c] + 1;
                        std::snprintf(l, sizeof l, "%d %d %d %d\n", a, b, d, d);
                        part.buf += l;
                    }
                }
                parts[w] = std::move(part.buf);
            });
        }
        for (auto& th : pool) th.join();
        for (auto& part : parts)
            if (!part.empty()) std::fwrite(part.data(), 1, part.size(), o.f);
    }
    const bool ok = std::ferror(o.f) == 0;
    if (std::fclose(o.f) != 0 || !ok) return fail(FVGB_ERR_IO, std::string("write failed: ") + path);
    return 0;
}

static int write_boundary(Solver& s, const char* path, double t, int preset) {
    Text o;
    o.f = std::fopen(path, "wb");
    if (!o.f) return fail(FVGB_ERR_IO, std::string("cannot write ") + path);
    char line[512];
    std::snprintf(line, sizeof line, "title= \"tecplot boundary file\"\nvariables= %s\n", variable_names(preset));
    o.put(line);
    for (int b = 0; b < s.om.NB; b++) {
        std::snprintf(line, sizeof line, "zone t= \"boundary %d %s\", solutiontime= %e, strandid= 0, i= %d, j= 1, f= point\n",
                      b + 1, s.om.set_name[b].c_str(), t, s.om.set_off[b + 1] - s.om.set_off[b]);
        o.put(line);
        int n1_old = -1;
        for (int k = s.om.set_off[b]; k < s.om.set_off[b + 1]; k++) {
            const int n0 = s.om.set_n0[k], n1 = s.om.set_n1[k];
            if (n0 != n1_old) node_line(o, s, n0, preset);
            node_line(o, s, n1, preset);
            n1_old = n1;
        }
    }
    o.flush();
    const bool ok = std::ferror(o.f) == 0;
    if (std::fclose(o.f) != 0 || !ok) return fail(FVGB_ERR_IO, std::string("write failed: ") + path);
    return 0;
}

}  // namespace fvgb

using namespace fvgb;

extern "C" int fvgb_node_field(fvgb_handle* h, double* out6) {
    if (!h) return fail(FVGB_ERR_ARG, "null handle");
    cudaSetDevice(h->s.p.device);
    int rc = node_field(h->s);
    if (rc) return rc;
    if (out6) std::copy(h->s.out->h_field.begin(), h->s.out->h_field.end(), out6);
    return 0;
}

extern "C" int fvgb_boundary_forces(fvgb_handle* h, double* cd, double* cl, double* cd_wall, double* cl_wall) {
    if (!h) return fail(FVGB_ERR_ARG, "null handle");
    cudaSetDevice(h->s.p.device);
    int rc = node_field(h->s);
    if (rc) return rc;
    forces(h->s, cd, cl, cd_wall, cl_wall);
    return 0;
}

extern "C" int fvgb_write_tecplot_volume(fvgb_handle* h, const char* path, const char* title, double t, int preset) {
    if (!h || !path) return fail(FVGB_ERR_ARG, "null argument");
    if (preset < 0 || preset > 2) return fail(FVGB_ERR_ARG, "preset is 0, 1 or 2");
    cudaSetDevice(h->s.p.device);
    int rc = node_field(h->s);
    if (rc) return rc;
    return write_volume(h->s, path, title ? title : "title", t, preset);
}

extern "C" int fvgb_write_tecplot_boundary(fvgb_handle* h, const char* path, double t, int preset) {
    if (!h || !path) return fail(FVGB_ERR_ARG, "null argument");
    if (preset < 0 || preset > 2) return fail(FVGB_ERR_ARG, "preset is 0, 1 or 2");
    cudaSetDevice(h->s.p.device);
    int rc = node_field(h->s);
    if (rc) return rc;
    return write_boundary(h->s, path, t, preset);
}

extern "C" int fvgb_colour_nodes(fvgb_handle* h, double range_lo, double range_hi, float** rgb_dev, float* rgb_host,
                                 float* node_value_host) {
    if (!h) return fail(FVGB_ERR_ARG, "null handle");
    Solver& s = h->s;
    cudaSetDevice(s.p.device);
    int rc = output_ready(s);
    if (rc) return rc;
    const int V = s.om.V;
    if (V > 0)
        dev::k_colour<<<(V + 255) / 256, 256, 0, s.stream>>>(s.d_U, s.out->d_node_ptr, s.out->d_node_cells, V,
                                                             (float)range_lo, (float)range_hi, s.out->d_rgb,
                                                             s.out->d_node_value);
    OK_(cudaGetLastError());
    s.launches += 1;
    if (rgb_dev) *rgb_dev = s.out->d_rgb;
    if (rgb_host)
        OK_(cudaMemcpyAsync(rgb_host, s.out->d_rgb, sizeof(float) * 3 * (size_t)V, cudaMemcpyDeviceToHost, s.stream));
    if (node_value_host)
        OK_(cudaMemcpyAsync(node_value_host, s.out->d_node_value, sizeof(float) * (size_t)V, cudaMemcpyDeviceToHost,
                            s.stream));
    OK_(cudaStreamSynchronize(s.stream));
    return 0;
}

extern "C" int fvgb_num_nodes(fvgb_handle* h, int* V) {
    if (!h || !V) return fail(FVGB_ERR_ARG, "null argument");
    *V = h->s.om.V;
    return 0;
}

// reps launches of each output kernel on the handle's stream, bracketed by CUDA events
extern "C" int fvgb_output_timed(fvgb_handle* h, int reps, double* ms_node_field, double* ms_colour) {
    if (!h || reps <= 0) return fail(FVGB_ERR_ARG, "bad arguments");
    Solver& s = h->s;
    cudaSetDevice(s.p.device);
    int rc = output_ready(s);
    if (rc) return rc;
    const int V = s.om.V;
    if (V == 0) return fail(FVGB_ERR_ARG, "mesh has no nodes");
    double p_inf, pdyn;
    farfield_reference(s.p, &p_inf, &pdyn);
    cudaEvent_t a, b, c;
    OK_(cudaEventCreate(&a));
    OK_(cudaEventCreate(&b));
    OK_(cudaEventCreate(&c));
    const int grid = (V + 255) / 256;
    OK_(cudaEventRecord(a, s.stream));
    for (int i = 0; i < reps; i++) launch_node_field(s, p_inf, pdyn);
    OK_(cudaEventRecord(b, s.stream));
    for (int i = 0; i < reps; i++)
        dev::k_colour<<<grid, 256, 0, s.stream>>>(s.d_U, s.out->d_node_ptr, s.out->d_node_cells, V, 0.5f, 1.5f,
                                                  s.out->d_rgb, s.out->d_node_value);
    OK_(cudaEventRecord(c, s.stream));
    OK_(cudaEventSynchronize(c));
    OK_(cudaGetLastError());
    float t1 = 0, t2 = 0;
    OK_(cudaEventElapsedTime(&t1, a, b));
    OK_(cudaEventElapsedTime(&t2, b, c));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaEventDestroy(c);
    s.launches += (long long)reps;
    if (ms_node_field) *ms_node_field = t1;
    if (ms_colour) *ms_colour = t2;
    return 0;
}

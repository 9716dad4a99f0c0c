// fvgb_rhs_noalloc: the first-order residual computed straight from
// caller-owned device arrays in the reference's layout, allocating nothing.
//
// Who needs this: a caller that already owns every device buffer and may not
// (or must not) allocate more, for instance an application that gives this
// step a fixed slice of a memory arena it manages itself, or a code path that
// cannot afford the device-wide synchronisation a cudaMalloc/cudaFree may
// cause.  Such a caller keeps the reference's SoA arrays on the device (as
// GPU::GPUSolver2 does) and passes their addresses; the only extra memory the
// computation needs -- one flux per edge -- lives in the file-scope device
// array below, which is part of the library image and exists on every GPU
// that loads the library until the process exits.
//
// Limits: at most kNoallocMaxEdges edges (32 MiB of edge fluxes); constant
// reconstruction and the Euler equations only (no gradients, no viscous
// terms).  Calls share the array: two calls that overlap on the GPU (different
// streams, or different threads) race on it and must be serialised by the
// caller.  Every edge's flux is written before it is read, so no clearing is
// needed between calls.
#include <cuda_runtime.h>

#include "internal.h"
#include "solver.h"

namespace fvgb {
namespace {

constexpr int kNoallocMaxEdges = 1 << 20;   // 1,048,576 edges -> 4 doubles each = 32 MiB

static __device__ __align__(256) double g_noalloc_edge_flux[4 * (size_t)kNoallocMaxEdges];

// The array's device address in the context current on the calling thread.  In host code
// the array's name is only a stand-in, never a device address, so every call asks the
// runtime for it (cudaGetSymbolAddress allocates nothing).  Nothing is cached: a cached
// address would go stale after cudaDeviceReset or when the caller switches to another
// context on the same device.  The first call in a context also loads the library's
// device code there, which is why that first call belongs before any stream capture.
int scratch_address(double** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_edge_flux);
    if (e != cudaSuccess) return fail(FVGB_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    *out = static_cast<double*>(p);
    return 0;
}

struct RefMesh {  // device pointers, reference layout and numbering
    int N, E, NB;
    const int* elem_edges;   // [4][N]
    const double* elem_volume;
    const int* edge_L;
    const int* edge_R;
    const int* edge_setID;
    const double* edge_length;
    const double* edge_normal;  // [2][E]
    const double* edge_xy;      // [2][E] (read on "dsr" edges only)
    const int* boundary_type;   // [NB]
};

__device__ __forceinline__ d4 load_ref(const double* U, int N, int c) {
    return mk4(U[c], U[(size_t)N + c], U[2 * (size_t)N + c], U[3 * (size_t)N + c]);
}

// edge_convection_flux_kernel (FVMR/src/space/Flux.cpp:230-303) with constant
// reconstruction, on the reference's arrays; fluxes go to the file-scope array
template <int FLUX>
__global__ void __launch_bounds__(256) k_noalloc_flux(RefMesh m, const double* __restrict__ U, dev::Gas g,
                                                      dev::BcData bc, double t_dsr, double* __restrict__ F) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m.E) return;
    const int L = m.edge_L[e], set = m.edge_setID[e];
    int R = m.edge_R[e];
    // indices outside the caller's arrays are not followed: such an edge's flux is NaN
    if (L < 0 || L >= m.N || R < -1 || R >= m.N || (set != -1 && (set < 1 || set > m.NB))) {
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
        for (int v = 0; v < 4; v++) F[(size_t)v * m.E + e] = nan;
        return;
    }
    const int bt = set != -1 ? m.boundary_type[set - 1] : -1;
    const double nx = m.edge_normal[e], ny = m.edge_normal[(size_t)m.E + e], len = m.edge_length[e];
    const d4 uL = load_ref(U, m.N, L);
    const dev::Prim wL = dev::to_prim(uL, g);
    d4 uR = mk4(0, 0, 0, 0);
    if (bt == BC_WALL_NONVISCOUS || bt == BC_SYMMETRY) {
        uR = dev::ghost_slip(uL, wL, nx, ny);
    } else if (bt == BC_WALL_ADIABAT) {
        uR = bc.wall_ref ? mk4(uL.x, -0.0, -0.0, uL.w) : mk4(uL.x, -uL.y, -uL.z, uL.w);
    } else if (bt == BC_INLET) {
        dev::ghost_farfield(wL, bc.inlet, bc.a_inlet, bc.son_inlet, nx, ny, g, uR);
    } else if (bt == BC_OUTLET) {
        dev::ghost_farfield(wL, bc.outlet, bc.a_outlet, bc.son_outlet, nx, ny, g, uR);
    } else if (bt == BC_INF) {
        dev::ghost_farfield(wL, bc.inf, bc.a_inf, bc.son_inf, nx, ny, g, uR);
    } else if (bt == BC_DSR) {
        if (dev::dsr_upstream_at(m.edge_xy[e], m.edge_xy[(size_t)m.E + e], t_dsr, bc))
            dev::ghost_farfield(wL, bc.inlet, bc.a_inlet, bc.son_inlet, nx, ny, g, uR);
        else
            dev::ghost_farfield(wL, bc.outlet, bc.a_outlet, bc.son_outlet, nx, ny, g, uR);
    } else if (R != -1) {  // interior and periodic edges: R holds the partner's cell
        uR = load_ref(U, m.N, R);
    }
    const dev::Prim wR = dev::to_prim(uR, g);
    const d4 f = (FLUX == 2002) ? dev::roe_flux(wL, wR, uL, uR, nx, ny, len, g) : dev::llf_flux(uL, uR, wL, wR, nx, ny, len, g);
    F[e] = f.x;
    F[(size_t)m.E + e] = f.y;
    F[2 * (size_t)m.E + e] = f.z;
    F[3 * (size_t)m.E + e] = f.w;
}

// add_edge_flux_to_element_flux (Flux.cpp:346-392) and the -1/vol of
// calculateFunctionF (FVMR/src/time/Evolve.cpp:106-111)
__global__ void __launch_bounds__(256) k_noalloc_gather(RefMesh m, const double* __restrict__ F,
                                                        double* __restrict__ rhs) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    double acc[4] = {0, 0, 0, 0};
    for (int j = 0; j < 4; j++) {
        const int e = m.elem_edges[(size_t)j * m.N + c];
        if (e < 0 || e >= m.E) continue;
        const double s = (c != m.edge_R[e]) ? 1.0 : -1.0;
        for (int v = 0; v < 4; v++) acc[v] = fma(s, F[(size_t)v * m.E + e], acc[v]);
    }
    const double mv = -1.0 / m.elem_volume[c];
    for (int v = 0; v < 4; v++) rhs[(size_t)v * m.N + c] = mv * acc[v];
}

}  // namespace
}  // namespace fvgb

using namespace fvgb;

// No counterpart in the reference: see include/fvgb.h.
extern "C" int fvgb_rhs_noalloc(const fvgb_mesh_soa* dev_mesh, const fvgb_params* p, const double* U_dev,
                                double* rhs_dev, void* stream) {
    if (!dev_mesh || !p || !U_dev || !rhs_dev) return fail(FVGB_ERR_ARG, "null argument");
    if (dev_mesh->num_edge < 0 || dev_mesh->num_element < 0) return fail(FVGB_ERR_ARG, "negative sizes");
    if (dev_mesh->num_edge > kNoallocMaxEdges)
        return fail(FVGB_ERR_ARG, "fvgb_rhs_noalloc: mesh has " + std::to_string(dev_mesh->num_edge) +
                                      " edges; this entry point holds at most " + std::to_string(kNoallocMaxEdges));
    if (p->reconstruct != 3001 || p->equation != 1)
        return fail(FVGB_ERR_UNSUPPORTED, "fvgb_rhs_noalloc: constant reconstruction (3001) and Euler (1) only");
    if (p->flux_scheme != 2001 && p->flux_scheme != 2002) return fail(FVGB_ERR_ARG, "invalid flux scheme");
    {  // every array the kernels may read must be there (a null device address would fault)
        const fvgb_mesh_soa& d = *dev_mesh;
        const bool e = d.num_edge > 0, n = d.num_element > 0;
        if ((n && (!d.elem_edges || !d.elem_volume)) ||
            (e && (!d.edge_L || !d.edge_R || !d.edge_setID || !d.edge_length || !d.edge_normal || !d.edge_xy)) ||
            (e && !d.boundary_type))
            return fail(FVGB_ERR_ARG, "fvgb_rhs_noalloc: a mesh array it reads is NULL");
    }
    double* F = nullptr;
    int rc = scratch_address(&F);
    if (rc) return rc;
    RefMesh m;
    m.N = dev_mesh->num_element;
    m.NB = dev_mesh->num_boundary;
    m.E = dev_mesh->num_edge;
    m.elem_edges = dev_mesh->elem_edges;
    m.elem_volume = dev_mesh->elem_volume;
    m.edge_L = dev_mesh->edge_L;
    m.edge_R = dev_mesh->edge_R;
    m.edge_setID = dev_mesh->edge_setID;
    m.edge_length = dev_mesh->edge_length;
    m.edge_normal = dev_mesh->edge_normal;
    m.edge_xy = dev_mesh->edge_xy;
    m.boundary_type = dev_mesh->boundary_type;
    const dev::Gas g = make_gas(*p);
    const dev::BcData bc = make_bc(*p);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (m.E > 0) {
        const int b = (m.E + 255) / 256;
        if (p->flux_scheme == 2002) k_noalloc_flux<2002><<<b, 256, 0, s>>>(m, U_dev, g, bc, p->dsr_time, F);
        else k_noalloc_flux<2001><<<b, 256, 0, s>>>(m, U_dev, g, bc, p->dsr_time, F);
    }
    if (m.N > 0) k_noalloc_gather<<<(m.N + 255) / 256, 256, 0, s>>>(m, F, rhs_dev);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(FVGB_ERR_CUDA, std::string("fvgb_rhs_noalloc launch: ") + cudaGetErrorString(e));
    return 0;
}

// Launchers of the step kernels (step_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "step_device.cuh"

namespace fvgb {
namespace dev {

// Time and time step of one solver, kept on the device so a step needs no host sync.
struct StepState {
    double t, T, dt, dt6, dt_raw;
    unsigned long long dtmin_bits;
    double t_old;  // t at the start of the step (the clock of the double-Mach-reflection boundary)
};

void launch_prim(cudaStream_t s, const d4* U, d4* U0, d4* prim, int N, const Gas& g, bool copy);
void launch_dt(cudaStream_t s, const d4* prim, const MeshView& m, const Gas& g, double value_1, double CFL,
               bool ns, double* alpha, double* alpha_vis, unsigned long long* dtmin, Status* st);
void launch_dt_final(cudaStream_t s, StepState* st, bool advance);
void launch_dt_local(cudaStream_t s, const d4* prim, const MeshView& m, const Gas& g, double value_1, double CFL,
                     bool ns, double* alpha, double* alpha_vis, double* dt_local, StepState* st, int cell0,
                     Status* status);
void launch_grad(cudaStream_t s, int gradient, bool barth, const d4* U, const MeshView& m, d4* Gx, d4* Gy,
                 const CellTape* tape = nullptr);
void launch_flux(cudaStream_t s, int scheme, bool linear, bool ns, const d4* U, const d4* Gx,
                 const d4* Gy, const MeshView& m, const Gas& g, const BcData& bc, d4* F, Status* st,
                 const EdgeTape* tape = nullptr);
void launch_update(cudaStream_t s, int kind, d4* U, const d4* U0, d4* K1, d4* rhs,
                   const d4* F, const MeshView& m, const StepState* st, const Gas& g, int* flag_list,
                   unsigned int* flag_count, int flag_cap, Status* status, d4* rec_R = nullptr,
                   const double* dt_local = nullptr, bool from_res = false);
// the fluxes of n edges of one colour (edges[0..n)), added into the cells' sums res (+F to L;
// -F to R where in_r[e]); with launch_update(from_res) in place of the edge-flux gather
void launch_flux_scatter(cudaStream_t s, int scheme, bool linear, bool ns, const d4* U, const d4* Gx, const d4* Gy,
                         const MeshView& m, const Gas& g, const BcData& bc, const int* edges, const int* in_r,
                         int n, d4* res, Status* st);
void launch_restrict(cudaStream_t s, d4* U, const MeshView& m, const int* cell_ref_of_dev,
                     const int* dev_of_cell_ref, int* flag_list, unsigned int* flag_count, int flag_cap,
                     int restrict_ref, const Gas& g, Status* st);
void launch_scatter_in(cudaStream_t s, const double* src, d4* U, const int* dev_of_ref, int N);
void launch_gather_out(cudaStream_t s, const d4* U, double* dst, const int* dev_of_ref, int N);
int residual_blocks(int N);
void launch_residual(cudaStream_t s, const d4* R, int N, int norm, d4* part, double* out);

}  // namespace dev
}  // namespace fvgb

// Kernels of one explicit step on one mesh (sm_103a, FP64): primitive
// variables and the global time step, gradients with the Barth limiter, edge
// fluxes, the residual gather fused with the Runge-Kutta stage update, and the
// positivity pass.  The bodies live in step_device.cuh (shared with the
// batched stage kernel); reference functions are cited there.
#include <cuda_runtime.h>

#include "step_device.cuh"
#include "step_kernels.cuh"

namespace fvgb {
namespace dev {

__global__ void __launch_bounds__(256) k_prim(const d4* __restrict__ U, d4* __restrict__ U0,
                                              d4* __restrict__ prim, int N, Gas g, int copy) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < N) prim_cell(c, U, U0, prim, g, copy != 0);
}

template <bool NS>
__global__ void __launch_bounds__(256) k_alpha(const d4* __restrict__ prim, MeshView m, Gas g, double value_1,
                                               double* __restrict__ alpha, double* __restrict__ alpha_vis,
                                               Status* st) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < m.E) alpha_edge<NS>(e, prim, m, g, value_1, alpha, alpha_vis, st);
}

// minimum over the cells of CFL vol / alpha (starting value 1e10, CalculateDt.cpp:74-85)
template <bool NS>
__global__ void __launch_bounds__(256) k_dt_cell(MeshView m, const double* __restrict__ alpha,
                                                 const double* __restrict__ alpha_vis, double CFL,
                                                 unsigned long long* dtmin) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double dtc = 1e10;
    if (c < m.N) dtc = dmin(dtc, dt_cell<NS>(c, m, alpha, alpha_vis, CFL));
    for (int o = 16; o > 0; o >>= 1) dtc = dmin(dtc, __shfl_xor_sync(0xffffffffu, dtc, o));
    __shared__ double sm[8];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = dtc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = sm[0];
        for (int i = 1; i < (int)(blockDim.x >> 5); i++) v = dmin(v, sm[i]);
        if (!neg(v) && !is_nan(v)) dmin_atomic(dtmin, v);
        else atomicMin(dtmin, 0ull);  // a negative or NaN time step stops the clock (dt = 0)
    }
}

// t clamp and advance of CIteration::iteration_device, FVMR/src/time/CIteration.cpp:134-139
__global__ void k_dt_final(StepState* s, int advance) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double dt = __longlong_as_double((long long)s->dtmin_bits);
    s->dt_raw = dt;
    if (advance) {
        if (s->t + dt > s->T) dt = s->T - s->t;
        s->t_old = s->t;
        s->t += dt;
        s->dt = dt;
        s->dt6 = dt / 6.0;
    }
    s->dtmin_bits = (unsigned long long)__double_as_longlong(1e10);
}

template <int GRAD, bool BARTH, bool REC>
__global__ void __launch_bounds__(256) k_grad(const d4* __restrict__ U, MeshView m, d4* __restrict__ Gx,
                                              d4* __restrict__ Gy, CellTape tape) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < m.N) grad_cell<GRAD, BARTH, REC>(c, U, m, Gx, Gy, tape);
}

template <int FLUX, bool LINEAR, bool NS, bool REC>
__global__ void __launch_bounds__(256) k_flux_interior(const d4* __restrict__ U, const d4* __restrict__ Gx,
                                                       const d4* __restrict__ Gy, MeshView m, Gas g,
                                                       d4* __restrict__ F, EdgeTape tape) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < m.E_int) flux_interior<FLUX, LINEAR, NS, REC>(e, U, Gx, Gy, m, g, F, tape);
}

template <int FLUX, bool LINEAR, bool NS, bool REC>
__global__ void __launch_bounds__(128) k_flux_boundary(const d4* __restrict__ U, const d4* __restrict__ Gx,
                                                       const d4* __restrict__ Gy, MeshView m, Gas g, BcData bc,
                                                       d4* __restrict__ F, Status* st, EdgeTape tape) {
    const int e = m.E_int + blockIdx.x * blockDim.x + threadIdx.x;
    if (e < m.E) flux_boundary<FLUX, LINEAR, NS, REC>(e, U, Gx, Gy, m, g, bc, F, st, tape);
}

template <int KIND, bool FROM_RES = false>
__global__ void __launch_bounds__(256) k_update(d4* __restrict__ U, const d4* __restrict__ U0, d4* __restrict__ K1,
                                                d4* __restrict__ rhs_out, const d4* __restrict__ F, MeshView m,
                                                const StepState* s, Gas g, int* __restrict__ flag_list,
                                                unsigned int* flag_count, int flag_cap, Status* st,
                                                d4* __restrict__ rec_R, const double* __restrict__ dt_local) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    if constexpr (KIND == STAGE_LOCAL) {  // evolve_explicit_localtimestep, Evolve.cpp:115-125
        update_cell<STAGE_EULER, FROM_RES>(c, U, U0, K1, rhs_out, F, m, __ldg(&dt_local[c]), 0.0, g, flag_list, flag_count,
                                 flag_cap, st, rec_R);
        return;
    }
    double dt = 0.0, dt6 = 0.0;
    if (KIND != STAGE_RHS) {
        dt = s->dt;
        dt6 = s->dt6;
    }
    update_cell<KIND, FROM_RES>(c, U, U0, K1, rhs_out, F, m, dt, dt6, g, flag_list, flag_count, flag_cap, st, rec_R);
}

// Edge-coloured scatter: the edges of one colour (no two of them write the same cell) compute
// their fluxes and add them straight into the cells' sums, +F to L and, where the edge is in R's
// edge list (interior edges; a periodic edge's partner cell sums its own partner edge), -F to R.
// The sums are res[c] for the update's FROM_RES form; each cell's sum is taken in colour order.
template <int FLUX, bool LINEAR, bool NS>
__global__ void __launch_bounds__(256) k_flux_scatter(const d4* __restrict__ U, const d4* __restrict__ Gx,
                                                      const d4* __restrict__ Gy, MeshView m, Gas g, BcData bc,
                                                      const int* __restrict__ edges, const int* __restrict__ in_r,
                                                      int n, d4* __restrict__ res, Status* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int e = __ldg(&edges[i]);
    const d4 f = e < m.E_int ? flux_interior_value<FLUX, LINEAR, NS>(e, U, Gx, Gy, m, g)
                             : flux_boundary_value<FLUX, LINEAR, NS>(e, U, Gx, Gy, m, g, bc, st);
    const int L = __ldg(&m.e_L[e]);
    d4 a = res[L];
    res[L] = mk4(a.x + f.x, a.y + f.y, a.z + f.z, a.w + f.w);
    if (__ldg(&in_r[e])) {
        const int R = __ldg(&m.e_R[e]);
        a = res[R];
        res[R] = mk4(a.x - f.x, a.y - f.y, a.z - f.z, a.w - f.w);
    }
}

// get_local_dt_host/device (CalculateDt.cpp:66-72, 182-186; CalculateDtGPU.cu:83-110): each
// cell's CFL vol / alpha; the clock moves by the dt of the reference's cell 0
// (CIteration.cpp:47-49, 110-113) and T does not bound it
template <bool NS>
__global__ void __launch_bounds__(256) k_dt_local(MeshView m, const double* __restrict__ alpha,
                                                  const double* __restrict__ alpha_vis, double CFL,
                                                  double* __restrict__ dt_local, StepState* s, int cell0) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    const double v = dt_cell<NS>(c, m, alpha, alpha_vis, CFL);
    dt_local[c] = v;
    if (c == cell0) {
        s->dt_raw = v;
        s->dt = v;
        s->dt6 = v / 6.0;
        s->t += v;
    }
}

__global__ void k_restrict(d4* U, MeshView m, const int* __restrict__ cell_ref_of_dev,
                           const int* __restrict__ dev_of_cell_ref, int* flag_list, unsigned int* flag_count,
                           int flag_cap, int restrict_ref, Gas g, Status* st) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    restrict_pass(U, m, cell_ref_of_dev, dev_of_cell_ref, m.N, flag_list, flag_count, flag_cap, restrict_ref, g, st);
}

// ---------------------------------------------------------------------------
// reference-order <-> device-order state copies, and the residual norms
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_scatter_in(const double* __restrict__ src, d4* __restrict__ U,
                                                    const int* __restrict__ dev_of_ref, int N) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    U[__ldg(&dev_of_ref[r])] = mk4(src[r], src[(size_t)N + r], src[2 * (size_t)N + r], src[3 * (size_t)N + r]);
}

__global__ void __launch_bounds__(256) k_gather_out(const d4* __restrict__ U, double* __restrict__ dst,
                                                    const int* __restrict__ dev_of_ref, int N) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    const d4 u = ld4(&U[__ldg(&dev_of_ref[r])]);
    dst[r] = u.x;
    dst[(size_t)N + r] = u.y;
    dst[2 * (size_t)N + r] = u.z;
    dst[3 * (size_t)N + r] = u.w;
}

// the larger of two norms, NaN if either is NaN.  The reference's Math::max ((a > b) ? a : b,
// FVMR/src/math/BasicAlgorithm.h:10-12) lets a NaN through only when it comes last in its cell
// order; here any NaN residual gives a NaN norm, so that the driver's isnan stop
// (CDriver.cpp:235-263) fires whatever the cell order.
__device__ __forceinline__ double max_nan(double a, double b) { return (is_nan(a) || is_nan(b)) ? a + b : fmax(a, b); }

// get_residual_host (FVMR/src/output/residual/Residual.cpp:4-43): per-block
// partial norms, then one block combines them in a fixed order (deterministic)
__global__ void __launch_bounds__(256) k_residual_partial(const d4* __restrict__ R, int N, int norm,
                                                          d4* __restrict__ part) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    d4 a = mk4(0, 0, 0, 0);
    if (c < N) {
        const d4 r = ld4(&R[c]);
        a = mk4(fabs(r.x), fabs(r.y), fabs(r.z), fabs(r.w));
        if (norm == 2) a = mk4(a.x * a.x, a.y * a.y, a.z * a.z, a.w * a.w);
    }
    __shared__ d4 sm[256];
    sm[threadIdx.x] = a;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            d4 x = sm[threadIdx.x], y = sm[threadIdx.x + s];
            if (norm == 0)
                sm[threadIdx.x] = mk4(max_nan(x.x, y.x), max_nan(x.y, y.y), max_nan(x.z, y.z), max_nan(x.w, y.w));
            else sm[threadIdx.x] = mk4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

__global__ void k_residual_final(const d4* __restrict__ part, int nb, int norm, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    d4 a = mk4(0, 0, 0, 0);
    for (int i = 0; i < nb; i++) {
        d4 y = part[i];
        if (norm == 0) a = mk4(max_nan(a.x, y.x), max_nan(a.y, y.y), max_nan(a.z, y.z), max_nan(a.w, y.w));
        else a = mk4(a.x + y.x, a.y + y.y, a.z + y.z, a.w + y.w);
    }
    if (norm == 2) a = mk4(sqrt(a.x), sqrt(a.y), sqrt(a.z), sqrt(a.w));
    out[0] = a.x;
    out[1] = a.y;
    out[2] = a.z;
    out[3] = a.w;
}

// ---------------------------------------------------------------------------
// launchers (host)
// ---------------------------------------------------------------------------
static inline int blocks(long long n, int t) { return (int)((n + t - 1) / t); }

void launch_prim(cudaStream_t s, const d4* U, d4* U0, d4* prim, int N, const Gas& g, bool copy) {
    if (N > 0) k_prim<<<blocks(N, 256), 256, 0, s>>>(U, U0, prim, N, g, copy ? 1 : 0);
}

void launch_dt(cudaStream_t s, const d4* prim, const MeshView& m, const Gas& g, double value_1, double CFL,
               bool ns, double* alpha, double* alpha_vis, unsigned long long* dtmin, Status* st) {
    if (m.E > 0) {
        if (ns) k_alpha<true><<<blocks(m.E, 256), 256, 0, s>>>(prim, m, g, value_1, alpha, alpha_vis, st);
        else k_alpha<false><<<blocks(m.E, 256), 256, 0, s>>>(prim, m, g, value_1, alpha, alpha_vis, st);
    }
    if (m.N > 0) {
        if (ns) k_dt_cell<true><<<blocks(m.N, 256), 256, 0, s>>>(m, alpha, alpha_vis, CFL, dtmin);
        else k_dt_cell<false><<<blocks(m.N, 256), 256, 0, s>>>(m, alpha, alpha_vis, CFL, dtmin);
    }
}

void launch_dt_final(cudaStream_t s, StepState* st, bool advance) { k_dt_final<<<1, 32, 0, s>>>(st, advance ? 1 : 0); }

void launch_dt_local(cudaStream_t s, const d4* prim, const MeshView& m, const Gas& g, double value_1, double CFL,
                     bool ns, double* alpha, double* alpha_vis, double* dt_local, StepState* st, int cell0,
                     Status* status) {
    if (m.E > 0) {
        if (ns) k_alpha<true><<<blocks(m.E, 256), 256, 0, s>>>(prim, m, g, value_1, alpha, alpha_vis, status);
        else k_alpha<false><<<blocks(m.E, 256), 256, 0, s>>>(prim, m, g, value_1, alpha, alpha_vis, status);
    }
    if (m.N > 0) {
        if (ns) k_dt_local<true><<<blocks(m.N, 256), 256, 0, s>>>(m, alpha, alpha_vis, CFL, dt_local, st, cell0);
        else k_dt_local<false><<<blocks(m.N, 256), 256, 0, s>>>(m, alpha, alpha_vis, CFL, dt_local, st, cell0);
    }
}

void launch_grad(cudaStream_t s, int gradient, bool barth, const d4* U, const MeshView& m, d4* Gx, d4* Gy,
                 const CellTape* tape) {
    if (m.N <= 0) return;
    const int b = blocks(m.N, 256);
    const CellTape none;
    if (tape && tape->gx && barth) {  // the adjoint's recorded forward
        if (gradient == 1) k_grad<1, true, true><<<b, 256, 0, s>>>(U, m, Gx, Gy, *tape);
        else k_grad<2, true, true><<<b, 256, 0, s>>>(U, m, Gx, Gy, *tape);
    } else if (gradient == 1) {
        if (barth) k_grad<1, true, false><<<b, 256, 0, s>>>(U, m, Gx, Gy, none);
        else k_grad<1, false, false><<<b, 256, 0, s>>>(U, m, Gx, Gy, none);
    } else {
        if (barth) k_grad<2, true, false><<<b, 256, 0, s>>>(U, m, Gx, Gy, none);
        else k_grad<2, false, false><<<b, 256, 0, s>>>(U, m, Gx, Gy, none);
    }
}

template <int FLUX, bool LINEAR, bool NS, bool REC = false>
static void flux_impl(cudaStream_t s, const d4* U, const d4* Gx, const d4* Gy, const MeshView& m,
                      const Gas& g, const BcData& bc, d4* F, Status* st, EdgeTape tape = EdgeTape()) {
    if (m.E_int > 0)
        k_flux_interior<FLUX, LINEAR, NS, REC><<<blocks(m.E_int, 256), 256, 0, s>>>(U, Gx, Gy, m, g, F, tape);
    if (m.E > m.E_int)
        k_flux_boundary<FLUX, LINEAR, NS, REC><<<blocks(m.E - m.E_int, 128), 128, 0, s>>>(U, Gx, Gy, m, g, bc, F, st,
                                                                                          tape);
}

void launch_flux(cudaStream_t s, int scheme, bool linear, bool ns, const d4* U, const d4* Gx,
                 const d4* Gy, const MeshView& m, const Gas& g, const BcData& bc, d4* F, Status* st,
                 const EdgeTape* tape) {
    if (tape && tape->v) {  // the adjoint's recorded forward
#define FVGB_REC(FL, LIN, NSV) flux_impl<FL, LIN, NSV, true>(s, U, Gx, Gy, m, g, bc, F, st, *tape)
        if (scheme == FLUX_ROE) {
            if (linear) { if (ns) FVGB_REC(FLUX_ROE, true, true); else FVGB_REC(FLUX_ROE, true, false); }
            else { if (ns) FVGB_REC(FLUX_ROE, false, true); else FVGB_REC(FLUX_ROE, false, false); }
        } else {
            if (linear) { if (ns) FVGB_REC(FLUX_LLF, true, true); else FVGB_REC(FLUX_LLF, true, false); }
            else { if (ns) FVGB_REC(FLUX_LLF, false, true); else FVGB_REC(FLUX_LLF, false, false); }
        }
#undef FVGB_REC
        return;
    }
    if (scheme == FLUX_ROE) {
        if (linear) {
            if (ns) flux_impl<FLUX_ROE, true, true>(s, U, Gx, Gy, m, g, bc, F, st);
            else flux_impl<FLUX_ROE, true, false>(s, U, Gx, Gy, m, g, bc, F, st);
        } else {
            if (ns) flux_impl<FLUX_ROE, false, true>(s, U, Gx, Gy, m, g, bc, F, st);
            else flux_impl<FLUX_ROE, false, false>(s, U, Gx, Gy, m, g, bc, F, st);
        }
    } else {
        if (linear) {
            if (ns) flux_impl<FLUX_LLF, true, true>(s, U, Gx, Gy, m, g, bc, F, st);
            else flux_impl<FLUX_LLF, true, false>(s, U, Gx, Gy, m, g, bc, F, st);
        } else {
            if (ns) flux_impl<FLUX_LLF, false, true>(s, U, Gx, Gy, m, g, bc, F, st);
            else flux_impl<FLUX_LLF, false, false>(s, U, Gx, Gy, m, g, bc, F, st);
        }
    }
}

void launch_update(cudaStream_t s, int kind, d4* U, const d4* U0, d4* K1, d4* rhs,
                   const d4* F, const MeshView& m, const StepState* st, const Gas& g, int* flag_list,
                   unsigned int* flag_count, int flag_cap, Status* status, d4* rec_R, const double* dt_local,
                   bool from_res) {
    if (m.N <= 0) return;
    const int b = blocks(m.N, 256);
#define FVGB_UPD(K)                                                                                                  \
    do {                                                                                                             \
        if (from_res)                                                                                                \
            k_update<K, true><<<b, 256, 0, s>>>(U, U0, K1, rhs, F, m, st, g, flag_list, flag_count, flag_cap, status, \
                                                rec_R, dt_local);                                                    \
        else                                                                                                         \
            k_update<K><<<b, 256, 0, s>>>(U, U0, K1, rhs, F, m, st, g, flag_list, flag_count, flag_cap, status,       \
                                          rec_R, dt_local);                                                          \
    } while (0)
    switch (kind) {
    case STAGE_LOCAL: FVGB_UPD(STAGE_LOCAL); break;
    case STAGE_RHS: FVGB_UPD(STAGE_RHS); break;
    case STAGE_EULER: FVGB_UPD(STAGE_EULER); break;
    case STAGE_RK3_1: FVGB_UPD(STAGE_RK3_1); break;
    case STAGE_RK3_2: FVGB_UPD(STAGE_RK3_2); break;
    case STAGE_RK3_3: FVGB_UPD(STAGE_RK3_3); break;
    case STAGE_SSP_1: FVGB_UPD(STAGE_SSP_1); break;
    case STAGE_SSP_2: FVGB_UPD(STAGE_SSP_2); break;
    default: FVGB_UPD(STAGE_SSP_3); break;
    }
#undef FVGB_UPD
}

void launch_flux_scatter(cudaStream_t s, int scheme, bool linear, bool ns, const d4* U, const d4* Gx, const d4* Gy,
                         const MeshView& m, const Gas& g, const BcData& bc, const int* edges, const int* in_r,
                         int n, d4* res, Status* st) {
    if (n <= 0) return;
    const int b = blocks(n, 256);
#define FVGB_SC(FL, LIN, NSV) \
    k_flux_scatter<FL, LIN, NSV><<<b, 256, 0, s>>>(U, Gx, Gy, m, g, bc, edges, in_r, n, res, st)
    if (scheme == FLUX_ROE) {
        if (linear) { if (ns) FVGB_SC(FLUX_ROE, true, true); else FVGB_SC(FLUX_ROE, true, false); }
        else { if (ns) FVGB_SC(FLUX_ROE, false, true); else FVGB_SC(FLUX_ROE, false, false); }
    } else {
        if (linear) { if (ns) FVGB_SC(FLUX_LLF, true, true); else FVGB_SC(FLUX_LLF, true, false); }
        else { if (ns) FVGB_SC(FLUX_LLF, false, true); else FVGB_SC(FLUX_LLF, false, false); }
    }
#undef FVGB_SC
}

void launch_restrict(cudaStream_t s, d4* U, const MeshView& m, const int* cell_ref_of_dev,
                     const int* dev_of_cell_ref, int* flag_list, unsigned int* flag_count, int flag_cap,
                     int restrict_ref, const Gas& g, Status* st) {
    k_restrict<<<1, 32, 0, s>>>(U, m, cell_ref_of_dev, dev_of_cell_ref, flag_list, flag_count, flag_cap, restrict_ref, g, st);
}

void launch_scatter_in(cudaStream_t s, const double* src, d4* U, const int* dev_of_ref, int N) {
    if (N > 0) k_scatter_in<<<blocks(N, 256), 256, 0, s>>>(src, U, dev_of_ref, N);
}

void launch_gather_out(cudaStream_t s, const d4* U, double* dst, const int* dev_of_ref, int N) {
    if (N > 0) k_gather_out<<<blocks(N, 256), 256, 0, s>>>(U, dst, dev_of_ref, N);
}

int residual_blocks(int N) { return blocks(N, 256); }

void launch_residual(cudaStream_t s, const d4* R, int N, int norm, d4* part, double* out) {
    const int nb = blocks(N, 256);
    if (nb > 0) k_residual_partial<<<nb, 256, 0, s>>>(R, N, norm, part);
    k_residual_final<<<1, 32, 0, s>>>(part, nb, norm, out);
}

}  // namespace dev
}  // namespace fvgb

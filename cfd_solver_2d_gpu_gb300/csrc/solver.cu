// One solver on one GPU: device memory, the captured step graph and the
// C ABI of include/fvgb.h.  Replaces GPU::GPUSolver2 (FVMR/src/solvers/GPUSolver2.cpp)
// and CIteration::iteration_device (FVMR/src/time/CIteration.cpp:89-161).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"
#include "layout.h"
#include "solver.h"
#include "step_kernels.cuh"

namespace fvgb {

namespace {
thread_local std::string g_error;
}

void set_error(const std::string& msg) { g_error = msg; }
int fail(int code, const std::string& msg) {
    set_error(msg);
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(FVGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));       \
    } while (0)

template <class T>
static int dalloc(T*& p, size_t n, std::vector<void*>& owned) {
    p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)&p, n * sizeof(T));
    if (e != cudaSuccess) return fail(FVGB_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    owned.push_back((void*)p);
    return 0;
}

template <class T>
static int dupload(T*& p, const std::vector<T>& v, std::vector<void*>& owned, cudaStream_t s) {
    int rc = dalloc(p, v.size(), owned);
    if (rc) return rc;
    if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return 0;
}

dev::Gas make_gas(const fvgb_params& p) {
    dev::Gas g;
    g.gamma = p.gamma;
    g.ga1 = p.gamma - 1.0;
    g.gam_over_ga1 = p.gamma / (p.gamma - 1.0);
    g.inv_ga1 = 1.0 / (p.gamma - 1.0);
    g.Etm_c = (p.gamma - 1.0) / p.gamma * 0.5;
    g.inv_gamma = 1.0 / p.gamma;
    g.R = p.R;
    g.Cv = p.R / (p.gamma - 1.0);
    g.Cp = g.Cv * p.gamma;
    g.inv_Cv = 1.0 / g.Cv;
    // get_Sutherland_C1_host_device, FVMR/src/space/viscous_flux/ViscousFluxGPU.h:26-28
    g.C1 = p.mu0 / std::pow(p.T0, 1.5) * (p.T0 + 110.4);
    return g;
}

dev::BcData make_bc(const fvgb_params& p) {
    dev::BcData b;
    std::memcpy(b.inf, p.inf, sizeof b.inf);
    std::memcpy(b.inlet, p.inlet, sizeof b.inlet);
    std::memcpy(b.outlet, p.outlet, sizeof b.outlet);
    auto a = [&](const double* s) { return s[0] > 0 ? std::sqrt(p.gamma * s[3] / s[0]) : 0.0; };
    auto son = [&](const double* s) { return s[0] > 0 ? s[3] / std::pow(s[0], p.gamma) : 0.0; };
    b.a_inf = a(p.inf);
    b.a_inlet = a(p.inlet);
    b.a_outlet = a(p.outlet);
    b.son_inf = son(p.inf);
    b.son_inlet = son(p.inlet);
    b.son_outlet = son(p.outlet);
    b.wall_ref = p.wall_bc_ref;
    b.dsr_x = p.dsr[0];
    b.sqrt3 = std::sqrt(3.0);  // CBoundaryDoubleShockReflect.cpp:7
    b.clock_t0 = b.clock_dt = nullptr;
    b.clock_frac = 0.0;
    return b;
}

static int check_params(const fvgb_params& p) {
    if (p.equation != 1 && p.equation != 2) return fail(FVGB_ERR_ARG, "physicsModel.equation must be 1 or 2");
    if (p.flux_scheme != 2001 && p.flux_scheme != 2002)
        return fail(FVGB_ERR_ARG, "invalid scheme (flux_conservation_scheme must be 2001 or 2002)");
    if (p.reconstruct != 3001 && p.reconstruct != 3002)
        return fail(FVGB_ERR_ARG, "invalid flag_reconstruct (3001 or 3002)");
    if (p.gradient != 1 && p.gradient != 2) return fail(FVGB_ERR_ARG, "invalid graident type (flag_gradient 1 or 2)");
    if (p.limiter != 0 && p.limiter != 1) return fail(FVGB_ERR_ARG, "invalid limiter type (flux_limiter 0 or 1)");
    if (p.time_advance != 3101 && p.time_advance != 3103 && p.time_advance != 3104)
        return fail(FVGB_ERR_ARG, "invalid temporal_choice (time_advance 3101, 3103 or 3104)");
    if (!(p.gamma > 1.0)) return fail(FVGB_ERR_ARG, "gamma must exceed 1");
    return 0;
}

int Solver::init(const fvgb_mesh_soa& m, const fvgb_params& prm) {
    p = prm;
    int rc = check_params(p);
    if (rc) return rc;
    if ((rc = validate_mesh(m))) return rc;  // host-only checks first: a bad mesh is refused without a device
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(FVGB_ERR_NO_DEVICE, "no CUDA device");
    if (p.device < 0 || p.device >= ndev) return fail(FVGB_ERR_ARG, "device ordinal out of range");
    CK(cudaSetDevice(p.device));
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    rc = build_layout(m, p, L);
    if (rc) return rc;
    if ((rc = keep_output_mesh(m))) return rc;
    N = L.N;
    E = L.E;
    gas = make_gas(p);
    bc = make_bc(p);
    // sqrt(length) for the time step lives in the spare geometry slot
    for (int i = 0; i < E; i++) L.e_geom[(size_t)i * 8 + 3] = std::sqrt(L.e_geom[(size_t)i * 8 + 2]);
    cudaStream_t s = stream;
    if ((rc = dupload(d_e_L, L.e_L, owned, s)) || (rc = dupload(d_e_R, L.e_R, owned, s)) ||
        (rc = dupload(d_e_bc, L.e_bc, owned, s)) || (rc = dupload(d_e_geom, L.e_geom, owned, s)) ||
        (rc = dupload(d_c_edge, L.c_edge, owned, s)) || (rc = dupload(d_c_nbr, L.c_nbr, owned, s)) ||
        (rc = dupload(d_c_nnb, L.c_nnb, owned, s)) || (rc = dupload(d_c_mvol, L.c_mvol, owned, s)) ||
        (rc = dupload(d_c_vol, L.c_vol, owned, s)) || (rc = dupload(d_c_vtx, L.c_vtx, owned, s)) ||
        (rc = dupload(d_dt_ptr, L.dt_ptr, owned, s)) || (rc = dupload(d_dt_edge, L.dt_edge, owned, s)) ||
        (rc = dupload(d_cell_ref, L.cell_ref, owned, s)) || (rc = dupload(d_cell_new, L.cell_new, owned, s)))
        return rc;
    if (p.gradient == 1) {
        if ((rc = dupload(d_c_lsq, L.c_lsq, owned, s))) return rc;
    } else {
        if ((rc = dupload(d_c_gg, L.c_gg, owned, s)) || (rc = dupload(d_c_ggout, L.c_ggout, owned, s)) ||
            (rc = dupload(d_c_ginv, L.c_ginv, owned, s)))
            return rc;
    }
    if (p.edge_colour &&
        ((rc = dupload(d_col_edge, L.col_edge, owned, s)) || (rc = dupload(d_e_in_r, L.e_in_r, owned, s))))
        return rc;
    const size_t n4 = (size_t)N;
    // the edge fluxes, or in the coloured scatter the cells' sums of them
    const size_t nF = std::max((size_t)E, p.edge_colour ? n4 : (size_t)0);
    if ((rc = dalloc(d_U, n4, owned)) || (rc = dalloc(d_U0, n4, owned)) || (rc = dalloc(d_Gx, n4, owned)) ||
        (rc = dalloc(d_Gy, n4, owned)) || (rc = dalloc(d_F, nF, owned)) || (rc = dalloc(d_prim, n4, owned)) ||
        (rc = dalloc(d_rhs, n4, owned)) || (rc = dalloc(d_alpha, (size_t)E, owned)) ||
        (rc = dalloc(d_alpha_vis, (size_t)E, owned)) || (rc = dalloc(d_flags, (size_t)kFlagCap, owned)) ||
        (rc = dalloc(d_flag_count, 1, owned)) || (rc = dalloc(d_state, 1, owned)) ||
        (rc = dalloc(d_status, 1, owned)) || (rc = dalloc(d_stage, 4 * n4, owned)) ||
        (rc = dalloc(d_res_part, (size_t)dev::residual_blocks(N) + 1, owned)) || (rc = dalloc(d_res_out, 4, owned)))
        return rc;
    if (p.time_advance == 3103 && (rc = dalloc(d_K1, n4, owned))) return rc;
    if (p.steady && (rc = dalloc(d_dt_local, (size_t)N, owned))) return rc;
    cell0_dev = N > 0 ? L.cell_new[0] : 0;
    if (!d_K1) d_K1 = d_U0;  // unused by the other integrators
    CK(cudaMemsetAsync(d_flag_count, 0, sizeof(unsigned int), s));
    CK(cudaMemsetAsync(d_status, 0, sizeof(dev::Status), s));
    CK(cudaMemsetAsync(d_Gx, 0, n4 * sizeof(d4), s));
    CK(cudaMemsetAsync(d_Gy, 0, n4 * sizeof(d4), s));
    dev::StepState st0{};
    st0.dtmin_bits = 0;
    {
        double big = 1e10;
        std::memcpy(&st0.dtmin_bits, &big, sizeof big);
    }
    CK(cudaMemcpyAsync(d_state, &st0, sizeof st0, cudaMemcpyHostToDevice, s));
    CK(cudaMallocHost((void**)&h_state, sizeof(dev::StepState)));
    *h_state = st0;
    mv.N = N;
    mv.E = E;
    mv.E_int = L.E_int;
    mv.e_L = d_e_L;
    mv.e_R = d_e_R;
    mv.e_bc = d_e_bc;
    mv.e_geom = d_e_geom;
    mv.c_edge = d_c_edge;
    mv.c_nbr = d_c_nbr;
    mv.c_nnb = d_c_nnb;
    mv.c_mvol = d_c_mvol;
    mv.c_vol = d_c_vol;
    mv.c_lsq = d_c_lsq;
    mv.c_vtx = d_c_vtx;
    mv.c_gg = d_c_gg;
    mv.c_ggout = d_c_ggout;
    mv.c_ginv = d_c_ginv;
    mv.dt_ptr = d_dt_ptr;
    mv.dt_edge = d_dt_edge;
    // initial field (FieldInitializer) in the reference order, then on the device
    std::vector<double> U0((size_t)4 * N);
    if (p.ic_type >= 1 && p.ic_type <= 4) {
        rc = initial_field(m, p, U0.data());
        if (rc) return rc;
        rc = set_state(U0.data());
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(s));
    return 0;
}

Solver::~Solver() {
    release_output();
    drop_graphs();
    if (h_state) cudaFreeHost(h_state);
    for (void* q : owned) cudaFree(q);
    if (stream) cudaStreamDestroy(stream);
}

bool Solver::needs_gradient() const { return p.reconstruct == 3002 || p.equation == 2; }

// event pair around one group of launches (profiling entry point only; never captured)
void Solver::mark(int cls, bool begin) {
    if (!prof) return;
    cudaEvent_t ev;
    cudaEventCreate(&ev);
    cudaEventRecord(ev, stream);
    if (begin) {
        prof->open[cls] = ev;
    } else {
        prof->pairs.push_back({cls, prof->open[cls], ev});
    }
}

// the residual of one stage: gradient + limiter, edge fluxes, gather + update
void Solver::enqueue_stage(int kind) {
    cudaStream_t s = stream;
    if (needs_gradient()) {
        mark(PROF_GRAD, true);
        dev::launch_grad(s, p.gradient, p.limiter == 1, d_U, mv, d_Gx, d_Gy, rec_ctape.gx ? &rec_ctape : nullptr);
        mark(PROF_GRAD, false);
        launches += 1;
    }
    mark(PROF_FLUX, true);
    dev::BcData b = bc;  // the stage's clock for the double-Mach-reflection boundary
    b.clock_t0 = &d_state->t_old;
    b.clock_dt = &d_state->dt;
    b.clock_frac = dev::dsr_stage_frac(kind);
    enqueue_residual(b, kind);
}

// the edge fluxes and the stage update of one stage: either every edge's flux to d_F and the
// per-cell gather in the reference's slot order, or ([gpu] edge_colour = 1) the fluxes added
// colour by colour into the cells' sums in d_F, which the update then reads
void Solver::enqueue_residual(const dev::BcData& b, int kind) {
    cudaStream_t s = stream;
    const bool coloured = p.edge_colour && !rec_tape.v;
    if (coloured) {
        cudaMemsetAsync(d_F, 0, sizeof(d4) * (size_t)N, s);
        const int nc = (int)L.col_ptr.size() - 1;
        for (int k = 0; k < nc; k++)
            dev::launch_flux_scatter(s, p.flux_scheme, p.reconstruct == 3002, p.equation == 2, d_U, d_Gx, d_Gy, mv,
                                     gas, b, d_col_edge + L.col_ptr[k], d_e_in_r, L.col_ptr[k + 1] - L.col_ptr[k],
                                     d_F, d_status);
        launches += nc;
    } else {
        dev::launch_flux(s, p.flux_scheme, p.reconstruct == 3002, p.equation == 2, d_U, d_Gx, d_Gy, mv, gas, b, d_F,
                         d_status, rec_tape.v ? &rec_tape : nullptr);
        launches += (mv.E_int > 0) + (mv.E > mv.E_int);
    }
    mark(PROF_FLUX, false);
    mark(PROF_UPDATE, true);
    dev::launch_update(s, kind, d_U, d_U0, d_K1, d_rhs, d_F, mv, d_state, gas, d_flags, d_flag_count, kFlagCap,
                       d_status, d_rec_R, d_dt_local, coloured);
    mark(PROF_UPDATE, false);
    launches += 1;
}

// one CIteration::iteration_device: dt, t clamp, stages, restrict
void Solver::enqueue_step() {
    cudaStream_t s = stream;
    const bool copy = p.time_advance != 3101 && !p.steady;
    mark(PROF_DT, true);
    dev::launch_prim(s, d_U, d_U0, d_prim, N, gas, copy);
    const double value_1 = std::max(4.0 / 3.0, p.gamma / p.Pr);
    if (p.steady) {  // CIteration.cpp:42-52 (host) and 109-121 (device)
        dev::launch_dt_local(s, d_prim, mv, gas, value_1, p.CFL, p.equation == 2, d_alpha, d_alpha_vis, d_dt_local,
                             d_state, cell0_dev, d_status);
        mark(PROF_DT, false);
        launches += 3;
        enqueue_stage(dev::STAGE_LOCAL);
        mark(PROF_RESTRICT, true);  // as iteration_host does (CIteration.cpp:79); iteration_device skips it
        dev::launch_restrict(s, d_U, mv, d_cell_ref, d_cell_new, d_flags, d_flag_count, kFlagCap, p.restrict_ref, gas,
                             d_status);
        mark(PROF_RESTRICT, false);
        launches += 1;
        return;
    }
    dev::launch_dt(s, d_prim, mv, gas, value_1, p.CFL, p.equation == 2, d_alpha, d_alpha_vis, &d_state->dtmin_bits,
                   d_status);
    dev::launch_dt_final(s, d_state, true);
    mark(PROF_DT, false);
    launches += 4;
    if (p.time_advance == 3101) {
        enqueue_stage(dev::STAGE_EULER);
    } else if (p.time_advance == 3103) {
        enqueue_stage(dev::STAGE_RK3_1);
        enqueue_stage(dev::STAGE_RK3_2);
        enqueue_stage(dev::STAGE_RK3_3);
    } else {
        enqueue_stage(dev::STAGE_SSP_1);
        enqueue_stage(dev::STAGE_SSP_2);
        enqueue_stage(dev::STAGE_SSP_3);
    }
    mark(PROF_RESTRICT, true);
    dev::launch_restrict(s, d_U, mv, d_cell_ref, d_cell_new, d_flags, d_flag_count, kFlagCap, p.restrict_ref, gas,
                         d_status);
    mark(PROF_RESTRICT, false);
    launches += 1;
}

// nsteps run launch by launch (no graph) with CUDA events around each kernel
// group on the solver's stream; returns the summed milliseconds per group
int Solver::profile_steps(double T, int nsteps, double* ms, int* count) {
    CK(cudaMemcpyAsync(&d_state->T, &T, sizeof(double), cudaMemcpyHostToDevice, stream));
    Prof pr;
    prof = &pr;
    for (int i = 0; i < nsteps; i++) enqueue_step();
    prof = nullptr;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
    for (int c = 0; c < PROF_NCLASS; c++) {
        ms[c] = 0.0;
        count[c] = 0;
    }
    for (auto& q : pr.pairs) {
        float t = 0.f;
        cudaEventElapsedTime(&t, q.a, q.b);
        ms[q.cls] += t;
        count[q.cls] += 1;
        cudaEventDestroy(q.a);
        cudaEventDestroy(q.b);
    }
    return check_status();
}

void Solver::drop_graphs() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (graph_exec_multi) cudaGraphExecDestroy(graph_exec_multi);
    graph_exec = graph_exec_multi = nullptr;
}

// The step captured once as a graph of one step and once as a graph of kGraphSteps
// steps back to back: long runs replay the second, so a graph boundary (and its launch)
// comes once every kGraphSteps steps instead of every step.
int Solver::build_graph() {
    if (graph_exec && graph_exec_multi) return 0;
    drop_graphs();
    auto capture = [&](int steps, cudaGraphExec_t* out) -> int {
        cudaGraph_t g = nullptr;
        const long long before = launches;
        CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < steps; i++) enqueue_step();
        cudaError_t e = cudaStreamEndCapture(stream, &g);
        if (e != cudaSuccess) return fail(FVGB_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        if (steps == 1) launches_per_step = launches - before;
        launches = before;
        e = cudaGraphInstantiate(out, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(FVGB_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        return 0;
    };
    int rc = capture(1, &graph_exec);
    if (!rc) rc = capture(kGraphSteps, &graph_exec_multi);
    if (rc) drop_graphs();
    return rc;
}

int Solver::check_status() {
    dev::Status st;
    CK(cudaMemcpyAsync(&st, d_status, sizeof st, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if (st.nan_cells > seen.nan_cells) {
        seen = st;
        return fail(FVGB_ERR_NAN, "NaN in the state (the reference stops here: Restrict.cpp:26-29)");
    }
    if (st.negative_dt > seen.negative_dt) {
        seen = st;
        return fail(FVGB_ERR_RANGE, "rho or p < 0 in the time step (CalculateDt.cpp:41-44)");
    }
    if (st.farfield_oor > seen.farfield_oor) {
        seen = st;
        return fail(FVGB_ERR_RANGE, "far-field ghost state out of range (Flux.cpp:157-160)");
    }
    seen = st;
    return 0;
}

int Solver::step_async(double T, int nsteps) {
    if (nsteps < 0) return fail(FVGB_ERR_ARG, "nsteps < 0");
    int rc = build_graph();
    if (rc) return rc;
    CK(cudaMemcpyAsync(&d_state->T, &T, sizeof(double), cudaMemcpyHostToDevice, stream));
    int i = 0;
    for (; i + kGraphSteps <= nsteps; i += kGraphSteps) CK(cudaGraphLaunch(graph_exec_multi, stream));
    for (; i < nsteps; i++) CK(cudaGraphLaunch(graph_exec, stream));
    launches += launches_per_step * nsteps;
    return 0;
}

int Solver::set_time(double t) {
    CK(cudaMemcpyAsync(&d_state->t, &t, sizeof(double), cudaMemcpyHostToDevice, stream));
    return 0;
}

int Solver::get_time(double* t, double* dt) {
    CK(cudaMemcpyAsync(h_state, d_state, sizeof(dev::StepState), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    if (t) *t = h_state->t;
    if (dt) *dt = h_state->dt;
    return 0;
}

// The device address of a page-locked host buffer (NULL for pageable memory): with
// unified addressing the scatter / gather kernels read and write such a buffer
// directly over the host link (NVLink-C2C on Grace), one coalesced pass and no
// staging copy.
static double* device_view(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost && a.devicePointer) ? static_cast<double*>(a.devicePointer) : nullptr;
}

// returns once U has been read (GPUSolver2::host_to_device's blocking copy), so the
// caller may reuse U at once
int Solver::set_state(const double* U) {
    if (const double* dv = device_view(U)) {
        dev::launch_scatter_in(stream, dv, d_U, d_cell_new, N);
    } else {
        CK(cudaMemcpyAsync(d_stage, U, (size_t)4 * N * sizeof(double), cudaMemcpyHostToDevice, stream));
        dev::launch_scatter_in(stream, d_stage, d_U, d_cell_new, N);
    }
    launches += 1;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
    return 0;
}

int Solver::get_state(double* U) {
    if (double* dv = device_view(U)) {
        dev::launch_gather_out(stream, d_U, dv, d_cell_new, N);
    } else {
        dev::launch_gather_out(stream, d_U, d_stage, d_cell_new, N);
        CK(cudaMemcpyAsync(U, d_stage, (size_t)4 * N * sizeof(double), cudaMemcpyDeviceToHost, stream));
    }
    launches += 1;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(stream));
    return 0;
}

int Solver::rhs(const double* U, double* R, double* gx, double* gy) {
    int rc = set_state(U);
    if (rc) return rc;
    if (needs_gradient() || gx || gy) {
        dev::launch_grad(stream, p.gradient, p.limiter == 1, d_U, mv, d_Gx, d_Gy);
        launches += 1;
    }
    dev::BcData b = bc;  // "dsr" edges at the handle's time t (the last step's end, or fvgb_step's t)
    b.clock_t0 = &d_state->t;
    b.clock_dt = &d_state->dt;
    b.clock_frac = 0.0;
    enqueue_residual(b, dev::STAGE_RHS);
    CK(cudaGetLastError());
    auto out = [&](const d4* src, double* dst) -> int {
        dev::launch_gather_out(stream, src, d_stage, d_cell_new, N);
        launches += 1;
        CK(cudaMemcpyAsync(dst, d_stage, (size_t)4 * N * sizeof(double), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        return 0;
    };
    if (R && (rc = out(d_rhs, R))) return rc;
    if (gx && (rc = out(d_Gx, gx))) return rc;
    if (gy && (rc = out(d_Gy, gy))) return rc;
    return check_status();
}

int Solver::dt(double* out) {
    dev::launch_prim(stream, d_U, d_U0, d_prim, N, gas, false);
    const double value_1 = std::max(4.0 / 3.0, p.gamma / p.Pr);
    dev::launch_dt(stream, d_prim, mv, gas, value_1, p.CFL, p.equation == 2, d_alpha, d_alpha_vis,
                   &d_state->dtmin_bits, d_status);
    dev::launch_dt_final(stream, d_state, false);
    launches += 4;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h_state, d_state, sizeof(dev::StepState), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    *out = h_state->dt_raw;
    return check_status();
}

int Solver::residual(int norm, double* out) {
    if (norm < 0 || norm > 2) return fail(FVGB_ERR_ARG, "norm must be 0, 1 or 2");
    dev::launch_residual(stream, d_rhs, N, norm, d_res_part, d_res_out);
    launches += 2;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, d_res_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    return 0;
}

}  // namespace fvgb

using namespace fvgb;

#define GUARD(h)                                                     \
    do {                                                             \
        if (!(h)) return fail(FVGB_ERR_ARG, "null handle");          \
        cudaError_t e0_ = cudaSetDevice((h)->s.p.device);            \
        if (e0_ != cudaSuccess) return fail(FVGB_ERR_CUDA, cudaGetErrorString(e0_)); \
    } while (0)

extern "C" int fvgb_create(const fvgb_mesh_soa* mesh, const fvgb_params* p, fvgb_handle** out) {
    if (!mesh || !p || !out) return fail(FVGB_ERR_ARG, "null argument");
    *out = nullptr;
    fvgb_handle* h = new fvgb_handle();
    int rc = h->s.init(*mesh, *p);
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return 0;
}

extern "C" void fvgb_destroy(fvgb_handle* h) {
    if (!h) return;
    cudaSetDevice(h->s.p.device);
    fvgb_adjoint_release(h);  // the adjoint workspace of this handle, if any
    delete h;
}

extern "C" int fvgb_set_state(fvgb_handle* h, const double* U) {
    GUARD(h);
    if (!U) return fail(FVGB_ERR_ARG, "null state");
    int rc = h->s.set_state(U);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->s.stream));
    return 0;
}

extern "C" int fvgb_get_state(fvgb_handle* h, double* U) {
    GUARD(h);
    if (!U) return fail(FVGB_ERR_ARG, "null state");
    return h->s.get_state(U);
}

extern "C" int fvgb_step(fvgb_handle* h, double* t, double T, int nsteps) {
    GUARD(h);
    if (!t) return fail(FVGB_ERR_ARG, "null time");
    int rc = h->s.set_time(*t);
    if (rc) return rc;
    if ((rc = h->s.step_async(T, nsteps))) return rc;
    if ((rc = h->s.get_time(t, nullptr))) return rc;
    return h->s.check_status();
}

extern "C" int fvgb_step_async(fvgb_handle* h, double T, int nsteps) {
    GUARD(h);
    return h->s.step_async(T, nsteps);
}

extern "C" int fvgb_set_time(fvgb_handle* h, double t) {
    GUARD(h);
    return h->s.set_time(t);
}

extern "C" int fvgb_set_cfl(fvgb_handle* h, double CFL) {
    GUARD(h);
    if (!(CFL > 0.0)) return fail(FVGB_ERR_ARG, "CFL must be positive");
    Solver& s = h->s;
    if (s.p.CFL == CFL) return 0;
    CK(cudaStreamSynchronize(s.stream));  // no launch of the old graph is still pending
    s.p.CFL = CFL;
    s.drop_graphs();  // the step was captured with the old value
    return 0;
}

extern "C" int fvgb_time(fvgb_handle* h, double* t, double* last_dt) {
    GUARD(h);
    return h->s.get_time(t, last_dt);
}

extern "C" int fvgb_synchronize(fvgb_handle* h) {
    GUARD(h);
    CK(cudaStreamSynchronize(h->s.stream));
    return h->s.check_status();
}

extern "C" int fvgb_rhs(fvgb_handle* h, const double* U, double* rhs, double* gx, double* gy) {
    GUARD(h);
    if (!U) return fail(FVGB_ERR_ARG, "null state");
    return h->s.rhs(U, rhs, gx, gy);
}

extern "C" int fvgb_dt(fvgb_handle* h, double* dt) {
    GUARD(h);
    if (!dt) return fail(FVGB_ERR_ARG, "null output");
    return h->s.dt(dt);
}

extern "C" int fvgb_residual(fvgb_handle* h, int norm, double out4[4]) {
    GUARD(h);
    if (!out4) return fail(FVGB_ERR_ARG, "null output");
    return h->s.residual(norm, out4);
}

extern "C" int fvgb_device_status(fvgb_handle* h, long long out4[4]) {
    GUARD(h);
    dev::Status st;
    CK(cudaMemcpyAsync(&st, h->s.d_status, sizeof st, cudaMemcpyDeviceToHost, h->s.stream));
    CK(cudaStreamSynchronize(h->s.stream));
    out4[0] = (long long)st.restricted;
    out4[1] = (long long)st.nan_cells;
    out4[2] = (long long)st.farfield_oor;
    out4[3] = (long long)st.negative_dt;
    return 0;
}

extern "C" int fvgb_device_state(fvgb_handle* h, double** U_dev, int* n_cells) {
    if (!h) return fail(FVGB_ERR_ARG, "null handle");
    if (U_dev) *U_dev = reinterpret_cast<double*>(h->s.d_U);
    if (n_cells) *n_cells = h->s.N;
    return 0;
}

extern "C" int fvgb_cell_permutation(fvgb_handle* h, int* perm) {
    if (!h || !perm) return fail(FVGB_ERR_ARG, "null argument");
    std::copy(h->s.L.cell_new.begin(), h->s.L.cell_new.end(), perm);
    return 0;
}

extern "C" int fvgb_edge_permutation(fvgb_handle* h, int* perm) {
    if (!h || !perm) return fail(FVGB_ERR_ARG, "null argument");
    std::copy(h->s.L.edge_new.begin(), h->s.L.edge_new.end(), perm);
    return 0;
}

extern "C" int fvgb_edge_colours(fvgb_handle* h, int* colour, int* ncolours) {
    GUARD(h);
    if (!colour || !ncolours) return fail(FVGB_ERR_ARG, "null argument");
    Solver& s = h->s;
    const int E = s.E;
    std::fill(colour, colour + E, -1);
    *ncolours = 0;
    if (!s.p.edge_colour) return 0;
    // the colour lists as the device holds them, mapped back to the reference's edge numbering
    std::vector<int> ce(E);
    CK(cudaMemcpy(ce.data(), s.d_col_edge, sizeof(int) * (size_t)E, cudaMemcpyDeviceToHost));
    const int nc = (int)s.L.col_ptr.size() - 1;
    for (int k = 0; k < nc; k++)
        for (int i = s.L.col_ptr[k]; i < s.L.col_ptr[k + 1]; i++) {
            const int e = ce[i];
            if (e < 0 || e >= E) return fail(FVGB_ERR_CUDA, "device colour list holds an edge outside the mesh");
            colour[s.L.edge_ref[e]] = k;
        }
    *ncolours = nc;
    return 0;
}

extern "C" int fvgb_layout_connectivity(fvgb_handle* h, int* elem_edges, int* elem_neighbors, int* edge_L, int* edge_R) {
    GUARD(h);
    Solver& s = h->s;
    const int N = s.N, E = s.E;
    // read back what the device holds and map it to the reference numbering
    std::vector<int> ce((size_t)3 * N), cn((size_t)3 * N), nnb(N), eL(E), eR(E);
    CK(cudaMemcpy(ce.data(), s.d_c_edge, ce.size() * sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(cn.data(), s.d_c_nbr, cn.size() * sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(nnb.data(), s.d_c_nnb, nnb.size() * sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(eL.data(), s.d_e_L, eL.size() * sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(eR.data(), s.d_e_R, eR.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (int r = 0; r < N; r++) {
        const int c = s.L.cell_new[r];
        for (int j = 0; j < 3; j++) {
            const int v = ce[(size_t)c * 3 + j];
            if (elem_edges) elem_edges[(size_t)j * N + r] = s.L.edge_ref[v >= 0 ? v : ~v];
            const int q = cn[(size_t)c * 3 + j];
            if (elem_neighbors) elem_neighbors[(size_t)j * N + r] = (j < nnb[c] && q >= 0) ? s.L.cell_ref[q] : -1;
        }
    }
    for (int r = 0; r < E; r++) {
        const int i = s.L.edge_new[r];
        if (edge_L) edge_L[r] = s.L.cell_ref[eL[i]];
        if (edge_R) edge_R[r] = eR[i] < 0 ? -1 : s.L.cell_ref[eR[i]];
    }
    return 0;
}

extern "C" long long fvgb_kernel_launches(fvgb_handle* h) { return h ? h->s.launches : -1; }

extern "C" int fvgb_step_timed(fvgb_handle* h, double T, int nsteps, double* ms_out) {
    GUARD(h);
    if (!ms_out || nsteps < 0) return fail(FVGB_ERR_ARG, "bad timing arguments");
    Solver& s = h->s;
    int rc = s.build_graph();
    if (rc) return rc;
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaStreamSynchronize(s.stream));
    CK(cudaEventRecord(a, s.stream));
    rc = s.step_async(T, nsteps);
    CK(cudaEventRecord(b, s.stream));
    CK(cudaEventSynchronize(b));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *ms_out = ms;
    if (rc) return rc;
    return s.check_status();
}

extern "C" int fvgb_profile_steps(fvgb_handle* h, double T, int nsteps, double ms_out[5], int count_out[5]) {
    GUARD(h);
    if (!ms_out || !count_out || nsteps < 0) return fail(FVGB_ERR_ARG, "bad profiling arguments");
    return h->s.profile_steps(T, nsteps, ms_out, count_out);
}

extern "C" const char* fvgb_last_error(void) { return g_error.c_str(); }

extern "C" const char* fvgb_version(void) { return "fvgb 0.1 (sm_103a, FP64)"; }

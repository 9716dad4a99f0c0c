// Batched form: many independent flow instances (meshes of uneven size)
// packed into one device layout and advanced together, one persistent
// cooperative kernel per Runge-Kutta stage, the whole step captured in a CUDA
// graph.  No counterpart in the reference (it runs one mesh per process);
// every instance computes exactly what the single-mesh path computes
// (step_device.cuh), so a batched instance is bit-identical to the same
// instance stepped alone.
//
// Packing: instance i owns cells [coff_i, coff_i+1); all interior/periodic
// edges of all instances come first, then all boundary edges, so the flux
// phase is branch-uniform except at one seam.  Each instance keeps its own
// time, time step (a segmented minimum over its cells) and boundary states.
//
// Phases of one stage kernel (grid barrier between phases):
//   [first stage]  primitive variables + U0 copy | spectral radii per edge |
//                  per-instance minimum of CFL vol / alpha | t clamp per instance
//   gradient + limiter | edge fluxes | gather + stage update
//   [last stage]   positivity pass (one thread, rare)
// The grid barrier spins with an iteration limit: on time-out it raises an
// error word the host reads, and every block returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"
#include "layout.h"
#include "solver.h"
#include "step_device.cuh"
#include "batch_stage.cuh"

namespace fvgb {

namespace {

#define BK(call)                                                                                      \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return fail(FVGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

StageFn pick(int kind, int flux, bool linear, int grad, bool barth, bool ns) {
    switch (kind) {
    case dev::STAGE_EULER: return batch_stage_euler(flux, linear, grad, barth, ns);
    case dev::STAGE_RK3_1: return batch_stage_rk3_1(flux, linear, grad, barth, ns);
    case dev::STAGE_RK3_2: return batch_stage_rk3_2(flux, linear, grad, barth, ns);
    case dev::STAGE_RK3_3: return batch_stage_rk3_3(flux, linear, grad, barth, ns);
    case dev::STAGE_SSP_1: return batch_stage_ssp_1(flux, linear, grad, barth, ns);
    case dev::STAGE_SSP_2: return batch_stage_ssp_2(flux, linear, grad, barth, ns);
    default: return batch_stage_ssp_3(flux, linear, grad, barth, ns);
    }
}

}  // namespace

struct Batch {
    static constexpr int kFlagCap = 4096;
    int n = 0;
    fvgb_params p{};
    std::vector<fvgb_params> ps;
    std::vector<Layout> layouts;
    std::vector<int> coff, eoff_int, eoff_bnd;
    int N = 0, E = 0, E_int = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> owned;
    dev::Gas gas{};
    dev::BatchView bv{};
    dev::InstState* d_inst = nullptr;
    dev::InstState* h_inst = nullptr;
    dev::GridBarrier* d_bar = nullptr;
    cudaGraphExec_t graph = nullptr;
    bool use_graph = true;
    int block = 256, grid = 0;
    long long launches = 0;
    std::vector<int> kinds;
    std::string tune_report;

    ~Batch() {
        if (graph) cudaGraphExecDestroy(graph);
        if (h_inst) cudaFreeHost(h_inst);
        for (void* q : owned) cudaFree(q);
        if (stream) cudaStreamDestroy(stream);
    }

    template <class T>
    int alloc(T*& ptr, size_t count) {
        ptr = nullptr;
        if (count == 0) count = 1;
        BK(cudaMalloc((void**)&ptr, count * sizeof(T)));
        owned.push_back((void*)ptr);
        return 0;
    }
    template <class T>
    int upload(T*& ptr, const std::vector<T>& v) {
        int rc = alloc(ptr, v.size());
        if (rc) return rc;
        if (!v.empty()) BK(cudaMemcpyAsync(ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, stream));
        return 0;
    }

    StageFn fn(int kind) const {
        return pick(kind, p.flux_scheme, p.reconstruct == 3002, p.gradient, p.limiter == 1, p.equation == 2);
    }

    int launch(int kind) {
        StageFn f = fn(kind);
        dev::Gas g = gas;
        dev::BatchView v = bv;
        void* args[] = {&v, &g};
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(block);
        cfg.stream = stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        BK(cudaLaunchKernelExC(&cfg, (const void*)f, args));
        launches += 1;
        return 0;
    }

    // grid = SMs x resident blocks of the largest stage kernel
    int size_grid() {
        int dev = 0, sms = 0;
        BK(cudaGetDevice(&dev));
        BK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        int per_sm = 1 << 30;
        for (int k : kinds) {
            int b = 0;
            BK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn(k), block, 0));
            per_sm = std::min(per_sm, b);
        }
        if (per_sm <= 0) return fail(FVGB_ERR_CUDA, "batched stage kernel does not fit on an SM");
        grid = sms * per_sm;
        return 0;
    }

    int capture() {
        if (graph) {
            cudaGraphExecDestroy(graph);
            graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        const long long before = launches;
        BK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        int rc = 0;
        for (int k : kinds)
            if (!rc) rc = launch(k);
        cudaError_t e = cudaStreamEndCapture(stream, &g);
        launches = before;
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return fail(FVGB_ERR_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(FVGB_ERR_CUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(e));
        return 0;
    }

    int check() {
        dev::Status st;
        unsigned int berr = 0;
        BK(cudaMemcpyAsync(&st, bv.status, sizeof st, cudaMemcpyDeviceToHost, stream));
        BK(cudaMemcpyAsync(&berr, &d_bar->error, sizeof berr, cudaMemcpyDeviceToHost, stream));
        BK(cudaStreamSynchronize(stream));
        if (berr) return fail(FVGB_ERR_TIMEOUT, "batched stage kernel: a grid barrier wait gave up");
        if (st.nan_cells) return fail(FVGB_ERR_NAN, "NaN in a batched instance");
        if (st.negative_dt) return fail(FVGB_ERR_RANGE, "rho or p < 0 in a batched instance's time step");
        if (st.farfield_oor) return fail(FVGB_ERR_RANGE, "far-field ghost out of range in a batched instance");
        return 0;
    }

    int step_async(int nsteps) {
        if (!graph && use_graph) {
            if (capture()) {
                // this driver cannot capture cooperative launches: launch stage by stage
                use_graph = false;
                cudaGetLastError();
            }
        }
        if (use_graph) {
            for (int i = 0; i < nsteps; i++) BK(cudaGraphLaunch(graph, stream));
            launches += (long long)kinds.size() * nsteps;
        } else {
            for (int i = 0; i < nsteps; i++)
                for (int k : kinds) {
                    int rc = launch(k);
                    if (rc) return rc;
                }
        }
        return 0;
    }

    int set_times(const double* t, const double* T) {
        BK(cudaMemcpyAsync(h_inst, d_inst, sizeof(dev::InstState) * n, cudaMemcpyDeviceToHost, stream));
        BK(cudaStreamSynchronize(stream));
        for (int i = 0; i < n; i++) {
            if (t) h_inst[i].t = t[i];
            if (T) h_inst[i].T = T[i];
        }
        BK(cudaMemcpyAsync(d_inst, h_inst, sizeof(dev::InstState) * n, cudaMemcpyHostToDevice, stream));
        return 0;
    }

    int get_times(double* t) {
        BK(cudaMemcpyAsync(h_inst, d_inst, sizeof(dev::InstState) * n, cudaMemcpyDeviceToHost, stream));
        BK(cudaStreamSynchronize(stream));
        for (int i = 0; i < n; i++) t[i] = h_inst[i].t;
        return 0;
    }

    // the project's own autotuner: block size x tile size x schedule, timed on this batch
    int tune(int trial_steps) {
        struct Cand { int block, tile_mult, dynamic; };
        const Cand cands[] = {{256, 1, 0}, {256, 4, 0}, {256, 16, 0}, {256, 4, 1}, {256, 16, 1},
                              {128, 1, 0}, {128, 8, 0}, {128, 8, 1}, {128, 32, 1}};
        // keep the state: tuning steps run on a copy
        d4* save = nullptr;
        int rc = alloc(save, (size_t)N);
        if (rc) return rc;
        std::vector<dev::InstState> inst0(n);
        BK(cudaMemcpyAsync(save, bv.U, sizeof(d4) * N, cudaMemcpyDeviceToDevice, stream));
        BK(cudaMemcpyAsync(inst0.data(), d_inst, sizeof(dev::InstState) * n, cudaMemcpyDeviceToHost, stream));
        BK(cudaStreamSynchronize(stream));
        double best = 1e300;
        Cand bestc = cands[0];
        tune_report.clear();
        cudaEvent_t a, b;
        BK(cudaEventCreate(&a));
        BK(cudaEventCreate(&b));
        for (const Cand& c : cands) {
            block = c.block;
            bv.tile = c.block * c.tile_mult;
            bv.dynamic = c.dynamic;
            if ((rc = size_grid())) return rc;
            if (graph) {
                cudaGraphExecDestroy(graph);
                graph = nullptr;
            }
            if ((rc = step_async(1))) return rc;  // warm-up (captures the graph)
            BK(cudaEventRecord(a, stream));
            if ((rc = step_async(trial_steps))) return rc;
            BK(cudaEventRecord(b, stream));
            BK(cudaEventSynchronize(b));
            float ms = 0;
            BK(cudaEventElapsedTime(&ms, a, b));
            if ((rc = check())) return rc;
            char line[160];
            std::snprintf(line, sizeof line, "block %d tile %d %s grid %d: %.3f ms/step\n", c.block,
                          c.block * c.tile_mult, c.dynamic ? "dynamic" : "static", grid, ms / trial_steps);
            tune_report += line;
            if (ms < best) {
                best = ms;
                bestc = c;
            }
            BK(cudaMemcpyAsync(bv.U, save, sizeof(d4) * N, cudaMemcpyDeviceToDevice, stream));
            BK(cudaMemcpyAsync(d_inst, inst0.data(), sizeof(dev::InstState) * n, cudaMemcpyHostToDevice, stream));
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        block = bestc.block;
        bv.tile = bestc.block * bestc.tile_mult;
        bv.dynamic = bestc.dynamic;
        if ((rc = size_grid())) return rc;
        if (graph) {
            cudaGraphExecDestroy(graph);
            graph = nullptr;
        }
        char line[160];
        std::snprintf(line, sizeof line, "chosen: block %d tile %d %s\n", block, bv.tile, bv.dynamic ? "dynamic" : "static");
        tune_report += line;
        BK(cudaStreamSynchronize(stream));
        return 0;
    }

    int init(int count, const fvgb_mesh_soa* const* meshes, const fvgb_params* params) {
        n = count;
        if (n <= 0) return fail(FVGB_ERR_ARG, "empty batch");
        p = params[0];
        ps.assign(params, params + n);
        for (int i = 0; i < n; i++) {
            const fvgb_params& q = params[i];
            if (q.equation != p.equation || q.flux_scheme != p.flux_scheme || q.reconstruct != p.reconstruct ||
                q.gradient != p.gradient || q.limiter != p.limiter || q.time_advance != p.time_advance ||
                q.gamma != p.gamma || q.R != p.R || q.lsq_det_ref != p.lsq_det_ref || q.wall_bc_ref != p.wall_bc_ref ||
                q.restrict_ref != p.restrict_ref)
                return fail(FVGB_ERR_ARG, "batched instances must share the scheme and the gas constants");
        }
        if (p.equation == 2)  // one Gas for the launch: the viscosity law and Pr are shared too
            for (int i = 0; i < n; i++)
                if (params[i].mu0 != p.mu0 || params[i].T0 != p.T0 || params[i].Pr != p.Pr)
                    return fail(FVGB_ERR_ARG, "batched Navier-Stokes instances must share mu0, T0 and Pr");
        for (int i = 0; i < n; i++) {
            if (params[i].steady)
                return fail(FVGB_ERR_UNSUPPORTED, "the batched form steps in time (time.is_steady = 0)");
            if (params[i].edge_colour)
                return fail(FVGB_ERR_UNSUPPORTED, "the batched form gathers the residual ([gpu] edge_colour = 0)");
        }
        if (p.time_advance != 3101 && p.time_advance != 3103 && p.time_advance != 3104)
            return fail(FVGB_ERR_ARG, "invalid time_advance");
        BK(cudaSetDevice(p.device));
        BK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        gas = make_gas(p);
        layouts.resize(n);
        coff.assign(n + 1, 0);
        eoff_int.assign(n + 1, 0);
        eoff_bnd.assign(n + 1, 0);
        for (int i = 0; i < n; i++) {
            fvgb_params q = params[i];
            int rc = build_layout(*meshes[i], q, layouts[i]);
            if (rc) return rc;
            const Layout& L = layouts[i];
            coff[i + 1] = coff[i] + L.N;
            eoff_int[i + 1] = eoff_int[i] + L.E_int;
            eoff_bnd[i + 1] = eoff_bnd[i] + (L.E - L.E_int);
        }
        N = coff[n];
        E_int = eoff_int[n];
        E = E_int + eoff_bnd[n];
        // packed arrays
        std::vector<int> eL(E), eR(E), ebc(E), einst(E), cedge((size_t)3 * N), cnbr((size_t)3 * N), cnnb(N), cinst(N);
        std::vector<double> geom((size_t)8 * E), mvol(N), vol(N), lsq((size_t)6 * N), vtx((size_t)6 * N);
        std::vector<double> gg(p.gradient == 2 ? (size_t)12 * N : 0), ginv(p.gradient == 2 ? N : 0);
        std::vector<int> ggout(p.gradient == 2 ? (size_t)3 * N : 0);
        std::vector<int> dtptr((size_t)N + 1, 0), dtedge, key(N), dev_of_key(N);
        auto gedge = [&](int i, int e) {  // instance-local edge -> packed edge
            const Layout& L = layouts[i];
            return e < L.E_int ? eoff_int[i] + e : E_int + eoff_bnd[i] + (e - L.E_int);
        };
        for (int i = 0; i < n; i++) {
            const Layout& L = layouts[i];
            const int c0 = coff[i];
            for (int e = 0; e < L.E; e++) {
                const int ge = gedge(i, e);
                eL[ge] = c0 + L.e_L[e];
                eR[ge] = L.e_R[e] < 0 ? -1 : c0 + L.e_R[e];
                ebc[ge] = L.e_bc[e];
                einst[ge] = i;
                std::memcpy(&geom[(size_t)ge * 8], &L.e_geom[(size_t)e * 8], 8 * sizeof(double));
                geom[(size_t)ge * 8 + 3] = std::sqrt(geom[(size_t)ge * 8 + 2]);
            }
            for (int c = 0; c < L.N; c++) {
                const int gc = c0 + c;
                cinst[gc] = i;
                cnnb[gc] = L.c_nnb[c];
                mvol[gc] = L.c_mvol[c];
                vol[gc] = L.c_vol[c];
                for (int j = 0; j < 3; j++) {
                    const int r = L.c_edge[(size_t)c * 3 + j];
                    const int ge = gedge(i, r >= 0 ? r : ~r);
                    cedge[(size_t)gc * 3 + j] = r >= 0 ? ge : ~ge;
                    const int q = L.c_nbr[(size_t)c * 3 + j];
                    cnbr[(size_t)gc * 3 + j] = q < 0 ? -1 : c0 + q;
                    if (p.gradient == 2) {
                        const int o = L.c_ggout[(size_t)c * 3 + j];
                        ggout[(size_t)gc * 3 + j] = o < 0 ? -1 : c0 + o;
                    }
                }
                std::memcpy(&lsq[(size_t)gc * 6], &L.c_lsq[(size_t)c * 6], 6 * sizeof(double));
                std::memcpy(&vtx[(size_t)gc * 6], &L.c_vtx[(size_t)c * 6], 6 * sizeof(double));
                if (p.gradient == 2) {
                    std::memcpy(&gg[(size_t)gc * 12], &L.c_gg[(size_t)c * 12], 12 * sizeof(double));
                    ginv[gc] = L.c_ginv[c];
                }
                dtptr[gc + 1] = dtptr[gc] + (L.dt_ptr[c + 1] - L.dt_ptr[c]);
                for (int k = L.dt_ptr[c]; k < L.dt_ptr[c + 1]; k++) dtedge.push_back(gedge(i, L.dt_edge[k]));
                key[gc] = c0 + L.cell_ref[c];  // instance-major, reference order within
            }
        }
        for (int c = 0; c < N; c++) dev_of_key[key[c]] = c;
        int rc;
        int *d_eL, *d_eR, *d_ebc, *d_einst, *d_cedge, *d_cnbr, *d_cnnb, *d_cinst, *d_dtptr, *d_dtedge, *d_key, *d_dok;
        int* d_ggout = nullptr;
        double *d_geom, *d_mvol, *d_vol, *d_lsq, *d_vtx, *d_gg = nullptr, *d_ginv = nullptr;
        if ((rc = upload(d_eL, eL)) || (rc = upload(d_eR, eR)) || (rc = upload(d_ebc, ebc)) ||
            (rc = upload(d_einst, einst)) || (rc = upload(d_cedge, cedge)) || (rc = upload(d_cnbr, cnbr)) ||
            (rc = upload(d_cnnb, cnnb)) || (rc = upload(d_cinst, cinst)) || (rc = upload(d_dtptr, dtptr)) ||
            (rc = upload(d_dtedge, dtedge)) || (rc = upload(d_key, key)) || (rc = upload(d_dok, dev_of_key)) ||
            (rc = upload(d_geom, geom)) || (rc = upload(d_mvol, mvol)) || (rc = upload(d_vol, vol)) ||
            (rc = upload(d_lsq, lsq)) || (rc = upload(d_vtx, vtx)))
            return rc;
        if (p.gradient == 2 && ((rc = upload(d_gg, gg)) || (rc = upload(d_ginv, ginv)) || (rc = upload(d_ggout, ggout))))
            return rc;
        dev::MeshView& m = bv.m;
        m.N = N;
        m.E = E;
        m.E_int = E_int;
        m.e_L = d_eL;
        m.e_R = d_eR;
        m.e_bc = d_ebc;
        m.e_geom = d_geom;
        m.c_edge = d_cedge;
        m.c_nbr = d_cnbr;
        m.c_nnb = d_cnnb;
        m.c_mvol = d_mvol;
        m.c_vol = d_vol;
        m.c_lsq = d_lsq;
        m.c_vtx = d_vtx;
        m.c_gg = d_gg;
        m.c_ggout = d_ggout;
        m.c_ginv = d_ginv;
        m.dt_ptr = d_dtptr;
        m.dt_edge = d_dtedge;
        bv.n_inst = n;
        bv.c_inst = d_cinst;
        bv.e_inst = d_einst;
        bv.cell_key = d_key;
        bv.dev_of_key = d_dok;
        if ((rc = alloc(bv.U, N)) || (rc = alloc(bv.U0, N)) || (rc = alloc(bv.Gx, N)) || (rc = alloc(bv.Gy, N)) ||
            (rc = alloc(bv.F, E)) || (rc = alloc(bv.prim, N)) || (rc = alloc(bv.rhs, N)) || (rc = alloc(bv.alpha, E)) ||
            (rc = alloc(bv.alpha_vis, E)) || (rc = alloc(bv.flags, kFlagCap)) || (rc = alloc(bv.flag_count, 1)) ||
            (rc = alloc(bv.status, 1)) || (rc = alloc(d_bar, 1)) || (rc = alloc(d_inst, n)))
            return rc;
        if (p.time_advance == 3103) {
            if ((rc = alloc(bv.K1, N))) return rc;
        } else {
            bv.K1 = bv.U0;
        }
        bv.inst = d_inst;
        {  // boundary data per instance; the double-Mach-reflection clock is the instance's
            std::vector<dev::BcData> bcs(n);
            for (int i = 0; i < n; i++) {
                bcs[i] = make_bc(params[i]);
                bcs[i].clock_t0 = &d_inst[i].t_old;
                bcs[i].clock_dt = &d_inst[i].dt;
            }
            dev::BcData* d_bc;
            if ((rc = upload(d_bc, bcs))) return rc;
            bv.bc = d_bc;
        }
        bv.flag_cap = kFlagCap;
        bv.bar = d_bar;
        bv.tile = 256;
        bv.dynamic = 0;
        bv.restrict_ref = p.restrict_ref;
        bv.value_1 = std::max(4.0 / 3.0, p.gamma / p.Pr);
        BK(cudaMemsetAsync(bv.flag_count, 0, sizeof(unsigned int), stream));
        BK(cudaMemsetAsync(bv.status, 0, sizeof(dev::Status), stream));
        BK(cudaMemsetAsync(d_bar, 0, sizeof(dev::GridBarrier), stream));
        BK(cudaMemsetAsync(bv.Gx, 0, sizeof(d4) * N, stream));
        BK(cudaMemsetAsync(bv.Gy, 0, sizeof(d4) * N, stream));
        BK(cudaMallocHost((void**)&h_inst, sizeof(dev::InstState) * n));
        for (int i = 0; i < n; i++) {
            dev::InstState s{};
            s.T = params[i].T_end;
            s.CFL = params[i].CFL;
            const double big = 1e10;
            std::memcpy(&s.dtmin_bits, &big, sizeof big);
            h_inst[i] = s;
        }
        BK(cudaMemcpyAsync(d_inst, h_inst, sizeof(dev::InstState) * n, cudaMemcpyHostToDevice, stream));
        kinds.clear();
        if (p.time_advance == 3101) kinds = {dev::STAGE_EULER};
        else if (p.time_advance == 3103) kinds = {dev::STAGE_RK3_1, dev::STAGE_RK3_2, dev::STAGE_RK3_3};
        else kinds = {dev::STAGE_SSP_1, dev::STAGE_SSP_2, dev::STAGE_SSP_3};
        if ((rc = size_grid())) return rc;
        // initial fields
        for (int i = 0; i < n; i++) {
            if (params[i].ic_type < 1 || params[i].ic_type > 4) continue;
            std::vector<double> U0((size_t)4 * layouts[i].N);
            if ((rc = initial_field(*meshes[i], params[i], U0.data()))) return rc;
            if ((rc = set_state(i, U0.data()))) return rc;
        }
        BK(cudaStreamSynchronize(stream));
        return 0;
    }

    int set_state(int i, const double* U) {
        if (i < 0 || i >= n) return fail(FVGB_ERR_ARG, "instance index out of range");
        const Layout& L = layouts[i];
        std::vector<d4> tmp(L.N);
        for (int r = 0; r < L.N; r++)
            tmp[L.cell_new[r]] = mk4(U[r], U[(size_t)L.N + r], U[2 * (size_t)L.N + r], U[3 * (size_t)L.N + r]);
        BK(cudaMemcpyAsync(bv.U + coff[i], tmp.data(), sizeof(d4) * L.N, cudaMemcpyHostToDevice, stream));
        BK(cudaStreamSynchronize(stream));
        return 0;
    }

    int get_state(int i, double* U) {
        if (i < 0 || i >= n) return fail(FVGB_ERR_ARG, "instance index out of range");
        const Layout& L = layouts[i];
        std::vector<d4> tmp(L.N);
        BK(cudaMemcpyAsync(tmp.data(), bv.U + coff[i], sizeof(d4) * L.N, cudaMemcpyDeviceToHost, stream));
        BK(cudaStreamSynchronize(stream));
        for (int r = 0; r < L.N; r++) {
            const d4 u = tmp[L.cell_new[r]];
            U[r] = u.x;
            U[(size_t)L.N + r] = u.y;
            U[2 * (size_t)L.N + r] = u.z;
            U[3 * (size_t)L.N + r] = u.w;
        }
        return 0;
    }
};

}  // namespace fvgb

using namespace fvgb;

struct fvgb_batch {
    Batch b;
};

extern "C" int fvgb_batch_create(int n, const fvgb_mesh_soa* const* meshes, const fvgb_params* params,
                                 fvgb_batch** out) {
    if (!meshes || !params || !out || n <= 0) return fail(FVGB_ERR_ARG, "bad batch arguments");
    *out = nullptr;
    fvgb_batch* h = new fvgb_batch();
    int rc = h->b.init(n, meshes, params);
    if (rc) {
        delete h;
        return rc;
    }
    *out = h;
    return 0;
}

extern "C" void fvgb_batch_destroy(fvgb_batch* h) { delete h; }

extern "C" int fvgb_batch_set_state(fvgb_batch* h, int i, const double* U) {
    if (!h || !U) return fail(FVGB_ERR_ARG, "null argument");
    return h->b.set_state(i, U);
}

extern "C" int fvgb_batch_get_state(fvgb_batch* h, int i, double* U) {
    if (!h || !U) return fail(FVGB_ERR_ARG, "null argument");
    return h->b.get_state(i, U);
}

extern "C" int fvgb_batch_step(fvgb_batch* h, double* t, const double* T, int nsteps) {
    if (!h || !t || nsteps < 0) return fail(FVGB_ERR_ARG, "bad arguments");
    int rc = h->b.set_times(t, T);
    if (rc) return rc;
    if ((rc = h->b.step_async(nsteps))) return rc;
    if ((rc = h->b.get_times(t))) return rc;
    return h->b.check();
}

extern "C" int fvgb_batch_step_timed(fvgb_batch* h, int nsteps, double* ms_out) {
    if (!h || !ms_out || nsteps < 0) return fail(FVGB_ERR_ARG, "bad arguments");
    Batch& b = h->b;
    cudaEvent_t a, e;
    BK(cudaEventCreate(&a));
    BK(cudaEventCreate(&e));
    if (b.use_graph && !b.graph) {
        int rc0 = b.step_async(0);  // captures the graph outside the timed region
        if (rc0) return rc0;
    }
    BK(cudaEventRecord(a, b.stream));
    int rc = b.step_async(nsteps);
    BK(cudaEventRecord(e, b.stream));
    BK(cudaEventSynchronize(e));
    float ms = 0;
    BK(cudaEventElapsedTime(&ms, a, e));
    cudaEventDestroy(a);
    cudaEventDestroy(e);
    *ms_out = ms;
    if (rc) return rc;
    return b.check();
}

extern "C" int fvgb_batch_tune(fvgb_batch* h, int trial_steps, char* report, int report_len) {
    if (!h || trial_steps <= 0) return fail(FVGB_ERR_ARG, "bad arguments");
    int rc = h->b.tune(trial_steps);
    if (report && report_len > 0) std::snprintf(report, (size_t)report_len, "%s", h->b.tune_report.c_str());
    return rc;
}

extern "C" int fvgb_batch_info(fvgb_batch* h, long long out[8]) {
    if (!h || !out) return fail(FVGB_ERR_ARG, "null argument");
    out[0] = h->b.n;
    out[1] = h->b.N;
    out[2] = h->b.E;
    out[3] = h->b.grid;
    out[4] = h->b.block;
    out[5] = h->b.launches;
    out[6] = h->b.bv.tile * (h->b.bv.dynamic ? -1 : 1);
    out[7] = h->b.use_graph ? 1 : 0;
    return 0;
}

// ---- the bounded barrier's give-up path, exercised without a fault ---------------
namespace fvgb {
namespace dev {
// every block but `absent` meets at grid_sync with the given poll limit; `absent`
// returns at once, so with absent >= 0 the others must give up and set the error word
__global__ void k_barrier_probe(GridBarrier* b, long long limit, int absent, int* passed) {
    if ((int)blockIdx.x == absent) return;
    const bool ok = grid_sync(b, limit);
    if (threadIdx.x == 0 && ok) atomicAdd(passed, 1);
}
}  // namespace dev
}  // namespace fvgb

extern "C" int fvgb_barrier_selftest(int device, int blocks, int absent_block, long long spin_limit, int* timed_out,
                                     int* blocks_passed) {
    using namespace fvgb;
    if (!timed_out || blocks <= 0 || blocks > 64 || spin_limit <= 0 || absent_block >= blocks)
        return fail(FVGB_ERR_ARG, "bad arguments");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(FVGB_ERR_NO_DEVICE, "no CUDA device");
    BK(cudaSetDevice(device));
    dev::GridBarrier* bar = nullptr;
    int* passed = nullptr;
    BK(cudaMalloc(&bar, sizeof(dev::GridBarrier)));
    if (cudaMalloc(&passed, sizeof(int)) != cudaSuccess) {
        cudaFree(bar);
        return fail(FVGB_ERR_CUDA, "cudaMalloc failed");
    }
    cudaMemset(bar, 0, sizeof(dev::GridBarrier));
    cudaMemset(passed, 0, sizeof(int));
    // a handful of 32-thread blocks: all resident at once
    dev::k_barrier_probe<<<blocks, 32>>>(bar, spin_limit, absent_block, passed);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    dev::GridBarrier hb{};
    int hp = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&hb, bar, sizeof hb, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&hp, passed, sizeof hp, cudaMemcpyDeviceToHost);
    cudaFree(bar);
    cudaFree(passed);
    if (e != cudaSuccess) return fail(FVGB_ERR_CUDA, std::string("barrier probe: ") + cudaGetErrorString(e));
    *timed_out = hb.error ? 1 : 0;
    if (blocks_passed) *blocks_passed = hp;
    return 0;
}

// One solver instance on one GPU (solver.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "internal.h"
#include "layout.h"
#include "step_kernels.cuh"

namespace fvgb {

dev::Gas make_gas(const fvgb_params& p);
dev::BcData make_bc(const fvgb_params& p);

struct Solver {
    static constexpr int kFlagCap = 4096;

    fvgb_params p{};
    Layout L;
    int N = 0, E = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph_exec = nullptr;        // one step
    cudaGraphExec_t graph_exec_multi = nullptr;  // kGraphSteps steps in one graph
    static constexpr int kGraphSteps = 8;
    std::vector<void*> owned;
    dev::Gas gas{};
    dev::BcData bc{};
    dev::MeshView mv{};
    long long launches = 0, launches_per_step = 0;
    dev::Status seen{};
    int adj_overlap = 1;  // fvgb_adjoint_overlap: recompute beside the reverse sweep where memory allows

    // layout
    int *d_e_L = nullptr, *d_e_R = nullptr, *d_e_bc = nullptr;
    double* d_e_geom = nullptr;
    int *d_c_edge = nullptr, *d_c_nbr = nullptr, *d_c_nnb = nullptr;
    double *d_c_mvol = nullptr, *d_c_vol = nullptr, *d_c_lsq = nullptr, *d_c_vtx = nullptr;
    double *d_c_gg = nullptr, *d_c_ginv = nullptr;
    int* d_c_ggout = nullptr;
    int *d_dt_ptr = nullptr, *d_dt_edge = nullptr;
    int *d_cell_ref = nullptr, *d_cell_new = nullptr;
    int *d_col_edge = nullptr, *d_e_in_r = nullptr;  // the edge colouring ([gpu] edge_colour = 1)
    // fields
    d4 *d_U = nullptr, *d_U0 = nullptr, *d_K1 = nullptr, *d_Gx = nullptr, *d_Gy = nullptr;
    d4 *d_F = nullptr, *d_prim = nullptr, *d_rhs = nullptr, *d_res_part = nullptr;
    d4* d_rec_R = nullptr;  // when set, the update kernels also write each stage's residual here
    dev::EdgeTape rec_tape;  // when set (.v), the flux kernels also write the adjoint's edge tape
    dev::CellTape rec_ctape;  // when set (.gx), the gradient kernel also writes the limiter record
    double *d_alpha = nullptr, *d_alpha_vis = nullptr, *d_stage = nullptr, *d_res_out = nullptr;
    double* d_dt_local = nullptr;  // per-cell dt of a steady run (time.is_steady = 1)
    int cell0_dev = 0;             // device index of the reference's cell 0 (its dt moves t in steady runs)
    int* d_flags = nullptr;
    unsigned int* d_flag_count = nullptr;
    dev::StepState* d_state = nullptr;
    dev::StepState* h_state = nullptr;
    dev::Status* d_status = nullptr;

    // what the output functions need (output.cu), in reference numbering: node
    // coordinates, the cells' nodes, and per boundary set its edges in set order
    struct OutputMesh {
        int V = 0, NB = 0;
        std::vector<double> node_xy;                 // 2V
        std::vector<int> elem_nodes;                 // 3N
        std::vector<int> set_off;                    // NB+1
        std::vector<int> set_n0, set_n1;             // per set edge: its two nodes
        std::vector<double> set_nx, set_ny, set_len;  // per set edge: normal and length
        std::vector<int> set_type;
        std::vector<std::string> set_name;
    } om;
    struct OutputState* out = nullptr;  // device node lists and buffers, made on first use
    int keep_output_mesh(const fvgb_mesh_soa& m);
    void release_output();

    // kernel groups timed by profile_steps()
    enum { PROF_DT = 0, PROF_GRAD = 1, PROF_FLUX = 2, PROF_UPDATE = 3, PROF_RESTRICT = 4, PROF_NCLASS = 5 };
    struct Prof {
        struct Pair { int cls; cudaEvent_t a, b; };
        cudaEvent_t open[PROF_NCLASS] = {};
        std::vector<Pair> pairs;
    };
    Prof* prof = nullptr;

    ~Solver();
    int init(const fvgb_mesh_soa& m, const fvgb_params& prm);
    void mark(int cls, bool begin);
    int profile_steps(double T, int nsteps, double* ms, int* count);
    bool needs_gradient() const;
    void enqueue_stage(int kind);
    void enqueue_residual(const dev::BcData& b, int kind);
    void enqueue_step();
    int build_graph();
    void drop_graphs();
    int check_status();
    int step_async(double T, int nsteps);
    int set_time(double t);
    int get_time(double* t, double* dt);
    int set_state(const double* U);
    int get_state(double* U);
    int rhs(const double* U, double* R, double* gx, double* gy);
    int dt(double* out);
    int residual(int norm, double* out);
};

}  // namespace fvgb

// the C ABI's opaque handle: one solver
struct fvgb_handle {
    fvgb::Solver s;
};


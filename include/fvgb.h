/* fvgb.h -- C ABI of the GB300 explicit finite-volume step (FP64, one GPU).
 *
 * This library replaces the reference's per-step path of FVMR
 * (OliveTIen/CFD_Solver_2D_GPU).  The reference has no plugin system; its
 * boundary is internal C++ (cited per entry point below).  Conventions:
 *   - every function returns 0 on success or a negative fvgb_status code and
 *     never exits the process (the reference calls exit(), e.g.
 *     FVMR/src/solvers/GPUSolver2.cpp:296-303, FVMR/src/gpu/GPUGlobalFunction.cu:18-34);
 *   - host arrays are in the reference's numbering and its [var][index] SoA
 *     layout (U[4][N] is 4 rows of N doubles);
 *   - one handle = one GPU, one CUDA stream, all device memory owned by the
 *     handle; a handle is used from one host thread at a time, and different
 *     handles may be used from different threads at once (the error message
 *     of fvgb_last_error is per thread).
 */
#ifndef FVGB_H
#define FVGB_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef enum fvgb_status {
    FVGB_OK = 0,
    FVGB_ERR_ARG = -1,       /* invalid argument or size */
    FVGB_ERR_IO = -2,        /* file cannot be read or written */
    FVGB_ERR_FORMAT = -3,    /* malformed .su2 / input.toml */
    FVGB_ERR_MESH = -4,      /* inconsistent mesh (periodic pairs, unknown boundary name, ...) */
    FVGB_ERR_CUDA = -5,      /* CUDA runtime error (message in fvgb_last_error) */
    FVGB_ERR_NAN = -6,       /* NaN in the state (the reference exits here: Restrict.cpp:26-29) */
    FVGB_ERR_RANGE = -7,     /* negative rho or p in the time-step (CalculateDt.cpp:41-44) or far-field state out of range (Flux.cpp:157-160) */
    FVGB_ERR_UNSUPPORTED = -8,/* option outside this path (e.g. double-Mach-reflection boundary) */
    FVGB_ERR_TIMEOUT = -9,   /* a bounded device wait gave up */
    FVGB_ERR_NO_DEVICE = -10
} fvgb_status;

/* The GlobalPara subset the step reads (FVMR/src/global/GlobalPara.cpp:4-90;
 * keys of input.toml per FVMR/src/input/TomlFileManager.cpp:110-170) plus
 * this library's mode switches. */
typedef struct fvgb_params {
    int equation;        /* physicsModel.equation: 1 Euler, 2 Navier-Stokes */
    int flux_scheme;     /* inviscid_flux_method.flux_conservation_scheme: 2001 LLF, 2002 Roe */
    int reconstruct;     /* inviscid_flux_method.flag_reconstruct: 3001 constant, 3002 linear */
    int gradient;        /* inviscid_flux_method.flag_gradient: 1 least squares, 2 Green-Gauss */
    int limiter;         /* inviscid_flux_method.flux_limiter: 0 none, 1 Barth */
    int time_advance;    /* time.time_advance: 3101 Euler, 3103 Kutta RK3, 3104 SSP-RK3 */
    int lsq_det_ref;     /* [gpu] lsq_det = "ref" (1) keeps MatrixKernel.h:48-49, "fixed" (0) corrects it */
    int wall_bc_ref;     /* [gpu] wall_bc = "ref" (1) keeps Flux.cpp:73-79, "mirror" (0) mirrors the velocity */
    int restrict_ref;    /* [gpu] restrict = "ref" (1) keeps Restrict.cpp:52, "fixed" (0) corrects it */
    int ic_type;         /* initialCondition.type: 1 uniform, 2 isentropic vortex, 3 shock tube,
                            4 double Mach reflection */
    int renumber;        /* [gpu] renumber: 0 keep the file order, 1 Morton order of cells and edges */
    int device;          /* CUDA device ordinal */
    double gamma, R, Pr, mu0, T0, CFL, T_end, Re;
    double inf[4], inlet[4], outlet[4];   /* rho, u, v, p */
    double vortex[3];    /* x, y, strength */
    double shock[4];     /* shock tube: x, y, normal x, normal y (defaults 0, 0, 1, 0) */
    double mesh_scale;   /* constant.mesh_scale_factor */
    int max_iteration;   /* output.maxIteration */
    /* [gpu] edge_colour = 1: the residual is scattered by edge colour (each colour's edges
     * add their fluxes into the cells' sums; no two edges of a colour share a cell) instead
     * of gathered per cell in the reference's slot order; the sums then run in colour order.
     * Plain path only (the batched form and the adjoint refuse it).  Default 0. */
    int edge_colour;
    double ref_area;     /* constant.referenceArea x mesh_scale_factor (TomlFileManager.cpp:128-131) */
    /* double Mach reflection (initialCondition.doubleShockReflection, FieldInitializer.cpp:93-108):
     * where the shock meets the wall (x, y) and its angle in degrees, [0, 90] */
    double dsr[3];
    /* the time at which fvgb_rhs_noalloc evaluates "dsr" boundary edges (it has no clock of its
     * own; the reference reads CBoundaryDoubleShockReflect's t + dt there, Flux.cpp:328-332).
     * The handle-based entry points keep their own clock and ignore it. */
    double dsr_time;
    /* time.is_steady = 1: local time stepping, each cell advanced by its own
     * CFL vol / alpha (CIteration.cpp:42-52, CalculateDt.cpp:66-72, 182-186,
     * Evolve.cpp:115-125); forward Euler, T is not a bound.  The step uses
     * time.CFL (default 0.6) as the reference does; time.CFL_steady is read into
     * CFL_steady (TomlFileManager.cpp:159-160) and not used by the step. */
    int steady;
    int pad2_;
    double CFL_steady;
} fvgb_params;

/* Reference-order mesh arrays, mirroring GPU::NodeSoA / ElementSoA / EdgeSoA /
 * BoundarySetMap (FVMR/src/gpu/datatype/*.h) as filled by
 * U2NITS::OldDataConverter (FVMR/src/solvers/OldDataConverter.cpp:35-195). */
typedef struct fvgb_mesh_soa {
    int num_node, num_element, num_edge, num_boundary;
    const double* node_xy;        /* [2][V] */
    const int* elem_nodes;        /* [4][N], slot 3 = -1 */
    const int* elem_edges;        /* [4][N], slot 3 = -1 */
    const int* elem_neighbors;    /* [4][N], -1 = none (periodic faces too) */
    const double* elem_xy;        /* [2][N] */
    const double* elem_volume;    /* [N] */
    const int* edge_nodes;        /* [2][E] */
    const int* edge_L;            /* [E] */
    const int* edge_R;            /* [E] (periodic: partner's L; boundary: -1) */
    const int* edge_setID;        /* [E] 1-based boundary set, -1 interior */
    const int* edge_periodicPair; /* [E] */
    const double* edge_length;    /* [E] */
    const double* edge_distance;  /* [E] */
    const double* edge_xy;        /* [2][E] */
    const double* edge_normal;    /* [2][E] */
    const int* boundary_type;     /* [NB] */
    /* each boundary set's edges in set order (VirtualBoundarySet_2D::pEdges, the
     * BoundaryV2 edge sets of OldDataConverter.cpp:179-193): set s holds
     * set_edge_list[set_edge_offsets[s] .. set_edge_offsets[s+1]); may be NULL, then
     * the edges of a set are taken in edge order */
    const int* set_edge_offsets;  /* [NB+1] */
    const int* set_edge_list;
    const char* const* set_names; /* [NB] marker names, may be NULL */
} fvgb_mesh_soa;

typedef struct fvgb_mesh fvgb_mesh;     /* host mesh owned by the library */
typedef struct fvgb_handle fvgb_handle; /* one solver on one GPU */
typedef struct fvgb_batch fvgb_batch;   /* many solvers packed into one launch per stage */

/* ---- configuration and mesh (host only; no GPU needed) ------------------ */

/* Defaults of FVMR/src/global/GlobalPara.cpp:4-90. */
int fvgb_params_default(fvgb_params* p);
/* Reads input.toml like TomlFileManager::treeToGlobalParameter
 * (FVMR/src/input/TomlFileManager.cpp:110-170, 200-265, mu0/Re 79-104).
 * mesh_name receives basic.filename (may be NULL). */
int fvgb_params_read_toml(const char* path, fvgb_params* p, char* mesh_name, int mesh_name_len);
/* What the driver loop reads from input.toml besides the step's parameters
 * (CDriver::start, FVMR/src/drivers/CDriver.cpp:31-184; keys per
 * TomlFileManager.cpp:110-148, defaults per GlobalPara.cpp:26-29, 74-82). */
typedef struct fvgb_run_config {
    int continue_run;            /* basic.continue: restart from the newest pause file */
    int step_per_print;          /* output.step_per_print */
    int step_per_output_field;   /* output.step_per_output_field */
    int step_per_output_hist;    /* output.step_per_output_hist */
    int start_output_field;      /* output.start_output_field */
    int max_iteration;           /* output.maxIteration */
    double tolerance_residual;   /* output.tolerace_residual (the reference's spelling) */
    char filename[256];          /* basic.filename: mesh <filename>.su2, outputs <filename>... */
    char mesh_file_type[16];     /* basic.meshFileType */
    int volume_preset;           /* output.outputScheme_volume_preset: 0 rho u v p, 1 + Cp, 2 + Ma (default 2) */
    int boundary_preset;         /* output.outputScheme_boundary_preset (default 1) */
    int time_strategy;           /* time.strategy: 0 none, 1 adaptive CFL (RoutineController) */
} fvgb_run_config;
int fvgb_run_config_read_toml(const char* path, fvgb_run_config* c);
/* The driver's adaptive CFL, RoutineController (FVMR/src/drivers/RoutineController.cpp:
 * 13-90) as CDriver::start applies it at each print event with the residual of rho
 * (CDriver.cpp:115-120): strategy 0 leaves CFL alone; strategy 1 records the first
 * residual, then (after step 1000) scales CFL by 0.75 when the residual exceeds ten
 * times the record, and (after step 5000) by 1.1 when it falls below half the
 * record (the record then x 0.9) and by 1.05 otherwise, each change with its
 * cool-down (500 / 1000 steps), CFL never below 0.5.  *applied = 1 when CFL
 * changed; pass the new value to fvgb_set_cfl. */
typedef struct fvgb_cfl_controller fvgb_cfl_controller;
int fvgb_cfl_controller_create(int strategy, fvgb_cfl_controller** out);
int fvgb_cfl_controller_apply(fvgb_cfl_controller* c, double residual_rho, int step, double* CFL, int* applied);
void fvgb_cfl_controller_destroy(fvgb_cfl_controller* c);
/* Reads and assembles an .su2 mesh with the reference's numbering
 * (SU2MeshReader::read_mesh_and_process, FVMR/src/input/SU2MeshReader.cpp:10-251,
 * FVM_2D::iniEdges.., FVMR/src/legacy/FVM_2D.cpp:36-198) in O(N). */
int fvgb_mesh_read_su2(const char* path, int equation, double scale, fvgb_mesh** out);
int fvgb_mesh_view(const fvgb_mesh* m, fvgb_mesh_soa* soa);
void fvgb_mesh_free(fvgb_mesh* m);
/* Synthetic .su2 writers for the benchmark meshes (no reference counterpart).
 * Square [0,L]^2 with n x n quads, periodic markers, interior nodes jittered
 * by U(-jitter*h, +jitter*h) from seed; O-grid around a cylinder. */
int fvgb_write_su2_periodic_square(const char* path, int n, double L, double jitter, unsigned long long seed);
int fvgb_write_su2_cylinder(const char* path, int n_theta, int n_r, double r0, double r1, double first_dr);
/* Initial field (FieldInitializer, FVMR/src/input/FieldInitializer.cpp:129-222) on host. */
int fvgb_initial_field(const fvgb_mesh_soa* mesh, const fvgb_params* p, double* U);

/* Continue ("pause") files, the reference's restart format: t, istep, CFL, the
 * nodes, the triangles with U and the boundary sets' edge IDs.  Written by
 * FieldWriter::writeContinueFile_1 (FVMR/src/output/FieldWriter.cpp:264-326) and
 * read by ContinueFileReader::readContinueFile_1 (FVMR/src/input/ContinueFileReader.cpp:
 * 19-158, 457-494), which rebuilds the mesh from the file alone.  This writer
 * uses 17 significant digits (the reference 6), so a restart continues bit for
 * bit; the reference reads these files and this reader reads the reference's.
 * fvgb_read_continue returns the mesh (its state through fvgb_continue_state),
 * t, istep and the saved CFL (-1 when the file has none; the reference then
 * keeps the input.toml value).  fvgb_write_continue takes a mesh from either
 * reader and U[4][N] in reference numbering. */
int fvgb_read_continue(const char* path, int equation, fvgb_mesh** out, double* t, int* istep, double* cfl);
int fvgb_continue_state(const fvgb_mesh* m, double* U);
int fvgb_write_continue(const fvgb_mesh* m, const char* path, double t, int istep, double cfl, const double* U);
/* The newest pause_<name>[<n>].dat in directory, by the reference's rule
 * (ContinueFileReader.cpp:24-53: largest n > 0); FVGB_ERR_IO when there is none. */
int fvgb_find_continue_file(const char* directory, const char* name, char* path_out, int path_len);

/* ---- one solver ----------------------------------------------------------- */

/* GPUSolver2::allocateMemory + initializeData (FVMR/src/solvers/GPUSolver2.cpp:54-165). */
int fvgb_create(const fvgb_mesh_soa* mesh, const fvgb_params* p, fvgb_handle** out);
void fvgb_destroy(fvgb_handle* h);
/* host <-> device state, reference numbering (GPUSolver2::host_to_device /
 * device_to_host, GPUSolver2.cpp:222-239).  Both return once U has been read or
 * written.  A page-locked U (cudaHostAlloc / cudaHostRegister) is read and written
 * by the permuting kernels directly over the host link, with no staging copy. */
int fvgb_set_state(fvgb_handle* h, const double* U);
int fvgb_get_state(fvgb_handle* h, double* U);
/* nsteps of CIteration::iteration_device (FVMR/src/time/CIteration.cpp:89-161):
 * dt, t clamp against T, RK stages, restrict.  *t is read and updated. */
int fvgb_step(fvgb_handle* h, double* t, double T, int nsteps);
/* the same, asynchronously: t stays on the device; read it with fvgb_time(). */
int fvgb_step_async(fvgb_handle* h, double T, int nsteps);
int fvgb_set_time(fvgb_handle* h, double t);
int fvgb_time(fvgb_handle* h, double* t, double* last_dt);
/* changes the CFL number of the following steps (GlobalPara::time::CFL, which the
 * reference's driver adjusts through RoutineController, CDriver.cpp:115-120); the
 * captured step is rebuilt at the next fvgb_step.  CFL must be positive. */
int fvgb_set_cfl(fvgb_handle* h, double CFL);
int fvgb_synchronize(fvgb_handle* h);
/* calculateFunctionF on a given state (FVMR/src/time/Evolve.cpp:98-112):
 * rhs[4][N]; grad_x/grad_y[4][N] (limited gradients) may be NULL. */
int fvgb_rhs(fvgb_handle* h, const double* U, double* rhs, double* grad_x, double* grad_y);
/* get_global_dt_host of the current state (FVMR/src/time/CalculateDt.cpp:87-102). */
int fvgb_dt(fvgb_handle* h, double* dt);
/* GPUSolver2::updateResidualVector (GPUSolver2.cpp:294-296) on the right-hand
 * side of the last stage: norm 0 = L-inf, 1 = L1, 2 = L2 (Residual.cpp:4-43). */
int fvgb_residual(fvgb_handle* h, int norm, double out4[4]);
/* device counters: [0] cells replaced by the positivity pass so far,
 * [1] NaN cells seen, [2] out-of-range far-field states, [3] negative rho/p in dt. */
int fvgb_device_status(fvgb_handle* h, long long out4[4]);
/* raw device pointers of the state U[4][N] (this library's cell order) and
 * the sizes, for callers that keep data on the GPU. */
int fvgb_device_state(fvgb_handle* h, double** U_dev, int* n_cells);
/* Cell permutation: perm[i] = this library's index of reference cell i. */
int fvgb_cell_permutation(fvgb_handle* h, int* perm);
int fvgb_edge_permutation(fvgb_handle* h, int* perm);
/* The edge colouring of [gpu] edge_colour = 1 (no counterpart in the reference,
 * which gathers the residual per cell): colour[i] = the colour of reference edge
 * i, read back from the device's colour lists, and *ncolours; with the option
 * off every colour is -1 and *ncolours = 0.  No two edges of a colour write the
 * same cell (an edge writes its L cell, and its R cell where it is one of R's
 * edges: interior edges, not periodic or boundary ones). */
int fvgb_edge_colours(fvgb_handle* h, int* colour, int* ncolours);
/* Device-side layout arrays mapped back to reference numbering, for checking
 * connectivity: elem_edges[3][N] (slot order), elem_neighbors[3][N] (the
 * valid face neighbours in slot order, then -1, as the gradient reads them),
 * edge_L[E], edge_R[E]. */
int fvgb_layout_connectivity(fvgb_handle* h, int* elem_edges, int* elem_neighbors, int* edge_L, int* edge_R);
/* Number of kernels this library launched on the handle's stream so far. */
long long fvgb_kernel_launches(fvgb_handle* h);
/* nsteps of fvgb_step_async bracketed by CUDA events on the handle's stream;
 * *ms_out = the device time between them.  t stays on the device. */
int fvgb_step_timed(fvgb_handle* h, double T, int nsteps, double* ms_out);
/* Runs nsteps like fvgb_step_async but launch by launch, with CUDA events on
 * the handle's stream around each kernel group; returns the summed time (ms)
 * and the number of timed groups for: [0] time step (4 kernels), [1] gradient
 * + limiter, [2] edge fluxes (interior + boundary), [3] gather + stage update,
 * [4] positivity pass.  (The reference times only whole iterations with
 * std::chrono, FVMR/src/drivers/CDriver.cpp:73-85.) */
int fvgb_profile_steps(fvgb_handle* h, double T, int nsteps, double ms_out[5], int count_out[5]);

/* ---- field output ----------------------------------------------------------
 * Node values of the current state, as FieldWriter::update_nodeField
 * (FVMR/src/output/FieldWriter.cpp:364-453) forms them for its Tecplot files:
 * per node the mean of its cells' rho, u, v, p (summed in cell order), then
 * Cp = (p - p_inf) / (1/2 rho_inf V_inf^2) and Ma.  out6[6][V] = rho, u, v, p,
 * Cp, Ma in reference node numbering (may be NULL).  Computed on the device. */
int fvgb_node_field(fvgb_handle* h, double* out6);
/* Pressure lift and drag coefficients per boundary set (ReferenceData::
 * calculate_edgeSet_force, FieldWriter.cpp:175-210: Cp of the edge's nodes
 * averaged, times length / referenceArea, along the edge normal) and their sums
 * over the wall sets (HistData::set_CDCL_wall, FieldWriter.cpp:611-632).  cd/cl
 * are [NB] (either may be NULL). */
int fvgb_boundary_forces(fvgb_handle* h, double* cd, double* cl, double* cd_wall, double* cl_wall);
/* Tecplot ASCII files of write_tecplot_volume_file / write_tecplot_boundary_file
 * (FieldWriter.cpp:44-172): preset 0 = x y rho u v p, 1 = + Cp, 2 = + Ma
 * (output.outputScheme_*_preset; the reference's defaults are 2 for the volume
 * and 1 for the boundary file). */
int fvgb_write_tecplot_volume(fvgb_handle* h, const char* path, const char* title, double t, int preset);
int fvgb_write_tecplot_boundary(fvgb_handle* h, const char* path, double t, int preset);
/* The field colouring of the reference's GUI (FVMR/src/gui/cuda/CudaGrid_kernels.cu:
 * 18-164, 225-245) without a graphics stack: per node the largest density of its
 * cells (the reference's racy max of rho x count, times 1/count, done here
 * deterministically), normalised by [range_lo, range_hi] (render.range_1/2)
 * and mapped through the reference's five-point colour map.  The colours
 * go to a device buffer owned by the handle, [V][3] floats (*rgb_dev, valid
 * until the next call or fvgb_destroy); rgb_host [V][3] and node_value_host [V]
 * receive copies when not NULL. */
int fvgb_colour_nodes(fvgb_handle* h, double range_lo, double range_hi, float** rgb_dev, float* rgb_host,
                      float* node_value_host);
int fvgb_num_nodes(fvgb_handle* h, int* V);
/* reps launches of the node-value kernel, then of the colouring kernel, each
 * series bracketed by CUDA events on the handle's stream (device ms per series). */
int fvgb_output_timed(fvgb_handle* h, int reps, double* ms_node_field, double* ms_colour);

/* ---- discrete adjoint ------------------------------------------------------
 * No counterpart in the reference.  Reverse-mode derivative of K steps of the
 * handle's own step map U_0 -> U_K (Euler or laminar Navier-Stokes equations,
 * Roe or LLF flux, least-squares or Green-Gauss gradients with or without the
 * Barth limiter, forward Euler, Kutta RK3 or SSP-RK3, every boundary kind; the
 * time step's dependence on the state included).  fvgb_adjoint_forward runs the K steps from U0 at time t0
 * keeping n_checkpoints states (sqrt(K) keeps memory at O(sqrt(K) N)) and
 * returns U_K; fvgb_adjoint_backward then maps a seed dL/dU_K to dL/dU_0
 * (both [4][N], reference numbering), recomputing each segment once.  The
 * handle's state afterwards is U_K.  Fails with FVGB_ERR_UNSUPPORTED outside
 * that scope, and when the positivity pass acted during the run.  A forward
 * with the same nsteps, n_checkpoints, overlap mode and CFL as the handle's
 * previous one reuses its workspace: the device buffers and the backward
 * sweep's captured graphs. */
int fvgb_adjoint_forward(fvgb_handle* h, int nsteps, int n_checkpoints, const double* U0, double t0, double* U_K,
                         double* ms_forward);
int fvgb_adjoint_backward(fvgb_handle* h, const double* seed_UK, double* grad_U0, double* ms_backward);
void fvgb_adjoint_release(fvgb_handle* h);
/* mode 1 (the default): fvgb_adjoint_forward lays out a second set of segment
 * records where the device has room for it and 1 GiB besides, and the backward
 * sweep recomputes each segment on the handle's stream beside the reverse of the
 * segment after it on a second stream.  Mode 0: one set, recomputation and
 * reverse one after the other.  The gradient is bitwise the same.  Takes effect
 * at the next fvgb_adjoint_forward; *overlapped (may be null) reports whether
 * the current adjoint workspace has the second set. */
int fvgb_adjoint_overlap(fvgb_handle* h, int mode, int* overlapped);
/* The residual's vector-Jacobian product grad_U = (dR/dU)^T seed_R at the state U,
 * where R is what fvgb_rhs returns for U (calculateFunctionF, FVMR/src/time/
 * Evolve.cpp:98-112): the reverse of the edge fluxes with their boundary ghosts,
 * the face reconstruction, the Barth limiter and the gradients, in the scope of
 * the adjoint above (steady runs included: R does not involve the time step).
 * These are the reverse kernels of one Runge-Kutta stage of fvgb_adjoint_backward,
 * run once on a recorded evaluation of R.  U, seed_R, grad_U: [4][N], reference
 * numbering; the handle's state becomes U, as with fvgb_rhs.  No counterpart in
 * the reference. */
int fvgb_rhs_vjp(fvgb_handle* h, const double* U, const double* seed_R, double* grad_U);

/* ---- batched instances -----------------------------------------------------
 * No counterpart in the reference (one mesh per process, the driver loop of
 * FVMR/src/drivers/CDriver.cpp:75-80 stepping it).  n independent instances of
 * the Euler or laminar Navier-Stokes step (their own meshes, far-field states,
 * CFL, time and end time; one shared scheme and gas, for Navier-Stokes the same
 * mu0, T0 and Pr) packed into one device layout and advanced by one
 * persistent cooperative kernel per Runge-Kutta stage, the step captured in a
 * CUDA graph.  Each instance gives bit for bit what fvgb_step gives for it
 * alone.  States are in each instance's reference numbering. */
int fvgb_batch_create(int n, const fvgb_mesh_soa* const* meshes, const fvgb_params* params, fvgb_batch** out);
void fvgb_batch_destroy(fvgb_batch* b);
int fvgb_batch_set_state(fvgb_batch* b, int i, const double* U);
int fvgb_batch_get_state(fvgb_batch* b, int i, double* U);
/* nsteps steps of every instance; t[n] is read and updated, T[n] (may be NULL
 * to keep the end times of the parameters) clamps each instance's time. */
int fvgb_batch_step(fvgb_batch* b, double* t, const double* T, int nsteps);
/* nsteps with the times kept on the device, bracketed by CUDA events. */
int fvgb_batch_step_timed(fvgb_batch* b, int nsteps, double* ms_out);
/* The autotuner: times block size x work-tile size x static or queued tile
 * schedule on trial_steps steps of this batch (state restored afterwards) and
 * keeps the fastest; report gets one line per candidate. */
int fvgb_batch_tune(fvgb_batch* b, int trial_steps, char* report, int report_len);
/* The persistent kernel's bounded grid barrier, exercised on its own: `blocks`
 * 32-thread blocks meet at one barrier with at most spin_limit polls each; block
 * absent_block (-1: none) never arrives, so the others give up, set the error word
 * and return.  *timed_out = that error word, *blocks_passed = the blocks whose wait
 * succeeded.  The GPU stays usable either way (nothing faults, every wait ends). */
int fvgb_barrier_selftest(int device, int blocks, int absent_block, long long spin_limit, int* timed_out,
                          int* blocks_passed);
/* [0] instances, [1] cells, [2] edges, [3] grid, [4] block, [5] kernel
 * launches, [6] tile size (negative: queued schedule), [7] 1 if the step runs
 * as a captured graph. */
int fvgb_batch_info(fvgb_batch* b, long long out[8]);

/* No counterpart in the reference.  The first-order residual (constant
 * reconstruction, Euler equations, Roe or LLF, every boundary type of this
 * path) computed from device arrays the caller owns, without allocating any
 * device or pinned memory: for callers that already manage every GPU buffer
 * themselves and may not add allocations of their own.  dev_mesh holds DEVICE
 * pointers to the reference-layout arrays (elem_edges, elem_volume, edge_L,
 * edge_R, edge_setID, edge_length, edge_normal, edge_xy and boundary_type
 * are read, none may be NULL; "dsr" edges are evaluated at p->dsr_time);
 * U_dev is U[4][N] and rhs_dev receives RHS[4][N] = -(1/vol) sum of edge
 * fluxes, both on the device; stream is a cudaStream_t (NULL = default
 * stream); the call only enqueues work.  The edge fluxes are kept in one
 * library-wide device array of 32 MiB (at most 1,048,576 edges; larger meshes
 * get FVGB_ERR_ARG).  Every call shares that array, so calls that overlap
 * on the GPU race on it and must be serialised by the caller.  Every call
 * looks up the array's device address in the current context
 * (cudaGetSymbolAddress: a runtime query, no allocation; nothing is cached,
 * so a device reset or a switch of context is safe); the first call in a
 * context also loads the library's device code there, so make that first
 * call before any stream capture begins.  Far-field ghost states out of
 * range are not reported by this call. */
int fvgb_rhs_noalloc(const fvgb_mesh_soa* dev_mesh, const fvgb_params* p, const double* U_dev, double* rhs_dev,
                     void* stream);

/* No counterpart in the reference.  The device's FP64 arithmetic rate in
 * GFLOP/s (an FMA counts two), measured with independent register FMA chains
 * on every SM (best of three timed launches): the roofline denominator for
 * kernels bound by the FP64 pipe. */
int fvgb_fp64_peak(int device, double* gflops);

/* No counterpart in the reference.  The device functions the kernels use in
 * place of most divisions and square roots (the hardware approximations
 * refined by a series step) evaluated on n host values x on the given device:
 * op 0 out[i] = 1/x[i], op 1 out[i] = 1/sqrt(x[i]), op 2 out[i] = sqrt(x[i]).
 * For accuracy tests. */
int fvgb_math_eval(int device, int op, int n, const double* x, double* out);

/* No counterpart in the reference.  The correctly rounded FP64 multiply (op 0)
 * and add (op 1) that run on the integer pipes (softfp64.cuh) evaluated on n
 * host pairs on the given device, beside the hardware instruction on the same
 * pairs: soft[i] and hw[i].  For bitwise tests. */
int fvgb_softfp64_eval(int device, int op, int n, const double* a, const double* b, double* soft, double* hw);
/* No counterpart in the reference.  The same functions compiled for the host
 * (the fallback is then the host's IEEE operation): out[i] = a[i] op b[i].  For
 * CPU tests. */
int fvgb_softfp64_host(int op, int n, const double* a, const double* b, double* out);
/* No counterpart in the reference.  G operations/s of independent FP64 chains,
 * eight per thread: out[0..3] multiply on the FP64 pipe alone, on the integer
 * pipes alone, 4 + 4 and 2 + 6 side by side in one thread; out[4..7] add the
 * same way (the last 6 + 2); out[8] the SM count, out[9] the maximum SM clock
 * in MHz. */
int fvgb_softfp64_rate(int device, double out[10]);

const char* fvgb_last_error(void);
const char* fvgb_version(void);

#ifdef __cplusplus
}
#endif
#endif

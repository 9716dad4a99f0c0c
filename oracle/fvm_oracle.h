/* fvm_oracle.h -- CPU restatement of FVMR's explicit finite-volume step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the parity tests, smoke()
 * and the CPU-baseline leg of bench.py check the CUDA path against.  The
 * product never links it.  Each function follows the reference's CPU path
 * operation by operation (file:line cited at each definition) and is built
 * with -ffp-contract=off so it is IEEE-exact and gives the same bits on x86
 * and Arm.  It is pinned against the reference itself compiled from source
 * (oracle/ref, binaries fvmr_ref_f64/f32).
 */
#ifndef FVM_ORACLE_H
#define FVM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct om_mesh {
    int N, E, V, NB;
    double* node_xy;     /* [2][V] */
    int* elem_nodes;     /* [4][N], slot 3 = -1 (triangles) */
    int* elem_edges;     /* [4][N], slot 3 = -1 */
    int* elem_nbrs;      /* [4][N], -1 = none (periodic faces included) */
    double* elem_xy;     /* [2][N] */
    double* elem_vol;    /* [N] */
    int* edge_nodes;     /* [2][E] */
    int* edge_L;         /* [E] */
    int* edge_R;         /* [E], -1 on non-periodic boundaries */
    int* edge_set;       /* [E], boundary set ID (1-based) or -1 */
    int* edge_pair;      /* [E], periodic partner edge or -1 */
    double* edge_len;    /* [E], rounded through float */
    double* edge_dist;   /* [E], distance of cell centres (float arithmetic) */
    double* edge_xy;     /* [2][E] */
    double* edge_normal; /* [2][E] */
    int* bc_type;        /* [NB] */
} om_mesh;

typedef struct om_params {
    int equation;      /* 1 Euler, 2 Navier-Stokes */
    int flux_scheme;   /* 2001 local Lax-Friedrichs, 2002 Roe */
    int reconstruct;   /* 3001 constant, 3002 linear */
    int gradient;      /* 1 least squares, 2 Green-Gauss */
    int limiter;       /* 0 none, 1 Barth */
    int time_advance;  /* 3101 forward Euler, 3103 Kutta RK3, 3104 SSP-RK3 */
    int lsq_det_ref;   /* 1: the reference's 2x2 determinant guard; 0: corrected */
    int wall_bc_ref;   /* 1: the reference's no-slip ghost state; 0: mirrored velocity */
    int restrict_ref;  /* 1: the reference's neighbour-volume sum; 0: corrected */
    int pad_;
    double gamma, R, Pr, mu0, T0, CFL, T_end;
    double inf[4], inlet[4], outlet[4]; /* rho, u, v, p */
    double shock[4];   /* shock tube: x, y, normal x, normal y */
    double dsr[3];     /* double Mach reflection: x, y where the shock meets the wall, angle (degrees) */
    double dsr_time;   /* CBoundaryDoubleShockReflect's t + dt: the time of "dsr" edges in om_rhs */
    int steady;        /* 1: local time stepping (time.is_steady), forward Euler with each cell's dt */
    int pad2_;
} om_params;

/* Reads an .su2 file and assembles the mesh exactly as the reference does.
 * Returns NULL and fills err on failure. */
om_mesh* om_mesh_read_su2(const char* path, int equation, double scale, char* err, int errlen);
void om_mesh_free(om_mesh* m);

/* Initial field: ic 1 uniform (inf), 2 isentropic vortex (vortex = x, y, strength),
 * 3 shock tube (params shock), 4 double Mach reflection (params dsr). */
int om_init_field(const om_mesh* m, const om_params* p, int ic, const double* vortex, double* U);
/* One residual evaluation: RHS = -(1/vol) * sum of edge fluxes; also the limited gradients. */
int om_rhs(const om_mesh* m, const om_params* p, const double* U, double* rhs, double* gx, double* gy);
/* Global time step of the state U (before the t-clamp). alpha may be NULL. */
int om_dt(const om_mesh* m, const om_params* p, const double* U, double* dt, double* alpha);
/* Positivity pass on U in place. Returns the number of cells replaced, -1 on NaN. */
int om_restrict(const om_mesh* m, const om_params* p, double* U);
/* nsteps steps of time_advance from time *t; U in place; dts[nsteps] may be NULL.
 * "dsr" edges are evaluated at each stage's time (p->dsr_time is not used).
 * Steady runs advance each cell by its own dt and t by cell 0's (dts: those). */
int om_run(const om_mesh* m, const om_params* p, double* U, int nsteps, double* t, double* dts, double* last_rhs);
/* Residual norm of an RHS field: norm 0 = L-infinity, 1 = L1, 2 = L2 (per variable). */
void om_residual(const om_mesh* m, const double* rhs, int norm, double* out4);
/* Node values for the Tecplot writers, FieldWriter::update_nodeField
 * (FVMR/src/output/FieldWriter.cpp:364-453): per node the mean of its cells'
 * U2ruvp values summed in cell order, then Cp against (p_inf, pdyn_inf) and Ma.
 * elem_nodes [4][N] (slot 3 ignored), U [4][N]; out [6][V] = rho u v p Cp Ma. */
void om_node_field(int N, int V, const int* elem_nodes, const double* U, double gamma, double p_inf,
                   double pdyn_inf, double* out);
/* ReferenceData::calculate_edgeSet_force (FieldWriter.cpp:175-210) per boundary
 * set, the sets' edges in set order (set_off [NB+1], set_list), and the sums
 * over wall sets (HistData::set_CDCL_wall, FieldWriter.cpp:611-632). */
void om_boundary_forces(int NB, const int* set_off, const int* set_list, const int* bc_type, int E,
                        const int* edge_nodes, const double* edge_normal, const double* edge_len,
                        const double* Cp, double ref_area, double* cd, double* cl, double* cd_wall,
                        double* cl_wall);
/* The GUI's field colouring (FVMR/src/gui/cuda/CudaGrid_kernels.cu:24-130) in
 * float arithmetic: node value = max over the node's cells of rho x count,
 * times 1/count; colour through the five-point map of CudaGrid.cpp:31-37.
 * rgb [V][3], node_value [V]. */
void om_colour_nodes(int N, int V, const int* elem_nodes, const double* U, float range_lo, float range_hi,
                     float* rgb, float* node_value);
/* Host threads for the per-cell and per-edge loops (results do not depend on
 * the count: every output value is computed by one thread in the reference's
 * order).  n <= 0 keeps the current count; returns the count in use. */
int om_set_threads(int n);
/* Freestream (rho,u,v,p) from Mach and angle of attack (degrees). */
void om_ruvp_from_mach(double Ma, double aoa_deg, double T0, double p0, double gamma, double R, double* ruvp);

#ifdef __cplusplus
}
#endif
#endif

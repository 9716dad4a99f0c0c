// The step kernels (sm_103a, FP64).  One thread per cell or per edge; states
// are d4 per cell (rho, rho u, rho v, rho E) so a gather of a
// neighbour's state is one 32-byte sector.
#pragma once
#include <cuda_runtime.h>

#include "physics.cuh"

namespace fvgb {
namespace dev {

enum { FLUX_LLF = 2001, FLUX_ROE = 2002 };

// Device view of one mesh layout (see layout.h for the meaning of each array).
struct MeshView {
    int N, E, E_int;
    const int* __restrict__ e_L;
    const int* __restrict__ e_R;
    const int* __restrict__ e_bc;
    const double* __restrict__ e_geom;   // [E][8]
    const int* __restrict__ c_edge;      // [N][3]
    const int* __restrict__ c_nbr;       // [N][3]
    const int* __restrict__ c_nnb;       // [N]
    const double* __restrict__ c_mvol;
    const double* __restrict__ c_vol;
    const double* __restrict__ c_lsq;    // [N][6]
    const double* __restrict__ c_vtx;    // [N][6]
    const double* __restrict__ c_gg;     // [N][12]
    const int* __restrict__ c_ggout;     // [N][3]
    const double* __restrict__ c_ginv;   // [N]
    const int* __restrict__ dt_ptr;
    const int* __restrict__ dt_edge;
};

// Boundary data of one solver instance.
struct BcData {
    double inf[4], inlet[4], outlet[4];   // rho, u, v, p
    double a_inf, a_inlet, a_outlet;       // sound speeds sqrt(gamma p / rho)
    double son_inf, son_inlet, son_outlet; // p / rho^gamma
    int wall_ref;                          // 1: the reference's no-slip ghost state
    // double Mach reflection ("dsr" edges): the far-field state is the inlet's upstream of
    // the moving shock and the outlet's downstream of it; the shock meets the boundary at
    // x = dsr_x + (y + 20 t) / sqrt3, t being the stage's time
    // *clock_t0 + clock_frac * *clock_dt (device words; null where no "dsr" edge exists)
    double dsr_x, sqrt3;
    const double* clock_t0;
    const double* clock_dt;
    double clock_frac;
};

// Status words written by the kernels (never a trap).
struct Status {
    unsigned long long restricted;   // cells replaced by the positivity pass
    unsigned long long nan_cells;    // NaN found in the state
    unsigned long long farfield_oor; // far-field ghost out of range
    unsigned long long negative_dt;  // negative rho or p in the time step
};

__device__ __forceinline__ d4 ld4(const d4* __restrict__ p) { return *p; }

__device__ __forceinline__ void dmin_atomic(unsigned long long* addr, double v) {
    // positive doubles order like their bit patterns
    atomicMin(addr, (unsigned long long)__double_as_longlong(v));
}

}  // namespace dev
}  // namespace fvgb

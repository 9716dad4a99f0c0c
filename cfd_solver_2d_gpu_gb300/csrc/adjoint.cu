// Discrete adjoint of the explicit step (no counterpart in the reference).
//
// For U_{n+1} = Step(U_n) (time step, Runge-Kutta stages; forward Euler 3101,
// Kutta RK3 3103 or SSP-RK3 3104; Euler or laminar Navier-Stokes equations; least-squares
// or Green-Gauss gradients with or without the Barth limiter; Roe or LLF flux; interior,
// periodic, slip and no-slip wall, symmetry, far-field, inlet, outlet and double-Mach-
// reflection edges) this
// computes lambda_0 = (dU_K/dU_0)^T lambda_K by reverse sweeps over the steps,
// each stage's vector-Jacobian product being the hand-written reverse of the
// forward kernels (adjoint_device.cuh).  The time step's dependence on the
// state (dt = CFL vol / alpha at the minimising cell) is included; the
// positivity pass is assumed inactive (the forward reports whether it acted).
//
// Memory: checkpoints of U every S = ceil(K / n_checkpoints) steps; during the
// reverse sweep each segment is recomputed once, keeping per step U_0, U_1, U_2,
// the stages' residuals, edge tapes and limiter records, so the sweep costs one
// extra forward pass and about K/S 4N + S (74 N + 117 E) doubles (sqrt(K)
// checkpoints: O(sqrt(K) N)).  Where the device has room for a second set of segment
// records (and fvgb_adjoint_overlap has not turned it off), the recomputation of segment
// i-1 runs on the solver's stream beside the reverse sweep of segment i on a second
// stream: both are branches of one CUDA graph, and the two sets of records
// alternate.  The kernels and their inputs are the same either way, so the gradient is
// bitwise the same; the small per-stage kernels of a 10^5-cell mesh leave enough of the
// SMs idle for the two sweeps to share them.
//
// Kernels of one stage VJP (all gathers, no atomics: deterministic):
//   k_adj_edge     per edge: mu = seed-weighted flux adjoint, flux VJP from the stage's tape
//   k_adj_cell     per cell: gather the face-state adjoints of its edges; limiter + LSQ VJP
//   k_adj_combine  per cell: gather the neighbours' LSQ adjoints; the stage's RK combination;
//                  block partials of lam_s . R_s (the time step's adjoint)
// and once a step k_adj_dt.  The recorded forward keeps, per stage, the input state, the
// residual R_s, the edge tape (face states and Roe intermediates) and the limiter record
// (gradient before the limiter, phi, 1/den, the limiting slot and vertex; step_device.cuh),
// so the reverse sweep recomputes none of them: on this part FP64 issue, not memory, is
// scarce (39 doubles a stage per edge and 16.5 per cell; 5 GB for 23 steps of the
// 256x256 mesh).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "adjoint_device.cuh"
#include "internal.h"
#include "solver.h"
#include "step_kernels.cuh"

namespace fvgb {
namespace dev {

// ---- per edge --------------------------------------------------------------
// 128-thread blocks, capped at 128 registers a thread so that four blocks fit on an SM
constexpr int kEdgeThreads = 128;

// mu = dLoss/dF_e (F_e enters R_L with +1/-vol and, when e is in R's edge list, R_R with
// -1/-vol), then the flux VJP from the stage's recorded tape: the face states and the
// Roe intermediates are read, not recomputed
// NS: the viscous flux's adjoints of the averaged state and gradients (viscous_vjp), already
// divided between the two sides (half each; a boundary edge's L side takes all), go to avu,
// avgx, avgy; Uin, Gx, Gy are the stage's input state and the gradients it read.
template <int FLUX, bool NS>
__global__ void __launch_bounds__(kEdgeThreads, 4) k_adj_edge(EdgeTape tp, MeshView m, Gas g, BcData bc,
                                                           const d4* __restrict__ lam,
                                                           const int* __restrict__ e_rlist, d4* __restrict__ aL,
                                                           d4* __restrict__ aR, const d4* __restrict__ Uin,
                                                           const d4* __restrict__ Gx, const d4* __restrict__ Gy,
                                                           d4* __restrict__ avu, d4* __restrict__ avgx,
                                                           d4* __restrict__ avgy) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m.E) return;
    const int L = __ldg(&m.e_L[e]), R = __ldg(&m.e_R[e]);
    const double* gm = &m.e_geom[(size_t)e * 8];
    const double nx = __ldg(&gm[0]), ny = __ldg(&gm[1]), len = __ldg(&gm[2]);
    const double mL = __ldg(&m.c_mvol[L]);
    const d4 lL = ld4(&lam[L]);
    d4 mu = mk4(mul(mL, lL.x), mul(mL, lL.y), mul(mL, lL.z), mul(mL, lL.w));
    if (__ldg(&e_rlist[e])) {
        const double mR = __ldg(&m.c_mvol[R]);
        const d4 lR = ld4(&lam[R]);
        mu = mk4(mu.x - mR * lR.x, mu.y - mR * lR.y, mu.z - mR * lR.z, mu.w - mR * lR.w);
    }
    const size_t E = (size_t)tp.E;
    const double* v = tp.v;
    auto t = [&](int f) { return __ldg(&v[(size_t)f * E + e]); };
    Prim wL{t(T_LR), t(T_LU), t(T_LV), t(T_LP), t(T_LIR)};
    Prim wR{t(T_RR), t(T_RU), t(T_RV), t(T_RP), t(T_RIR)};
    const d4 fL = mk4(wL.r, t(T_ULY), t(T_ULZ), t(T_ULW));
    const d4 fR = mk4(wR.r, t(T_URY), t(T_URZ), t(T_URW));
    Prim bwL, bwR;
    d4 bfL, bfR;
    if constexpr (FLUX == FLUX_ROE) {
        RoeRec r;
        r.ruL = t(T_RUL); r.ruR = t(T_RUR); r.HL = t(T_HL); r.HR = t(T_HR); r.irm = t(T_IRM); r.rm = t(T_RM);
        r.rrorl = t(T_RRORL); r.w = t(T_W); r.um = t(T_UM); r.vm = t(T_VM); r.Hm = t(T_HM); r.am2 = t(T_AM2);
        r.iam = t(T_IAM); r.am = t(T_AM); r.un = t(T_UN); r.sel = t(T_SEL); r.Mstar = t(T_MSTAR); r.dE = t(T_DE);
        r.Etm = t(T_ETM); r.ae = t(T_AE); r.dUroe = t(T_DUROE); r.dProe = t(T_DPROE); r.dUr = t(T_DUR);
        r.sub = (__ldg(&tp.flags[e]) & 4) != 0;
        roe_rev(wL, wR, fL, fR, nx, ny, len, g, r, mu, bwL, bwR, bfL, bfR);
    } else {
        llf_rev(fL, fR, wL, wR, nx, ny, len, g, mu, bwL, bwR, bfL, bfR);
    }
    to_prim_vjp(fR, wR, g, bwR, bfR);
    if (NS) {
        d4 ua = ld4(&Uin[L]), gxa = ld4(&Gx[L]), gya = ld4(&Gy[L]);
        const bool two = e < m.E_int;
        if (two) {  // get_U_Gradient_mean / get_U_mean: averages of both sides
            const d4 ur = ld4(&Uin[R]), gxr = ld4(&Gx[R]), gyr = ld4(&Gy[R]);
            ua = mk4(0.5 * (ua.x + ur.x), 0.5 * (ua.y + ur.y), 0.5 * (ua.z + ur.z), 0.5 * (ua.w + ur.w));
            gxa = mk4(0.5 * (gxa.x + gxr.x), 0.5 * (gxa.y + gxr.y), 0.5 * (gxa.z + gxr.z), 0.5 * (gxa.w + gxr.w));
            gya = mk4(0.5 * (gya.x + gyr.x), 0.5 * (gya.y + gyr.y), 0.5 * (gya.z + gyr.z), 0.5 * (gya.w + gyr.w));
        }
        d4 bu, bgx, bgy;
        viscous_vjp(ua, gxa, gya, nx, ny, len, g, mu, bu, bgx, bgy);
        const double f = two ? 0.5 : 1.0;
        avu[e] = mk4(f * bu.x, f * bu.y, f * bu.z, f * bu.w);
        avgx[e] = mk4(f * bgx.x, f * bgx.y, f * bgx.z, f * bgx.w);
        avgy[e] = mk4(f * bgy.x, f * bgy.y, f * bgy.z, f * bgy.w);
    }
    if (e >= m.E_int) {  // a boundary edge: the ghost is a function of the L face state
        const int bt = __ldg(&m.e_bc[e]);
        if (bt == BC_WALL_ADIABAT) {  // no-slip adiabatic wall (Flux.cpp:73-79): (rho, -rho u or 0, -rho v or 0, rho E)
            bfL.x += bfR.x;
            bfL.w += bfR.w;
            if (!bc.wall_ref) { bfL.y -= bfR.y; bfL.z -= bfR.z; }
        } else if (bt == BC_DSR) {  // double Mach reflection: the side the forward took (tape flag bit 3)
            if (__ldg(&tp.flags[e]) & 8) ghost_farfield_vjp(wL, bc.inlet, bc.a_inlet, bc.son_inlet, nx, ny, g, bfR, bwL);
            else ghost_farfield_vjp(wL, bc.outlet, bc.a_outlet, bc.son_outlet, nx, ny, g, bfR, bwL);
        } else if (bt == BC_INLET) ghost_farfield_vjp(wL, bc.inlet, bc.a_inlet, bc.son_inlet, nx, ny, g, bfR, bwL);
        else if (bt == BC_OUTLET) ghost_farfield_vjp(wL, bc.outlet, bc.a_outlet, bc.son_outlet, nx, ny, g, bfR, bwL);
        else if (bt == BC_INF) ghost_farfield_vjp(wL, bc.inf, bc.a_inf, bc.son_inf, nx, ny, g, bfR, bwL);
        else ghost_slip_vjp(fL, wL, nx, ny, bfR, bfL, bwL);  // slip wall, symmetry
        bfR = mk4(0, 0, 0, 0);
    }
    to_prim_vjp(fL, wL, g, bwL, bfL);
    aL[e] = bfL;
    aR[e] = bfR;
}

// ---- per cell: gather face-state adjoints, then limiter + LSQ VJP ---------------
// The limiter's choices and the gradient before it come from the stage's record
// (grad_cell<1, true, true>); nothing of the forward is recomputed.
// GRAD 1: least squares, the transpose goes to the neighbour differences (bdU); GRAD 2:
// Green-Gauss, phi_f = g_C U_c + (1 - g_C) U_F on faces with a cell F beyond them (U_c on the
// others), grad = (1/vol) sum phi_f S_f: the U_c part joins lam_dir, the U_F parts go to bgg
// (one per face), and the limiter's bound adjoints still go to bdU.
template <bool LINEAR, bool BARTH, int GRAD, bool NS>
__global__ void __launch_bounds__(256) k_adj_cell(MeshView m, const d4* __restrict__ aL, const d4* __restrict__ aR,
                                                  const int* __restrict__ aflag, CellTape ct,
                                                  d4* __restrict__ lam_dir, d4* __restrict__ bdU,
                                                  d4* __restrict__ bgg, const d4* __restrict__ avu,
                                                  const d4* __restrict__ avgx, const d4* __restrict__ avgy) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    double lu[4] = {0, 0, 0, 0}, lgx[4] = {0, 0, 0, 0}, lgy[4] = {0, 0, 0, 0};
    const int b = __ldg(&m.dt_ptr[c]), en = __ldg(&m.dt_ptr[c + 1]);
    for (int k = b; k < en; k++) {
        const int e = __ldg(&m.dt_edge[k]);
        const bool isL = __ldg(&m.e_L[e]) == c;
        const d4 a = isL ? ld4(&aL[e]) : ld4(&aR[e]);
        const double av[4] = {a.x, a.y, a.z, a.w};
        const int fl = __ldg(&aflag[e]);
        const bool used = isL ? (fl & 1) : (fl & 2);
        const double* gm = &m.e_geom[(size_t)e * 8];
        const double dx = isL ? __ldg(&gm[4]) : __ldg(&gm[6]);
        const double dy = isL ? __ldg(&gm[5]) : __ldg(&gm[7]);
#pragma unroll
        for (int v = 0; v < 4; v++) {
            lu[v] += av[v];
            if (LINEAR && used) {
                lgx[v] = fma(av[v], dx, lgx[v]);
                lgy[v] = fma(av[v], dy, lgy[v]);
            }
        }
        if (NS) {  // the viscous flux read this cell's state and gradients
            const d4 u = ld4(&avu[e]), x = ld4(&avgx[e]), y = ld4(&avgy[e]);
            lu[0] += u.x; lu[1] += u.y; lu[2] += u.z; lu[3] += u.w;
            lgx[0] += x.x; lgx[1] += x.y; lgx[2] += x.z; lgx[3] += x.w;
            lgy[0] += y.x; lgy[1] += y.y; lgy[2] += y.z; lgy[3] += y.w;
        }
    }
    double bd[3][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
    double bgx_all[4] = {0, 0, 0, 0}, bgy_all[4] = {0, 0, 0, 0};  // adjoint of the unlimited gradient
    if (LINEAR) {
        const int nnb = __ldg(&m.c_nnb[c]);
        const double* B = &m.c_lsq[(size_t)c * 6];
        double b0[3], b1[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            b0[k] = __ldg(&B[k]);
            b1[k] = __ldg(&B[3 + k]);
        }
        double vx[3] = {0, 0, 0}, vy[3] = {0, 0, 0}, gxr[4] = {0, 0, 0, 0}, gyr[4] = {0, 0, 0, 0};
        double phi[4] = {1, 1, 1, 1}, rden[4] = {0, 0, 0, 0};
        int code = 0;
        if (BARTH) {
            const double* X = &m.c_vtx[(size_t)c * 6];
#pragma unroll
            for (int j = 0; j < 3; j++) {
                vx[j] = __ldg(&X[2 * j]);
                vy[j] = __ldg(&X[2 * j + 1]);
            }
            code = __ldg(&ct.code[c]);
            if (code) {
                const d4 a = ld4(&ct.gx[c]), bb = ld4(&ct.gy[c]), p = ld4(&ct.phi[c]), r = ld4(&ct.rden[c]);
                gxr[0] = a.x; gxr[1] = a.y; gxr[2] = a.z; gxr[3] = a.w;
                gyr[0] = bb.x; gyr[1] = bb.y; gyr[2] = bb.z; gyr[3] = bb.w;
                phi[0] = p.x; phi[1] = p.y; phi[2] = p.z; phi[3] = p.w;
                rden[0] = r.x; rden[1] = r.y; rden[2] = r.z; rden[3] = r.w;
            }
        }
#pragma unroll
        for (int v = 0; v < 4; v++) {
            double bgx = lgx[v], bgy = lgy[v];
            const int cv = code >> (5 * v);
            if (BARTH && (cv & 1)) {
                // gx_lim = phi gx, gy_lim = phi gy, phi = num / den, den = d(vertex jj) +- eps,
                // num = U(slot kk) - Uc
                const int kk = ((cv >> 1) & 3) - 1, jj = (cv >> 3) & 3;
                const double b_phi = fma(bgy, gyr[v], mul(bgx, gxr[v]));
                bgx = mul(bgx, phi[v]);
                bgy = mul(bgy, phi[v]);
                const double b_num = mul(b_phi, rden[v]);
                const double b_den = -mul(mul(b_phi, phi[v]), rden[v]);
                const double vxj = jj == 0 ? vx[0] : (jj == 1 ? vx[1] : vx[2]);
                const double vyj = jj == 0 ? vy[0] : (jj == 1 ? vy[1] : vy[2]);
                bgx = fma(b_den, vxj, bgx);
                bgy = fma(b_den, vyj, bgy);
#pragma unroll
                for (int k = 0; k < 3; k++)
                    if (k == kk) bd[k][v] += b_num;
            }
            if (GRAD == 1) {
#pragma unroll
                for (int k = 0; k < 3; k++)
                    if (k < nnb) bd[k][v] = fma(b0[k], bgx, fma(b1[k], bgy, bd[k][v]));
            }
            bgx_all[v] = bgx;
            bgy_all[v] = bgy;
        }
        if (GRAD == 2) {
            const double* W = &m.c_gg[(size_t)c * 12];
            const double ginv = __ldg(&m.c_ginv[c]);
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const int out = __ldg(&m.c_ggout[c * 3 + j]);
                const double gC = __ldg(&W[4 * j]), gC1 = __ldg(&W[4 * j + 1]);
                const double Sx = __ldg(&W[4 * j + 2]), Sy = __ldg(&W[4 * j + 3]);
                double bf[4];
#pragma unroll
                for (int v = 0; v < 4; v++) {
                    const double b_phif = ginv * (Sx * bgx_all[v] + Sy * bgy_all[v]);
                    lu[v] += out >= 0 ? gC * b_phif : b_phif;
                    bf[v] = out >= 0 ? gC1 * b_phif : 0.0;
                }
                bgg[(size_t)c * 3 + j] = mk4(bf[0], bf[1], bf[2], bf[3]);
            }
        }
    }
    lam_dir[c] = mk4(lu[0], lu[1], lu[2], lu[3]);
    for (int k = 0; k < 3; k++) bdU[(size_t)c * 3 + k] = mk4(bd[k][0], bd[k][1], bd[k][2], bd[k][3]);
}

// ---- per cell: neighbours' LSQ adjoints and the stage's Runge-Kutta combination ------
// U_s = a U_0 + b (c U_in + dt R(U_in)):  lam_in = b (c lam_s + dt J^T lam_s);  acc0 (+)= a lam_s.
// (c = 1 for forward Euler and SSP-RK3; the Kutta stages pass their residual's seed as lam_s
// with c = 0 and combine the results with k_adj_lincomb.)
// acc_mode 0: acc0 = a lam_s; 1: acc0 += a lam_s; 2: nothing; 3 (a = 0, the first stage, whose
// input is U_0 itself): lam_in += acc0.  dot_part[block] = sum over the block's cells of
// lam_s . R_s (= d loss / d dt through this stage, divided by b), summed in a fixed order.
__global__ void __launch_bounds__(256) k_adj_combine(MeshView m, const int* __restrict__ rev,
                                                     const d4* __restrict__ lam_dir, const d4* __restrict__ bdU,
                                                     const d4* __restrict__ lam_s, const d4* __restrict__ R_s,
                                                     const double* __restrict__ dt_p, double a, double b, double ci,
                                                     int acc_mode, d4* __restrict__ lam_in, d4* __restrict__ acc0,
                                                     int linear, double* __restrict__ dot_part,
                                                     const int* __restrict__ ggrev, const d4* __restrict__ bgg) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double dot = 0.0;
    if (c < m.N) {
        const d4 ld = ld4(&lam_dir[c]);
        double r[4] = {ld.x, ld.y, ld.z, ld.w};
        if (linear) {
            const int nnb = __ldg(&m.c_nnb[c]);
            for (int k = 0; k < nnb; k++) {
                const d4 own = ld4(&bdU[(size_t)c * 3 + k]);  // d/dU_c of U_k - U_c
                r[0] -= own.x; r[1] -= own.y; r[2] -= own.z; r[3] -= own.w;
                const int q = __ldg(&m.c_nbr[c * 3 + k]);
                const d4 other = ld4(&bdU[(size_t)q * 3 + __ldg(&rev[c * 3 + k])]);  // c is a neighbour of q
                r[0] += other.x; r[1] += other.y; r[2] += other.z; r[3] += other.w;
            }
            if (bgg) {  // Green-Gauss: c is the cell beyond face ggrev[c][k] of its k-th face cell
                for (int k = 0; k < 3; k++) {
                    const int q = __ldg(&m.c_ggout[c * 3 + k]);
                    if (q < 0) continue;
                    const d4 o = ld4(&bgg[(size_t)q * 3 + __ldg(&ggrev[c * 3 + k])]);
                    r[0] += o.x; r[1] += o.y; r[2] += o.z; r[3] += o.w;
                }
            }
        }
        const double dt = *dt_p;
        const d4 ls = ld4(&lam_s[c]);
        const d4 rs = ld4(&R_s[c]);
        dot = fma(ls.x, rs.x, fma(ls.y, rs.y, fma(ls.z, rs.z, mul(ls.w, rs.w))));
        d4 li = mk4(mul(b, fma(dt, r[0], mul(ci, ls.x))), mul(b, fma(dt, r[1], mul(ci, ls.y))),
                    mul(b, fma(dt, r[2], mul(ci, ls.z))), mul(b, fma(dt, r[3], mul(ci, ls.w))));
        if (acc_mode == 0) {
            acc0[c] = mk4(mul(a, ls.x), mul(a, ls.y), mul(a, ls.z), mul(a, ls.w));
        } else if (acc_mode == 1) {
            const d4 o = acc0[c];
            acc0[c] = mk4(fma(a, ls.x, o.x), fma(a, ls.y, o.y), fma(a, ls.z, o.z), fma(a, ls.w, o.w));
        } else if (acc_mode == 3) {
            const d4 o = acc0[c];
            li = mk4(o.x + li.x, o.y + li.y, o.z + li.z, o.w + li.w);
        }
        lam_in[c] = li;
    }
    for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
    __shared__ double sm[8];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = dot;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < 8; i++) t += sm[i];
        dot_part[blockIdx.x] = t;
    }
}

// out = c0 x0 + c1 x1 + c2 x2 + c3 x3 per cell (null terms skipped): the Kutta stages' seeds
__global__ void __launch_bounds__(256) k_adj_lincomb(int n, d4* out, double c0, const d4* x0,
                                                     double c1, const d4* x1, double c2, const d4* x2, double c3,
                                                     const d4* x3) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double cs[4] = {c0, c1, c2, c3};
    const d4* xs[4] = {x0, x1, x2, x3};
    double r[4] = {0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (!xs[k]) continue;
        const d4 x = ld4(&xs[k][c]);
        r[0] = fma(cs[k], x.x, r[0]);
        r[1] = fma(cs[k], x.y, r[1]);
        r[2] = fma(cs[k], x.z, r[2]);
        r[3] = fma(cs[k], x.w, r[3]);
    }
    out[c] = mk4(r[0], r[1], r[2], r[3]);
}

// smallest cell index whose CFL vol / alpha equals the step's minimum
__global__ void __launch_bounds__(256) k_adj_argmin(MeshView m, const double* __restrict__ alpha,
                                                    const double* __restrict__ alpha_vis, int ns, double CFL,
                                                    const unsigned long long* dtmin, int* out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    const double d = dmin(1e10, ns ? dt_cell<true>(c, m, alpha, alpha_vis, CFL) : dt_cell<false>(c, m, alpha, nullptr, CFL));
    if ((unsigned long long)__double_as_longlong(d) == *dtmin) atomicMin(out, c);
}

// lambda_dt = sum over stages of b_s (lam_s . R_s), the combine kernel's block partials
// reduced in a fixed order (thread-strided sums, then a shared-memory tree); then thread 0 adds
// lambda_dt d(dt)/dU_0 to lam, dt = CFL vol_c / alpha_c at the minimising cell c
constexpr int kDtThreads = 256;
__global__ void __launch_bounds__(kDtThreads) k_adj_dt(const double* __restrict__ part, int nb, int nstages,
                                                       double b0, double b1, double b2, const d4* __restrict__ U0,
                                                       MeshView m, Gas g, double CFL, const int* cstar,
                                                       const double* dt_info, d4* lam, int ns, double value_1) {
    // lt = sum over the stages of b_s (sum of the stage's block partials): each thread sums its
    // share of every stage, then the warps and the block reduce in a fixed order
    __shared__ double red[kDtThreads / 32];
    double x = 0.0;
    for (int st = 0; st < nstages; st++) {
        const double bs = st == 0 ? b0 : (st == 1 ? b1 : b2);
        double y = 0.0;
        for (int i = threadIdx.x; i < nb; i += kDtThreads) y += part[(size_t)st * nb + i];
        x = fma(bs, y, x);
    }
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    double lt = 0.0;
    for (int i = 0; i < kDtThreads / 32; i++) lt += red[i];
    const int c = *cstar;
    if (c < 0 || c >= m.N) return;
    if (dt_info[0] != dt_info[1]) return;  // clamped to the end time: dt does not depend on U
    if (lt == 0.0) return;
    // d dt / d U at the argmin cell: dt = CFL vol / alpha, alpha = the cell's sum over its edges
    // (k_alpha, dt_cell); one lane per edge, the sums and the updates of lam in the edge order
    const int k0 = m.dt_ptr[c], ne = m.dt_ptr[c + 1] - k0;
    if (ne > 32) return;  // a cell has at most four edge slots
    const bool act = lane < ne;
    const int e = act ? m.dt_edge[k0 + lane] : 0;
    const int L = act ? m.e_L[e] : 0, R = act ? m.e_R[e] : -1;
    Prim wl{}, wr{};
    d4 w = mk4(0, 0, 0, 0);
    double term = 0.0, nxl = 0.0, nyl = 0.0, ir = 0.0, sq = 0.0, un = 0.0, gm2 = 0.0, gm3 = 0.0;
    if (act) {
        wl = to_prim(U0[L], g);
        w = mk4(wl.r, wl.u, wl.v, wl.p);
        if (R != -1) {
            wr = to_prim(U0[R], g);
            w = mk4(mul(0.5, w.x + wr.r), mul(0.5, w.y + wr.u), mul(0.5, w.z + wr.v), mul(0.5, w.w + wr.p));
        }
        const double* gm = &m.e_geom[(size_t)e * 8];
        gm2 = gm[2];
        gm3 = gm[3];
        nxl = mul(gm[0], gm2);
        nyl = mul(gm[1], gm2);
        un = fma(w.y, nxl, mul(w.z, nyl));
        ir = rcp(w.x);
        sq = sqrt(mul(mul(g.gamma, w.w), ir));
        term = fma(sq, gm3, fabs(un));
        if (ns) {  // the viscous spectral radius (k_alpha<true>, dt_cell<true>)
            const double T = mul(w.w / g.R, ir);
            const double mu = mul(mul(g.C1, mul(T, sqrt(T))), rcp(T + 110.4));
            term = mul(mul(mul(mul(2.0, gm2), value_1), mu), ir);  // alpha_vis; scaled by 1/vol below
        }
    }
    const double vol = m.c_vol[c];
    double alpha = 0.0;
    for (int k = 0; k < ne; k++) {  // the cell's sum in the edge order, as dt_cell forms it
        const double tk = __shfl_sync(0xffffffffu, term, k);
        const double sk = ns ? __shfl_sync(0xffffffffu, fma(sq, gm3, fabs(un)), k) : tk;
        alpha += sk;
        if (ns) alpha = fma(tk, rcp(vol), alpha);
    }
    const double dt = mul(mul(CFL, vol), rcp(alpha));
    const double b_alpha = mul(lt, -mul(dt, rcp(alpha)));
    d4 buL = mk4(0, 0, 0, 0), buR = mk4(0, 0, 0, 0);
    if (act) {
        const double b_un = mul(b_alpha, sgn(un));
        const double b_s = mul(b_alpha, gm3);
        const double b_p = sq > 0 ? mul(mul(b_s, g.gamma), ir) / (2.0 * sq) : 0.0;
        const double b_ir = sq > 0 ? mul(mul(b_s, g.gamma), w.w) / (2.0 * sq) : 0.0;
        Prim bw{};
        bw.r = -mul(mul(b_ir, ir), ir);
        bw.u = mul(b_un, nxl);
        bw.v = mul(b_un, nyl);
        bw.p = b_p;
        if (ns) {  // alpha_vis = 2 L value_1 mu(T) / rho / vol, T = p / (R rho)
            const double T = mul(w.w / g.R, ir);
            const double mu = mul(mul(g.C1, mul(T, sqrt(T))), rcp(T + 110.4));
            const double b_av = mul(b_alpha, rcp(vol));
            const double kk = mul(mul(2.0, gm2), value_1);
            const double b_mu = mul(mul(b_av, kk), ir);
            const double b_T = mul(mul(b_mu, mu), 1.5 / T - 1.0 / (T + 110.4));
            const double b_irv = fma(mul(b_av, kk), mu, mul(b_T, w.w) / g.R);
            bw.r = fma(-mul(b_irv, ir), ir, bw.r);
            bw.p = fma(b_T, ir / g.R, bw.p);
        }
        const double f = (R != -1) ? 0.5 : 1.0;
        const Prim bc{mul(f, bw.r), mul(f, bw.u), mul(f, bw.v), mul(f, bw.p), 0.0};
        to_prim_vjp(U0[L], wl, g, bc, buL);
        if (R != -1) to_prim_vjp(U0[R], wr, g, bc, buR);
    }
    for (int k = 0; k < ne; k++) {  // the updates of lam in the edge order (edges share cells)
        if (lane == k) {
            d4 o = lam[L];
            lam[L] = mk4(o.x + buL.x, o.y + buL.y, o.z + buL.z, o.w + buL.w);
            if (R != -1) {
                o = lam[R];
                lam[R] = mk4(o.x + buR.x, o.y + buR.y, o.z + buR.z, o.w + buR.w);
            }
        }
        __syncwarp();
    }
}

// seed in the reference's numbering -> device order (and back for the gradient)
__global__ void __launch_bounds__(256) k_adj_copy(const d4* __restrict__ src, d4* __restrict__ dst, int N) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < N) dst[c] = src[c];
}

}  // namespace dev

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
#define AK(call)                                                                                      \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return fail(FVGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

static inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

struct Adjoint {
    Solver* s = nullptr;
    int K = 0, S = 0, nseg = 0, nst = 0;
    std::vector<void*> owned;
    std::vector<d4*> chk;          // U at the start of each segment
    double* d_chk_t = nullptr;     // t at the start of each segment
    std::vector<d4*> seg_states;   // per step of a segment: U_0, U_1, U_2
    std::vector<d4*> seg_R;           // per stage of a segment's steps: the residual R(U_in)
    std::vector<double*> seg_tape;    // per stage of a segment's steps: the edge tape (kTapeFields x E)
    std::vector<int*> seg_tflags;
    std::vector<dev::CellTape> seg_ctape;  // per stage: the limiter record (Barth only)
    std::vector<d4*> seg_gx, seg_gy;  // per stage (Navier-Stokes): the limited gradients the viscous flux read
    d4 *d_avu = nullptr, *d_avgx = nullptr, *d_avgy = nullptr;  // per edge: viscous adjoints of U, Gx, Gy
    const d4 *vis_gx = nullptr, *vis_gy = nullptr;  // the stage in hand's gradients (set by step_vjp)
    double* d_seg_dt = nullptr;    // per step: dt, dt_raw
    int* d_seg_cstar = nullptr;    // per step: the minimising cell
    d4 *d_lam = nullptr, *d_lam_in = nullptr, *d_acc0 = nullptr, *d_aL = nullptr, *d_aR = nullptr;
    d4 *d_k_a2 = nullptr, *d_k_a1 = nullptr, *d_k_seed = nullptr;  // Kutta RK3: lam_U2, lam_U1, a seed
    d4* d_bgg = nullptr;    // Green-Gauss: per face, the adjoint of the cell beyond it
    int* d_ggrev = nullptr; // Green-Gauss: the matching face of the cell beyond
    d4 *d_lamdir = nullptr, *d_bdU = nullptr, *d_keepU = nullptr;
    int *d_rlist = nullptr, *d_rev = nullptr;
    double* d_dotp = nullptr;
    double* d_one = nullptr;  // 1.0: the time step of rhs_vjp's reverse
    bool ready = false;
    bool last_kept = false;  // the segment buffers (set 0) hold the last segment's steps
    // segment records: nsets sets of S steps x nst stages; record_step writes set rec_set,
    // step_vjp reads set rev_set
    int nsets = 1, rec_set = 0, rev_set = 0;
    cudaStream_t rstream = nullptr;     // the reverse sweep's stream beside a recomputation
    cudaStream_t vjp_stream = nullptr;  // where the VJPs are enqueued (null: the solver's stream)
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // what the workspace was laid out for: a forward with the same steps, checkpoints, overlap
    // mode and CFL (captured by value in the graphs) reuses it, graphs included
    int req_ncheck = 0, req_overlap = 0;
    double req_cfl = 0.0;
    bool reusable(int nsteps, int ncheck) const {
        return K == nsteps && req_ncheck == ncheck && req_overlap == s->adj_overlap && req_cfl == s->p.CFL;
    }
    size_t at(int set, int slot, int si) const { return ((size_t)set * S + slot) * nst + si; }
    size_t step_at(int set, int slot) const { return (size_t)set * S + slot; }
    cudaStream_t vstream() const { return vjp_stream ? vjp_stream : s->stream; }
    int seg_len(int i) const { return std::min(S, K - i * S); }
    long long restricted_before = 0;
    double ms_fwd = 0, ms_bwd = 0;

    // CUDA graphs of a segment's reverse-sweep work (its recorded recomputation, where needed,
    // and the VJPs of its steps), captured once per shape and replayed: a segment enqueues
    // several hundred short kernels and copies whose launch gaps the graph removes.  The VJPs
    // exchange the adjoint buffers d_lam and d_lam_in on the host as they are enqueued, so a
    // graph belongs to the assignment of the two buffers at the segment's start and records
    // the assignment it leaves.
    struct SegGraph {
        int n = 0;        // steps reversed
        int nrec = 0;     // steps recorded (before the reverse, or beside it when overlap)
        bool overlap = false;
        int rev = 0, rec = 0;  // the record sets read and written
        d4* lam0 = nullptr;
        d4* lam_out = nullptr;
        d4* lam_in_out = nullptr;
        cudaGraphExec_t exec = nullptr;
        long long launches = 0;
    };
    std::vector<SegGraph> seg_graphs;

    ~Adjoint() {
        for (auto& g : seg_graphs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        for (void* q : owned) cudaFree(q);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (rstream) cudaStreamDestroy(rstream);
    }
    template <class T>
    int alloc(T*& p, size_t n) {
        p = nullptr;
        AK(cudaMalloc((void**)&p, (n ? n : 1) * sizeof(T)));
        owned.push_back((void*)p);
        return 0;
    }

    // the records of one segment (S steps x nst stages) in set `set`
    int alloc_set(int set) {
        const int N = s->N, E = s->E;
        int rc;
        for (int k = 0; k < S; k++)
            for (int si = 0; si < nst; si++) {
                const size_t i = at(set, k, si);
                if ((rc = alloc(seg_states[i], N)) || (rc = alloc(seg_R[i], N)) ||
                    (rc = alloc(seg_tape[i], (size_t)dev::kTapeFields * E)) || (rc = alloc(seg_tflags[i], E)))
                    return rc;
                if (!seg_gx.empty() && ((rc = alloc(seg_gx[i], N)) || (rc = alloc(seg_gy[i], N)))) return rc;
                if (!seg_ctape.empty()) {
                    dev::CellTape& t = seg_ctape[i];
                    if ((rc = alloc(t.gx, N)) || (rc = alloc(t.gy, N)) || (rc = alloc(t.phi, N)) ||
                        (rc = alloc(t.rden, N)) || (rc = alloc(t.code, N)))
                        return rc;
                }
            }
        return 0;
    }

    // rhs_only: the workspace of one recorded residual (rhs_vjp), whatever the time scheme
    int setup(Solver* solver, int nsteps, int ncheck, bool rhs_only = false) {
        s = solver;
        const fvgb_params& p = s->p;
        if (p.equation != 1 && p.equation != 2) return fail(FVGB_ERR_ARG, "invalid equation");
        if (p.steady && !rhs_only)
            return fail(FVGB_ERR_UNSUPPORTED, "the adjoint covers time-accurate runs (time.is_steady = 0)");
        if (p.edge_colour)
            return fail(FVGB_ERR_UNSUPPORTED, "the adjoint differentiates the gathered residual ([gpu] edge_colour = 0)");
        if (p.flux_scheme != 2001 && p.flux_scheme != 2002) return fail(FVGB_ERR_ARG, "invalid flux scheme");
        if (p.time_advance != 3101 && p.time_advance != 3103 && p.time_advance != 3104)
            return fail(FVGB_ERR_ARG, "invalid time_advance");
        for (int e = s->L.E_int; e < s->E; e++) {
            const int bt = s->L.e_bc[e];
            if (bt != BC_WALL_NONVISCOUS && bt != BC_WALL_ADIABAT && bt != BC_SYMMETRY && bt != BC_INLET && bt != BC_OUTLET && bt != BC_INF && bt != BC_DSR)
                return fail(FVGB_ERR_UNSUPPORTED, "unknown boundary type");
        }
        K = nsteps;
        req_ncheck = ncheck;
        req_overlap = s->adj_overlap;
        req_cfl = p.CFL;
        ncheck = std::max(1, std::min(ncheck, K));
        S = (K + ncheck - 1) / ncheck;
        nseg = (K + S - 1) / S;
        nst = (rhs_only || p.time_advance == 3101) ? 1 : 3;
        const int N = s->N, E = s->E;
        // R-list flag per edge (interior non-periodic edges appear in R's edge list)
        std::vector<int> rlist(E, 0);
        for (int c = 0; c < N; c++)
            for (int j = 0; j < 3; j++) {
                const int r = s->L.c_edge[(size_t)c * 3 + j];
                if (r < 0) rlist[~r] = 1;
            }
        // reverse neighbour slots: c is the rev[c][k]-th neighbour of its k-th neighbour
        std::vector<int> rev((size_t)3 * N, 0);
        for (int c = 0; c < N; c++)
            for (int k = 0; k < s->L.c_nnb[c]; k++) {
                const int q = s->L.c_nbr[(size_t)c * 3 + k];
                for (int j = 0; j < s->L.c_nnb[q]; j++)
                    if (s->L.c_nbr[(size_t)q * 3 + j] == c) rev[(size_t)c * 3 + k] = j;
            }
        int rc;
        if ((rc = alloc(d_rlist, E)) || (rc = alloc(d_rev, 3 * (size_t)N))) return rc;
        AK(cudaMemcpyAsync(d_rlist, rlist.data(), sizeof(int) * E, cudaMemcpyHostToDevice, s->stream));
        AK(cudaMemcpyAsync(d_rev, rev.data(), sizeof(int) * 3 * (size_t)N, cudaMemcpyHostToDevice, s->stream));
        chk.assign(nseg, nullptr);
        for (int i = 0; i < nseg; i++)
            if ((rc = alloc(chk[i], N))) return rc;
        if ((rc = alloc(d_chk_t, nseg))) return rc;
        // two sets of segment records are laid out; the second is allocated only where it fits
        const bool grads = p.reconstruct == 3002 || p.equation == 2;  // the step computes gradients
        const size_t per = (size_t)S * nst;
        seg_states.assign(2 * per, nullptr);
        seg_R.assign(2 * per, nullptr);
        seg_tape.assign(2 * per, nullptr);
        seg_tflags.assign(2 * per, nullptr);
        seg_ctape.assign(grads && p.limiter == 1 ? 2 * per : 0, dev::CellTape());
        if (p.equation == 2) {
            seg_gx.assign(2 * per, nullptr);
            seg_gy.assign(2 * per, nullptr);
            if ((rc = alloc(d_avu, E)) || (rc = alloc(d_avgx, E)) || (rc = alloc(d_avgy, E))) return rc;
        }
        const bool want2 = !rhs_only && s->adj_overlap && nseg > 1;
        size_t free0 = 0, free1 = 0, total = 0;
        if (want2) AK(cudaMemGetInfo(&free0, &total));
        if ((rc = alloc_set(0))) return rc;
        nsets = 1;
        if (want2) {
            AK(cudaMemGetInfo(&free1, &total));
            const size_t used = free0 > free1 ? free0 - free1 : 0;
            if (free1 > used + ((size_t)1 << 30)) {  // room for a second set and 1 GiB besides
                if ((rc = alloc_set(1))) return rc;
                AK(cudaStreamCreateWithFlags(&rstream, cudaStreamNonBlocking));
                AK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
                AK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
                nsets = 2;
            }
        }
        const int nb = nblk(N, 256);
        if ((rc = alloc(d_seg_dt, 4 * (size_t)S)) || (rc = alloc(d_seg_cstar, 2 * (size_t)S)) || (rc = alloc(d_lam, N)) ||
            (rc = alloc(d_lam_in, N)) || (rc = alloc(d_acc0, N)) || (rc = alloc(d_aL, E)) || (rc = alloc(d_aR, E)) ||
            (rc = alloc(d_lamdir, N)) || (rc = alloc(d_keepU, N)) || (rc = alloc(d_bdU, 3 * (size_t)N)) ||
            (rc = alloc(d_dotp, (size_t)nb * 3)))
            return rc;
        if (p.time_advance == 3103 && !rhs_only &&
            ((rc = alloc(d_k_a2, N)) || (rc = alloc(d_k_a1, N)) || (rc = alloc(d_k_seed, N))))
            return rc;
        if ((rc = alloc(d_one, 1))) return rc;
        static const double kOne = 1.0;
        AK(cudaMemcpyAsync(d_one, &kOne, sizeof(double), cudaMemcpyHostToDevice, s->stream));
        if (p.reconstruct == 3002 && p.gradient == 2) {
            // ggrev[c][k]: the face of cell q = ggout[c][k] whose far cell is c; where c and q
            // share several faces (tiny periodic meshes), the m-th such face of c is paired with
            // the m-th of q
            std::vector<int> ggrev((size_t)3 * N, 0);
            const std::vector<int>& go = s->L.c_ggout;
            for (int c = 0; c < N; c++)
                for (int k = 0; k < 3; k++) {
                    const int q = go[(size_t)c * 3 + k];
                    if (q < 0) continue;
                    int m = 0;
                    for (int k2 = 0; k2 < k; k2++) m += go[(size_t)c * 3 + k2] == q;
                    int j = 0;
                    for (; j < 3; j++)
                        if (go[(size_t)q * 3 + j] == c && m-- == 0) break;
                    if (j == 3) return fail(FVGB_ERR_MESH, "Green-Gauss face cells are not mutual");
                    ggrev[(size_t)c * 3 + k] = j;
                }
            if ((rc = alloc(d_ggrev, 3 * (size_t)N)) || (rc = alloc(d_bgg, 3 * (size_t)N))) return rc;
            AK(cudaMemcpyAsync(d_ggrev, ggrev.data(), sizeof(int) * 3 * (size_t)N, cudaMemcpyHostToDevice,
                               s->stream));
            AK(cudaStreamSynchronize(s->stream));
        }
        return 0;
    }

    // one forward step launched kernel by kernel, keeping what the reverse sweep needs
    int record_step(int slot) {
        Solver& v = *s;
        cudaStream_t st = v.stream;
        const bool copy = v.p.time_advance != 3101;
        AK(cudaMemcpyAsync(seg_states[at(rec_set, slot, 0)], v.d_U, sizeof(d4) * v.N, cudaMemcpyDeviceToDevice, st));
        dev::launch_prim(st, v.d_U, v.d_U0, v.d_prim, v.N, v.gas, copy);
        const double value_1 = std::max(4.0 / 3.0, v.p.gamma / v.p.Pr);
        dev::launch_dt(st, v.d_prim, v.mv, v.gas, value_1, v.p.CFL, v.p.equation == 2, v.d_alpha, v.d_alpha_vis,
                       &v.d_state->dtmin_bits, v.d_status);
        AK(cudaMemsetAsync(d_seg_cstar + step_at(rec_set, slot), 0x7f, sizeof(int), st));
        dev::k_adj_argmin<<<nblk(v.N, 256), 256, 0, st>>>(v.mv, v.d_alpha, v.d_alpha_vis, v.p.equation == 2 ? 1 : 0,
                                                          v.p.CFL, &v.d_state->dtmin_bits, d_seg_cstar + step_at(rec_set, slot));
        dev::launch_dt_final(st, v.d_state, true);
        AK(cudaMemcpyAsync(d_seg_dt + 2 * step_at(rec_set, slot), &v.d_state->dt, sizeof(double), cudaMemcpyDeviceToDevice, st));
        AK(cudaMemcpyAsync(d_seg_dt + 2 * step_at(rec_set, slot) + 1, &v.d_state->dt_raw, sizeof(double), cudaMemcpyDeviceToDevice, st));
        // each stage's residual and edge tape go to the segment's buffers (kept for the reverse sweep)
        auto stage = [&](int si, int kind) {
            v.d_rec_R = seg_R[at(rec_set, slot, si)];
            v.rec_tape.v = seg_tape[at(rec_set, slot, si)];
            v.rec_tape.flags = seg_tflags[at(rec_set, slot, si)];
            v.rec_tape.E = v.E;
            if (!seg_ctape.empty()) v.rec_ctape = seg_ctape[at(rec_set, slot, si)];
            v.enqueue_stage(kind);
            if (!seg_gx.empty()) {  // the gradients this stage's viscous fluxes read
                AK(cudaMemcpyAsync(seg_gx[at(rec_set, slot, si)], v.d_Gx, sizeof(d4) * v.N, cudaMemcpyDeviceToDevice,
                                   st));
                AK(cudaMemcpyAsync(seg_gy[at(rec_set, slot, si)], v.d_Gy, sizeof(d4) * v.N, cudaMemcpyDeviceToDevice,
                                   st));
            }
            return 0;
        };
        if (v.p.time_advance == 3101) {
            if (int rc = stage(0, dev::STAGE_EULER)) return rc;
        } else {
            const bool kutta = v.p.time_advance == 3103;
            if (int rc = stage(0, kutta ? dev::STAGE_RK3_1 : dev::STAGE_SSP_1)) return rc;
            AK(cudaMemcpyAsync(seg_states[at(rec_set, slot, 1)], v.d_U, sizeof(d4) * v.N, cudaMemcpyDeviceToDevice, st));
            if (int rc = stage(1, kutta ? dev::STAGE_RK3_2 : dev::STAGE_SSP_2)) return rc;
            AK(cudaMemcpyAsync(seg_states[at(rec_set, slot, 2)], v.d_U, sizeof(d4) * v.N, cudaMemcpyDeviceToDevice, st));
            if (int rc = stage(2, kutta ? dev::STAGE_RK3_3 : dev::STAGE_SSP_3)) return rc;
        }
        v.d_rec_R = nullptr;
        v.rec_tape = dev::EdgeTape();
        v.rec_ctape = dev::CellTape();
        dev::launch_restrict(st, v.d_U, v.mv, v.d_cell_ref, v.d_cell_new, v.d_flags, v.d_flag_count, Solver::kFlagCap,
                             v.p.restrict_ref, v.gas, v.d_status);
        AK(cudaGetLastError());
        return 0;
    }

    // one stage VJP: lam_s (seed, default d_lam) -> lam_in (out, default d_lam_in), acc0,
    // partial lam_s . R_s in dot slot; tape and ct: the stage's records of its input state
    int stage_vjp(const d4* Uin, const dev::EdgeTape& tape, const dev::CellTape& ct, const d4* Rs,
                  const double* dt_p, double a, double b, int acc_mode, int dot_slot, const d4* seed = nullptr,
                  d4* out = nullptr, double ci = 1.0) {
        if (!seed) seed = d_lam;
        if (!out) out = d_lam_in;
        Solver& v = *s;
        cudaStream_t st = vstream();
        const bool ns = v.p.equation == 2;
        const bool linear = v.p.reconstruct == 3002 || ns;  // the step computes (and reads) gradients
        const int nbE = nblk(v.E, dev::kEdgeThreads), nbN = nblk(v.N, 256);
        double* dp = d_dotp + (size_t)dot_slot * nbN;
#define FVGB_ADJ_EDGE(FL, NSV)                                                                                  \
    dev::k_adj_edge<FL, NSV><<<nbE, dev::kEdgeThreads, 0, st>>>(tape, v.mv, v.gas, v.bc, seed, d_rlist, d_aL, d_aR, \
                                                                Uin, vis_gx, vis_gy, d_avu, d_avgx, d_avgy)
        if (v.p.flux_scheme == 2002) { if (ns) FVGB_ADJ_EDGE(dev::FLUX_ROE, true); else FVGB_ADJ_EDGE(dev::FLUX_ROE, false); }
        else { if (ns) FVGB_ADJ_EDGE(dev::FLUX_LLF, true); else FVGB_ADJ_EDGE(dev::FLUX_LLF, false); }
#undef FVGB_ADJ_EDGE
        const int* fl = tape.flags;
        const bool gg = linear && v.p.gradient == 2;
#define FVGB_ADJ_CELL(LIN, BAR, GR, NSV)                                                                           \
    dev::k_adj_cell<LIN, BAR, GR, NSV><<<nbN, 256, 0, st>>>(v.mv, d_aL, d_aR, fl, ct, d_lamdir, d_bdU, d_bgg, d_avu, \
                                                           d_avgx, d_avgy)
        if (!linear) FVGB_ADJ_CELL(false, false, 1, false);
        else if (ns) {
            if (v.p.limiter == 1) { if (gg) FVGB_ADJ_CELL(true, true, 2, true); else FVGB_ADJ_CELL(true, true, 1, true); }
            else { if (gg) FVGB_ADJ_CELL(true, false, 2, true); else FVGB_ADJ_CELL(true, false, 1, true); }
        } else if (v.p.limiter == 1) {
            if (gg) FVGB_ADJ_CELL(true, true, 2, false);
            else FVGB_ADJ_CELL(true, true, 1, false);
        } else {
            if (gg) FVGB_ADJ_CELL(true, false, 2, false);
            else FVGB_ADJ_CELL(true, false, 1, false);
        }
#undef FVGB_ADJ_CELL
        dev::k_adj_combine<<<nbN, 256, 0, st>>>(v.mv, d_rev, d_lamdir, d_bdU, seed, Rs, dt_p, a, b, ci, acc_mode,
                                                out, d_acc0, linear ? 1 : 0, dp, gg ? d_ggrev : nullptr,
                                                gg ? d_bgg : nullptr);
        AK(cudaGetLastError());
        return 0;
    }

    // lam (adjoint of U_{n+1}) -> lam (adjoint of U_n) for the step kept in slot
    int step_vjp(int slot) {
        Solver& v = *s;
        cudaStream_t st = vstream();
        const double* dtp = d_seg_dt + 2 * step_at(rev_set, slot);
        const int nbN = nblk(v.N, 256);
        auto R = [&](int si) { return seg_R[at(rev_set, slot, si)]; };
        auto ctp = [&](int si) {
            return seg_ctape.empty() ? dev::CellTape() : seg_ctape[at(rev_set, slot, si)];
        };
        // the stage's recorded gradients for the viscous reverse (Navier-Stokes)
        auto use = [&](int si) {
            vis_gx = seg_gx.empty() ? nullptr : seg_gx[at(rev_set, slot, si)];
            vis_gy = seg_gy.empty() ? nullptr : seg_gy[at(rev_set, slot, si)];
        };
        auto tp = [&](int si) {
            dev::EdgeTape t;
            t.v = seg_tape[at(rev_set, slot, si)];
            t.flags = seg_tflags[at(rev_set, slot, si)];
            t.E = v.E;
            return t;
        };
        int rc;
        double b0 = 1.0, b1 = 0.0, b2 = 0.0;  // b_s of the stages in reverse order
        if (v.p.time_advance == 3101) {
            // U1 = U0 + dt R(U0): a = 0, b = 1
            use(0);
            if ((rc = stage_vjp(seg_states[at(rev_set, slot, 0)], tp(0), ctp(0), R(0), dtp, 0.0, 1.0, 2, 0))) return rc;
            std::swap(d_lam, d_lam_in);
        } else if (v.p.time_advance == 3103) {
            // Kutta RK3: k1 = R(U0), U1 = U0 + dt/2 k1; k2 = R(U1), U2 = U0 - dt k1 + 2 dt k2;
            // k3 = R(U2), U3 = U0 + dt/6 (k1 + 4 k2 + k3).  With L3 = lam (adjoint of U3), the
            // residuals' seeds (adjoints of the k, divided by dt) are
            //   s3 = L3/6,  s2 = 2/3 L3 + 2 L2,  s1 = L3/6 - L2 + L1/2,
            // L2 = dt J2^T s3 and L1 = dt J1^T s2 being the adjoints of U2 and U1, and
            //   lam_U0 = L3 + L2 + L1 + dt J0^T s1;  d loss / d dt = s3.k3 + s2.k2 + s1.k1.
            const d4* U0 = seg_states[at(rev_set, slot, 0)];
            const d4* U1 = seg_states[at(rev_set, slot, 1)];
            const d4* U2 = seg_states[at(rev_set, slot, 2)];
            const int nbk = nblk(v.N, 256);
            // L2 = dt J2^T (L3/6): seed L3, b = 1/6, no identity term
            use(2);
            if ((rc = stage_vjp(U2, tp(2), ctp(2), R(2), dtp, 0.0, 1.0 / 6.0, 2, 0, d_lam, d_k_a2, 0.0))) return rc;
            dev::k_adj_lincomb<<<nbk, 256, 0, st>>>(v.N, d_k_seed, 2.0 / 3.0, d_lam, 2.0, d_k_a2, 0.0, nullptr, 0.0,
                                                    nullptr);
            // L1 = dt J1^T s2
            use(1);
            if ((rc = stage_vjp(U1, tp(1), ctp(1), R(1), dtp, 0.0, 1.0, 2, 1, d_k_seed, d_k_a1, 0.0))) return rc;
            dev::k_adj_lincomb<<<nbk, 256, 0, st>>>(v.N, d_k_seed, 1.0 / 6.0, d_lam, -1.0, d_k_a2, 0.5, d_k_a1, 0.0,
                                                    nullptr);
            // dt J0^T s1, then lam_U0
            use(0);
            if ((rc = stage_vjp(U0, tp(0), ctp(0), R(0), dtp, 0.0, 1.0, 2, 2, d_k_seed, d_lam_in, 0.0))) return rc;
            dev::k_adj_lincomb<<<nbk, 256, 0, st>>>(v.N, d_lam, 1.0, d_lam, 1.0, d_k_a2, 1.0, d_k_a1, 1.0, d_lam_in);
            AK(cudaGetLastError());
            b0 = 1.0 / 6.0;  // slot 0 holds L3 . k3
            b1 = 1.0;
            b2 = 1.0;
        } else {
            const d4* U0 = seg_states[at(rev_set, slot, 0)];
            const d4* U1 = seg_states[at(rev_set, slot, 1)];
            const d4* U2 = seg_states[at(rev_set, slot, 2)];
            // U3 = 1/3 U0 + 2/3 (U2 + dt R(U2))
            use(2);
            if ((rc = stage_vjp(U2, tp(2), ctp(2), R(2), dtp, 1.0 / 3.0, 2.0 / 3.0, 0, 0))) return rc;
            std::swap(d_lam, d_lam_in);
            // U2 = 3/4 U0 + 1/4 (U1 + dt R(U1))
            use(1);
            if ((rc = stage_vjp(U1, tp(1), ctp(1), R(1), dtp, 0.75, 0.25, 1, 1))) return rc;
            std::swap(d_lam, d_lam_in);
            // U1 = U0 + dt R(U0); U0 also feeds stages 2 and 3 directly (acc0)
            use(0);
            if ((rc = stage_vjp(U0, tp(0), ctp(0), R(0), dtp, 0.0, 1.0, 3, 2))) return rc;
            std::swap(d_lam, d_lam_in);
            b0 = 2.0 / 3.0;
            b1 = 0.25;
            b2 = 1.0;
        }
        dev::k_adj_dt<<<1, dev::kDtThreads, 0, st>>>(d_dotp, nbN, nst, b0, b1, b2, seg_states[at(rev_set, slot, 0)],
                                                    v.mv, v.gas, v.p.CFL, d_seg_cstar + step_at(rev_set, slot), dtp, d_lam,
                                                    v.p.equation == 2 ? 1 : 0,
                                                    std::max(4.0 / 3.0, v.p.gamma / v.p.Pr));
        AK(cudaGetLastError());
        return 0;
    }

    // (dR/dU)^T seed at U, R = fvgb_rhs(U): one recorded evaluation of R made as
    // Solver::rhs makes it ("dsr" edges at the handle's time), then the stage reverse
    // with dt = 1 and no identity term (b = 1, ci = 0: lam_in = J^T seed exactly)
    int rhs_vjp(const double* U, const double* seed, double* grad) {
        Solver& v = *s;
        cudaStream_t st = v.stream;
        int rc;
        if ((rc = v.set_state(U))) return rc;
        const bool ns = v.p.equation == 2;
        const dev::CellTape ct = seg_ctape.empty() ? dev::CellTape() : seg_ctape[0];
        if (v.needs_gradient()) {
            dev::launch_grad(st, v.p.gradient, v.p.limiter == 1, v.d_U, v.mv, v.d_Gx, v.d_Gy, ct.gx ? &ct : nullptr);
            v.launches += 1;
        }
        dev::BcData b = v.bc;
        b.clock_t0 = &v.d_state->t;
        b.clock_dt = &v.d_state->dt;
        b.clock_frac = 0.0;
        dev::EdgeTape tp;
        tp.v = seg_tape[0];
        tp.flags = seg_tflags[0];
        tp.E = v.E;
        dev::launch_flux(st, v.p.flux_scheme, v.p.reconstruct == 3002, ns, v.d_U, v.d_Gx, v.d_Gy, v.mv, v.gas, b,
                         v.d_F, v.d_status, &tp);
        dev::launch_update(st, dev::STAGE_RHS, v.d_U, v.d_U0, v.d_K1, seg_R[0], v.d_F, v.mv, v.d_state, v.gas,
                           v.d_flags, v.d_flag_count, Solver::kFlagCap, v.d_status);
        v.launches += 1 + (v.mv.E_int > 0) + (v.mv.E > v.mv.E_int);
        AK(cudaMemcpyAsync(v.d_stage, seed, sizeof(double) * 4 * v.N, cudaMemcpyHostToDevice, st));
        dev::launch_scatter_in(st, v.d_stage, d_lam, v.d_cell_new, v.N);
        vis_gx = ns ? v.d_Gx : nullptr;  // the viscous reverse reads the gradients of this evaluation
        vis_gy = ns ? v.d_Gy : nullptr;
        if ((rc = stage_vjp(v.d_U, tp, ct, seg_R[0], d_one, 0.0, 1.0, 2, 0, d_lam, d_lam_in, 0.0))) return rc;
        v.launches += 4;
        dev::launch_gather_out(st, d_lam_in, v.d_stage, v.d_cell_new, v.N);
        AK(cudaMemcpyAsync(grad, v.d_stage, sizeof(double) * 4 * v.N, cudaMemcpyDeviceToHost, st));
        AK(cudaStreamSynchronize(st));
        return v.check_status();
    }

    // the state and time at the start of segment i
    int load_segment(int i) {
        Solver& v = *s;
        AK(cudaMemcpyAsync(v.d_U, chk[i], sizeof(d4) * v.N, cudaMemcpyDeviceToDevice, v.stream));
        AK(cudaMemcpyAsync(&v.d_state->t, d_chk_t + i, sizeof(double), cudaMemcpyDeviceToDevice, v.stream));
        return 0;
    }

    // runs segment i's steps kernel by kernel, keeping each step's states (record_step)
    int record_segment(int i) {
        Solver& v = *s;
        AK(cudaMemcpyAsync(&v.d_state->T, &v.p.T_end, sizeof(double), cudaMemcpyHostToDevice, v.stream));
        const int n = std::min(S, K - i * S);
        int rc;
        for (int k = 0; k < n; k++)
            if ((rc = record_step(k))) return rc;
        return 0;
    }

    // segment work of the reverse sweep (see SegGraph): records nrec steps of a segment into
    // set rec_set (its checkpoint already loaded) and reverses the n steps held in set rev_set.
    // Sequential: the recording first, then the reverse, on the solver's stream (the same
    // segment, rec_set == rev_set).  Overlap: the reverse of one segment on rstream beside the
    // recording of the one before it on the solver's stream (rec_set != rev_set), forked and
    // joined with events inside the captured graph.
    int run_graph(int n, int nrec, bool overlap) {
        Solver& v = *s;
        for (const SegGraph& g : seg_graphs)
            if (g.n == n && g.nrec == nrec && g.overlap == overlap && g.rev == rev_set && g.rec == rec_set &&
                g.lam0 == d_lam) {
                AK(cudaGraphLaunch(g.exec, v.stream));
                d_lam = g.lam_out;
                d_lam_in = g.lam_in_out;
                v.launches += g.launches;
                return 0;
            }
        SegGraph g;
        g.n = n;
        g.nrec = nrec;
        g.overlap = overlap;
        g.rev = rev_set;
        g.rec = rec_set;
        g.lam0 = d_lam;
        d4* const lam_in0 = d_lam_in;
        const long long before = v.launches;
        AK(cudaStreamBeginCapture(v.stream, cudaStreamCaptureModeThreadLocal));
        int rc = 0;
        cudaError_t ce = cudaSuccess;
        if (overlap) {
            ce = cudaEventRecord(ev_fork, v.stream);
            if (ce == cudaSuccess) ce = cudaStreamWaitEvent(rstream, ev_fork, 0);
            if (ce == cudaSuccess) vjp_stream = rstream;
        }
        if (ce == cudaSuccess) {
            for (int k = 0; k < nrec && !rc; k++) rc = record_step(k);
            for (int k = n - 1; k >= 0 && !rc; k--) rc = step_vjp(k);
        }
        if (vjp_stream) {  // join the reverse branch whatever happened, so that the capture can end
            vjp_stream = nullptr;
            const cudaError_t c1 = cudaEventRecord(ev_join, rstream);
            const cudaError_t c2 = c1 == cudaSuccess ? cudaStreamWaitEvent(v.stream, ev_join, 0) : c1;
            if (ce == cudaSuccess) ce = c2;
        }
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(v.stream, &graph);
        if (rc || ce != cudaSuccess || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            d_lam = g.lam0;
            d_lam_in = lam_in0;
            v.launches = before;
            if (rc) return rc;
            return fail(FVGB_ERR_CUDA, std::string("adjoint graph capture: ") +
                                           cudaGetErrorString(ce != cudaSuccess ? ce : e));
        }
        g.launches = v.launches - before;
        v.launches = before;
        g.lam_out = d_lam;
        g.lam_in_out = d_lam_in;
        // no node priorities: with the reverse branch first wherever both branches had blocks
        // waiting (cudaGraphInstantiateFlagUseNodePriority, the reverse captured from a stream
        // of the highest priority) the 500-step sweep of the 256x256 mesh took 285 ms, without
        // them 276 ms
        const cudaError_t ei = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) return fail(FVGB_ERR_CUDA, std::string("adjoint graph instantiate: ") + cudaGetErrorString(ei));
        seg_graphs.push_back(g);
        AK(cudaGraphLaunch(g.exec, v.stream));
        v.launches += g.launches;
        return 0;
    }

    int forward(const double* U0, double t0, double* UK) {
        Solver& v = *s;
        int rc;
        if ((rc = v.set_state(U0))) return rc;
        if ((rc = v.set_time(t0))) return rc;
        {
            dev::Status stt;
            AK(cudaMemcpyAsync(&stt, v.d_status, sizeof stt, cudaMemcpyDeviceToHost, v.stream));
            AK(cudaStreamSynchronize(v.stream));
            restricted_before = (long long)stt.restricted;
        }
        cudaEvent_t a, b;
        AK(cudaEventCreate(&a));
        AK(cudaEventCreate(&b));
        AK(cudaEventRecord(a, v.stream));
        for (int i = 0; i < nseg; i++) {
            AK(cudaMemcpyAsync(chk[i], v.d_U, sizeof(d4) * v.N, cudaMemcpyDeviceToDevice, v.stream));
            AK(cudaMemcpyAsync(d_chk_t + i, &v.d_state->t, sizeof(double), cudaMemcpyDeviceToDevice, v.stream));
            const int n = std::min(S, K - i * S);
            if (i + 1 < nseg) {
                if ((rc = v.step_async(v.p.T_end, n))) return rc;
            } else {  // the reverse sweep starts here: keep its states now, in set 0
                rec_set = 0;
                if ((rc = record_segment(i))) return rc;
            }
        }
        AK(cudaEventRecord(b, v.stream));
        AK(cudaEventSynchronize(b));
        float ms = 0;
        AK(cudaEventElapsedTime(&ms, a, b));
        ms_fwd = ms;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        if ((rc = v.check_status())) return rc;
        if (UK && (rc = v.get_state(UK))) return rc;
        last_kept = true;
        ready = true;
        return 0;
    }

    int backward(const double* seed, double* grad) {
        if (!ready) return fail(FVGB_ERR_ARG, "fvgb_adjoint_backward before fvgb_adjoint_forward");
        Solver& v = *s;
        cudaStream_t st = v.stream;
        int rc;
        // keep the forward's final state and time
        double t_end = 0;
        if ((rc = v.get_time(&t_end, nullptr))) return rc;
        AK(cudaMemcpyAsync(d_keepU, v.d_U, sizeof(d4) * v.N, cudaMemcpyDeviceToDevice, st));
        // seed -> device order
        AK(cudaMemcpyAsync(v.d_stage, seed, sizeof(double) * 4 * v.N, cudaMemcpyHostToDevice, st));
        dev::launch_scatter_in(st, v.d_stage, d_lam, v.d_cell_new, v.N);
        cudaEvent_t a, b;
        AK(cudaEventCreate(&a));
        AK(cudaEventCreate(&b));
        AK(cudaEventRecord(a, st));
        if (nsets == 2) {
            // segment i's records in set cur; the one before it recorded into the other set
            // beside its reverse.  The last segment's records are still those the forward sweep
            // kept in set 0, unless a backward sweep has used the sets since.
            int cur = 0;
            if (!last_kept) {
                rec_set = rev_set = 0;
                if ((rc = load_segment(nseg - 1))) return rc;
                AK(cudaMemcpyAsync(&v.d_state->T, &v.p.T_end, sizeof(double), cudaMemcpyHostToDevice, st));
                if ((rc = run_graph(0, seg_len(nseg - 1), false))) return rc;
            }
            for (int i = nseg - 1; i >= 0; i--) {
                rev_set = cur;
                rec_set = 1 - cur;
                const int nrec = i > 0 ? seg_len(i - 1) : 0;
                if (nrec) {
                    if ((rc = load_segment(i - 1))) return rc;
                    AK(cudaMemcpyAsync(&v.d_state->T, &v.p.T_end, sizeof(double), cudaMemcpyHostToDevice, st));
                }
                if ((rc = run_graph(seg_len(i), nrec, nrec > 0))) return rc;
                cur = 1 - cur;
            }
        } else {
            rec_set = rev_set = 0;
            for (int i = nseg - 1; i >= 0; i--) {
                // the last segment's states are still those the forward sweep recorded
                const bool rec = i + 1 < nseg || !last_kept;
                if (rec) {
                    if ((rc = load_segment(i))) return rc;
                    AK(cudaMemcpyAsync(&v.d_state->T, &v.p.T_end, sizeof(double), cudaMemcpyHostToDevice, st));
                }
                if ((rc = run_graph(seg_len(i), rec ? seg_len(i) : 0, false))) return rc;
            }
        }
        last_kept = nseg == 1;
        AK(cudaEventRecord(b, st));
        AK(cudaEventSynchronize(b));
        float ms = 0;
        AK(cudaEventElapsedTime(&ms, a, b));
        ms_bwd = ms;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        dev::Status stt;
        AK(cudaMemcpyAsync(&stt, v.d_status, sizeof stt, cudaMemcpyDeviceToHost, st));
        AK(cudaStreamSynchronize(st));
        // restore the forward's final state and time
        AK(cudaMemcpyAsync(v.d_U, d_keepU, sizeof(d4) * v.N, cudaMemcpyDeviceToDevice, st));
        if ((rc = v.set_time(t_end))) return rc;
        // gradient -> reference order
        dev::launch_gather_out(st, d_lam, v.d_stage, v.d_cell_new, v.N);
        AK(cudaMemcpyAsync(grad, v.d_stage, sizeof(double) * 4 * v.N, cudaMemcpyDeviceToHost, st));
        AK(cudaStreamSynchronize(st));
        if ((long long)stt.restricted != restricted_before)
            return fail(FVGB_ERR_UNSUPPORTED, "the positivity pass acted during the run; the adjoint assumes it does not");
        return v.check_status();
    }
};

}  // namespace fvgb

using namespace fvgb;

namespace {
struct AdjHandle {
    fvgb_handle* owner;
    Adjoint adj;
};
// One adjoint workspace per handle, and one for fvgb_rhs_vjp kept between calls.  A handle is
// used by one thread at a time, but different handles may be used from different threads, so
// the registries themselves are guarded; the work on a workspace runs outside the lock.
std::mutex g_adj_mu;
std::vector<AdjHandle*> g_adj;
std::vector<AdjHandle*> g_adj_rhs;
AdjHandle* find_adj(fvgb_handle* h, std::vector<AdjHandle*>& reg = g_adj) {
    std::lock_guard<std::mutex> lk(g_adj_mu);
    for (auto* a : reg)
        if (a->owner == h) return a;
    return nullptr;
}
void add_adj(AdjHandle* a, std::vector<AdjHandle*>& reg) {
    std::lock_guard<std::mutex> lk(g_adj_mu);
    reg.push_back(a);
}
void drop_adj(fvgb_handle* h, std::vector<AdjHandle*>& reg) {
    AdjHandle* a = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_adj_mu);
        for (auto it = reg.begin(); it != reg.end(); ++it)
            if ((*it)->owner == h) {
                a = *it;
                reg.erase(it);
                break;
            }
    }
    delete a;
}
}  // namespace

extern "C" int fvgb_adjoint_forward(fvgb_handle* h, int nsteps, int n_checkpoints, const double* U0, double t0,
                                    double* U_K, double* ms_forward) {
    if (!h || !U0 || nsteps <= 0) return fail(FVGB_ERR_ARG, "bad adjoint arguments");
    cudaSetDevice(h->s.p.device);
    // the workspace of the previous forward serves again when laid out for the same run
    AdjHandle* a = find_adj(h);
    if (a && !a->adj.reusable(nsteps, n_checkpoints)) {
        drop_adj(h, g_adj);
        a = nullptr;
    }
    const bool fresh = a == nullptr;
    int rc = 0;
    if (fresh) {
        a = new AdjHandle{h, Adjoint()};
        rc = a->adj.setup(&h->s, nsteps, n_checkpoints);
    }
    if (!rc) rc = a->adj.forward(U0, t0, U_K);
    if (rc) {
        if (fresh) delete a;
        else drop_adj(h, g_adj);
        return rc;
    }
    if (fresh) add_adj(a, g_adj);
    if (ms_forward) *ms_forward = a->adj.ms_fwd;
    return 0;
}

extern "C" int fvgb_adjoint_backward(fvgb_handle* h, const double* seed_UK, double* grad_U0, double* ms_backward) {
    if (!h || !seed_UK || !grad_U0) return fail(FVGB_ERR_ARG, "bad adjoint arguments");
    cudaSetDevice(h->s.p.device);
    AdjHandle* a = find_adj(h);
    if (!a) return fail(FVGB_ERR_ARG, "fvgb_adjoint_backward before fvgb_adjoint_forward");
    int rc = a->adj.backward(seed_UK, grad_U0);
    if (ms_backward) *ms_backward = a->adj.ms_bwd;
    return rc;
}

extern "C" int fvgb_adjoint_overlap(fvgb_handle* h, int mode, int* overlapped) {
    if (!h || (mode != 0 && mode != 1)) return fail(FVGB_ERR_ARG, "fvgb_adjoint_overlap: mode is 0 or 1");
    h->s.adj_overlap = mode;
    if (overlapped) {
        AdjHandle* a = find_adj(h);
        *overlapped = a && a->adj.nsets == 2 ? 1 : 0;
    }
    return 0;
}

extern "C" void fvgb_adjoint_release(fvgb_handle* h) {
    drop_adj(h, g_adj);
    drop_adj(h, g_adj_rhs);
}

// No counterpart in the reference: see include/fvgb.h.
extern "C" int fvgb_rhs_vjp(fvgb_handle* h, const double* U, const double* seed_R, double* grad_U) {
    if (!h || !U || !seed_R || !grad_U) return fail(FVGB_ERR_ARG, "null argument");
    cudaSetDevice(h->s.p.device);
    AdjHandle* a = find_adj(h, g_adj_rhs);
    if (!a) {
        a = new AdjHandle{h, Adjoint()};
        if (int rc = a->adj.setup(&h->s, 1, 1, true)) {
            delete a;
            return rc;
        }
        add_adj(a, g_adj_rhs);
    }
    return a->adj.rhs_vjp(U, seed_R, grad_U);
}

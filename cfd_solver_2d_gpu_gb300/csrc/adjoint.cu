// Discrete adjoint of the explicit step (no counterpart in the reference).
//
// For U_{n+1} = Step(U_n) (time step, Runge-Kutta stages; forward Euler 3101 or
// SSP-RK3 3104; Euler equations; least-squares gradients with or without the
// Barth limiter; Roe flux; interior, periodic and slip-wall edges) this
// computes lambda_0 = (dU_K/dU_0)^T lambda_K by reverse sweeps over the steps,
// each stage's vector-Jacobian product being the hand-written reverse of the
// forward kernels (adjoint_device.cuh).  The time step's dependence on the
// state (dt = CFL vol / alpha at the minimising cell) is included; the
// positivity pass is assumed inactive (the forward reports whether it acted).
//
// Memory: checkpoints of U every S = ceil(K / n_checkpoints) steps; during the
// reverse sweep each segment is recomputed once, keeping U_0, U_1, U_2 of each
// of its steps, so the sweep costs one extra forward pass and O((K/S + 3 S) N)
// states (sqrt(K) checkpoints: O(sqrt(K) N)).
//
// Kernels of one stage VJP (all gathers, no atomics: deterministic):
//   primal gradient + limiter of the stage input (k_grad)
//   k_adj_edge     per edge: face states, flux, flux VJP, mu = seed-weighted flux adjoint, F.mu
//   k_adj_cell     per cell: gather the face-state adjoints of its edges; limiter + LSQ VJP
//   k_adj_combine  per cell: gather the neighbours' LSQ adjoints; the stage's RK combination
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "adjoint_device.cuh"
#include "internal.h"
#include "solver.h"
#include "step_kernels.cuh"

namespace fvgb {
namespace dev {

// ---- per edge --------------------------------------------------------------
template <bool LINEAR>
__global__ void __launch_bounds__(256) k_adj_edge(const d4* __restrict__ U, const d4* __restrict__ Gx,
                                                  const d4* __restrict__ Gy, MeshView m, Gas g,
                                                  const d4* __restrict__ lam, const int* __restrict__ e_rlist,
                                                  d4* __restrict__ aL, d4* __restrict__ aR, int* __restrict__ aflag,
                                                  double* __restrict__ dot_part) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double dot = 0.0;
    if (e < m.E) {
        const int L = __ldg(&m.e_L[e]), R = __ldg(&m.e_R[e]);
        const double* gm = &m.e_geom[(size_t)e * 8];
        const double nx = __ldg(&gm[0]), ny = __ldg(&gm[1]), len = __ldg(&gm[2]);
        // mu = dLoss/dF_e: F_e enters R_L with +1/-vol and, when e is in R's edge list, R_R with -1/-vol
        const double mL = __ldg(&m.c_mvol[L]);
        const d4 lL = ld4(&lam[L]);
        d4 mu = mk4(mL * lL.x, mL * lL.y, mL * lL.z, mL * lL.w);
        if (__ldg(&e_rlist[e])) {
            const double mR = __ldg(&m.c_mvol[R]);
            const d4 lR = ld4(&lam[R]);
            mu = mk4(mu.x - mR * lR.x, mu.y - mR * lR.y, mu.z - mR * lR.z, mu.w - mR * lR.w);
        }
        const d4 uL = ld4(&U[L]);
        d4 gxL = mk4(0, 0, 0, 0), gyL = gxL;
        if (LINEAR) {
            gxL = ld4(&Gx[L]);
            gyL = ld4(&Gy[L]);
        }
        Prim wL;
        const d4 fL = face_state<LINEAR>(uL, gxL, gyL, __ldg(&gm[4]), __ldg(&gm[5]), g, wL);
        int flag = 0;  // bit 0 / bit 1: the L / R face state is the linear reconstruction
        if (LINEAR) {
            const Prim t = to_prim(lin(uL, gxL, gyL, __ldg(&gm[4]), __ldg(&gm[5])), g);
            if (!out_of_range(t.r, t.p)) flag |= 1;
        }
        d4 bfL = mk4(0, 0, 0, 0), bfR = mk4(0, 0, 0, 0);
        Prim bwL{}, bwR{};
        if (e < m.E_int) {
            const d4 uR = ld4(&U[R]);
            d4 gxR = mk4(0, 0, 0, 0), gyR = gxR;
            if (LINEAR) {
                gxR = ld4(&Gx[R]);
                gyR = ld4(&Gy[R]);
            }
            Prim wR;
            const d4 fR = face_state<LINEAR>(uR, gxR, gyR, __ldg(&gm[6]), __ldg(&gm[7]), g, wR);
            if (LINEAR) {
                const Prim t = to_prim(lin(uR, gxR, gyR, __ldg(&gm[6]), __ldg(&gm[7])), g);
                if (!out_of_range(t.r, t.p)) flag |= 2;
            }
            const d4 F = roe_flux(wL, wR, nx, ny, len, g);
            dot = F.x * mu.x + F.y * mu.y + F.z * mu.z + F.w * mu.w;
            roe_flux_vjp(wL, wR, nx, ny, len, g, mu, bwL, bwR);
            to_prim_vjp(fR, wR, g, bwR, bfR);
            to_prim_vjp(fL, wL, g, bwL, bfL);
        } else {  // slip wall / symmetry: the ghost is a function of the L face state
            const d4 fR = ghost_slip(fL, wL, nx, ny);
            const Prim wR = to_prim(fR, g);
            const d4 F = roe_flux(wL, wR, nx, ny, len, g);
            dot = F.x * mu.x + F.y * mu.y + F.z * mu.z + F.w * mu.w;
            roe_flux_vjp(wL, wR, nx, ny, len, g, mu, bwL, bwR);
            d4 bgR = mk4(0, 0, 0, 0);
            to_prim_vjp(fR, wR, g, bwR, bgR);
            ghost_slip_vjp(fL, wL, nx, ny, bgR, bfL, bwL);
            to_prim_vjp(fL, wL, g, bwL, bfL);
        }
        aL[e] = bfL;
        aR[e] = bfR;
        aflag[e] = flag;
    }
    // deterministic block partial of sum_e F_e . mu_e
    for (int o = 16; o > 0; o >>= 1) dot += __shfl_down_sync(0xffffffffu, dot, o);
    __shared__ double sm[8];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = dot;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sm[i];
        dot_part[blockIdx.x] = s;
    }
}

// ---- per cell: gather face-state adjoints, then limiter + LSQ VJP ---------------
template <bool LINEAR, bool BARTH>
__global__ void __launch_bounds__(256) k_adj_cell(const d4* __restrict__ U, MeshView m, const d4* __restrict__ aL,
                                                  const d4* __restrict__ aR, const int* __restrict__ aflag,
                                                  d4* __restrict__ lam_dir, d4* __restrict__ bdU) {
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
        for (int v = 0; v < 4; v++) {
            lu[v] += av[v];
            if (LINEAR && used) {
                lgx[v] = fma(av[v], dx, lgx[v]);
                lgy[v] = fma(av[v], dy, lgy[v]);
            }
        }
    }
    lam_dir[c] = mk4(lu[0], lu[1], lu[2], lu[3]);
    double bd[3][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
    if (LINEAR) {
        // recompute the raw gradient and the limiter's choices (grad_cell, least squares)
        const d4 uc = ld4(&U[c]);
        const int nnb = __ldg(&m.c_nnb[c]);
        const double ucv[4] = {uc.x, uc.y, uc.z, uc.w};
        double dU[3][4];
        for (int k = 0; k < 3; k++) {
            const int q = __ldg(&m.c_nbr[c * 3 + k]);
            const d4 un = (k < nnb) ? ld4(&U[q]) : uc;
            const double unv[4] = {un.x, un.y, un.z, un.w};
            for (int v = 0; v < 4; v++) dU[k][v] = unv[v] - ucv[v];
        }
        const double* B = &m.c_lsq[(size_t)c * 6];
        double b0[3], b1[3];
        for (int k = 0; k < 3; k++) {
            b0[k] = __ldg(&B[k]);
            b1[k] = __ldg(&B[3 + k]);
        }
        const double* X = &m.c_vtx[(size_t)c * 6];
        double vx[3], vy[3];
        for (int j = 0; j < 3; j++) {
            vx[j] = __ldg(&X[2 * j]);
            vy[j] = __ldg(&X[2 * j + 1]);
        }
        for (int v = 0; v < 4; v++) {
            const double gx = fma(b0[2], dU[2][v], fma(b0[1], dU[1][v], b0[0] * dU[0][v]));
            const double gy = fma(b1[2], dU[2][v], fma(b1[1], dU[1][v], b1[0] * dU[0][v]));
            double bgx = lgx[v], bgy = lgy[v];
            if (BARTH) {
                double np = 0.0, nn = 0.0;
                int kp = -1, kn = -1;  // neighbour slot giving hi - Uc / lo - Uc (-1: the cell itself, 0)
                for (int k = 0; k < 3; k++) {
                    if (k < nnb) {
                        if (dlt(np, dU[k][v])) { np = dU[k][v]; kp = k; }
                        if (dlt(dU[k][v], nn)) { nn = dU[k][v]; kn = k; }
                    }
                }
                double d[3];
                for (int j = 0; j < 3; j++) d[j] = fma(gx, vx[j], gy * vy[j]);
                int jh = 0, jl = 0;
                for (int j = 1; j < 3; j++) {
                    if (dlt(d[jh], d[j])) jh = j;
                    if (dlt(d[j], d[jl])) jl = j;
                }
                const double dp = d[jh] + kEps, dn = d[jl] - kEps;
                const bool lim_p = pos(d[jh]) && dlt(np, dp);
                const bool lim_n = neg(d[jl]) && dlt(dn, nn);
                if (lim_p || lim_n) {
                    const bool use_p = lim_p && (!lim_n || dlt(nn * dp, np * dn));
                    const double num = use_p ? np : nn, den = use_p ? dp : dn;
                    const int kk = use_p ? kp : kn, jj = use_p ? jh : jl;
                    const double rden = rcp(den);
                    const double phi = num * rden;
                    // gx_lim = phi gx, gy_lim = phi gy
                    const double b_phi = bgx * gx + bgy * gy;
                    bgx *= phi;
                    bgy *= phi;
                    const double b_num = b_phi * rden;
                    const double b_den = -b_phi * phi * rden;
                    bgx = fma(b_den, vx[jj], bgx);
                    bgy = fma(b_den, vy[jj], bgy);
                    if (kk >= 0) bd[kk][v] += b_num;
                }
            }
            for (int k = 0; k < 3; k++)
                if (k < nnb) bd[k][v] = fma(b0[k], bgx, fma(b1[k], bgy, bd[k][v]));
        }
    }
    for (int k = 0; k < 3; k++) bdU[(size_t)c * 3 + k] = mk4(bd[k][0], bd[k][1], bd[k][2], bd[k][3]);
}

// ---- per cell: neighbours' LSQ adjoints and the stage's Runge-Kutta combination ------
// U_s = a U_0 + b (U_in + dt R(U_in)):  lam_in = b (lam_s + dt J^T lam_s);  acc0 (+)= a lam_s
__global__ void __launch_bounds__(256) k_adj_combine(MeshView m, const int* __restrict__ rev,
                                                     const d4* __restrict__ lam_dir, const d4* __restrict__ bdU,
                                                     const d4* __restrict__ lam_s, const double* __restrict__ dt_p,
                                                     double a, double b, int acc_mode, d4* __restrict__ lam_in,
                                                     d4* __restrict__ acc0, int linear) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
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
    }
    const double dt = *dt_p;
    const d4 ls = ld4(&lam_s[c]);
    lam_in[c] = mk4(b * fma(dt, r[0], ls.x), b * fma(dt, r[1], ls.y), b * fma(dt, r[2], ls.z), b * fma(dt, r[3], ls.w));
    if (acc_mode == 0) acc0[c] = mk4(a * ls.x, a * ls.y, a * ls.z, a * ls.w);
    else if (acc_mode == 1) {
        const d4 o = acc0[c];
        acc0[c] = mk4(fma(a, ls.x, o.x), fma(a, ls.y, o.y), fma(a, ls.z, o.z), fma(a, ls.w, o.w));
    }
}

// lam = acc0 + lam_in (the first stage's input is U_0 itself)
__global__ void __launch_bounds__(256) k_adj_add(int N, const d4* __restrict__ acc0, d4* __restrict__ lam) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const d4 a = acc0[c], l = lam[c];
    lam[c] = mk4(a.x + l.x, a.y + l.y, a.z + l.z, a.w + l.w);
}

// lambda_dt = sum over stages of b_s (F . mu)_s, partials summed in a fixed order
__global__ void k_adj_lamdt(const double* __restrict__ part, int nb, int nstages, const double* __restrict__ bs,
                            double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double t = 0.0;
    for (int s = 0; s < nstages; s++) {
        double x = 0.0;
        for (int i = 0; i < nb; i++) x += part[(size_t)s * nb + i];
        t = fma(bs[s], x, t);
    }
    *out = t;
}

// smallest cell index whose CFL vol / alpha equals the step's minimum
__global__ void __launch_bounds__(256) k_adj_argmin(MeshView m, const double* __restrict__ alpha, double CFL,
                                                    const unsigned long long* dtmin, int* out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m.N) return;
    const double d = dmin(1e10, dt_cell<false>(c, m, alpha, nullptr, CFL));
    if ((unsigned long long)__double_as_longlong(d) == *dtmin) atomicMin(out, c);
}

// dt = CFL vol_c / alpha_c at the minimising cell c: adds lambda_dt d(dt)/dU_0 to lam
__global__ void k_adj_dt(const d4* __restrict__ U0, MeshView m, Gas g, double CFL, const int* cstar,
                         const double* dt_info, const double* lamdt, d4* lam) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int c = *cstar;
    if (c < 0 || c >= m.N) return;
    if (dt_info[0] != dt_info[1]) return;  // clamped to the end time: dt does not depend on U
    const double lt = *lamdt;
    if (lt == 0.0) return;
    double alpha = 0.0;
    for (int k = m.dt_ptr[c]; k < m.dt_ptr[c + 1]; k++) {
        const int e = m.dt_edge[k];
        const int L = m.e_L[e], R = m.e_R[e];
        const Prim wl = to_prim(U0[L], g);
        d4 w = mk4(wl.r, wl.u, wl.v, wl.p);
        if (R != -1) {
            const Prim wr = to_prim(U0[R], g);
            w = mk4(0.5 * (w.x + wr.r), 0.5 * (w.y + wr.u), 0.5 * (w.z + wr.v), 0.5 * (w.w + wr.p));
        }
        const double* gm = &m.e_geom[(size_t)e * 8];
        const double un = w.y * (gm[0] * gm[2]) + w.z * (gm[1] * gm[2]);
        alpha += fabs(un) + sqrt(g.gamma * w.w * rcp(w.x)) * gm[3];
    }
    const double vol = m.c_vol[c];
    const double dt = CFL * vol * rcp(alpha);
    const double b_alpha = lt * (-dt * rcp(alpha));
    for (int k = m.dt_ptr[c]; k < m.dt_ptr[c + 1]; k++) {
        const int e = m.dt_edge[k];
        const int L = m.e_L[e], R = m.e_R[e];
        const Prim wl = to_prim(U0[L], g);
        Prim wr{};
        d4 w = mk4(wl.r, wl.u, wl.v, wl.p);
        if (R != -1) {
            wr = to_prim(U0[R], g);
            w = mk4(0.5 * (w.x + wr.r), 0.5 * (w.y + wr.u), 0.5 * (w.z + wr.v), 0.5 * (w.w + wr.p));
        }
        const double* gm = &m.e_geom[(size_t)e * 8];
        const double nxl = gm[0] * gm[2], nyl = gm[1] * gm[2];
        const double un = w.y * nxl + w.z * nyl;
        const double ir = rcp(w.x);
        const double s = sqrt(g.gamma * w.w * ir);
        const double b_un = b_alpha * sgn(un);
        const double b_s = b_alpha * gm[3];
        const double b_p = s > 0 ? b_s * g.gamma * ir / (2.0 * s) : 0.0;
        const double b_ir = s > 0 ? b_s * g.gamma * w.w / (2.0 * s) : 0.0;
        Prim bw{};
        bw.r = -b_ir * ir * ir;
        bw.u = b_un * nxl;
        bw.v = b_un * nyl;
        bw.p = b_p;
        const double f = (R != -1) ? 0.5 : 1.0;
        Prim bc{f * bw.r, f * bw.u, f * bw.v, f * bw.p, 0.0};
        d4 bu = mk4(0, 0, 0, 0);
        to_prim_vjp(U0[L], wl, g, bc, bu);
        d4 o = lam[L];
        lam[L] = mk4(o.x + bu.x, o.y + bu.y, o.z + bu.z, o.w + bu.w);
        if (R != -1) {
            bu = mk4(0, 0, 0, 0);
            to_prim_vjp(U0[R], wr, g, bc, bu);
            o = lam[R];
            lam[R] = mk4(o.x + bu.x, o.y + bu.y, o.z + bu.z, o.w + bu.w);
        }
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
    std::vector<double> chk_t;     // t at the start of each segment
    std::vector<d4*> seg_states;   // per step of a segment: U_0, U_1, U_2
    double* d_seg_dt = nullptr;    // per step: dt, dt_raw
    int* d_seg_cstar = nullptr;    // per step: the minimising cell
    d4 *d_lam = nullptr, *d_lam_in = nullptr, *d_acc0 = nullptr, *d_aL = nullptr, *d_aR = nullptr;
    d4 *d_lamdir = nullptr, *d_bdU = nullptr, *d_keepU = nullptr;
    int *d_aflag = nullptr, *d_rlist = nullptr, *d_rev = nullptr;
    double *d_dotp = nullptr, *d_lamdt = nullptr, *d_bs = nullptr;
    bool ready = false;
    long long restricted_before = 0;
    double ms_fwd = 0, ms_bwd = 0;

    ~Adjoint() {
        for (void* q : owned) cudaFree(q);
    }
    template <class T>
    int alloc(T*& p, size_t n) {
        p = nullptr;
        AK(cudaMalloc((void**)&p, (n ? n : 1) * sizeof(T)));
        owned.push_back((void*)p);
        return 0;
    }

    int setup(Solver* solver, int nsteps, int ncheck) {
        s = solver;
        const fvgb_params& p = s->p;
        if (p.equation != 1) return fail(FVGB_ERR_UNSUPPORTED, "the adjoint covers the Euler equations");
        if (p.flux_scheme != 2002) return fail(FVGB_ERR_UNSUPPORTED, "the adjoint covers the Roe flux");
        if (p.time_advance != 3101 && p.time_advance != 3104)
            return fail(FVGB_ERR_UNSUPPORTED, "the adjoint covers forward Euler (3101) and SSP-RK3 (3104)");
        if (p.reconstruct == 3002 && p.gradient != 1)
            return fail(FVGB_ERR_UNSUPPORTED, "the adjoint covers least-squares gradients");
        for (int e = s->L.E_int; e < s->E; e++) {
            const int bt = s->L.e_bc[e];
            if (bt != 6001 && bt != 6021)
                return fail(FVGB_ERR_UNSUPPORTED, "the adjoint covers interior, periodic and slip-wall edges");
        }
        K = nsteps;
        ncheck = std::max(1, std::min(ncheck, K));
        S = (K + ncheck - 1) / ncheck;
        nseg = (K + S - 1) / S;
        nst = p.time_advance == 3101 ? 1 : 3;
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
        chk_t.assign(nseg, 0.0);
        for (int i = 0; i < nseg; i++)
            if ((rc = alloc(chk[i], N))) return rc;
        seg_states.assign((size_t)S * nst, nullptr);
        for (auto& q : seg_states)
            if ((rc = alloc(q, N))) return rc;
        const int nb = nblk(E, 256);
        if ((rc = alloc(d_seg_dt, 2 * (size_t)S)) || (rc = alloc(d_seg_cstar, S)) || (rc = alloc(d_lam, N)) ||
            (rc = alloc(d_lam_in, N)) || (rc = alloc(d_acc0, N)) || (rc = alloc(d_aL, E)) || (rc = alloc(d_aR, E)) ||
            (rc = alloc(d_lamdir, N)) || (rc = alloc(d_keepU, N)) || (rc = alloc(d_bdU, 3 * (size_t)N)) || (rc = alloc(d_aflag, E)) ||
            (rc = alloc(d_dotp, (size_t)nb * 3)) || (rc = alloc(d_lamdt, 1)) || (rc = alloc(d_bs, 3)))
            return rc;
        return 0;
    }

    // one forward step launched kernel by kernel, keeping what the reverse sweep needs
    int record_step(int slot) {
        Solver& v = *s;
        cudaStream_t st = v.stream;
        const bool copy = v.p.time_advance != 3101;
        AK(cudaMemcpyAsync(seg_states[(size_t)slot * nst], v.d_U, sizeof(d4) * v.N, cudaMemcpyDeviceToDevice, st));
        dev::launch_prim(st, v.d_U, v.d_U0, v.d_prim, v.N, v.gas, copy);
        const double value_1 = std::max(4.0 / 3.0, v.p.gamma / v.p.Pr);
        dev::launch_dt(st, v.d_prim, v.mv, v.gas, value_1, v.p.CFL, false, v.d_alpha, v.d_alpha_vis,
                       &v.d_state->dtmin_bits, v.d_status);
        AK(cudaMemsetAsync(d_seg_cstar + slot, 0x7f, sizeof(int), st));
        dev::k_adj_argmin<<<nblk(v.N, 256), 256, 0, st>>>(v.mv, v.d_alpha, v.p.CFL, &v.d_state->dtmin_bits,
                                                          d_seg_cstar + slot);
        dev::launch_dt_final(st, v.d_state, true);
        AK(cudaMemcpyAsync(d_seg_dt + 2 * slot, &v.d_state->dt, sizeof(double), cudaMemcpyDeviceToDevice, st));
        AK(cudaMemcpyAsync(d_seg_dt + 2 * slot + 1, &v.d_state->dt_raw, sizeof(double), cudaMemcpyDeviceToDevice, st));
        if (v.p.time_advance == 3101) {
            v.enqueue_stage(dev::STAGE_EULER);
        } else {
            v.enqueue_stage(dev::STAGE_SSP_1);
            AK(cudaMemcpyAsync(seg_states[(size_t)slot * nst + 1], v.d_U, sizeof(d4) * v.N, cudaMemcpyDeviceToDevice, st));
            v.enqueue_stage(dev::STAGE_SSP_2);
            AK(cudaMemcpyAsync(seg_states[(size_t)slot * nst + 2], v.d_U, sizeof(d4) * v.N, cudaMemcpyDeviceToDevice, st));
            v.enqueue_stage(dev::STAGE_SSP_3);
        }
        dev::launch_restrict(st, v.d_U, v.mv, v.d_cell_ref, v.d_cell_new, v.d_flags, v.d_flag_count, Solver::kFlagCap,
                             v.p.restrict_ref, v.gas, v.d_status);
        AK(cudaGetLastError());
        return 0;
    }

    // one stage VJP: lam_s (d_lam) -> lam_in (d_lam_in), acc0, partial F.mu in dot slot
    int stage_vjp(const d4* Uin, const double* dt_p, double a, double b, int acc_mode, int dot_slot) {
        Solver& v = *s;
        cudaStream_t st = v.stream;
        const bool linear = v.p.reconstruct == 3002;
        if (linear) dev::launch_grad(st, 1, v.p.limiter == 1, Uin, v.mv, v.d_Gx, v.d_Gy);
        const int nbE = nblk(v.E, 256), nbN = nblk(v.N, 256);
        double* dp = d_dotp + (size_t)dot_slot * nbE;
        if (linear)
            dev::k_adj_edge<true><<<nbE, 256, 0, st>>>(Uin, v.d_Gx, v.d_Gy, v.mv, v.gas, d_lam, d_rlist, d_aL, d_aR,
                                                       d_aflag, dp);
        else
            dev::k_adj_edge<false><<<nbE, 256, 0, st>>>(Uin, v.d_Gx, v.d_Gy, v.mv, v.gas, d_lam, d_rlist, d_aL, d_aR,
                                                        d_aflag, dp);
        if (!linear) dev::k_adj_cell<false, false><<<nbN, 256, 0, st>>>(Uin, v.mv, d_aL, d_aR, d_aflag, d_lamdir, d_bdU);
        else if (v.p.limiter == 1)
            dev::k_adj_cell<true, true><<<nbN, 256, 0, st>>>(Uin, v.mv, d_aL, d_aR, d_aflag, d_lamdir, d_bdU);
        else dev::k_adj_cell<true, false><<<nbN, 256, 0, st>>>(Uin, v.mv, d_aL, d_aR, d_aflag, d_lamdir, d_bdU);
        dev::k_adj_combine<<<nbN, 256, 0, st>>>(v.mv, d_rev, d_lamdir, d_bdU, d_lam, dt_p, a, b, acc_mode, d_lam_in,
                                                d_acc0, linear ? 1 : 0);
        AK(cudaGetLastError());
        return 0;
    }

    // lam (adjoint of U_{n+1}) -> lam (adjoint of U_n) for the step kept in slot
    int step_vjp(int slot) {
        Solver& v = *s;
        cudaStream_t st = v.stream;
        const double* dtp = d_seg_dt + 2 * slot;
        const int nbN = nblk(v.N, 256), nbE = nblk(v.E, 256);
        int rc;
        if (v.p.time_advance == 3101) {
            // U1 = U0 + dt R(U0): a = 0, b = 1
            if ((rc = stage_vjp(seg_states[(size_t)slot], dtp, 0.0, 1.0, 2, 0))) return rc;
            const double bs[3] = {1.0, 0.0, 0.0};
            AK(cudaMemcpyAsync(d_bs, bs, sizeof bs, cudaMemcpyHostToDevice, st));
            std::swap(d_lam, d_lam_in);
        } else {
            const d4* U0 = seg_states[(size_t)slot * 3];
            const d4* U1 = seg_states[(size_t)slot * 3 + 1];
            const d4* U2 = seg_states[(size_t)slot * 3 + 2];
            // U3 = 1/3 U0 + 2/3 (U2 + dt R(U2))
            if ((rc = stage_vjp(U2, dtp, 1.0 / 3.0, 2.0 / 3.0, 0, 0))) return rc;
            std::swap(d_lam, d_lam_in);
            // U2 = 3/4 U0 + 1/4 (U1 + dt R(U1))
            if ((rc = stage_vjp(U1, dtp, 0.75, 0.25, 1, 1))) return rc;
            std::swap(d_lam, d_lam_in);
            // U1 = U0 + dt R(U0)
            if ((rc = stage_vjp(U0, dtp, 0.0, 1.0, 2, 2))) return rc;
            std::swap(d_lam, d_lam_in);
            dev::k_adj_add<<<nbN, 256, 0, st>>>(v.N, d_acc0, d_lam);
            const double bs[3] = {2.0 / 3.0, 0.25, 1.0};
            AK(cudaMemcpyAsync(d_bs, bs, sizeof bs, cudaMemcpyHostToDevice, st));
        }
        dev::k_adj_lamdt<<<1, 32, 0, st>>>(d_dotp, nbE, nst, d_bs, d_lamdt);
        dev::k_adj_dt<<<1, 32, 0, st>>>(seg_states[(size_t)slot * nst], v.mv, v.gas, v.p.CFL, d_seg_cstar + slot, dtp,
                                        d_lamdt, d_lam);
        AK(cudaGetLastError());
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
            double t;
            if ((rc = v.get_time(&t, nullptr))) return rc;
            chk_t[i] = t;
            const int n = std::min(S, K - i * S);
            if ((rc = v.step_async(v.p.T_end, n))) return rc;
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
        for (int i = nseg - 1; i >= 0; i--) {
            AK(cudaMemcpyAsync(v.d_U, chk[i], sizeof(d4) * v.N, cudaMemcpyDeviceToDevice, st));
            if ((rc = v.set_time(chk_t[i]))) return rc;
            AK(cudaMemcpyAsync(&v.d_state->T, &v.p.T_end, sizeof(double), cudaMemcpyHostToDevice, st));
            const int n = std::min(S, K - i * S);
            for (int k = 0; k < n; k++)
                if ((rc = record_step(k))) return rc;
            for (int k = n - 1; k >= 0; k--)
                if ((rc = step_vjp(k))) return rc;
        }
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
std::vector<AdjHandle*> g_adj;  // one adjoint workspace per handle (handles are single-threaded)
AdjHandle* find_adj(fvgb_handle* h) {
    for (auto* a : g_adj)
        if (a->owner == h) return a;
    return nullptr;
}
}  // namespace

extern "C" int fvgb_adjoint_forward(fvgb_handle* h, int nsteps, int n_checkpoints, const double* U0, double t0,
                                    double* U_K, double* ms_forward) {
    if (!h || !U0 || nsteps <= 0) return fail(FVGB_ERR_ARG, "bad adjoint arguments");
    cudaSetDevice(h->s.p.device);
    AdjHandle* a = find_adj(h);
    if (a) {
        g_adj.erase(std::find(g_adj.begin(), g_adj.end(), a));
        delete a;
    }
    a = new AdjHandle{h, Adjoint()};
    int rc = a->adj.setup(&h->s, nsteps, n_checkpoints);
    if (!rc) rc = a->adj.forward(U0, t0, U_K);
    if (rc) {
        delete a;
        return rc;
    }
    g_adj.push_back(a);
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

extern "C" void fvgb_adjoint_release(fvgb_handle* h) {
    AdjHandle* a = find_adj(h);
    if (a) {
        g_adj.erase(std::find(g_adj.begin(), g_adj.end(), a));
        delete a;
    }
}

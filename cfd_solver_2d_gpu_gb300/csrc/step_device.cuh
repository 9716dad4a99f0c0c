// Per-cell and per-edge bodies of the step (sm_103a, FP64).  The single-mesh
// kernels (step_kernels.cu) and the batched persistent stage kernel
// (batch.cu) call the same functions; reference functions are cited at each.
#pragma once
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace fvgb {
namespace dev {

enum StageKind {
    STAGE_RHS = 0,     // residual only
    STAGE_EULER = 1,   // forward Euler (3101)
    STAGE_RK3_1 = 2,   // Kutta RK3 (3103) stages
    STAGE_RK3_2 = 3,
    STAGE_RK3_3 = 4,
    STAGE_SSP_1 = 5,   // SSP-RK3 (3104) stages
    STAGE_SSP_2 = 6,
    STAGE_SSP_3 = 7,
    STAGE_LOCAL = 8,   // forward Euler with each cell's own dt (time.is_steady = 1)
};

__host__ __device__ constexpr bool final_stage(int kind) {
    return kind == STAGE_EULER || kind == STAGE_RK3_3 || kind == STAGE_SSP_3 || kind == STAGE_LOCAL;
}

// The stage's time offset, in units of dt, at which the double-Mach-reflection boundary is
// evaluated: CIteration.cpp:61-62 set its clock to (t, 0) for the step, and
// evolve_rk3_globaltimestep (Evolve.cpp:43-77) sets dt, then 0.5 dt, before its second and
// third residuals.  SSP-RK3's stages sit at t, t + dt and t + dt/2 as well.
__host__ __device__ constexpr double dsr_stage_frac(int kind) {
    return (kind == STAGE_RK3_2 || kind == STAGE_SSP_2) ? 1.0 : (kind == STAGE_RK3_3 || kind == STAGE_SSP_3) ? 0.5 : 0.0;
}

// ---- time step ---------------------------------------------------------------

// update_host_ruvp_Uold, FVMR/src/time/CIteration.cpp:163-180 (plus U0 <- U)
__device__ __forceinline__ void prim_cell(int c, const d4* __restrict__ U, d4* __restrict__ U0, d4* __restrict__ prim,
                                          const Gas& g, bool copy) {
    const d4 u = ld4(&U[c]);
    const Prim w = to_prim(u, g);
    prim[c] = mk4(w.r, w.u, w.v, w.p);
    if (copy) U0[c] = u;
}

// spectral radius of one edge, update_alphaC_host, FVMR/src/time/CalculateDt.cpp:207-248
template <bool NS>
__device__ __forceinline__ void alpha_edge(int e, const d4* __restrict__ prim, const MeshView& m, const Gas& g,
                                           double value_1, double* __restrict__ alpha, double* __restrict__ alpha_vis,
                                           Status* st) {
    const int L = __ldg(&m.e_L[e]), R = __ldg(&m.e_R[e]);
    d4 w = ld4(&prim[L]);
    if (R != -1) {
        const d4 wr = ld4(&prim[R]);
        w = mk4(mul(0.5, w.x + wr.x), mul(0.5, w.y + wr.y), mul(0.5, w.z + wr.z), mul(0.5, w.w + wr.w));
    }
    if (neg(w.x) || neg(w.w)) atomicAdd(&st->negative_dt, 1ull);
    const double* gm = &m.e_geom[(size_t)e * 8];
    const double nx = __ldg(&gm[0]), ny = __ldg(&gm[1]), len = __ldg(&gm[2]), sqrt_len = __ldg(&gm[3]);
    const double un = fma(w.y, mul(nx, len), mul(w.z, mul(ny, len)));
    const double ir = rcp(w.x);
    alpha[e] = fma(sq(mul(mul(g.gamma, w.w), ir)), sqrt_len, absd(un));
    if (NS) {
        const double T = w.w / g.R * ir;
        const double mu = mul(mul(g.C1, mul(T, sq(T))), rcp(T + 110.4));
        alpha_vis[e] = 2.0 * len * value_1 * mu * ir;
    }
}

// CFL vol / alpha of one cell, get_minimus_dt_by_alphaC, CalculateDt.cpp:74-85: the cell's
// sum over the edges touching it, in the reference's edge order
template <bool NS>
__device__ __forceinline__ double dt_cell(int c, const MeshView& m, const double* __restrict__ alpha,
                                          const double* __restrict__ alpha_vis, double CFL) {
    const int b = __ldg(&m.dt_ptr[c]), e_ = __ldg(&m.dt_ptr[c + 1]);
    const double vol = __ldg(&m.c_vol[c]);
    const double ivol = NS ? rcp(vol) : 0.0;
    double a = 0.0;
    for (int k = b; k < e_; k++) {
        const int e = __ldg(&m.dt_edge[k]);
        a += __ldg(&alpha[e]);
        if (NS) a = fma(__ldg(&alpha_vis[e]), ivol, a);
    }
    return CFL * vol * rcp(a);
}

// ---- gradients and the Barth limiter (Gradient, FVMR/src/space/gradient/Gradient.cpp:116-158)

// the discrete adjoint's record of one stage's limited least-squares gradients: per cell
// the gradient before the limiter, per variable phi and 1/den of the limiting ratio,
// and a code word (per variable five bits: limited, the neighbour slot + 1 giving the
// bound (0: the cell itself), the vertex)
struct CellTape {
    d4* gx = nullptr;
    d4* gy = nullptr;
    d4* phi = nullptr;
    d4* rden = nullptr;
    int* code = nullptr;
};

template <int GRAD, bool BARTH, bool REC = false>
__device__ __forceinline__ void grad_cell(int c, const d4* __restrict__ U, const MeshView& m, d4* __restrict__ Gx,
                                          d4* __restrict__ Gy, CellTape tape = CellTape()) {
    const d4 uc = ld4(&U[c]);
    const int nnb = __ldg(&m.c_nnb[c]);
    d4 un[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int q = __ldg(&m.c_nbr[c * 3 + k]);
        un[k] = (k < nnb) ? ld4(&U[q]) : uc;
    }
    double gx[4], gy[4];
    const double ucv[4] = {uc.x, uc.y, uc.z, uc.w};
    // neighbour differences U_k - U_c (valid neighbours in slot order), shared by the
    // least-squares gradient and the limiter's bounds
    double dU[3][4];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double unv[4] = {un[k].x, un[k].y, un[k].z, un[k].w};
#pragma unroll
        for (int v = 0; v < 4; v++) dU[k][v] = unv[v] - ucv[v];
    }
    if (GRAD == 1) {
        // GradientLeastSquare_2 (Gradient.cpp:160-246) with the weights B = (A^T A)^-1 A^T
        // precomputed per cell: grad = B dU, summed over the valid neighbours in slot order
        const double* B = &m.c_lsq[(size_t)c * 6];
        double b0[3], b1[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            b0[k] = __ldg(&B[k]);
            b1[k] = __ldg(&B[3 + k]);
        }
#pragma unroll
        for (int v = 0; v < 4; v++) {
            // absent neighbours carry B = 0 and dU = 0
            gx[v] = fma(b0[2], dU[2][v], fma(b0[1], dU[1][v], mul(b0[0], dU[0][v])));
            gy[v] = fma(b1[2], dU[2][v], fma(b1[1], dU[1][v], mul(b1[0], dU[0][v])));
        }
    } else {
        // GradientGreenGauss_2 (Gradient.cpp:248-458) with precomputed face weights
        const double* W = &m.c_gg[(size_t)c * 12];
        double sx[4] = {0, 0, 0, 0}, sy[4] = {0, 0, 0, 0};
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const int out = __ldg(&m.c_ggout[c * 3 + j]);
            const double gC = __ldg(&W[4 * j]), gC1 = __ldg(&W[4 * j + 1]);
            const double Sx = __ldg(&W[4 * j + 2]), Sy = __ldg(&W[4 * j + 3]);
            d4 uf = uc;
            if (out >= 0) uf = ld4(&U[out]);
            const double ufv[4] = {uf.x, uf.y, uf.z, uf.w};
#pragma unroll
            for (int v = 0; v < 4; v++) {
                const double phif = (out >= 0) ? fma(gC, ucv[v], mul(gC1, ufv[v])) : ucv[v];
                sx[v] = fma(phif, Sx, sx[v]);
                sy[v] = fma(phif, Sy, sy[v]);
            }
        }
        const double ginv = __ldg(&m.c_ginv[c]);
#pragma unroll
        for (int v = 0; v < 4; v++) {
            gx[v] = mul(ginv, sx[v]);
            gy[v] = mul(ginv, sy[v]);
        }
    }
    static_assert(!REC || BARTH, "the adjoint's record covers the Barth limiter");
    double gxr[4], gyr[4], phiv[4] = {1, 1, 1, 1}, rdv[4] = {0, 0, 0, 0};
    int code = 0;
    if constexpr (REC) {
#pragma unroll
        for (int v = 0; v < 4; v++) {
            gxr[v] = gx[v];
            gyr[v] = gy[v];
        }
    }
    if (BARTH) {
        // LimiterBarth, Gradient.cpp:58-114:
        //   phi = min over the vertices of min(1, (hi - Uc)/(d + eps)) for d > 0 and
        //   min(1, (lo - Uc)/(d - eps)) for d < 0, d = U(vertex) - Uc.
        // hi - Uc and lo - Uc are the largest / smallest of 0 and the neighbour
        // differences.  Division and rounding are monotonic, so the minimum over the
        // positive vertices is taken at the largest d (and over the negative ones at
        // the smallest d); of the two candidates only the smaller ratio is divided
        // out (compared by cross-multiplication), and none when neither is below 1.
        // All comparisons run on the integer pipe (okey).
        const double* X = &m.c_vtx[(size_t)c * 6];
        double vx[3], vy[3];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            vx[j] = __ldg(&X[2 * j]);
            vy[j] = __ldg(&X[2 * j + 1]);
        }
#pragma unroll
        for (int v = 0; v < 4; v++) {
            double np = 0.0, nn = 0.0;  // hi - Uc >= 0, lo - Uc <= 0
            int kp = -1, kn = -1;       // (REC) the slot giving np / nn, -1: the cell itself
#pragma unroll
            for (int k = 0; k < 3; k++) {
                if (k < nnb) {
                    if constexpr (REC) {
                        if (dlt(np, dU[k][v])) { np = dU[k][v]; kp = k; }
                        if (dlt(dU[k][v], nn)) { nn = dU[k][v]; kn = k; }
                    } else {
                        np = dmax(np, dU[k][v]);
                        nn = dmin(nn, dU[k][v]);
                    }
                }
            }
            const double d0 = fma(gx[v], vx[0], mul(gy[v], vy[0]));
            const double d1 = fma(gx[v], vx[1], mul(gy[v], vy[1]));
            const double d2 = fma(gx[v], vx[2], mul(gy[v], vy[2]));
            const double dhi = dmax(dmax(d0, d1), d2), dlo = dmin(dmin(d0, d1), d2);
            int jh = 0, jl = 0;  // (REC) the vertices giving dhi / dlo, as dmax / dmin choose them
            if constexpr (REC) {
                jh = dlt(d0, d1) ? 1 : 0;
                jh = dlt(jh ? d1 : d0, d2) ? 2 : jh;
                jl = dlt(d1, d0) ? 1 : 0;
                jl = dlt(d2, jl ? d1 : d0) ? 2 : jl;
            }
            const double dp = dhi + kEps, dn = dlo - kEps;
            const bool lim_p = pos(dhi) && dlt(np, dp);  // ratio np/dp below 1
            const bool lim_n = neg(dlo) && dlt(dn, nn);  // ratio nn/dn below 1
            if (lim_p || lim_n) {
                // both limited: np/dp < nn/dn  <=>  np*dn > nn*dp  (dp > 0 > dn)
                const bool use_p = lim_p && (!lim_n || dlt(mul(nn, dp), mul(np, dn)));
                const double num = use_p ? np : nn, den = use_p ? dp : dn;
                const double rd = rcp(den);
                const double phi = mul(num, rd);
                if constexpr (REC) {
                    phiv[v] = phi;
                    rdv[v] = rd;
                    code |= (1 | (((use_p ? kp : kn) + 1) << 1) | ((use_p ? jh : jl) << 3)) << (5 * v);
                }
                gx[v] = mul(gx[v], phi);
                gy[v] = mul(gy[v], phi);
            }
        }
    }
    Gx[c] = mk4(gx[0], gx[1], gx[2], gx[3]);
    Gy[c] = mk4(gy[0], gy[1], gy[2], gy[3]);
    if constexpr (REC) {
        tape.gx[c] = mk4(gxr[0], gxr[1], gxr[2], gxr[3]);
        tape.gy[c] = mk4(gyr[0], gyr[1], gyr[2], gyr[3]);
        tape.phi[c] = mk4(phiv[0], phiv[1], phiv[2], phiv[3]);
        tape.rden[c] = mk4(rdv[0], rdv[1], rdv[2], rdv[3]);
        tape.code[c] = code;
    }
}

// ---- edge fluxes: edge_convection_flux_kernel, FVMR/src/space/Flux.cpp:230-303, and
// viscous_flux_kernel, FVMR/src/space/viscous_flux/ViscousFlux.cpp:63-168

// get_Uvector_reconstruct_2 (Flux.cpp:41-55): linear reconstruction at the face,
// falling back to the cell value when rho or p leave their range
template <bool LINEAR>
__device__ __forceinline__ d4 face_state(const d4 u, const d4 gx, const d4 gy, double dx, double dy, const Gas& g,
                                         Prim& w) {
    if (!LINEAR) {
        w = to_prim(u, g);
        return u;
    }
    const d4 f = lin(u, gx, gy, dx, dy);
    w = to_prim(f, g);
    if (out_of_range(w.r, w.p)) {
        w = to_prim(u, g);
        return u;
    }
    return f;
}

// face_state that also reports whether the linear reconstruction was kept
template <bool LINEAR>
__device__ __forceinline__ d4 face_state_used(const d4 u, const d4 gx, const d4 gy, double dx, double dy,
                                              const Gas& g, Prim& w, bool& used) {
    used = false;
    if (!LINEAR) {
        w = to_prim(u, g);
        return u;
    }
    const d4 f = lin(u, gx, gy, dx, dy);
    w = to_prim(f, g);
    if (out_of_range(w.r, w.p)) {
        w = to_prim(u, g);
        return u;
    }
    used = true;
    return f;
}

// ---- the discrete adjoint's tape of one stage's Roe edge fluxes (Euler equations):
// per edge the two face states (primitive and conserved), the Roe flux's intermediates
// (RoeRec) and a flag word (bit 0 / 1: the L / R face state is the linear
// reconstruction; bit 2: |un| < am), field-major so that each field is one coalesced row
enum TapeField : int {
    T_LR, T_LU, T_LV, T_LP, T_LIR, T_RR, T_RU, T_RV, T_RP, T_RIR, T_ULY, T_ULZ, T_ULW, T_URY, T_URZ, T_URW,
    T_RUL, T_RUR, T_HL, T_HR, T_IRM, T_RM, T_RRORL, T_W, T_UM, T_VM, T_HM, T_AM2, T_IAM, T_AM, T_UN, T_SEL,
    T_MSTAR, T_DE, T_ETM, T_AE, T_DUROE, T_DPROE, T_DUR, kTapeFields
};
struct EdgeTape {
    double* v = nullptr;   // [kTapeFields][E]
    int* flags = nullptr;  // [E]
    int E = 0;
};

__device__ __forceinline__ void tape_put(const EdgeTape& t, int e, const Prim& L, const Prim& R, const d4 UL,
                                         const d4 UR, const RoeRec& r, int flags) {
    const size_t E = (size_t)t.E;
    double* v = t.v;
    const double vals[kTapeFields] = {L.r,    L.u,   L.v,     L.p,   L.ir,    R.r,    R.u,   R.v,     R.p,    R.ir,
                                      UL.y,   UL.z,  UL.w,    UR.y,  UR.z,    UR.w,   r.ruL, r.ruR,   r.HL,   r.HR,
                                      r.irm,  r.rm,  r.rrorl, r.w,   r.um,    r.vm,   r.Hm,  r.am2,   r.iam,  r.am,
                                      r.un,   r.sel, r.Mstar, r.dE,  r.Etm,   r.ae,   r.dUroe, r.dProe, r.dUr};
#pragma unroll
    for (int f = 0; f < kTapeFields; f++) v[(size_t)f * E + e] = vals[f];
    t.flags[e] = flags | (r.sub ? 4 : 0);
}

// the tape entry of an LLF edge: the two face states only (the reverse rebuilds the rest)
__device__ __forceinline__ void tape_put_faces(const EdgeTape& t, int e, const Prim& L, const Prim& R, const d4 UL,
                                               const d4 UR, int flags) {
    const size_t E = (size_t)t.E;
    double* v = t.v;
    const double vals[T_RUL] = {L.r, L.u, L.v, L.p, L.ir, R.r, R.u, R.v, R.p, R.ir, UL.y, UL.z, UL.w, UR.y, UR.z, UR.w};
#pragma unroll
    for (int f = 0; f < T_RUL; f++) v[(size_t)f * E + e] = vals[f];
    t.flags[e] = flags;
}

// the flux of a recorded edge and its tape entry
template <int FLUX>
__device__ __forceinline__ d4 flux_rec(const Prim& wL, const Prim& wR, const d4 fL, const d4 fR, double nx, double ny,
                                       double len, const Gas& g, const EdgeTape& tape, int e, int flags) {
    if constexpr (FLUX == FLUX_ROE) {
        RoeRec r;
        const d4 F = roe_core<true>(wL, wR, fL, fR, nx, ny, len, g, &r);
        tape_put(tape, e, wL, wR, fL, fR, r, flags);
        return F;
    } else {
        tape_put_faces(tape, e, wL, wR, fL, fR, flags);
        return llf_flux(fL, fR, wL, wR, nx, ny, len, g);
    }
}

// the flux of an interior or periodic edge (R reconstructed at the partner's midpoint for
// periodic ones)
template <int FLUX, bool LINEAR, bool NS>
__device__ __forceinline__ d4 flux_interior_value(int e, const d4* __restrict__ U, const d4* __restrict__ Gx,
                                                  const d4* __restrict__ Gy, const MeshView& m, const Gas& g) {
    const int L = __ldg(&m.e_L[e]), R = __ldg(&m.e_R[e]);
    const double2* gm = reinterpret_cast<const double2*>(&m.e_geom[(size_t)e * 8]);
    const double2 n01 = __ldg(&gm[0]), l23 = __ldg(&gm[1]);
    const double nx = n01.x, ny = n01.y, len = l23.x;
    const d4 uL = ld4(&U[L]), uR = ld4(&U[R]);
    d4 gxL, gyL, gxR, gyR;
    if (LINEAR || NS) {
        gxL = ld4(&Gx[L]);
        gyL = ld4(&Gy[L]);
        gxR = ld4(&Gx[R]);
        gyR = ld4(&Gy[R]);
    }
    Prim wL, wR;
    d4 fL, fR;
    if (LINEAR) {
        const double2 dL = __ldg(&gm[2]), dR = __ldg(&gm[3]);
        fL = face_state<true>(uL, gxL, gyL, dL.x, dL.y, g, wL);
        fR = face_state<true>(uR, gxR, gyR, dR.x, dR.y, g, wR);
    } else {
        fL = face_state<false>(uL, gxL, gyL, 0, 0, g, wL);
        fR = face_state<false>(uR, gxR, gyR, 0, 0, g, wR);
    }
    d4 flux = (FLUX == FLUX_ROE) ? roe_flux(wL, wR, fL, fR, nx, ny, len, g) : llf_flux(fL, fR, wL, wR, nx, ny, len, g);
    if (NS) {
        // get_U_Gradient_mean / get_U_mean (ViscousFluxGPU.cu:7-87): averages of both sides
        const d4 ua = mk4(0.5 * (uL.x + uR.x), 0.5 * (uL.y + uR.y), 0.5 * (uL.z + uR.z), 0.5 * (uL.w + uR.w));
        const d4 gxa = mk4(0.5 * (gxL.x + gxR.x), 0.5 * (gxL.y + gxR.y), 0.5 * (gxL.z + gxR.z), 0.5 * (gxL.w + gxR.w));
        const d4 gya = mk4(0.5 * (gyL.x + gyR.x), 0.5 * (gyL.y + gyR.y), 0.5 * (gyL.z + gyR.z), 0.5 * (gyL.w + gyR.w));
        viscous_flux(flux, ua, gxa, gya, nx, ny, len, g);
    }
    return flux;
}

// an interior or periodic edge: its flux to F[e]; with REC (Roe, Euler) the edge's tape entry
// is written as well
template <int FLUX, bool LINEAR, bool NS, bool REC = false>
__device__ __forceinline__ void flux_interior(int e, const d4* __restrict__ U, const d4* __restrict__ Gx,
                                              const d4* __restrict__ Gy, const MeshView& m, const Gas& g,
                                              d4* __restrict__ F, EdgeTape tape = EdgeTape()) {
    if constexpr (!REC) {
        F[e] = flux_interior_value<FLUX, LINEAR, NS>(e, U, Gx, Gy, m, g);
        return;
    }
    const int L = __ldg(&m.e_L[e]), R = __ldg(&m.e_R[e]);
    const double2* gm = reinterpret_cast<const double2*>(&m.e_geom[(size_t)e * 8]);
    const double2 n01 = __ldg(&gm[0]), l23 = __ldg(&gm[1]);
    const double nx = n01.x, ny = n01.y, len = l23.x;
    const d4 uL = ld4(&U[L]), uR = ld4(&U[R]);
    d4 gxL, gyL, gxR, gyR;
    if (LINEAR || NS) {
        gxL = ld4(&Gx[L]);
        gyL = ld4(&Gy[L]);
        gxR = ld4(&Gx[R]);
        gyR = ld4(&Gy[R]);
    }
    Prim wL, wR;
    d4 fL, fR;
    if constexpr (REC) {
        bool usedL = false, usedR = false;
        double dLx = 0, dLy = 0, dRx = 0, dRy = 0;
        if (LINEAR) {
            const double2 dL = __ldg(&gm[2]), dR = __ldg(&gm[3]);
            dLx = dL.x; dLy = dL.y; dRx = dR.x; dRy = dR.y;
        }
        fL = face_state_used<LINEAR>(uL, gxL, gyL, dLx, dLy, g, wL, usedL);
        fR = face_state_used<LINEAR>(uR, gxR, gyR, dRx, dRy, g, wR, usedR);
        d4 flux = flux_rec<FLUX>(wL, wR, fL, fR, nx, ny, len, g, tape, e, (usedL ? 1 : 0) | (usedR ? 2 : 0));
        if (NS) {
            const d4 ua = mk4(0.5 * (uL.x + uR.x), 0.5 * (uL.y + uR.y), 0.5 * (uL.z + uR.z), 0.5 * (uL.w + uR.w));
            const d4 gxa = mk4(0.5 * (gxL.x + gxR.x), 0.5 * (gxL.y + gxR.y), 0.5 * (gxL.z + gxR.z), 0.5 * (gxL.w + gxR.w));
            const d4 gya = mk4(0.5 * (gyL.x + gyR.x), 0.5 * (gyL.y + gyR.y), 0.5 * (gyL.z + gyR.z), 0.5 * (gyL.w + gyR.w));
            viscous_flux(flux, ua, gxa, gya, nx, ny, len, g);
        }
        F[e] = flux;
        return;
    }
}

// The double-Mach-reflection boundary (Flux.cpp:21-26 and 280-287): the edge is upstream of
// the shock when its midpoint lies left of shock_x + (y + 20 t) / sqrt(3)
// (CBoundaryDoubleShockReflect::isUpStreamOfShock_atBoundary, CBoundaryDoubleShockReflect.cpp:
// 36-49, shock speed 20 from CBoundaryDoubleShockReflect.h:15), t being the stage's time
// get_t_plus_dt(); rounded operation by operation, without contraction, as the reference.
__device__ __forceinline__ bool dsr_upstream_at(double x, double y, double t, const BcData& bc) {
    const double right = __dadd_rn(bc.dsr_x, __ddiv_rn(__dadd_rn(y, __dmul_rn(20.0, t)), bc.sqrt3));
    return x < right;
}
__device__ __forceinline__ bool dsr_upstream(double x, double y, const BcData& bc) {
    return dsr_upstream_at(x, y, __dadd_rn(*bc.clock_t0, __dmul_rn(bc.clock_frac, *bc.clock_dt)), bc);
}

// a boundary edge with a ghost state (walls, far field, inlet, outlet, symmetry,
// double Mach reflection); with REC
// (Roe, Euler) the tape entry of slip-wall, symmetry, far-field, inlet and outlet edges is
// written as well
// the flux of a boundary edge with a ghost state (walls, far field, inlet, outlet, symmetry,
// double Mach reflection)
template <int FLUX, bool LINEAR, bool NS>
__device__ __forceinline__ d4 flux_boundary_value(int e, const d4* __restrict__ U, const d4* __restrict__ Gx,
                                                  const d4* __restrict__ Gy, const MeshView& m, const Gas& g,
                                                  const BcData& bc, Status* st) {
    const int L = __ldg(&m.e_L[e]);
    const int bt = __ldg(&m.e_bc[e]);
    const double* gm = &m.e_geom[(size_t)e * 8];
    const double nx = __ldg(&gm[0]), ny = __ldg(&gm[1]), len = __ldg(&gm[2]);
    const d4 uL = ld4(&U[L]);
    d4 gxL = mk4(0, 0, 0, 0), gyL = gxL;
    if (LINEAR || NS) {
        gxL = ld4(&Gx[L]);
        gyL = ld4(&Gy[L]);
    }
    Prim wL;
    const d4 fL = face_state<LINEAR>(uL, gxL, gyL, __ldg(&gm[4]), __ldg(&gm[5]), g, wL);
    d4 fR = mk4(0, 0, 0, 0);
    switch (bt) {
    case BC_SYMMETRY:  // symmetry
    case BC_WALL_NONVISCOUS:  // slip wall, get_UR_wallNonViscous
        fR = ghost_slip(fL, wL, nx, ny);
        break;
    case BC_WALL_ADIABAT:  // no-slip adiabatic wall, get_UR_wall_adiabat (Flux.cpp:73-79)
        fR = bc.wall_ref ? mk4(fL.x, -0.0, -0.0, fL.w) : mk4(fL.x, -fL.y, -fL.z, fL.w);
        break;
    case BC_INLET:
        if (!ghost_farfield(wL, bc.inlet, bc.a_inlet, bc.son_inlet, nx, ny, g, fR)) atomicAdd(&st->farfield_oor, 1ull);
        break;
    case BC_OUTLET:
        if (!ghost_farfield(wL, bc.outlet, bc.a_outlet, bc.son_outlet, nx, ny, g, fR)) atomicAdd(&st->farfield_oor, 1ull);
        break;
    case BC_INF:
        if (!ghost_farfield(wL, bc.inf, bc.a_inf, bc.son_inf, nx, ny, g, fR)) atomicAdd(&st->farfield_oor, 1ull);
        break;
    case BC_DSR: {  // boundary edges keep their midpoint in the slots of the absent R offset
        const bool up = dsr_upstream(__ldg(&gm[6]), __ldg(&gm[7]), bc);
        const bool ok = up ? ghost_farfield(wL, bc.inlet, bc.a_inlet, bc.son_inlet, nx, ny, g, fR)
                           : ghost_farfield(wL, bc.outlet, bc.a_outlet, bc.son_outlet, nx, ny, g, fR);
        if (!ok) atomicAdd(&st->farfield_oor, 1ull);
        break;
    }
    default:
        break;
    }
    const Prim wR = to_prim(fR, g);
    d4 flux = (FLUX == FLUX_ROE) ? roe_flux(wL, wR, fL, fR, nx, ny, len, g) : llf_flux(fL, fR, wL, wR, nx, ny, len, g);
    if (NS) viscous_flux(flux, uL, gxL, gyL, nx, ny, len, g);  // boundary: the L cell's values
    return flux;
}

template <int FLUX, bool LINEAR, bool NS, bool REC = false>
__device__ __forceinline__ void flux_boundary(int e, const d4* __restrict__ U, const d4* __restrict__ Gx,
                                              const d4* __restrict__ Gy, const MeshView& m, const Gas& g,
                                              const BcData& bc, d4* __restrict__ F, Status* st,
                                              EdgeTape tape = EdgeTape()) {
    if constexpr (!REC) {
        F[e] = flux_boundary_value<FLUX, LINEAR, NS>(e, U, Gx, Gy, m, g, bc, st);
        return;
    }
    const int L = __ldg(&m.e_L[e]);
    const int bt = __ldg(&m.e_bc[e]);
    const double* gm = &m.e_geom[(size_t)e * 8];
    const double nx = __ldg(&gm[0]), ny = __ldg(&gm[1]), len = __ldg(&gm[2]);
    const d4 uL = ld4(&U[L]);
    d4 gxL = mk4(0, 0, 0, 0), gyL = gxL;
    if (LINEAR || NS) {
        gxL = ld4(&Gx[L]);
        gyL = ld4(&Gy[L]);
    }
    Prim wL;
    if constexpr (REC) {
        if (bt == BC_WALL_NONVISCOUS || bt == BC_SYMMETRY || bt == BC_WALL_ADIABAT || bt == BC_INLET || bt == BC_OUTLET || bt == BC_INF || bt == BC_DSR) {
        bool usedL = false;
        int dsr_flag = 0;  // bit 3: a "dsr" edge took the inlet state
        const d4 fL = face_state_used<LINEAR>(uL, gxL, gyL, __ldg(&gm[4]), __ldg(&gm[5]), g, wL, usedL);
        d4 fR;
        if (bt == BC_WALL_NONVISCOUS || bt == BC_SYMMETRY) {
            fR = ghost_slip(fL, wL, nx, ny);
        } else if (bt == BC_WALL_ADIABAT) {  // get_UR_wall_adiabat (Flux.cpp:73-79)
            fR = bc.wall_ref ? mk4(fL.x, -0.0, -0.0, fL.w) : mk4(fL.x, -fL.y, -fL.z, fL.w);
        } else if (bt == BC_DSR) {
            const bool up = dsr_upstream(__ldg(&gm[6]), __ldg(&gm[7]), bc);
            dsr_flag = up ? 8 : 0;
            const bool ok = up ? ghost_farfield(wL, bc.inlet, bc.a_inlet, bc.son_inlet, nx, ny, g, fR)
                               : ghost_farfield(wL, bc.outlet, bc.a_outlet, bc.son_outlet, nx, ny, g, fR);
            if (!ok) atomicAdd(&st->farfield_oor, 1ull);
        } else {
            const bool ok = bt == BC_INLET   ? ghost_farfield(wL, bc.inlet, bc.a_inlet, bc.son_inlet, nx, ny, g, fR)
                            : bt == BC_OUTLET ? ghost_farfield(wL, bc.outlet, bc.a_outlet, bc.son_outlet, nx, ny, g, fR)
                                         : ghost_farfield(wL, bc.inf, bc.a_inf, bc.son_inf, nx, ny, g, fR);
            if (!ok) atomicAdd(&st->farfield_oor, 1ull);
        }
        const Prim wR = to_prim(fR, g);
        d4 flux = flux_rec<FLUX>(wL, wR, fL, fR, nx, ny, len, g, tape, e, (usedL ? 1 : 0) | dsr_flag);
        if (NS) viscous_flux(flux, uL, gxL, gyL, nx, ny, len, g);  // boundary: the L cell's values
        F[e] = flux;
        return;
        }
    }
    // kinds the record does not cover: the flux alone
    F[e] = flux_boundary_value<FLUX, LINEAR, NS>(e, U, Gx, Gy, m, g, bc, st);
}

// ---- residual gather + stage update.  add_edge_flux_to_element_flux (Flux.cpp:346-392)
// sums the cell's edges in slot order with sign -1 where the cell is R;
// calculateFunctionF scales by -1/vol (Evolve.cpp:106-111); the stage combinations
// are those of Evolve.cpp:12-23 (Euler), 58-86 (Kutta RK3) and the Shu-Osher SSP-RK3.
// Returns true when the new state needs the positivity pass.
// With FROM_RES the cell's sum of signed edge fluxes is already in F[c] (the edge-coloured
// scatter, k_flux_scatter, accumulated it colour by colour) and is read instead of gathered.
template <int KIND, bool FROM_RES = false>
__device__ __forceinline__ void update_cell(int c, d4* __restrict__ U, const d4* __restrict__ U0, d4* __restrict__ K1,
                                            d4* __restrict__ rhs_out, const d4* __restrict__ F, const MeshView& m,
                                            double dt, double dt6, const Gas& g, int* __restrict__ flag_list,
                                            unsigned int* flag_count, int flag_cap, Status* st,
                                            d4* __restrict__ rec_R = nullptr) {
    d4 acc;
    if constexpr (FROM_RES) {
        acc = ld4(&F[c]);
    } else {
        const int r0 = __ldg(&m.c_edge[c * 3]);
        const d4 f0 = ld4(&F[r0 >= 0 ? r0 : ~r0]);
        acc = (r0 >= 0) ? f0 : mk4(negd(f0.x), negd(f0.y), negd(f0.z), negd(f0.w));  // 0 + s f0 == s f0
#pragma unroll
        for (int j = 1; j < 3; j++) {
            // a - f == a + (-f) exactly: the sign flipped on the integer pipe (negd), one FP64
            // add a component whichever side of the edge the cell is on
            const int r = __ldg(&m.c_edge[c * 3 + j]);
            d4 f = ld4(&F[r >= 0 ? r : ~r]);
            if (r < 0) f = mk4(negd(f.x), negd(f.y), negd(f.z), negd(f.w));
            acc.x += f.x; acc.y += f.y; acc.z += f.z; acc.w += f.w;
        }
    }
    const double mv = __ldg(&m.c_mvol[c]);
    const d4 k = mk4(mul(mv, acc.x), mul(mv, acc.y), mul(mv, acc.z), mul(mv, acc.w));
    if (rec_R) rec_R[c] = k;  // the stage's residual, kept for the adjoint
    if (KIND == STAGE_RHS) {
        rhs_out[c] = k;
        return;
    }
    d4 un;
    if (KIND == STAGE_EULER) {
        const d4 u = U[c];
        un = mk4(fma(dt, k.x, u.x), fma(dt, k.y, u.y), fma(dt, k.z, u.z), fma(dt, k.w, u.w));
    } else if (KIND == STAGE_RK3_1) {
        const d4 u0 = ld4(&U0[c]);
        const double h = 0.5 * dt;
        un = mk4(fma(h, k.x, u0.x), fma(h, k.y, u0.y), fma(h, k.z, u0.z), fma(h, k.w, u0.w));
        K1[c] = k;
    } else if (KIND == STAGE_RK3_2) {
        const d4 u0 = ld4(&U0[c]);
        const d4 k1 = K1[c];
        const double d2 = 2.0 * dt;
        un = mk4(fma(d2, k.x, fma(-dt, k1.x, u0.x)), fma(d2, k.y, fma(-dt, k1.y, u0.y)),
                 fma(d2, k.z, fma(-dt, k1.z, u0.z)), fma(d2, k.w, fma(-dt, k1.w, u0.w)));
        K1[c] = mk4(fma(4.0, k.x, k1.x), fma(4.0, k.y, k1.y), fma(4.0, k.z, k1.z), fma(4.0, k.w, k1.w));
    } else if (KIND == STAGE_RK3_3) {
        const d4 u0 = ld4(&U0[c]);
        const d4 a = K1[c];
        un = mk4(fma(dt6, a.x + k.x, u0.x), fma(dt6, a.y + k.y, u0.y), fma(dt6, a.z + k.z, u0.z),
                 fma(dt6, a.w + k.w, u0.w));
    } else if (KIND == STAGE_SSP_1) {
        const d4 u = U[c];
        un = mk4(fma(dt, k.x, u.x), fma(dt, k.y, u.y), fma(dt, k.z, u.z), fma(dt, k.w, u.w));
    } else if (KIND == STAGE_SSP_2) {
        const d4 u0 = ld4(&U0[c]);
        const d4 u = U[c];
        un = mk4(fma(0.75, u0.x, mul(0.25, fma(dt, k.x, u.x))), fma(0.75, u0.y, mul(0.25, fma(dt, k.y, u.y))),
                 fma(0.75, u0.z, mul(0.25, fma(dt, k.z, u.z))), fma(0.75, u0.w, mul(0.25, fma(dt, k.w, u.w))));
    } else {  // STAGE_SSP_3
        const d4 u0 = ld4(&U0[c]);
        const d4 u = U[c];
        const double a = 1.0 / 3.0, b = 2.0 / 3.0;
        un = mk4(fma(a, u0.x, mul(b, fma(dt, k.x, u.x))), fma(a, u0.y, mul(b, fma(dt, k.y, u.y))),
                 fma(a, u0.z, mul(b, fma(dt, k.z, u.z))), fma(a, u0.w, mul(b, fma(dt, k.w, u.w))));
    }
    U[c] = un;
    if (final_stage(KIND)) {
        rhs_out[c] = k;
        // detection half of modifyElementFieldU2d (FVMR/src/space/restrict/Restrict.cpp:20-38)
        const Prim w = to_prim(un, g);
        if (is_nan(w.r) || is_nan(w.u) || is_nan(w.v) || is_nan(w.p)) {
            atomicAdd(&st->nan_cells, 1ull);
        } else if (out_of_range(w.r, w.p)) {
            const unsigned int slot = atomicAdd(flag_count, 1u);
            if ((int)slot < flag_cap) flag_list[slot] = c;
        }
    }
}

// ---- positivity pass, modifyElementFieldU2d_kernel (Restrict.cpp:20-90): flagged cells
// are replaced, in the reference's cell order and in place, by the volume-weighted mean
// of their face neighbours.  Run by one thread: the pass is rare and its order matters
// when flagged cells are neighbours.  cell_key orders cells as the reference does.
__device__ __forceinline__ void restrict_pass(d4* U, const MeshView& m, const int* __restrict__ cell_key,
                                              const int* __restrict__ dev_of_key, int n_keys, int* flag_list,
                                              unsigned int* flag_count, int flag_cap, int restrict_ref, const Gas& g,
                                              Status* st) {
    const unsigned int n = *flag_count;
    if (n == 0) return;
    auto fix = [&](int c) {
        double sum[4] = {0, 0, 0, 0}, vs = 0.0;
        int nv = 0;
        for (int k = 0; k < 3; k++) {
            const int q = m.c_nbr[c * 3 + k];
            if (q < 0) continue;
            nv++;
            const double vol = m.c_vol[q];
            const d4 uq = U[q];
            const double uv[4] = {uq.x, uq.y, uq.z, uq.w};
            for (int v = 0; v < 4; v++) {
                sum[v] += uv[v] * vol;
                if (restrict_ref) vs += vol;  // Restrict.cpp:52 adds the volume once per variable
            }
            if (!restrict_ref) vs += vol;
        }
        if (nv == 0) return;
        U[c] = mk4(sum[0] / vs, sum[1] / vs, sum[2] / vs, sum[3] / vs);
        atomicAdd(&st->restricted, 1ull);
    };
    if ((int)n <= flag_cap) {
        for (unsigned int i = 1; i < n; i++) {  // insertion sort by the reference's order
            const int x = flag_list[i];
            const int kx = cell_key[x];
            int j = (int)i - 1;
            while (j >= 0 && cell_key[flag_list[j]] > kx) {
                flag_list[j + 1] = flag_list[j];
                j--;
            }
            flag_list[j + 1] = x;
        }
        for (unsigned int i = 0; i < n; i++) fix(flag_list[i]);
    } else {  // too many to list: scan every cell in the reference's order
        for (int r = 0; r < n_keys; r++) {
            const int c = dev_of_key[r];
            const Prim w = to_prim(U[c], g);
            if (out_of_range(w.r, w.p)) fix(c);
        }
    }
    *flag_count = 0;
}

}  // namespace dev
}  // namespace fvgb

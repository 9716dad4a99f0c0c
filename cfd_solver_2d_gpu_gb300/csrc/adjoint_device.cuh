// Reverse-mode derivatives (vector-Jacobian products) of the device physics,
// written by hand against the exact operation sequence of physics.cuh and
// step_device.cuh, so the adjoint is the derivative of the forward map this
// library computes.  No counterpart in the reference (it has no adjoint).
#pragma once
#include <cuda_runtime.h>

#include "step_device.cuh"

namespace fvgb {
namespace dev {

__device__ __forceinline__ double sgn(double x) { return pos(x) ? 1.0 : (neg(x) ? -1.0 : 0.0); }

// adjoint of to_prim: (bw.r, bw.u, bw.v, bw.p, bw.ir) -> dL/dU added to bU
__device__ __forceinline__ void to_prim_vjp(const d4 U, const Prim& w, const Gas& g, const Prim& bw, d4& bU) {
    const double q = U.w * w.ir - 0.5 * (w.u * w.u + w.v * w.v);
    const double b_q = bw.p * w.r * g.ga1;
    double b_ir = bw.ir + b_q * U.w;
    const double b_u = bw.u - b_q * w.u;
    const double b_v = bw.v - b_q * w.v;
    bU.w += b_q * w.ir;
    bU.y += b_u * w.ir;
    b_ir += b_u * U.y;
    bU.z += b_v * w.ir;
    b_ir += b_v * U.z;
    bU.x += bw.r + bw.p * g.ga1 * q - b_ir * w.ir * w.ir;
}

// adjoint of roe_flux (physics.cuh): bF -> adjoints of the two primitive states
__device__ __forceinline__ void roe_flux_vjp(const Prim& L, const Prim& R, double nx, double ny, double area,
                                             const Gas& g, const d4 bF, Prim& bL, Prim& bR) {
    // ---- forward, exactly as roe_flux ----
    const double unL = nx * L.u + ny * L.v, unR = nx * R.u + ny * R.v;
    const double ruL = L.r * unL, ruR = R.r * unR;
    const double V2L = L.u * L.u + L.v * L.v, V2R = R.u * R.u + R.v * R.v;
    const double EL = L.p * L.ir, ER = R.p * R.ir;
    const double HL = fma(g.gam_over_ga1, EL, 0.5 * V2L);
    const double HR = fma(g.gam_over_ga1, ER, 0.5 * V2R);
    const double prod = R.r * L.r;
    const double irm = rsqrt(prod);
    const double rm = prod * irm;
    const double rrorl = R.r * irm;
    const double w = rcp(rrorl + 1.0);
    const double Xu = fma(R.u, rrorl, L.u), Xv = fma(R.v, rrorl, L.v), XH = fma(HR, rrorl, HL);
    const double um = Xu * w, vm = Xv * w, Hm = XH * w;
    const double Vm2 = um * um + vm * vm;
    const double am2 = g.ga1 * (Hm - 0.5 * Vm2);
    const double iam = rsqrt(am2);
    const double am = am2 * iam;
    const double un = um * nx + vm * ny;
    const double eig1 = fabs(un), eig2 = fabs(un + am), eig3 = fabs(un - am);
    const double dE = (HR - ER) - (HL - EL);
    const double Etm = fma(g.Etm_c, Vm2, Hm * g.inv_gamma);
    const double dW0 = R.r - L.r;
    const double du = R.u - L.u, dv = R.v - L.v;
    const double dW1 = fma(rm, du, dW0 * um);
    const double dW2 = fma(rm, dv, dW0 * vm);
    const double dW3 = fma(rm, dE, dW0 * Etm);
    const double Mstar = (eig2 - eig3) * 0.5 * iam;
    const double dun = fma(nx, du, ny * dv);
    const double dp = R.p - L.p;
    const double astar = (eig2 + eig3) * 0.5;
    const double ae = astar - eig1;
    const double iam2 = iam * iam;
    const double dUroe = fma(Mstar, dun, ae * dp * irm * iam2);
    const double dProe = fma(Mstar, dp, ae * rm * dun);
    const double dUr = dUroe * rm;
    const double h = 0.5 * area;
    // ---- reverse ----
    const double bC0 = h * bF.x, bC1 = h * bF.y, bC2 = h * bF.z, bC3 = h * bF.w;  // central part
    const double bD0 = -bC0, bD1 = -bC1, bD2 = -bC2, bD3 = -bC3;                   // dissipation
    double b_eig1 = bD0 * dW0 + bD1 * dW1 + bD2 * dW2 + bD3 * dW3;
    double b_dW0 = bD0 * eig1, b_dW1 = bD1 * eig1, b_dW2 = bD2 * eig1, b_dW3 = bD3 * eig1;
    const double b_dUr = bD0 + bD1 * um + bD2 * vm + bD3 * Hm;
    double b_um = bD1 * dUr, b_vm = bD2 * dUr, b_Hm = bD3 * dUr;
    const double b_dProe = bD1 * nx + bD2 * ny + bD3 * un;
    double b_un = bD3 * dProe;
    const double b_dUroe = b_dUr * rm;
    double b_rm = b_dUr * dUroe;
    double b_Mstar = b_dProe * dp;
    double b_dp = b_dProe * Mstar;
    double b_ae = b_dProe * rm * dun;
    b_rm += b_dProe * ae * dun;
    double b_dun = b_dProe * ae * rm;
    b_Mstar += b_dUroe * dun;
    b_dun += b_dUroe * Mstar;
    b_ae += b_dUroe * dp * irm * iam2;
    b_dp += b_dUroe * ae * irm * iam2;
    double b_irm = b_dUroe * ae * dp * iam2;
    double b_iam = b_dUroe * ae * dp * irm * 2.0 * iam;
    const double b_astar = b_ae;
    b_eig1 -= b_ae;
    double b_Rp = b_dp, b_Lp = -b_dp;
    double b_du = b_dun * nx, b_dv = b_dun * ny;
    double b_eig2 = b_Mstar * 0.5 * iam, b_eig3 = -b_Mstar * 0.5 * iam;
    b_iam += b_Mstar * (eig2 - eig3) * 0.5;
    b_eig2 += 0.5 * b_astar;
    b_eig3 += 0.5 * b_astar;
    b_rm += b_dW3 * dE;
    const double b_dE = b_dW3 * rm;
    b_dW0 += b_dW3 * Etm;
    const double b_Etm = b_dW3 * dW0;
    b_rm += b_dW2 * dv;
    b_dv += b_dW2 * rm;
    b_dW0 += b_dW2 * vm;
    b_vm += b_dW2 * dW0;
    b_rm += b_dW1 * du;
    b_du += b_dW1 * rm;
    b_dW0 += b_dW1 * um;
    b_um += b_dW1 * dW0;
    double b_Ru = b_du, b_Lu = -b_du, b_Rv = b_dv, b_Lv = -b_dv;
    double b_Rr = b_dW0, b_Lr = -b_dW0;
    double b_Vm2 = b_Etm * g.Etm_c;
    b_Hm += b_Etm * g.inv_gamma;
    double b_HR = b_dE, b_ER = -b_dE, b_HL = -b_dE, b_EL = b_dE;
    b_un += b_eig1 * sgn(un);
    const double s2 = sgn(un + am), s3 = sgn(un - am);
    b_un += b_eig2 * s2 + b_eig3 * s3;
    const double b_am = b_eig2 * s2 - b_eig3 * s3;
    b_um += b_un * nx;
    b_vm += b_un * ny;
    double b_am2 = b_am * iam;
    b_iam += b_am * am2;
    b_am2 += b_iam * (-0.5 * iam * iam2);
    b_Hm += b_am2 * g.ga1;
    b_Vm2 += -0.5 * g.ga1 * b_am2;
    b_um += 2.0 * um * b_Vm2;
    b_vm += 2.0 * vm * b_Vm2;
    const double b_w = b_um * Xu + b_vm * Xv + b_Hm * XH;
    const double bXu = b_um * w, bXv = b_vm * w, bXH = b_Hm * w;
    b_Ru += bXu * rrorl;
    b_Lu += bXu;
    b_Rv += bXv * rrorl;
    b_Lv += bXv;
    b_HR += bXH * rrorl;
    b_HL += bXH;
    double b_rrorl = bXu * R.u + bXv * R.v + bXH * HR - b_w * w * w;
    b_Rr += b_rrorl * irm;
    b_irm += b_rrorl * R.r;
    double b_prod = b_rm * irm;
    b_irm += b_rm * prod;
    b_prod += b_irm * (-0.5 * irm * irm * irm);
    b_Rr += b_prod * L.r;
    b_Lr += b_prod * R.r;
    // central flux (ruL + ruR, ruL uL + ruR uR + nx psum, ruL vL + ruR vR + ny psum, ruL HL + ruR HR)
    const double b_ruL = bC0 + bC1 * L.u + bC2 * L.v + bC3 * HL;
    const double b_ruR = bC0 + bC1 * R.u + bC2 * R.v + bC3 * HR;
    b_Lu += bC1 * ruL;
    b_Ru += bC1 * ruR;
    b_Lv += bC2 * ruL;
    b_Rv += bC2 * ruR;
    b_HL += bC3 * ruL;
    b_HR += bC3 * ruR;
    const double b_psum = bC1 * nx + bC2 * ny;
    b_Lp += b_psum;
    b_Rp += b_psum;
    b_EL += b_HL * g.gam_over_ga1;
    b_ER += b_HR * g.gam_over_ga1;
    const double b_V2L = 0.5 * b_HL, b_V2R = 0.5 * b_HR;
    b_Lp += b_EL * L.ir;
    b_Rp += b_ER * R.ir;
    const double b_Lir = b_EL * L.p, b_Rir = b_ER * R.p;
    b_Lu += 2.0 * L.u * b_V2L;
    b_Lv += 2.0 * L.v * b_V2L;
    b_Ru += 2.0 * R.u * b_V2R;
    b_Rv += 2.0 * R.v * b_V2R;
    b_Lr += b_ruL * unL;
    b_Rr += b_ruR * unR;
    const double b_unL = b_ruL * L.r, b_unR = b_ruR * R.r;
    b_Lu += b_unL * nx;
    b_Lv += b_unL * ny;
    b_Ru += b_unR * nx;
    b_Rv += b_unR * ny;
    bL.r = b_Lr; bL.u = b_Lu; bL.v = b_Lv; bL.p = b_Lp; bL.ir = b_Lir;
    bR.r = b_Rr; bR.u = b_Ru; bR.v = b_Rv; bR.p = b_Rp; bR.ir = b_Rir;
}

// face_state (step_device.cuh) that also reports whether the linear reconstruction was kept
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

// adjoint of ghost_slip (physics.cuh): bUR -> bUL (ghost_slip reads UL.x, UL.w and the
// primitive velocity of UL)
__device__ __forceinline__ void ghost_slip_vjp(const d4 UL, const Prim& wL, double nx, double ny, const d4 bUR,
                                               d4& bUL, Prim& bwL) {
    const double unL = wL.u * nx + wL.v * ny;
    const double utL = wL.u * ny - wL.v * nx;
    const double uxR = -unL * nx + utL * ny;
    const double uyR = -unL * ny - utL * nx;
    bUL.x += bUR.x + bUR.y * uxR + bUR.z * uyR;
    bUL.w += bUR.w;
    const double b_uxR = bUR.y * UL.x, b_uyR = bUR.z * UL.x;
    const double b_unL = -b_uxR * nx - b_uyR * ny;
    const double b_utL = b_uxR * ny - b_uyR * nx;
    bwL.u += b_unL * nx + b_utL * ny;
    bwL.v += b_unL * ny - b_utL * nx;
}

}  // namespace dev
}  // namespace fvgb

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
    const double q = fma(-0.5, fma(w.u, w.u, mul(w.v, w.v)), mul(U.w, w.ir));
    const double b_q = mul(mul(bw.p, w.r), g.ga1);
    double b_ir = fma(b_q, U.w, bw.ir);
    const double b_u = fma(-b_q, w.u, bw.u);
    const double b_v = fma(-b_q, w.v, bw.v);
    bU.w = fma(b_q, w.ir, bU.w);
    bU.y = fma(b_u, w.ir, bU.y);
    b_ir = fma(b_u, U.y, b_ir);
    bU.z = fma(b_v, w.ir, bU.z);
    b_ir = fma(b_v, U.z, b_ir);
    bU.x += fma(-mul(b_ir, w.ir), w.ir, fma(mul(bw.p, g.ga1), q, bw.r));
}

// adjoint of roe_flux (physics.cuh): bF -> adjoints of the two primitive states (bL, bR,
// including 1/rho in .ir) and of the conserved face states the flux reads directly
// (bUL, bUR: the momenta through the mass flux, rho E through H and dE); all four are
// overwritten.  r holds the forward's intermediates (roe_core<true>); the few cheap ones
// not kept are recomputed with roe_core's operations, and the reverse follows the
// forward backwards through the factorisations roe_core uses.
__device__ __forceinline__ void roe_rev(const Prim& L, const Prim& R, const d4 UL, const d4 UR, double nx, double ny,
                                        double area, const Gas& g, const RoeRec& r, const d4 bF, Prim& bL, Prim& bR,
                                        d4& bUL, d4& bUR) {
    const double ruL = r.ruL, ruR = r.ruR, HL = r.HL, HR = r.HR, irm = r.irm, rm = r.rm, rrorl = r.rrorl, w = r.w;
    const double um = r.um, vm = r.vm, Hm = r.Hm, am2 = r.am2, iam = r.iam, un = r.un, sel = r.sel;
    const double Mstar = r.Mstar, dE = r.dE, Etm = r.Etm, ae = r.ae, dUroe = r.dUroe, dProe = r.dProe, dUr = r.dUr;
    const bool sub = r.sub;
    const double sL = UL.w + L.p, sR = UR.w + R.p;
    const double prod = mul(R.r, L.r);
    const double Xu = fma(R.u, rrorl, L.u), Xv = fma(R.v, rrorl, L.v), XH = fma(HR, rrorl, HL);
    const double eig1 = fabs(un);
    const double dW0 = R.r - L.r;
    const double du = R.u - L.u, dv = R.v - L.v;
    const double dW1 = fma(rm, du, mul(dW0, um));
    const double dW2 = fma(rm, dv, mul(dW0, vm));
    const double dW3 = fma(rm, dE, mul(dW0, Etm));
    const double dun = fma(nx, du, mul(ny, dv));
    const double dp = R.p - L.p;
    const double iam2 = mul(iam, iam);
    const double t1 = mul(ae, dp), t12 = mul(t1, irm);  // dUroe's second term is t12 iam2
    const double t3 = mul(ae, rm);                      // dProe's second term is t3 dun
    const double h = mul(0.5, area);
    // ---- reverse ----
    const double bC0 = mul(h, bF.x), bC1 = mul(h, bF.y), bC2 = mul(h, bF.z), bC3 = mul(h, bF.w);  // central part
    // dissipation: the sign flips on the integer pipe (negd), since these feed integer-pipe
    // products that cannot absorb a negation the way an FP64 instruction's operand does
    const double bD0 = negd(bC0), bD1 = negd(bC1), bD2 = negd(bC2), bD3 = negd(bC3);
    double b_eig1 = fma(bD3, dW3, fma(bD2, dW2, fma(bD1, dW1, mul(bD0, dW0))));
    double b_dW0 = mul(bD0, eig1);
    const double b_dW1 = mul(bD1, eig1), b_dW2 = mul(bD2, eig1), b_dW3 = mul(bD3, eig1);
    const double b_dUr = fma(bD3, Hm, fma(bD2, vm, fma(bD1, um, bD0)));
    double b_um = mul(bD1, dUr), b_vm = mul(bD2, dUr), b_Hm = mul(bD3, dUr);
    const double b_dProe = fma(bD3, un, fma(bD2, ny, mul(bD1, nx)));
    double b_un = mul(bD3, dProe);
    // dUr = dUroe rm
    const double b_dUroe = mul(b_dUr, rm);
    double b_rm = mul(b_dUr, dUroe);
    // dProe = Mstar dp + t3 dun
    double b_Mstar = mul(b_dProe, dp);
    double b_dp = mul(b_dProe, Mstar);
    const double b_t3 = mul(b_dProe, dun);
    double b_dun = mul(b_dProe, t3);
    double b_ae = mul(b_t3, rm);
    b_rm = fma(b_t3, ae, b_rm);
    // dUroe = Mstar dun + t12 iam2
    b_Mstar = fma(b_dUroe, dun, b_Mstar);
    b_dun = fma(b_dUroe, Mstar, b_dun);
    const double b_iam2 = mul(b_dUroe, t12);
    const double b_t12 = mul(b_dUroe, iam2);
    double b_irm = mul(b_t12, t1);
    const double b_t1 = mul(b_t12, irm);
    b_ae = fma(b_t1, dp, b_ae);
    b_dp = fma(b_t1, ae, b_dp);
    double b_iam = mul(mul(2.0, iam), b_iam2);
    // ae = astar - eig1; astar = am or eig1
    double b_am = sub ? b_ae : 0.0;
    b_eig1 += sub ? -b_ae : 0.0;  // astar = eig1 when not sub: the two cancel
    // dp, dun, dW*, dE, Etm
    double b_Rp = b_dp, b_Lp = -b_dp;
    double b_du = mul(b_dun, nx), b_dv = mul(b_dun, ny);
    b_rm += fma(b_dW1, du, fma(b_dW2, dv, mul(b_dW3, dE)));
    const double b_dE = mul(b_dW3, rm);
    const double b_Etm = mul(b_dW3, dW0);
    b_dW0 += fma(b_dW1, um, fma(b_dW2, vm, mul(b_dW3, Etm)));
    b_dv = fma(b_dW2, rm, b_dv);
    b_vm = fma(b_dW2, dW0, b_vm);
    b_du = fma(b_dW1, rm, b_du);
    b_um = fma(b_dW1, dW0, b_um);
    double b_Rr = b_dW0, b_Lr = -b_dW0;
    double b_Ru = b_du, b_Lu = -b_du, b_Rv = b_dv, b_Lv = -b_dv;
    double b_Vm2 = mul(b_Etm, g.Etm_c);
    b_Hm = fma(b_Etm, g.inv_gamma, b_Hm);
    // dE = URw Rir - ULw Lir
    double b_URw = mul(b_dE, R.ir), b_ULw = -mul(b_dE, L.ir);
    double b_Rir = mul(b_dE, UR.w), b_Lir = -mul(b_dE, UL.w);
    // Mstar = sel iam; sel = un (sub) or copysign(am, un)
    const double b_sel = mul(b_Mstar, iam);
    b_iam = fma(b_Mstar, sel, b_iam);
    if (sub) b_un += b_sel;
    else b_am += b_sel * copysign(1.0, un);
    // eig1 = |un|; un = um nx + vm ny
    b_un += b_eig1 * sgn(un);
    b_um += b_un * nx;
    b_vm += b_un * ny;
    // am = am2 iam; iam = am2^(-1/2); am2 = ga1 (Hm - Vm2/2); Vm2 = um^2 + vm^2
    double b_am2 = mul(b_am, iam);
    b_iam = fma(b_am, am2, b_iam);
    b_am2 = fma(-mul(mul(0.5, b_iam), iam), iam2, b_am2);
    b_Hm = fma(b_am2, g.ga1, b_Hm);
    b_Vm2 = fma(-mul(0.5, g.ga1), b_am2, b_Vm2);
    b_um = fma(mul(2.0, um), b_Vm2, b_um);
    b_vm = fma(mul(2.0, vm), b_Vm2, b_vm);
    // (um, vm, Hm) = (Xu, Xv, XH) w
    const double b_w = fma(b_Hm, XH, fma(b_vm, Xv, mul(b_um, Xu)));
    const double bXu = mul(b_um, w), bXv = mul(b_vm, w), bXH = mul(b_Hm, w);
    b_Ru = fma(bXu, rrorl, b_Ru);
    b_Lu += bXu;
    b_Rv = fma(bXv, rrorl, b_Rv);
    b_Lv += bXv;
    double b_HR = mul(bXH, rrorl), b_HL = bXH;
    double b_rrorl = fma(-mul(b_w, w), w, fma(bXH, HR, fma(bXv, R.v, mul(bXu, R.u))));
    // rrorl = Rr irm; rm = prod irm; irm = prod^(-1/2); prod = Rr Lr
    b_Rr = fma(b_rrorl, irm, b_Rr);
    b_irm = fma(b_rrorl, R.r, b_irm);
    double b_prod = mul(b_rm, irm);
    b_irm = fma(b_rm, prod, b_irm);
    b_prod = fma(-mul(mul(mul(0.5, b_irm), irm), irm), irm, b_prod);
    b_Rr = fma(b_prod, L.r, b_Rr);
    b_Lr = fma(b_prod, R.r, b_Lr);
    // central flux (ruL + ruR, ruL uL + ruR uR + nx psum, ruL vL + ruR vR + ny psum, ruL HL + ruR HR)
    const double b_ruL = fma(bC3, HL, fma(bC2, L.v, fma(bC1, L.u, bC0)));
    const double b_ruR = fma(bC3, HR, fma(bC2, R.v, fma(bC1, R.u, bC0)));
    b_Lu = fma(bC1, ruL, b_Lu);
    b_Ru = fma(bC1, ruR, b_Ru);
    b_Lv = fma(bC2, ruL, b_Lv);
    b_Rv = fma(bC2, ruR, b_Rv);
    b_HL = fma(bC3, ruL, b_HL);
    b_HR = fma(bC3, ruR, b_HR);
    const double b_psum = fma(bC2, ny, mul(bC1, nx));
    b_Lp += b_psum;
    b_Rp += b_psum;
    // H = (rho E + p) / rho
    b_ULw = fma(b_HL, L.ir, b_ULw);
    b_Lp = fma(b_HL, L.ir, b_Lp);
    b_Lir = fma(b_HL, sL, b_Lir);
    b_URw = fma(b_HR, R.ir, b_URw);
    b_Rp = fma(b_HR, R.ir, b_Rp);
    b_Rir = fma(b_HR, sR, b_Rir);
    bL.r = b_Lr; bL.u = b_Lu; bL.v = b_Lv; bL.p = b_Lp; bL.ir = b_Lir;
    bR.r = b_Rr; bR.u = b_Ru; bR.v = b_Rv; bR.p = b_Rp; bR.ir = b_Rir;
    // mass fluxes n . (rho u)
    bUL = mk4(0.0, mul(b_ruL, nx), mul(b_ruL, ny), b_ULw);
    bUR = mk4(0.0, mul(b_ruR, nx), mul(b_ruR, ny), b_URw);
}

// the same with the forward recomputed (for a caller without the recorded intermediates)
__device__ __forceinline__ void roe_flux_vjp(const Prim& L, const Prim& R, const d4 UL, const d4 UR, double nx,
                                             double ny, double area, const Gas& g, const d4 bF, Prim& bL, Prim& bR,
                                             d4& bUL, d4& bUR) {
    RoeRec r;
    roe_core<true>(L, R, UL, UR, nx, ny, area, g, &r);
    roe_rev(L, R, UL, UR, nx, ny, area, g, r, bF, bL, bR, bUL, bUR);
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

// adjoint of llf_flux (physics.cuh; LocalLaxFriedrichs.cpp:4-47): bF -> adjoints of the two
// primitive face states (bL, bR, 1/rho in .ir) and of the conserved ones (bUL, bUR), all four
// overwritten.  The flux is rebuilt from the face states; max(aL, aR) passes its adjoint to the
// side dmax chose.
__device__ __forceinline__ void llf_rev(const d4 UL, const d4 UR, const Prim& L, const Prim& R, double nx, double ny,
                                        double length, const Gas& g, const d4 bF, Prim& bL, Prim& bR, d4& bUL,
                                        d4& bUR) {
    const double unL = fma(nx, L.u, ny * L.v), unR = fma(nx, R.u, ny * R.v);
    const double ruL = fma(nx, UL.y, ny * UL.z), ruR = fma(nx, UR.y, ny * UR.z);
    const double hl = (UL.w + L.p) * L.ir, hr = (UR.w + R.p) * R.ir;
    const double sL = sqrt(g.gamma * L.p * L.ir), sR = sqrt(g.gamma * R.p * R.ir);
    const double aL = fabs(unL) + sL, aR = fabs(unR) + sR;
    const double lm = dmax(aL, aR);
    const double h = 0.5 * length;
    const d4 m = mk4(h * bF.x, h * bF.y, h * bF.z, h * bF.w);
    const double b_lm = -(m.x * (UR.x - UL.x) + m.y * (UR.y - UL.y) + m.z * (UR.z - UL.z) + m.w * (UR.w - UL.w));
    bUL = mk4(lm * m.x, lm * m.y, lm * m.z, lm * m.w);
    bUR = mk4(-lm * m.x, -lm * m.y, -lm * m.z, -lm * m.w);
    const double b_ruL = m.x + m.y * L.u + m.z * L.v + m.w * hl;
    const double b_ruR = m.x + m.y * R.u + m.z * R.v + m.w * hr;
    bL = Prim{0, m.y * ruL, m.z * ruL, nx * m.y + ny * m.z, 0};
    bR = Prim{0, m.y * ruR, m.z * ruR, nx * m.y + ny * m.z, 0};
    // h = (rho E + p) / rho
    const double b_hl = m.w * ruL, b_hr = m.w * ruR;
    bUL.w += b_hl * L.ir; bL.p += b_hl * L.ir; bL.ir += b_hl * (UL.w + L.p);
    bUR.w += b_hr * R.ir; bR.p += b_hr * R.ir; bR.ir += b_hr * (UR.w + R.p);
    // ru = n . (rho u)
    bUL.y += nx * b_ruL; bUL.z += ny * b_ruL;
    bUR.y += nx * b_ruR; bUR.z += ny * b_ruR;
    // lm = max(aL, aR), a = |un| + sqrt(gamma p / rho)
    const bool right = dlt(aL, aR);
    const double b_aL = right ? 0.0 : b_lm, b_aR = right ? b_lm : 0.0;
    const double b_unL = b_aL * sgn(unL), b_unR = b_aR * sgn(unR);
    bL.u += nx * b_unL; bL.v += ny * b_unL;
    bR.u += nx * b_unR; bR.v += ny * b_unR;
    if (sL > 0) { bL.p += b_aL * g.gamma * L.ir / (2.0 * sL); bL.ir += b_aL * g.gamma * L.p / (2.0 * sL); }
    if (sR > 0) { bR.p += b_aR * g.gamma * R.ir / (2.0 * sR); bR.ir += b_aR * g.gamma * R.p / (2.0 * sR); }
}

// adjoint of viscous_flux (physics.cuh): bF -> adjoints of the averaged state U and of the
// averaged gradients gx, gy (only bF.y, .z, .w matter; the mass flux has no viscous part);
// the forward's intermediates are recomputed with its operations, then reversed
__device__ __forceinline__ void viscous_vjp(const d4 U, const d4 gx, const d4 gy, double nx, double ny, double area,
                                            const Gas& g, const d4 bF, d4& bU, d4& bgx, d4& bgy) {
    const double ir = rcp(U.x);
    const double u = U.y * ir, v = U.z * ir, E = U.w * ir;
    const double dudx = ir * (gx.y - u * gx.x);
    const double dvdx = ir * (gx.z - v * gx.x);
    const double dudy = ir * (gy.y - u * gy.x);
    const double dvdy = ir * (gy.z - v * gy.x);
    const double dEdx = ir * (gx.w - E * gx.x);
    const double dEdy = ir * (gy.w - E * gy.x);
    const double iCv = g.inv_Cv;
    const double T = iCv * (E - 0.5 * (u * u + v * v));
    const double dTdx = (dEdx - u * dudx - v * dvdx) * iCv;
    const double dTdy = (dEdy - u * dudy - v * dvdy) * iCv;
    const double mu = g.C1 * (T * sqrt(T)) * rcp(T + 110.4);
    const double div = dudx + dvdy;
    const double NMD = -2.0 / 3.0;
    const double txx = mu * fma(NMD, div, 2.0 * dudx);
    const double tyy = mu * fma(NMD, div, 2.0 * dvdy);
    const double txy = mu * (dudy + dvdx);
    const double akmu = g.Cp * (mu * (1.0 / 0.72));
    // F.y -= (txx nx + txy ny) A; F.z -= (txy nx + tyy ny) A; F.w -= (Phix nx + Phiy ny) A
    double b_txx = -area * nx * bF.y, b_txy = -area * (ny * bF.y + nx * bF.z), b_tyy = -area * ny * bF.z;
    const double b_Phix = -area * nx * bF.w, b_Phiy = -area * ny * bF.w;
    double b_u = 0, b_v = 0, b_E = 0, b_ir = 0, b_mu = 0;
    // Phix = akmu dTdx + u txx + v txy, Phiy = akmu dTdy + u txy + v tyy
    const double b_akmu = b_Phix * dTdx + b_Phiy * dTdy;
    const double b_dTdx = b_Phix * akmu, b_dTdy = b_Phiy * akmu;
    b_u += b_Phix * txx + b_Phiy * txy;
    b_v += b_Phix * txy + b_Phiy * tyy;
    b_txx += b_Phix * u;
    b_txy += b_Phix * v + b_Phiy * u;
    b_tyy += b_Phiy * v;
    b_mu += b_akmu * g.Cp * (1.0 / 0.72);
    // stresses
    b_mu += b_txx * fma(NMD, div, 2.0 * dudx) + b_tyy * fma(NMD, div, 2.0 * dvdy) + b_txy * (dudy + dvdx);
    const double b_div = mu * NMD * (b_txx + b_tyy);
    double b_dudx = 2.0 * mu * b_txx + b_div, b_dvdy = 2.0 * mu * b_tyy + b_div;
    double b_dudy = mu * b_txy, b_dvdx = mu * b_txy;
    // Sutherland: mu = C1 T^1.5 / (T + 110.4)
    double b_T = b_mu * mu * (1.5 / T - 1.0 / (T + 110.4));
    // temperature gradients
    const double b_dEdx = iCv * b_dTdx, b_dEdy = iCv * b_dTdy;
    b_u -= iCv * (b_dTdx * dudx + b_dTdy * dudy);
    b_v -= iCv * (b_dTdx * dvdx + b_dTdy * dvdy);
    b_dudx -= iCv * b_dTdx * u;
    b_dvdx -= iCv * b_dTdx * v;
    b_dudy -= iCv * b_dTdy * u;
    b_dvdy -= iCv * b_dTdy * v;
    // T = (E - (u^2 + v^2)/2) / Cv
    b_E += iCv * b_T;
    b_u -= iCv * b_T * u;
    b_v -= iCv * b_T * v;
    // derivatives of u, v, E from the conserved gradients
    bgx = mk4(0, ir * b_dudx, ir * b_dvdx, ir * b_dEdx);
    bgy = mk4(0, ir * b_dudy, ir * b_dvdy, ir * b_dEdy);
    bgx.x = -ir * (b_dudx * u + b_dvdx * v + b_dEdx * E);
    bgy.x = -ir * (b_dudy * u + b_dvdy * v + b_dEdy * E);
    b_ir += b_dudx * (gx.y - u * gx.x) + b_dvdx * (gx.z - v * gx.x) + b_dEdx * (gx.w - E * gx.x) +
            b_dudy * (gy.y - u * gy.x) + b_dvdy * (gy.z - v * gy.x) + b_dEdy * (gy.w - E * gy.x);
    b_u -= ir * (b_dudx * gx.x + b_dudy * gy.x);
    b_v -= ir * (b_dvdx * gx.x + b_dvdy * gy.x);
    b_E -= ir * (b_dEdx * gx.x + b_dEdy * gy.x);
    // u = rho u / rho, v, E likewise
    bU = mk4(0, b_u * ir, b_v * ir, b_E * ir);
    b_ir += b_u * U.y + b_v * U.z + b_E * U.w;
    bU.x = -b_ir * ir * ir;
}

// adjoint of ghost_farfield (physics.cuh; get_UR_farField, FVMR/src/space/Flux.cpp:81-163):
// bUR, the adjoint of the ghost's conserved state, onto the interior face state's primitive
// variables (bw; .ir carries the 1/rho the sound speed reads).  The branch is re-evaluated
// with the forward's operations on the same inputs, so it is the forward's branch.
__device__ __forceinline__ void ghost_farfield_vjp(const Prim& e, const double* fs, double fa, double fson,
                                                   double nx, double ny, const Gas& g, const d4 bUR, Prim& bw) {
    const double ae = sqrt(g.gamma * e.p * e.ir);
    const double qnf = fs[1] * nx + fs[2] * ny;
    const double qne = e.u * nx + e.v * ny;
    const double rf = qnf - 2.0 * fa * g.inv_ga1;
    const double re = qne + 2.0 * ae * g.inv_ga1;
    const double qn = 0.5 * (re + rf);
    const double as = g.ga1 * (re - rf) * 0.25;
    if (qn <= -as) return;  // supersonic inflow: the ghost is the far-field state
    double r0, u0, v0, son = 0.0, X = 0.0;
    const bool outflow = !(qn < 0);
    if (qn < as) {
        double qtx, qty;
        if (!outflow) {
            son = fson;
            qtx = fs[1] - qnf * nx;
            qty = fs[2] - qnf * ny;
        } else {
            son = e.p / pow(e.r, g.gamma);
            qtx = e.u - qne * nx;
            qty = e.v - qne * ny;
        }
        X = as * as / son * g.inv_gamma;
        r0 = pow(X, g.inv_ga1);
        u0 = qtx + qn * nx;
        v0 = qty + qn * ny;
    } else {
        r0 = e.r; u0 = e.u; v0 = e.v;
    }
    // to_cons: (r, r u, r v, p/(gamma-1) + r (u^2 + v^2)/2)
    const double br0 = bUR.x + bUR.y * u0 + bUR.z * v0 + 0.5 * bUR.w * (u0 * u0 + v0 * v0);
    const double bu0 = (bUR.y + bUR.w * u0) * r0;
    const double bv0 = (bUR.z + bUR.w * v0) * r0;
    const double bp0 = bUR.w * g.inv_ga1;
    if (!(qn < as)) {  // supersonic outflow: the ghost is the interior state
        bw.r += br0; bw.u += bu0; bw.v += bv0; bw.p += bp0;
        return;
    }
    // p0 = as^2 r0 / gamma, r0 = X^(1/(gamma-1)), X = as^2 / (son gamma)
    double b_as = bp0 * 2.0 * as * r0 * g.inv_gamma;
    const double b_r0 = br0 + bp0 * as * as * g.inv_gamma;
    const double b_X = b_r0 * g.inv_ga1 * r0 / X;
    b_as += b_X * 2.0 * as / son * g.inv_gamma;
    const double b_son = -b_X * X / son;
    // u0 = qtx + qn nx, v0 = qty + qn ny
    const double b_qn = bu0 * nx + bv0 * ny;
    double b_qne = 0.0;
    if (outflow) {  // qtx = u - qne nx, qty = v - qne ny, son = p / r^gamma
        bw.u += bu0;
        bw.v += bv0;
        b_qne -= bu0 * nx + bv0 * ny;
        bw.p += b_son * son / e.p;
        bw.r -= b_son * g.gamma * son / e.r;
    }
    // qn = (re + rf)/2, as = (gamma-1)(re - rf)/4, re = qne + 2 ae/(gamma-1)
    const double b_re = 0.5 * b_qn + 0.25 * g.ga1 * b_as;
    b_qne += b_re;
    const double b_ae = 2.0 * g.inv_ga1 * b_re;
    bw.u += b_qne * nx;
    bw.v += b_qne * ny;
    // ae = sqrt(gamma p ir)
    bw.p += b_ae * g.gamma * e.ir / (2.0 * ae);
    bw.ir += b_ae * g.gamma * e.p / (2.0 * ae);
}

}  // namespace dev
}  // namespace fvgb

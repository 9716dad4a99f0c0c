// Device-side physics of the explicit step, FP64.
//
// Each function computes what the cited reference function computes.  The
// formulas are rearranged to spend fewer FP64 divides and square roots (the
// FP64 pipe, not HBM, bounds this step on GB300): one reciprocal of rho per
// state instead of three divides, one reciprocal square root for the Roe
// average, T*sqrt(T) for T^1.5, square roots from the reciprocal square root.  Results differ from the reference's by a few
// ulp per operation; decisions (range checks, limiter bounds, far-field
// branches) are taken on the same quantities in the same way.
#pragma once
#include <cuda_runtime.h>

#include "bc_types.h"
#include "softfp64.cuh"

// Where the kernels multiply (a plain product, not a fused multiply-add), they call mul():
// the correctly rounded product computed on the integer pipes (softfp64.cuh), which run
// beside the FP64 pipe that bounds these kernels on GB300.  The result is the IEEE
// product bit for bit either way; FVGB_SOFT_MUL=0 at build time puts the products back on
// the FP64 pipe (the same bits, for side-by-side timing).
#ifndef FVGB_SOFT_MUL
#define FVGB_SOFT_MUL 1
#endif

namespace fvgb {

// cell state (rho, rho u, rho v, rho E): 32-byte aligned so one state is one sector
typedef double4_32a d4;
__host__ __device__ __forceinline__ d4 mk4(double x, double y, double z, double w) {
    d4 r;
    r.x = x;
    r.y = y;
    r.z = z;
    r.w = w;
    return r;
}

namespace dev {

constexpr double kEps = 1e-10;                  // FVMR/src/math/CommonValue.h:24
constexpr double kRhoMax = 300.0;               // CommonValue.h:27
constexpr double kPMax = 400.0 * 101325.0;      // CommonValue.h:30

struct Gas {
    double gamma, ga1, gam_over_ga1, inv_ga1, Etm_c, inv_gamma;  // derived constants
    double R, Cv, Cp, inv_Cv, C1;                                 // viscous constants
};

struct Prim {
    double r, u, v, p, ir;  // rho, u, v, p, 1/rho
};

// ---- comparisons on the integer pipe ------------------------------------
// A GB300 SM issues 2 FP64 lane-operations per clock but 64 integer ones, so
// comparisons, minima and maxima of doubles are done on their bit patterns.
// okey() maps a double to an int64 whose signed order is the order of the
// doubles (for non-NaN values, with -0 just below +0); min/max select one of
// their arguments, so their results are exact.
__device__ __forceinline__ long long okey(double x) {
    const long long b = __double_as_longlong(x);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool dlt(double a, double b) { return okey(a) < okey(b); }
__device__ __forceinline__ double dmax(double a, double b) { return okey(a) < okey(b) ? b : a; }
__device__ __forceinline__ double dmin(double a, double b) { return okey(b) < okey(a) ? b : a; }
// x > 0 and x < 0 in the IEEE sense (both false for -0 and +0)
__device__ __forceinline__ bool pos(double x) { return __double_as_longlong(x) > 0; }
__device__ __forceinline__ bool neg(double x) {
    const long long b = __double_as_longlong(x);
    return b < 0 && (b << 1) != 0;
}
__device__ __forceinline__ bool is_nan(double x) {
    return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}

// -x, |x| and copysign(x, y) as sign-bit operations on the integer pipe (exact; NaN
// payloads kept).  Written in C++ -- a unary minus, fabs, or even an integer XOR or AND of
// the bits -- the compiler issues them as an FP64 add, one FP64-pipe slot each; inline PTX
// keeps them on the integer pipe.
__device__ __forceinline__ double negd(double x) {
    double r;
    asm("{ .reg .b64 t; mov.b64 t, %1; xor.b64 t, t, 0x8000000000000000; mov.b64 %0, t; }" : "=d"(r) : "d"(x));
    return r;
}
__device__ __forceinline__ double absd(double x) {
    double r;
    asm("{ .reg .b64 t; mov.b64 t, %1; and.b64 t, t, 0x7fffffffffffffff; mov.b64 %0, t; }" : "=d"(r) : "d"(x));
    return r;
}
__device__ __forceinline__ double copysignd(double x, double y) {
    double r;
    asm("{ .reg .b64 a, b; mov.b64 a, %1; mov.b64 b, %2; and.b64 a, a, 0x7fffffffffffffff;"
        " and.b64 b, b, 0x8000000000000000; or.b64 a, a, b; mov.b64 %0, a; }"
        : "=d"(r) : "d"(x), "d"(y));
    return r;
}

// a * b, rounded once to nearest even, never contracted into a fused multiply-add
__device__ __forceinline__ double mul(double a, double b) {
#if FVGB_SOFT_MUL
    return soft::dmul(a, b);
#else
    return __dmul_rn(a, b);
#endif
}

// 1/x: the hardware's approximate reciprocal y (relative error e = 1 - x y,
// |e| < 2^-22) refined by the cubic series 1/x = y (1 + e + e^2 + O(e^3)), one
// fused multiply-add fewer than two Newton steps for the same accuracy: the
// truncation y e^3 is below 2^-66, so the result is within ~1 ulp of the
// correctly rounded value for normal x.
__device__ __forceinline__ double rcp(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
}

// 1/sqrt(x) and sqrt(x) for normal x > 0: the hardware's approximate reciprocal square root
// y (relative error below 2^-22) refined by the series (1 - e)^(-1/2) = 1 + e/2 + 3e^2/8 +
// O(e^3), e = 1 - x y^2, whose truncation is below 2^-63; sqrt(x) = x rsq(x).  Both are
// within ~1.5 ulp of the correctly rounded value.  Zero, subnormal, negative, infinite and
// NaN arguments call the library functions out of line (a real branch: see softfp64.cuh).
static __device__ __noinline__ double rsq_rare(double x) { return rsqrt(x); }
static __device__ __noinline__ double sq_rare(double x) { return sqrt(x); }
__device__ __forceinline__ bool normal_pos(double x) {
    return (unsigned long long)__double_as_longlong(x) - 0x0010000000000000ull < 0x7fe0000000000000ull;
}
__device__ __forceinline__ double rsq(double x) {
    if (!normal_pos(x)) return rsq_rare(x);
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x, mul(y, y), 1.0);
    return fma(mul(y, e), fma(0.375, e, 0.5), y);
}
__device__ __forceinline__ double sq(double x) {
    if (!normal_pos(x)) return sq_rare(x);
    return mul(x, rsq(x));
}

// U2ruvp_host, FVMR/src/math/PhysicalKernel.h:11-18; the pressure as
// (gamma-1) (rho E - (rho u u + rho v v)/2), equal to the reference's
// rho (gamma-1) (E/rho - (u u + v v)/2) with four FP64 operations instead of six
__device__ __forceinline__ Prim to_prim(const d4 U, const Gas& g) {
    Prim w;
    w.ir = rcp(U.x);
    w.r = U.x;
    w.u = mul(U.y, w.ir);
    w.v = mul(U.z, w.ir);
    w.p = mul(g.ga1, fma(-0.5, fma(U.y, w.u, mul(U.z, w.v)), U.w));
    return w;
}

// ruvp2U_host, PhysicalKernel.h:20-27
__device__ __forceinline__ d4 to_cons(double r, double u, double v, double p, const Gas& g) {
    return mk4(r, r * u, r * v, p * g.inv_ga1 + 0.5 * r * (u * u + v * v));
}

// Restrict::outOfRange, FVMR/src/space/restrict/Restrict.h:15-23: rho or p
// below 1e-10 or above 300 / 400 atm (NaN counts as in range, as in the
// reference, where every comparison with NaN is false)
__device__ __forceinline__ bool out_of_range(double r, double p) {
    const long long kr = okey(r), kp = okey(p);
    const bool r_nan = is_nan(r), p_nan = is_nan(p);
    return (!r_nan && (kr < okey(kEps) || kr > okey(kRhoMax))) || (!p_nan && (kp < okey(kEps) || kp > okey(kPMax)));
}

// get_U_reconstruct_singleValue (linear), FVMR/src/space/Flux.cpp:28-39
__device__ __forceinline__ d4 lin(const d4 U, const d4 gx, const d4 gy, double dx, double dy) {
    return mk4(fma(gy.x, dy, fma(gx.x, dx, U.x)), fma(gy.y, dy, fma(gx.y, dx, U.y)),
                        fma(gy.z, dy, fma(gx.z, dx, U.z)), fma(gy.w, dy, fma(gx.w, dx, U.w)));
}

// The forward values the Roe flux's reverse (roe_rev, adjoint_device.cuh) reads, kept
// per edge by the recorded forward of the discrete adjoint so that the reverse sweep
// need not recompute them (memory is cheap next to FP64 issue on this part).
struct RoeRec {
    double ruL, ruR, HL, HR, irm, rm, rrorl, w, um, vm, Hm, am2, iam, am, un, sel, Mstar, dE, Etm, ae, dUroe,
        dProe, dUr;
    bool sub;
};

// ConvectRoeCommon2d + RoeDissapationTerm2d, FVMR/src/space/convection/Roe.cpp:380-538
// (entropy fix off, static mesh).  L, R: the face states' primitive variables; UL, UR
// the same states conserved.  Exact identities save FP64 work: the mass flux is
// n . (rho u) from the momentum, the total enthalpy H = gamma/(gamma-1) p/rho + V^2/2
// is (rho E + p)/rho, H - p/rho is rho E/rho, and with a > 0
// (|un + a| + |un - a|)/2 = max(|un|, a), (|un + a| - |un - a|)/2 = un if |un| < a,
// else a sgn(un).  With REC the intermediates also go to *rec.
template <bool REC>
__device__ __forceinline__ d4 roe_core(const Prim& L, const Prim& R, const d4 UL, const d4 UR, double nx, double ny,
                                       double area, const Gas& g, RoeRec* rec) {
    const double ruL = fma(nx, UL.y, mul(ny, UL.z)), ruR = fma(nx, UR.y, mul(ny, UR.z));
    const double HL = mul(UL.w + L.p, L.ir), HR = mul(UR.w + R.p, R.ir);
    const double psum = L.p + R.p;
    // central part 0.5 (F_L + F_R).n, scaled by 0.5 area at the end
    d4 F = mk4(ruL + ruR, fma(ruL, L.u, fma(ruR, R.u, mul(nx, psum))), fma(ruL, L.v, fma(ruR, R.v, mul(ny, psum))),
               fma(ruL, HL, mul(ruR, HR)));
    // Roe averages: rm = sqrt(rR rL), rrorl = sqrt(rR/rL) = rR / rm
    const double prod = mul(R.r, L.r);
    const double irm = rsq(prod);
    const double rm = mul(prod, irm);
    const double rrorl = mul(R.r, irm);
    const double w = rcp(rrorl + 1.0);
    const double um = mul(fma(R.u, rrorl, L.u), w);
    const double vm = mul(fma(R.v, rrorl, L.v), w);
    const double Hm = mul(fma(HR, rrorl, HL), w);
    const double Vm2 = fma(um, um, mul(vm, vm));
    const double am2 = mul(g.ga1, fma(-0.5, Vm2, Hm));
    const double iam = rsq(am2);
    const double am = mul(am2, iam);
    const double un = fma(um, nx, mul(vm, ny));
    const double eig1 = absd(un);
    const bool sub = dlt(eig1, am);                      // |un| < am
    const double astar = sub ? am : eig1;                // (eig2 + eig3) / 2 = dmax(eig1, am)
    const double sel = sub ? un : copysignd(am, un);
    const double Mstar = mul(sel, iam);                  // (eig2 - eig3) / (2 am)
    const double dE = fma(UR.w, R.ir, -mul(UL.w, L.ir));  // (HR - ER) - (HL - EL)
    const double Etm = fma(g.Etm_c, Vm2, mul(Hm, g.inv_gamma));
    const double dW0 = R.r - L.r;
    const double du = R.u - L.u, dv = R.v - L.v;
    const double dW1 = fma(rm, du, mul(dW0, um));
    const double dW2 = fma(rm, dv, mul(dW0, vm));
    const double dW3 = fma(rm, dE, mul(dW0, Etm));
    const double dun = fma(nx, du, mul(ny, dv));
    const double dp = R.p - L.p;
    const double ae = astar - eig1;
    const double dUroe = fma(Mstar, dun, mul(mul(mul(ae, dp), irm), mul(iam, iam)));
    const double dProe = fma(Mstar, dp, mul(mul(ae, rm), dun));
    const double dUr = mul(dUroe, rm);
    const double h = mul(0.5, area);
    F.x = mul(h, F.x - fma(eig1, dW0, dUr));
    F.y = mul(h, F.y - fma(eig1, dW1, fma(dUr, um, mul(dProe, nx))));
    F.z = mul(h, F.z - fma(eig1, dW2, fma(dUr, vm, mul(dProe, ny))));
    F.w = mul(h, F.w - fma(eig1, dW3, fma(dUr, Hm, mul(dProe, un))));
    if (REC) {
        rec->ruL = ruL; rec->ruR = ruR; rec->HL = HL; rec->HR = HR; rec->irm = irm; rec->rm = rm;
        rec->rrorl = rrorl; rec->w = w; rec->um = um; rec->vm = vm; rec->Hm = Hm; rec->am2 = am2; rec->iam = iam;
        rec->am = am; rec->un = un; rec->sel = sel; rec->Mstar = Mstar; rec->dE = dE; rec->Etm = Etm; rec->ae = ae;
        rec->dUroe = dUroe; rec->dProe = dProe; rec->dUr = dUr; rec->sub = sub;
    }
    return F;
}

__device__ __forceinline__ d4 roe_flux(const Prim& L, const Prim& R, const d4 UL, const d4 UR, double nx, double ny,
                                       double area, const Gas& g) {
    return roe_core<false>(L, R, UL, UR, nx, ny, area, g, nullptr);
}

// LocalLaxFriedrichs, FVMR/src/space/convection/LocalLaxFriedrichs.cpp:4-47
// (the mass flux and the total enthalpy from the conserved states, as in roe_flux)
__device__ __forceinline__ d4 llf_flux(const d4 UL, const d4 UR, const Prim& L, const Prim& R,
                                            double nx, double ny, double length, const Gas& g) {
    const double unL = fma(nx, L.u, mul(ny, L.v)), unR = fma(nx, R.u, mul(ny, R.v));
    const double ruL = fma(nx, UL.y, mul(ny, UL.z)), ruR = fma(nx, UR.y, mul(ny, UR.z));
    const double hl = mul(UL.w + L.p, L.ir);
    const double hr = mul(UR.w + R.p, R.ir);
    const double aL = absd(unL) + sq(mul(mul(g.gamma, L.p), L.ir));
    const double aR = absd(unR) + sq(mul(mul(g.gamma, R.p), R.ir));
    const double lm = dmax(aL, aR);
    const double hlen = mul(0.5, length);
    return mk4(mul(hlen, ruL + ruR - mul(lm, UR.x - UL.x)),
               mul(hlen, fma(ruL, L.u, mul(nx, L.p)) + fma(ruR, R.u, mul(nx, R.p)) - mul(lm, UR.y - UL.y)),
               mul(hlen, fma(ruL, L.v, mul(ny, L.p)) + fma(ruR, R.v, mul(ny, R.p)) - mul(lm, UR.z - UL.z)),
               mul(hlen, fma(ruL, hl, mul(ruR, hr)) - mul(lm, UR.w - UL.w)));
}

// get_UR_wallNonViscous, FVMR/src/space/Flux.cpp:57-71
__device__ __forceinline__ d4 ghost_slip(const d4 UL, const Prim& L, double nx, double ny) {
    const double unL = L.u * nx + L.v * ny;
    const double utL = L.u * ny - L.v * nx;
    const double uxR = -unL * nx + utL * ny;
    const double uyR = -unL * ny - utL * nx;
    return mk4(UL.x, UL.x * uxR, UL.x * uyR, UL.w);
}

// get_UR_farField, FVMR/src/space/Flux.cpp:81-163.  fs = far-field state
// (rho, u, v, p), fa = its sound speed, fson = p / rho^gamma of it.
// Returns false if the boundary state is out of range (the reference exits).
__device__ __forceinline__ bool ghost_farfield(const Prim& e, const double* fs, double fa, double fson, double nx,
                                               double ny, const Gas& g, d4& UR) {
    const double ae = sqrt(g.gamma * e.p * e.ir);
    const double qnf = fs[1] * nx + fs[2] * ny;
    const double qne = e.u * nx + e.v * ny;
    const double rf = qnf - 2.0 * fa * g.inv_ga1;
    const double re = qne + 2.0 * ae * g.inv_ga1;
    const double qn = 0.5 * (re + rf);
    const double as = g.ga1 * (re - rf) * 0.25;
    double r0, u0, v0, p0;
    if (qn <= -as) {
        r0 = fs[0]; u0 = fs[1]; v0 = fs[2]; p0 = fs[3];
    } else if (qn < as) {
        double son, qtx, qty;
        if (qn < 0) {  // subsonic inflow
            son = fson;
            qtx = fs[1] - qnf * nx;
            qty = fs[2] - qnf * ny;
        } else {       // subsonic outflow
            son = e.p / pow(e.r, g.gamma);
            qtx = e.u - qne * nx;
            qty = e.v - qne * ny;
        }
        r0 = pow(as * as / son * g.inv_gamma, g.inv_ga1);
        u0 = qtx + qn * nx;
        v0 = qty + qn * ny;
        p0 = as * as * r0 * g.inv_gamma;
    } else {
        r0 = e.r; u0 = e.u; v0 = e.v; p0 = e.p;
    }
    UR = to_cons(r0, u0, v0, p0, g);
    return !out_of_range(r0, p0);
}

// viscous_flux_kernel, FVMR/src/space/viscous_flux/ViscousFlux.cpp:63-168 with the
// helpers of ViscousFluxGPU.cu:7-124 and Sutherland's law of ViscousFluxGPU.h:26-32;
// the Prandtl number is the reference's constant 0.72.
__device__ __forceinline__ void viscous_flux(d4& F, const d4 U, const d4 gx, const d4 gy,
                                             double nx, double ny, double area, const Gas& g) {
    const double ir = rcp(U.x);
    const double u = U.y * ir, v = U.z * ir, E = U.w * ir;
    const double dudx = ir * (gx.y - u * gx.x);
    const double dvdx = ir * (gx.z - v * gx.x);
    const double dudy = ir * (gy.y - u * gy.x);
    const double dvdy = ir * (gy.z - v * gy.x);
    const double dEdx = ir * (gx.w - E * gx.x);
    const double dEdy = ir * (gy.w - E * gy.x);
    const double T = g.inv_Cv * (E - 0.5 * (u * u + v * v));
    const double dTdx = (dEdx - u * dudx - v * dvdx) * g.inv_Cv;
    const double dTdy = (dEdy - u * dudy - v * dvdy) * g.inv_Cv;
    const double mu = mul(mul(g.C1, mul(T, sq(T))), rcp(T + 110.4));
    const double div = dudx + dvdy;
    const double NMD = -2.0 / 3.0;
    const double txx = mu * fma(NMD, div, 2.0 * dudx);
    const double tyy = mu * fma(NMD, div, 2.0 * dvdy);
    const double txy = mu * (dudy + dvdx);
    const double akmu = g.Cp * (mu * (1.0 / 0.72));
    const double Phix = fma(akmu, dTdx, fma(u, txx, v * txy));
    const double Phiy = fma(akmu, dTdy, fma(u, txy, v * tyy));
    F.y -= (txx * nx + txy * ny) * area;
    F.z -= (txy * nx + tyy * ny) * area;
    F.w -= (Phix * nx + Phiy * ny) * area;
}

}  // namespace dev
}  // namespace fvgb

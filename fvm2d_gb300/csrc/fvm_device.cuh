// fvm_device.cuh -- per-edge / per-triangle / per-vertex arithmetic of the
// fvm2d hot path as device functions templated on the state type R
// (double: plain method; float: FP32 state and fluxes).
//
// Each function restates one reference routine operation by operation, in
// the order the Fortran evaluates it (left-to-right, integer powers as
// multiplications).  The FP64 translation unit is compiled with
// --fmad=false, so with IEEE sqrt and division these reproduce the CPU
// arithmetic bit for bit; pow/erf/exp/atan2/sin/cos are CUDA's and agree
// with glibc to a few ulp.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "fvm_internal.h"

namespace fvm {

__device__ __forceinline__ float msqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double msqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float merf(float x) { return erff(x); }
__device__ __forceinline__ double merf(double x) { return erf(x); }
// FP32: the fast hardware approximations (a few ulp), like the approximate
// division and square root of the FP32 build
__device__ __forceinline__ float mexp(float x) { return __expf(x); }
__device__ __forceinline__ double mexp(double x) { return exp(x); }
__device__ __forceinline__ float mpow(float x, float y) { return __powf(x, y); }
__device__ __forceinline__ double mpow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float mfabs(float x) { return fabsf(x); }
// Division: IEEE in FP64; in FP32 the two-instruction approximation
// (reciprocal and multiply; the divisors here are states, limiter sums and
// sound speeds, far from the range where it loses accuracy)
__device__ __forceinline__ float mdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double mdiv(double a, double b) { return a / b; }
__device__ __forceinline__ double mfabs(double x) { return fabs(x); }

// Fortran dmin1/dmax1 on non-NaN operands
template <typename R>
__device__ __forceinline__ R dmin1(R a, R b) { return b < a ? b : a; }
template <typename R>
__device__ __forceinline__ R dmax1(R a, R b) { return b > a ? b : a; }
template <typename R>
__device__ __forceinline__ R sq(R x) { return x * x; }
template <typename R>
__device__ __forceinline__ R cube(R x) { return (x * x) * x; }
template <typename R>
__device__ __forceinline__ R pow6(R x) { R x3 = (x * x) * x; return x3 * x3; }

template <typename R>
__device__ __forceinline__ R comp(const R4<R> &a, int k) {
  return k == 0 ? a.x : (k == 1 ? a.y : (k == 2 ? a.z : a.w));
}

// ---------------------------------------------------------------- recon.f
template <typename R>
__device__ __forceinline__ R limit_albada(R ul, R ur, R eps) {
  if (ul * ur <= R(0)) return R(0);
  R top = (sq(ul) + eps) * ur + (sq(ur) + eps) * ul;
  R bot = sq(ul) + sq(ur) + R(2) * eps;
  return top / bot;
}
// FP32: the same value without a branch (bot >= 2 eps > 0), so the warp
// does not diverge on the sign test, and with the numerator factored:
// (ul^2 + eps) ur + (ur^2 + eps) ul = (ul + ur)(ul ur + eps), the same value
// in fewer operations, the product reused for the sign test (the flux pass
// 0.206 -> 0.200 ms on 8 x 1024x384).  Its FP32 rounding differs from the
// written order, which the FP64 form keeps.
template <>
__device__ __forceinline__ float limit_albada<float>(float ul, float ur, float eps) {
  const float p = ul * ur;
  const float top = (ul + ur) * (p + eps);
  const float bot = fmaf(ul, ul, fmaf(ur, ur, 2.0f * eps));
  const float r = __fdividef(top, bot);
  return (p <= 0.0f) ? 0.0f : r;
}

// recon.f:4-50 for one variable
template <typename R>
__device__ __forceinline__ void recon1(R p1, R p2, R gx1, R gy1, R gx2, R gy2, R dx, R dy,
                                       int ilimit, R a11, R a12, R a21, R a22, R eps,
                                       R &pl, R &pr) {
  R dqp = p2 - p1;
  if (ilimit == 1) {
    R dql = a21 * (dx * gx1 + dy * gy1) + a22 * dqp;
    R si = limit_albada(dql, dqp, eps);
    pl = p1 + R(0.5) * si;
    R dqr = a21 * (dx * gx2 + dy * gy2) + a22 * dqp;
    R sj = limit_albada(dqr, dqp, eps);
    pr = p2 - R(0.5) * sj;
  } else {
    R dql = dx * gx1 + dy * gy1;
    R si = a11 * dql + a12 * dqp;
    pl = p1 + R(0.5) * si;
    R dqr = dx * gx2 + dy * gy2;
    R sj = a11 * dqr + a12 * dqp;
    pr = p2 - R(0.5) * sj;
  }
}

// ---------------------------------------------------------- roe_flux.f
// Returns false when the Roe-average sound speed squared is not positive
// (roe_flux.f:60-65).
template <typename R>
__device__ __forceinline__ bool roe_flux(R ct, R st, R length, const R pl4[4], const R pr4[4],
                                         R GAMMA, R GAMMA1, R flux[4]) {
  R rl = pl4[0], ul = pl4[1], vl = pl4[2], pl = pl4[3];
  R al2 = mdiv(GAMMA * pl, rl);
  R ql2 = sq(ul) + sq(vl);
  R hl = mdiv(al2, GAMMA1) + R(0.5) * ql2;
  R rr = pr4[0], ur = pr4[1], vr = pr4[2], pr = pr4[3];
  R ar2 = mdiv(GAMMA * pr, rr);
  R qr2 = sq(ur) + sq(vr);
  R hr = mdiv(ar2, GAMMA1) + R(0.5) * qr2;
  R unl = ul * ct + vl * st;
  R Fc0 = rl * unl;
  R Fc1 = pl * ct + rl * ul * unl;
  R Fc2 = pl * st + rl * vl * unl;
  R Fc3 = rl * hl * unl;
  R rl12 = msqrt(rl), rr12 = msqrt(rr);
  R rd = mdiv(R(1), rl12 + rr12);
  R ua = (ul * rl12 + ur * rr12) * rd;
  R va = (vl * rl12 + vr * rr12) * rd;
  R ha = (hl * rl12 + hr * rr12) * rd;
  R qa2 = sq(ua) + sq(va);
  R aa2 = GAMMA1 * (ha - R(0.5) * qa2);
  bool ok = aa2 > R(0);
  R aa = msqrt(aa2);
  R una = ua * ct + va * st;
  R vna = -ua * st + va * ct;
  R l1 = dmin1(una - aa, R(0));
  R l2 = dmin1(una, R(0));
  R l3 = l2;
  R l4 = dmin1(una + aa, R(0));
  R du1 = rr - rl;
  R du2 = rr * ur - rl * ul;
  R du3 = rr * vr - rl * vl;
  R du4 = mdiv(pr - pl, GAMMA1) + R(0.5) * (rr * qr2 - rl * ql2);
  R m1 = mdiv(ct * du2 + st * du3 - una * du1, aa);
  R m2 = mdiv(GAMMA1 * (du4 - ua * du2 - va * du3 + qa2 * du1), sq(aa));
  R a4 = R(0.5) * (m1 + m2);
  R a1 = R(0.5) * (m2 - m1);
  R a3 = du1 - a1 - a4;
  R a2 = mdiv(st * du2 - ct * du3 + vna * du1, aa);
  R a1l1 = a1 * l1, a2l2 = a2 * l2, a3l3 = a3 * l3, a4l4 = a4 * l4;
  R aact = aa * ct, aast = aa * st;
  R Fd0 = a1l1 + a3l3 + a4l4;
  R Fd1 = a1l1 * (ua - aact) + a2l2 * aa * st + a3l3 * ua + a4l4 * (ua + aact);
  R Fd2 = a1l1 * (va - aast) - a2l2 * aa * ct + a3l3 * va + a4l4 * (va + aast);
  R Fd3 = a1l1 * (ha - una * aa) + a2l2 * aa * vna + a3l3 * R(0.5) * qa2 + a4l4 * (ha + una * aa);
  flux[0] = (Fc0 + Fd0) * length;
  flux[1] = (Fc1 + Fd1) * length;
  flux[2] = (Fc2 + Fd2) * length;
  flux[3] = (Fc3 + Fd3) * length;
  return ok;
}

// FP32: the same flux with fewer special-function operations.  The four
// divisions by the Roe-average sound speed (and its square) become products
// with one reciprocal square root, which also gives the sound speed
// (aa = aa2 / sqrt(aa2)); the divisions by gamma - 1 become products with
// its reciprocal, formed once per call (loop-invariant in the edge loops).
// Same operations otherwise; FP32 rounding differs from the written order,
// which the FP64 form keeps.
template <>
__device__ __forceinline__ bool roe_flux<float>(float ct, float st, float length,
                                                const float pl4[4], const float pr4[4],
                                                float GAMMA, float GAMMA1, float flux[4]) {
  const float ig1 = __fdividef(1.0f, GAMMA1);
  const float rl = pl4[0], ul = pl4[1], vl = pl4[2], pl = pl4[3];
  const float al2 = __fdividef(GAMMA * pl, rl);
  const float ql2 = ul * ul + vl * vl;
  const float hl = al2 * ig1 + 0.5f * ql2;
  const float rr = pr4[0], ur = pr4[1], vr = pr4[2], pr = pr4[3];
  const float ar2 = __fdividef(GAMMA * pr, rr);
  const float qr2 = ur * ur + vr * vr;
  const float hr = ar2 * ig1 + 0.5f * qr2;
  const float unl = ul * ct + vl * st;
  const float Fc0 = rl * unl;
  const float Fc1 = pl * ct + rl * ul * unl;
  const float Fc2 = pl * st + rl * vl * unl;
  const float Fc3 = rl * hl * unl;
  const float rl12 = sqrtf(rl), rr12 = sqrtf(rr);
  const float rd = __fdividef(1.0f, rl12 + rr12);
  const float ua = (ul * rl12 + ur * rr12) * rd;
  const float va = (vl * rl12 + vr * rr12) * rd;
  const float ha = (hl * rl12 + hr * rr12) * rd;
  const float qa2 = ua * ua + va * va;
  const float aa2 = GAMMA1 * (ha - 0.5f * qa2);
  const bool ok = aa2 > 0.0f;
  const float iaa = rsqrtf(aa2);
  const float aa = aa2 * iaa;
  const float una = ua * ct + va * st;
  const float vna = -ua * st + va * ct;
  const float l1 = dmin1(una - aa, 0.0f);
  const float l2 = dmin1(una, 0.0f);
  const float l3 = l2;
  const float l4 = dmin1(una + aa, 0.0f);
  const float du1 = rr - rl;
  const float du2 = rr * ur - rl * ul;
  const float du3 = rr * vr - rl * vl;
  const float du4 = (pr - pl) * ig1 + 0.5f * (rr * qr2 - rl * ql2);
  const float m1 = (ct * du2 + st * du3 - una * du1) * iaa;
  const float m2 = GAMMA1 * (du4 - ua * du2 - va * du3 + qa2 * du1) * (iaa * iaa);
  const float a4 = 0.5f * (m1 + m2);
  const float a1 = 0.5f * (m2 - m1);
  const float a3 = du1 - a1 - a4;
  const float a2 = (st * du2 - ct * du3 + vna * du1) * iaa;
  const float a1l1 = a1 * l1, a2l2 = a2 * l2, a3l3 = a3 * l3, a4l4 = a4 * l4;
  const float aact = aa * ct, aast = aa * st;
  const float Fd0 = a1l1 + a3l3 + a4l4;
  const float Fd1 = a1l1 * (ua - aact) + a2l2 * aa * st + a3l3 * ua + a4l4 * (ua + aact);
  const float Fd2 = a1l1 * (va - aast) - a2l2 * aa * ct + a3l3 * va + a4l4 * (va + aast);
  const float Fd3 = a1l1 * (ha - una * aa) + a2l2 * aa * vna + a3l3 * 0.5f * qa2 +
                    a4l4 * (ha + una * aa);
  flux[0] = (Fc0 + Fd0) * length;
  flux[1] = (Fc1 + Fd1) * length;
  flux[2] = (Fc2 + Fd2) * length;
  flux[3] = (Fc3 + Fd3) * length;
  return ok;
}

// --------------------------------------------------------- kfvs_flux.f
template <typename R>
__device__ __forceinline__ void kfvs_flux(R ct, R st, R length, const R pl4[4], const R pr4[4],
                                          R GAMMA1, R PI, R flux[4]) {
  R rl = pl4[0], ul = pl4[1], vl = pl4[2], pl = pl4[3];
  R ql2 = sq(ul) + sq(vl);
  R el = mdiv(pl, GAMMA1) + R(0.5) * rl * ql2;
  R rr = pr4[0], ur = pr4[1], vr = pr4[2], pr = pr4[3];
  R qr2 = sq(ur) + sq(vr);
  R er = mdiv(pr, GAMMA1) + R(0.5) * rr * qr2;
  R unl = ul * ct + vl * st;
  R unr = ur * ct + vr * st;
  R vnl = -ul * st + vl * ct;
  R vnr = -ur * st + vr * ct;
  R betal = mdiv(R(0.5) * rl, pl);
  R sl = unl * msqrt(betal);
  R Al = R(0.5) * (R(1) + merf(sl));
  R Bl = mdiv(R(0.5) * mexp(-sq(sl)), msqrt(PI * betal));
  R Fp0 = rl * (unl * Al + Bl);
  R Fp1 = (pl + rl * sq(unl)) * Al + rl * unl * Bl;
  R Fp2 = rl * (unl * Al + Bl) * vnl;
  R Fp3 = (el + pl) * unl * Al + (el + R(0.5) * pl) * Bl;
  R betar = mdiv(R(0.5) * rr, pr);
  R sr = unr * msqrt(betar);
  R Ar = R(0.5) * (R(1) - merf(sr));
  R Br = mdiv(R(0.5) * mexp(-sq(sr)), msqrt(PI * betar));
  R Fm0 = rr * (unr * Ar - Br);
  R Fm1 = (pr + rr * sq(unr)) * Ar - rr * unr * Br;
  R Fm2 = rr * (unr * Ar - Br) * vnr;
  R Fm3 = (er + pr) * unr * Ar - (er + R(0.5) * pr) * Br;
  R Ff0 = Fp0 + Fm0, Ff1 = Fp1 + Fm1, Ff2 = Fp2 + Fm2, Ff3 = Fp3 + Fm3;
  flux[0] = Ff0 * length;
  flux[1] = (ct * Ff1 - st * Ff2) * length;
  flux[2] = (st * Ff1 + ct * Ff2) * length;
  flux[3] = Ff3 * length;
}

// --------------------------------------------------------- hllc_flux.f
// rotate_back = 0 reproduces hllc_flux.f:149-154 (normal/tangential momentum
// flux added as x/y); 1 rotates it back to x/y.
template <typename R>
__device__ __forceinline__ void hllc_flux(R ct, R st, R length, const R pl4[4], const R pr4[4],
                                          R gamma, R GAMMA1, int rotate_back, R flux[4]) {
  R rl = pl4[0];
  R ul = pl4[1] * ct + pl4[2] * st;
  R vl = -pl4[1] * st + pl4[2] * ct;
  R pl = pl4[3];
  R al = msqrt(mdiv(gamma * pl, rl));
  R El = mdiv(pl, GAMMA1) + R(0.5) * rl * (sq(ul) + sq(vl));
  R rr = pr4[0];
  R ur = pr4[1] * ct + pr4[2] * st;
  R vr = -pr4[1] * st + pr4[2] * ct;
  R pr = pr4[3];
  R ar = msqrt(mdiv(gamma * pr, rr));
  R Er = mdiv(pr, GAMMA1) + R(0.5) * rr * (sq(ur) + sq(vr));
  R rbar = R(0.5) * (rl + rr);
  R abar = R(0.5) * (al + ar);
  R Ppv = R(0.5) * (pl + pr - (ur - ul) * rbar * abar);
  R Upv = R(0.5) * (ul + ur - mdiv(pr - pl, rbar * abar));
  R prmax, prmin;
  if (pl > pr) {
    prmax = pl;
    prmin = pr;
  } else {
    prmax = pr;
    prmin = pl;
  }
  R Q = mdiv(prmax, prmin);
  R pstar, ustar;
  if (Q < R(2) && prmin < Ppv && Ppv < prmax) {
    pstar = Ppv;
    ustar = Upv;
  } else if (Ppv < prmin) {
    R z = R(0.5) * (gamma - R(1)) / gamma;
    R a1 = al + ar - R(0.5) * (gamma - R(1)) * (ur - ul);
    R a2 = al / mpow(pl, z) + ar / mpow(pr, z);
    pstar = mpow(a1 / a2, R(1) / z);
    R Plr = mpow(pl / pr, z);
    R b1 = Plr * ul / al + ur / ar + R(2) * (Plr - R(1)) / (gamma - R(1));
    R b2 = Plr / al + R(1) / ar;
    ustar = b1 / b2;
  } else {
    R po = dmax1(R(0), Ppv);
    R Ml = R(2) / (gamma + R(1)) / rl;
    R Nl = (gamma - R(1)) * pl / (gamma + R(1));
    R gl = msqrt(Ml / (po + Nl));
    R Mr = R(2) / (gamma + R(1)) / rr;
    R Nr = (gamma - R(1)) * pr / (gamma + R(1));
    R gr = msqrt(Mr / (po + Nr));
    R a1 = gl * pl + gr * pr - (ur - ul);
    R a2 = gl + gr;
    pstar = a1 / a2;
    ustar = R(0.5) * (ul + ur + (pstar - pr) * gr - (pstar - pl) * gl);
  }
  R ql = (pstar <= pl) ? R(1) : msqrt(R(1) + mdiv(R(0.5) * (gamma + R(1)) * (mdiv(pstar, pl) - R(1)), gamma));
  R qr = (pstar <= pr) ? R(1) : msqrt(R(1) + mdiv(R(0.5) * (gamma + R(1)) * (mdiv(pstar, pr) - R(1)), gamma));
  R Sl = ul - al * ql;
  R Ss = ustar;
  R Sr = ur + ar * qr;
  // hllc_flux.f:105-147: F(U_L) if 0 <= Sl; F_L + Sl (U*_L - U_L) if
  // Sl <= 0 <= Ss; F_R + Sr (U*_R - U_R) if Ss <= 0 <= Sr; else F(U_R).
  // The side is chosen first and its terms computed once, with the same
  // operations as the branch it stands for, so a warp whose edges fall in
  // different cases does not run both sides.
  const bool c1 = R(0) <= Sl;
  const bool c2 = !c1 && Sl <= R(0) && R(0) <= Ss;
  const bool c3 = !c1 && !c2 && Ss <= R(0) && R(0) <= Sr;
  const bool left = c1 || c2, star = c2 || c3;
  const R rk = left ? rl : rr, uk = left ? ul : ur, vk = left ? vl : vr;
  const R pk = left ? pl : pr, Ek = left ? El : Er, Sk = left ? Sl : Sr;
  R f0 = rk * uk, f1 = pk + rk * sq(uk), f2 = rk * uk * vk, f3 = (Ek + pk) * uk;
  if (star) {
    R fact = mdiv(rk * (Sk - uk), Sk - Ss);
    R du0 = fact - rk;
    R du1 = fact * Ss - rk * uk;
    R du2 = fact * vk - rk * vk;
    R t1 = mdiv(Ek, rk) + (Ss - uk) * (Ss + mdiv(mdiv(pk, rk), Sk - uk));
    R du3 = fact * t1 - Ek;
    f0 = f0 + Sk * du0;
    f1 = f1 + Sk * du1;
    f2 = f2 + Sk * du2;
    f3 = f3 + Sk * du3;
  }
  if (rotate_back) {
    R fn = f1, ft = f2;
    f1 = ct * fn - st * ft;
    f2 = st * fn + ct * ft;
  }
  flux[0] = f0 * length;
  flux[1] = f1 * length;
  flux[2] = f2 * length;
  flux[3] = f3 * length;
}

// ------------------------------------------------------ farfield_flux.f
// Contributions flux1 (to n1) and flux2 (to n2) of one farfield edge.
template <typename R>
__device__ __forceinline__ void farfield_flux(const MeshConst &mc, double cl, double2 x1,
                                              double2 x2, const R4<R> &P1, const R4<R> &P2,
                                              R flux1[4], R flux2[4]) {
  const R GAMMA = MCR(R, gamma), gamma1 = MCR(R, gamma1);
  R uinf, vinf, q2inf, pinf, rinf;
  if (mc.mach_inf < 1.0 && mc.vortex == 1) {
    // point-vortex correction (farfield_flux.f:28-44), evaluated in FP64
    double dx = 0.5 * (x1.x + x2.x) - mc.xref;
    double dy = 0.5 * (x1.y + x2.y) - mc.yref;
    double dref = sqrt(dx * dx + dy * dy);
    double theta = atan2(dy, dx);
    double circ = 0.5 * mc.q_inf * cl;
    double fact1 = circ * sqrt(1.0 - mc.mach_inf * mc.mach_inf);
    double fact2 = 2.0 * mc.pi * dref;
    double s3 = mc.mach_inf * sin(theta - mc.aoa);
    double fact3 = 1.0 - s3 * s3;
    double fact = fact1 / (fact2 * fact3);
    double ui = mc.u_inf + fact * sin(theta);
    double vi = mc.v_inf - fact * cos(theta);
    double q2 = ui * ui + vi * vi;
    double fact4 = 1.0 + 0.5 * mc.gamma1 * (mc.q_inf * mc.q_inf - q2) / (mc.a_inf * mc.a_inf);
    double ri = mc.r_inf * pow(fact4, 1.0 / mc.gamma1);
    double pi_ = mc.p_inf * pow(ri / mc.r_inf, mc.gamma);
    uinf = R(ui);
    vinf = R(vi);
    q2inf = R(q2);
    rinf = R(ri);
    pinf = R(pi_);
  } else {
    uinf = MCR(R, u_inf);
    vinf = MCR(R, v_inf);
    q2inf = sq(uinf) + sq(vinf);
    pinf = MCR(R, p_inf);
    rinf = MCR(R, r_inf);
  }
  R Uout[4] = {rinf, rinf * uinf, rinf * vinf, pinf / gamma1 + R(0.5) * rinf * q2inf};
  R ra = R(0.5) * (P1.x + P2.x);
  R ua = R(0.5) * (P1.y + P2.y);
  R va = R(0.5) * (P1.z + P2.z);
  R pa = R(0.5) * (P1.w + P2.w);
  R qa2 = sq(ua) + sq(va);
  R aa2 = GAMMA * pa / ra;
  R aa = msqrt(GAMMA * pa / ra);
  R ha = aa2 / gamma1 + R(0.5) * qa2;
  R Uin1[4] = {P1.x, P1.x * P1.y, P1.x * P1.z,
               P1.w / gamma1 + R(0.5) * P1.x * (sq(P1.y) + sq(P1.z))};
  R Uin2[4] = {P2.x, P2.x * P2.y, P2.x * P2.z,
               P2.w / gamma1 + R(0.5) * P2.x * (sq(P2.y) + sq(P2.z))};
  R ct = R(x2.y - x1.y);
  R st = -R(x2.x - x1.x);
  R lent = msqrt(sq(ct) + sq(st));
  ct = ct / lent;
  st = st / lent;
  R una = ua * ct + va * st;
  R vna = -ua * st + va * ct;
  R l1 = una, l2 = una, l3 = una + aa, l4 = una - aa;
  R lp1 = dmax1(l1, R(0)), lp2 = lp1, lp3 = dmax1(l3, R(0)), lp4 = dmax1(l4, R(0));
  R lm1 = l1 - lp1, lm2 = l2 - lp2, lm3 = l3 - lp3, lm4 = l4 - lp4;
  R T[4][4], S[4][4];
  R t1 = R(0.5) * ra / aa;
  R m2 = qa2 / aa2;
  T[0][0] = R(1);  T[1][0] = ua;       T[2][0] = va;       T[3][0] = R(0.5) * qa2;
  T[0][1] = R(0);  T[1][1] = ra * st;  T[2][1] = -ra * ct; T[3][1] = -ra * vna;
  T[0][2] = t1;    T[1][2] = t1 * (ua + aa * ct);
  T[2][2] = t1 * (va + aa * st);       T[3][2] = t1 * (ha + aa * una);
  T[0][3] = t1;    T[1][3] = t1 * (ua - aa * ct);
  T[2][3] = t1 * (va - aa * st);       T[3][3] = t1 * (ha - aa * una);
  t1 = R(0.5) * gamma1 * m2 * aa / ra;
  R t2 = una / ra, t3 = gamma1 * ua / aa, t4 = gamma1 * va / aa, t5 = gamma1 / (ra * aa);
  S[0][0] = R(1) - R(0.5) * gamma1 * m2;
  S[1][0] = vna / ra;
  S[2][0] = t1 - t2;
  S[3][0] = t1 + t2;
  S[0][1] = t3 / aa;
  S[1][1] = st / ra;
  S[2][1] = (ct - t3) / ra;
  S[3][1] = -(ct + t3) / ra;
  S[0][2] = t4 / aa;
  S[1][2] = -ct / ra;
  S[2][2] = (st - t4) / ra;
  S[3][2] = -(st + t4) / ra;
  S[0][3] = -gamma1 / aa2;
  S[1][3] = R(0);
  S[2][3] = t5;
  S[3][3] = t5;
  const R lp[4] = {lp1, lp2, lp3, lp4};
  const R lm[4] = {lm1, lm2, lm3, lm4};
#pragma unroll
  for (int i = 0; i < 4; i++) {
    R jacp[4], jacm[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      R a = R(0), b = R(0);
#pragma unroll
      for (int k = 0; k < 4; k++) {
        a = a + (lp[k] * T[i][k]) * S[k][j];
        b = b + (lm[k] * T[i][k]) * S[k][j];
      }
      jacp[j] = a;
      jacm[j] = b;
    }
    R f1 = R(0), f2 = R(0);
#pragma unroll
    for (int j = 0; j < 4; j++) {
      f1 = f1 + jacp[j] * Uin1[j] + jacm[j] * Uout[j];
      f2 = f2 + jacp[j] * Uin2[j] + jacm[j] * Uout[j];
    }
    flux1[i] = R(0.5) * lent * f1;
    flux2[i] = R(0.5) * lent * f2;
  }
}

// ------------------------------------------------------------ viscosity.f
template <typename R>
__device__ __forceinline__ R sutherland_viscosity(const MeshConst &mc, R density, R pressure) {
  R temp = mdiv(mdiv(pressure, density), MCR(R, gas_const));
  R num = MCR(R, t_inf) + MCR(R, sconst);
  R den = temp + MCR(R, sconst);
  return mdiv(mpow(mdiv(temp, MCR(R, t_inf)), R(1.5)) * mdiv(num, den), MCR(R, rey));
}

template <typename R>
__device__ __forceinline__ R mu_turb(const MeshConst &mc, R mu_lam, R density, R nu_tilde) {
  R chi = mdiv(nu_tilde * density, mu_lam);
  R chi3 = cube(chi);
  R fv1 = mdiv(chi3, chi3 + MCR(R, cv11));
  return density * nu_tilde * fv1;
}

// ------------------------------------------------------------ time_step.f
template <typename R>
__device__ __forceinline__ R time_step(const MeshConst &mc, const R4<R> &P, R mu, R drmin) {
  R q = msqrt(sq(P.y) + sq(P.z));
  R a = msqrt(mdiv(MCR(R, gamma) * P.w, P.x));
  R dr = drmin;
  if (mc.iflow != 1) {
    R dtv = mdiv(R(2) * MCR(R, gamma) * mu, P.x * MCR(R, prandtl));
    return mdiv(MCR(R, cfl) * sq(dr), dr * (q + a) + dtv);
  }
  return mdiv(MCR(R, cfl) * dr, q + a);
}

// ---------------------------------------------------- update.f, convert.f
template <typename R>
__device__ __forceinline__ void prim2con(const R4<R> &P, R gamma1, R c[4]) {
  c[0] = P.x;
  c[1] = P.x * P.y;
  c[2] = P.x * P.z;
  c[3] = mdiv(P.w, gamma1) + R(0.5) * P.x * (sq(P.y) + sq(P.z));
}

template <typename R>
__device__ __forceinline__ R4<R> rk_update(const MeshConst &mc, int irk, const R4<R> &Po,
                                           const R4<R> &Pc, R dt, R cvarea,
                                           const R res[4], bool noslip) {
  const R gamma1 = MCR(R, gamma1);
  R a = MCR(R, airk[irk - 1]), b = MCR(R, birk[irk - 1]);
  R c0[4], c1[4], cn[4];
  prim2con(Po, gamma1, c0);
  prim2con(Pc, gamma1, c1);
  R f = mdiv(dt, cvarea);
#pragma unroll
  for (int j = 0; j < 4; j++) cn[j] = a * c0[j] + b * (c1[j] - f * res[j]);
  if (noslip) {
    cn[1] = R(0);
    cn[2] = R(0);
  }
  R4<R> out;
  out.x = cn[0];
  out.y = mdiv(cn[1], cn[0]);
  out.z = mdiv(cn[2], cn[0]);
  out.w = gamma1 * (cn[3] - mdiv(R(0.5) * (sq(cn[1]) + sq(cn[2])), cn[0]));
  return out;
}

// --------------------------------------------------------- sa_model.f
template <typename R>
__device__ __forceinline__ R update_sa(const MeshConst &mc, R nut, R rho, R mul, R wd,
                                       R dt, R cvarea, R divf, R omega) {
  R chi = mdiv(nut * rho, mul);
  R chi3 = cube(chi);
  R fv1 = mdiv(chi3, chi3 + MCR(R, cv11));
  R fv2 = mdiv(R(1), cube(R(1) + mdiv(chi, MCR(R, cv2))));
  R r = mdiv(mdiv(nut, wd), wd * MCR(R, kolm2));
  R fv3 = mdiv((R(1) + chi * fv1) * (R(1) - fv2), dmax1(chi, R(0.001)));
  R S = fv3 * mfabs(omega) + r * fv2;
  r = mdiv(r, S);
  r = dmin1(r, R(2));
  R g = r + MCR(R, cw2) * (pow6(r) - r);
  R fw = g * mpow(mdiv(MCR(R, cw31), pow6(g) + MCR(R, cw32)), mdiv(R(1), R(6)));
  R source = MCR(R, cb1) * S * nut;
  R fact = R(1) + MCR(R, cw1) * fw * mdiv(nut, wd) * mdiv(dt, wd);
  return mdiv(nut - mdiv(dt, cvarea) * divf + dt * source, fact);
}

}  // namespace fvm

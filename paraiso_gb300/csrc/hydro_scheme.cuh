// hydro_scheme.cuh -- the examples/Hydro finite-volume scheme as device
// functions, one C operation per OM Arith node in the builder's order, so a
// translation unit compiled without multiply-add contraction reproduces the
// generated code's rounding exactly.
//
// Reference: examples/Hydro/Hydro.hs:37-127 (primitive <-> conserved algebra,
// fluxes, sound speed), examples/Hydro/HydroMain.hs:134-276 (proceed,
// proceedSingle, addFlux, interpolate, hllc).  std::max / std::min follow
// the generated C++ (Language/Paraiso/Generator/PlanTrans.hs:692-693).
#pragma once

#include <cuda_runtime.h>

namespace om {
namespace hs {

template <class R> __device__ __forceinline__ R omax(R a, R b) { return (a < b) ? b : a; }
template <class R> __device__ __forceinline__ R omin(R a, R b) { return (b < a) ? b : a; }

template <class R> struct Prim { R rho, v0, v1, p; };
// 16-byte aligned: a record in shared memory moves as one 128-bit access
// (FP32) or two (FP64), free of bank conflicts
template <class R> struct alignas(16) Flux { R fd, fm0, fm1, fe; };

// kineticEnergy x = 0.5 * contract (\i -> velocity x !i * momentum x !i)
template <class R> __device__ __forceinline__ R kinetic(R v0, R v1, R m0, R m1) {
  return R(0.5) * ((R(0) + v0 * m0) + v1 * m1);
}

// energy of a primitive record: Ek + 1/(gamma-1) * p
template <class R> __device__ __forceinline__ R energy_prim(R g, R rho, R v0, R v1, R p) {
  const R m0 = rho * v0, m1 = rho * v1;
  return kinetic(v0, v1, m0, m1) + (R(1) / (g - R(1))) * p;
}

// fluxes along axis AX of a primitive record
template <int AX, class R>
__device__ __forceinline__ Flux<R> flux_prim(R g, R rho, R v0, R v1, R p) {
  const R m0 = rho * v0, m1 = rho * v1;
  const R e = kinetic(v0, v1, m0, m1) + (R(1) / (g - R(1))) * p;
  const R h = e + p;
  const R va = AX == 0 ? v0 : v1;
  Flux<R> f;
  f.fd = AX == 0 ? m0 : m1;
  f.fm0 = m0 * va + p * (AX == 0 ? R(1) : R(0));
  f.fm1 = m1 * va + p * (AX == 1 ? R(1) : R(0));
  f.fe = h * va;
  return f;
}

// fluxes along AX of a conserved record (velocity m/rho, p = (g-1)(E-Ek))
template <int AX, class R>
__device__ __forceinline__ Flux<R> flux_cons(R g, R rho, R m0, R m1, R e) {
  const R v0 = m0 / rho, v1 = m1 / rho;
  const R p = (g - R(1)) * (e - kinetic(v0, v1, m0, m1));
  const R h = e + p;
  const R va = AX == 0 ? v0 : v1;
  Flux<R> f;
  f.fd = AX == 0 ? m0 : m1;
  f.fm0 = m0 * va + p * (AX == 0 ? R(1) : R(0));
  f.fm1 = m1 * va + p * (AX == 1 ? R(1) : R(0));
  f.fe = h * va;
  return f;
}

// soundSpeed' dens pres = sqrt (kGamma * pres / dens)
template <class R> __device__ __forceinline__ R sound(R g, R rho, R p) {
  return sqrt((g * p) / rho);
}

// hllcQ sp p, condition as written in HydroMain.hs
template <class R> __device__ __forceinline__ R hllc_q(R g, R sp, R p) {
  const R t = sqrt(R(1) + (g + R(1)) / (R(2) * g) * (sp / p - R(1)));
  return (p <= sp) ? R(1) : t;
}

template <int AX, class R>
__device__ __forceinline__ Flux<R> star_flux(R g, R sstar, R shock, R rho, R v0, R v1,
                                             R p) {
  const R speed = AX == 0 ? v0 : v1;
  const R dens = rho * (shock - speed) / (shock - sstar);
  const R mome0 = dens * (AX == 0 ? sstar : v0);
  const R mome1 = dens * (AX == 1 ? sstar : v1);
  const R e = energy_prim(g, rho, v0, v1, p);
  const R enrg = dens * (e / rho + (sstar - speed) * (sstar + p / rho / (shock - speed)));
  return flux_cons<AX>(g, dens, mome0, mome1, enrg);
}

// The wall record's fluxes of hllc i left right (HydroMain.hs:237-268).
// cl, cr: sound speeds of the two states.
template <int AX, class R>
__device__ __forceinline__ Flux<R> hllc(R g, const Prim<R> &L, R cl, const Prim<R> &Rt,
                                        R cr) {
  const R densMid = (L.rho + Rt.rho) / R(2);
  const R soundMid = (cl + cr) / R(2);
  const R uL = AX == 0 ? L.v0 : L.v1;
  const R uR = AX == 0 ? Rt.v0 : Rt.v1;
  const R psraw = (L.p + Rt.p) / R(2) - densMid * soundMid * (uR - uL);
  const R presStar = omax(R(0), psraw);
  const R qL = hllc_q(g, presStar, L.p), qR = hllc_q(g, presStar, Rt.p);
  const R shockLeft = uL - cl * qL;
  const R shockRight = uR + cr * qR;
  const R shockStar = (Rt.p - L.p + L.rho * uL * (shockLeft - uL) -
                       Rt.rho * uR * (shockRight - uR)) /
                      (L.rho * (shockLeft - uL) - Rt.rho * (shockRight - uR));
  // select (0 < SL) L (select (0 < S*) L* (select (0 < SR) R* R)): pick the
  // side first, then evaluate one physical or star flux on it, so a warp
  // whose faces take different cases does not run both star states
  const bool posL = R(0) < shockLeft, posS = R(0) < shockStar, posR = R(0) < shockRight;
  const bool useL = posL || posS;
  const bool star = useL ? !posL : posR;
  const R xr = useL ? L.rho : Rt.rho, x0 = useL ? L.v0 : Rt.v0, x1 = useL ? L.v1 : Rt.v1,
          xp = useL ? L.p : Rt.p;
  const R shock = useL ? shockLeft : shockRight;
  const Flux<R> fs = star_flux<AX>(g, shockStar, shock, xr, x0, x1, xp);
  const Flux<R> fp = flux_prim<AX>(g, xr, x0, x1, xp);
  return star ? fs : fp;
}

template <class R> __device__ __forceinline__ R absmaller(R a, R b) {
  return (a * b <= R(0)) ? R(0) : ((fabs(a) < fabs(b)) ? a : b);
}

// interpolateSingle 2 (minmod MUSCL): face value left (l) and right (r)
template <class R>
__device__ __forceinline__ void muscl(R x0, R x1, R x2, R x3, R &l, R &r) {
  const R d01 = x1 - x0, d12 = x2 - x1, d23 = x3 - x2;
  const R d1 = absmaller(d01, d12);
  const R d2 = absmaller(d12, d23);
  l = x1 + d1 / R(2);
  r = x2 - d2 / R(2);
}

// Conservative update of base state b by the axis-1 walls, then the axis-0
// walls (foldl1 (.) over the axes applies axis 1 first), then
// bindPrimitive (max 1e-2 rho) v (max 1e-2 p).  cons (optional): the new
// conserved state (rho, m0, m1, E) before the primitive recovery.
template <class R>
__device__ __forceinline__ Prim<R> update(R g, const Prim<R> &b, R dtdx0, R dtdx1,
                                          const Flux<R> &l0, const Flux<R> &r0,
                                          const Flux<R> &l1, const Flux<R> &r1,
                                          R *cons = nullptr) {
  const R m0 = b.rho * b.v0, m1 = b.rho * b.v1;
  const R e = kinetic(b.v0, b.v1, m0, m1) + (R(1) / (g - R(1))) * b.p;
  const R d1 = b.rho + dtdx1 * (l1.fd - r1.fd);
  const R a0 = m0 + dtdx1 * (l1.fm0 - r1.fm0);
  const R a1 = m1 + dtdx1 * (l1.fm1 - r1.fm1);
  const R e1 = e + dtdx1 * (l1.fe - r1.fe);
  const R d2 = d1 + dtdx0 * (l0.fd - r0.fd);
  const R b0 = a0 + dtdx0 * (l0.fm0 - r0.fm0);
  const R b1 = a1 + dtdx0 * (l0.fm1 - r0.fm1);
  const R e2 = e1 + dtdx0 * (l0.fe - r0.fe);
  if (cons) {
    cons[0] = d2;
    cons[1] = b0;
    cons[2] = b1;
    cons[3] = e2;
  }
  const R v0 = b0 / d2, v1 = b1 / d2;
  const R pn = (g - R(1)) * (e2 - kinetic(v0, v1, b0, b1));
  Prim<R> q;
  q.rho = omax(R(1e-2), d2);
  q.v0 = v0;
  q.v1 = v1;
  q.p = omax(R(1e-2), pn);
  return q;
}

// per-cell CFL timescale min_i dR_i / (c + |v_i|)   (HydroMain.hs:150-153)
template <class R>
__device__ __forceinline__ R timescale(R g, R dR0, R dR1, R rho, R v0, R v1, R p) {
  const R c = sound(g, rho, p);
  const R t0 = dR0 / (c + fabs(v0));
  const R t1 = dR1 / (c + fabs(v1));
  return omin(t0, t1);
}

}  // namespace hs

// ---------------------------------------------------------------------------
// The production FP32 algebra of the same scheme.  The exact build above
// repeats the generated operation order (bit-exact with the oracle); this
// one is equal to it up to rounding and is held to the FP64 oracle by
// tolerance:
//  * 1/(gamma-1) and (gamma+1)/(2 gamma) are formed once per launch;
//  * a reciprocal is shared where the generated code divides twice by the
//    same value;
//  * the star state's flux is taken in closed form: its recovered velocity
//    is S* along the wall and the side's own velocity across it (m/rho of
//    the star record), so no division recovers it, and its pressure is the
//    equation of state of the star record, as bindConserved gives it
//    (HydroMain.hs:272-282, Hydro.hs:110-118);
//  * the physical and star fluxes share one flux formula applied to the
//    selected state (density, normal velocity, energy, pressure).
// The timescale and the MUSCL reconstruction stay those of hs:: (the reverse
// sweep recomputes both and must find the forward's values).
// ---------------------------------------------------------------------------
namespace hf {

using hs::Flux;
using hs::Prim;
using hs::omax;

template <class R> struct Consts {
  R g, gm1, gm1inv, qc;  // gamma, gamma-1, 1/(gamma-1), (gamma+1)/(2 gamma)
};

template <class R> __device__ __forceinline__ Consts<R> consts(R g) {
  Consts<R> k;
  k.g = g;
  k.gm1 = g - R(1);
  k.gm1inv = R(1) / k.gm1;
  k.qc = (g + R(1)) / (R(2) * g);
  return k;
}

// hllc i left right (HydroMain.hs:237-268), hllcQ as written (:270-271)
template <int AX, class R>
__device__ __forceinline__ Flux<R> hllc(const Consts<R> &k, const Prim<R> &L, R cl,
                                        const Prim<R> &Rt, R cr) {
  const R uL = AX == 0 ? L.v0 : L.v1;
  const R uR = AX == 0 ? Rt.v0 : Rt.v1;
  const R densMid = R(0.5) * (L.rho + Rt.rho);
  const R soundMid = R(0.5) * (cl + cr);
  const R presStar = omax(R(0), R(0.5) * (L.p + Rt.p) - densMid * soundMid * (uR - uL));
  const R tL = sqrt(R(1) + k.qc * (presStar / L.p - R(1)));
  const R tR = sqrt(R(1) + k.qc * (presStar / Rt.p - R(1)));
  const R qL = (L.p <= presStar) ? R(1) : tL;
  const R qR = (Rt.p <= presStar) ? R(1) : tR;
  const R shockLeft = uL - cl * qL;
  const R shockRight = uR + cr * qR;
  const R aL = L.rho * (shockLeft - uL), aR = Rt.rho * (shockRight - uR);
  const R shockStar = (Rt.p - L.p + aL * uL - aR * uR) / (aL - aR);
  const bool posL = R(0) < shockLeft, posS = R(0) < shockStar, posR = R(0) < shockRight;
  const bool useL = posL || posS;
  const bool star = useL ? !posL : posR;
  const R r = useL ? L.rho : Rt.rho, p = useL ? L.p : Rt.p;
  const R x0 = useL ? L.v0 : Rt.v0, x1 = useL ? L.v1 : Rt.v1;
  const R un = AX == 0 ? x0 : x1, ut = AX == 0 ? x1 : x0;
  const R shock = useL ? shockLeft : shockRight;
  const R E = R(0.5) * r * (un * un + ut * ut) + k.gm1inv * p;
  // starState: density r (S-u)/(S-S*), energy density ((E/r) + (S*-u)(S* +
  // p/(r (S-u)))), velocity (S*, ut)
  const R su = shock - un;
  const R rr = R(1) / r;
  const R dens = r * su / (shock - shockStar);
  const R enrg = dens * (E * rr + (shockStar - un) * (shockStar + p * rr / su));
  const R pst = k.gm1 * (enrg - R(0.5) * dens * (shockStar * shockStar + ut * ut));
  const R fr = star ? dens : r, fu = star ? shockStar : un;
  const R fE = star ? enrg : E, fp = star ? pst : p;
  const R mn = fr * fu;
  Flux<R> f;
  f.fd = mn;
  const R fn = mn * fu + fp, ft = fr * ut * fu;
  f.fm0 = AX == 0 ? fn : ft;
  f.fm1 = AX == 0 ? ft : fn;
  f.fe = (fE + fp) * fu;
  return f;
}

// the conservative update of hs::update (axis 1 walls, then axis 0 walls,
// then bindPrimitive with the 1e-2 floors), one reciprocal of the density
template <class R>
__device__ __forceinline__ Prim<R> update(const Consts<R> &k, const Prim<R> &b, R dtdx0, R dtdx1,
                                          const Flux<R> &l0, const Flux<R> &r0,
                                          const Flux<R> &l1, const Flux<R> &r1,
                                          R *cons = nullptr) {
  const R m0 = b.rho * b.v0, m1 = b.rho * b.v1;
  const R e = R(0.5) * (b.v0 * m0 + b.v1 * m1) + k.gm1inv * b.p;
  const R d1 = b.rho + dtdx1 * (l1.fd - r1.fd);
  const R a0 = m0 + dtdx1 * (l1.fm0 - r1.fm0);
  const R a1 = m1 + dtdx1 * (l1.fm1 - r1.fm1);
  const R e1 = e + dtdx1 * (l1.fe - r1.fe);
  const R d2 = d1 + dtdx0 * (l0.fd - r0.fd);
  const R b0 = a0 + dtdx0 * (l0.fm0 - r0.fm0);
  const R b1 = a1 + dtdx0 * (l0.fm1 - r0.fm1);
  const R e2 = e1 + dtdx0 * (l0.fe - r0.fe);
  if (cons) {
    cons[0] = d2;
    cons[1] = b0;
    cons[2] = b1;
    cons[3] = e2;
  }
  const R rd = R(1) / d2;
  const R v0 = b0 * rd, v1 = b1 * rd;
  const R pn = k.gm1 * (e2 - R(0.5) * (v0 * b0 + v1 * b1));
  Prim<R> q;
  q.rho = omax(R(1e-2), d2);
  q.v0 = v0;
  q.v1 = v1;
  q.p = omax(R(1e-2), pn);
  return q;
}

}  // namespace hf
}  // namespace om
